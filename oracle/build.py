"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/liboracle.so``: the C restatement ``oracle/cvx_oracle.c`` (host code, built on
  whichever machine runs the tests).  ``-ffp-contract=off`` keeps every ``a*b+c`` a separate
  multiply and add, which is what the reference CPU build does on x86-64; without it gcc fuses
  them on aarch64 and the restatement would no longer reproduce the reference bit for bit.
* ``oracle/_ref/``: the reference's own code, built by ``oracle/build_ref.sh``.  Where the reference
  tree is present (the development machine) the script stages the reference CPU voxelizer's source
  files into ``oracle/_ref/src`` and builds everything from the tree; elsewhere (the GPU machine, which
  receives ``oracle/_ref`` with the repository snapshot) it builds ``libref_cpu.so`` from the staged
  sources (and the reference's command-line program, relinked against libcvx.so), and the prebuilt
  device-code files are used as they are.  The reference tree is found
  through the ``CVX_REFERENCE_ROOT`` environment variable, else as a checkout named ``reference``
  next to this repository.
* ``oracle/_build/libref_gpu_runner.so``: ``oracle/ref_gpu_runner.cu``, the driver-API loader
  that runs the reference's kernels from ``oracle/_ref/*.cubin`` (only where nvcc exists).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REFERENCE_ROOT = os.environ.get("CVX_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                      "reference")


def _run(cmd):
    subprocess.run(cmd, check=True)


def foreign_binary(path: str) -> bool:
    """True if `path` is an ELF file built for another CPU architecture than this machine's."""
    import platform
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if len(head) < 20 or head[:4] != b"\x7fELF" or want is None:
        return False
    return int.from_bytes(head[18:20], "little") != want


def _stale(out: str, src: str) -> bool:
    return not os.path.exists(out) or foreign_binary(out) or os.path.getmtime(out) < os.path.getmtime(src)


def build_oracle() -> str:
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "liboracle.so")
    src = os.path.join(HERE, "cvx_oracle.c")
    if _stale(out, src):
        _run(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11",
              src, "-o", out, "-lm"])
    return out


def build_reference() -> None:
    """Compile the reference's code into oracle/_ref: from the reference tree when it is present,
    else the CPU voxelizer from the sources staged in oracle/_ref/src (when its build is missing or
    was made for another CPU architecture)."""
    if os.path.isfile(os.path.join(REFERENCE_ROOT, "src", "cpu_voxelizer.cpp")):
        _run(["bash", os.path.join(HERE, "build_ref.sh"), REFERENCE_ROOT])
        return
    staged = os.path.join(REF_OUT, "src", "cpu_voxelizer.cpp")
    if os.path.isfile(staged) and (_stale(os.path.join(REF_OUT, "libref_cpu.so"), staged) or
                                   _stale(os.path.join(REF_OUT, "cuda_voxelizer_relinked"), staged)):
        _run(["bash", os.path.join(HERE, "build_ref.sh"), "--staged"])


def build_gpu_runner() -> str | None:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        return None
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "libref_gpu_runner.so")
    src = os.path.join(HERE, "ref_gpu_runner.cu")
    if _stale(out, src):
        _run([nvcc, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
              "-gencode", "arch=compute_103a,code=sm_103a", src, "-o", out, "-lcuda"])
    return out


def build_all() -> None:
    build_oracle()
    build_reference()
    build_gpu_runner()


if __name__ == "__main__":
    build_all()
    print("oracle build done", file=sys.stderr)
