"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/liboracle.so``: the C restatement ``oracle/cvx_oracle.c`` (host code, built on
  whichever machine runs the tests).  ``-ffp-contract=off`` keeps every ``a*b+c`` a separate
  multiply and add, which is what the reference CPU build does on x86-64; without it gcc fuses
  them on aarch64 and the restatement would no longer reproduce the reference bit for bit.
* ``oracle/_ref/``: the reference's own code, built from its sources by ``oracle/build_ref.sh``
  when the reference tree is present (only on the development machine; elsewhere the prebuilt
  device-code files in ``oracle/_ref`` are used as they are).
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
REFERENCE_ROOT = os.environ.get("CVX_REFERENCE_ROOT", "/root/reference")


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
    """Compile the reference's code into oracle/_ref when its sources are present."""
    if os.path.isfile(os.path.join(REFERENCE_ROOT, "src", "cpu_voxelizer.cpp")):
        _run(["bash", os.path.join(HERE, "build_ref.sh"), REFERENCE_ROOT])


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
