"""Build libcvx.so in-tree (cuda_voxelizer_gb300/_lib/) with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into one shared library with the C ABI
of include/cvx.h and the C++ drop-in symbols of include/cvx_dropin.h.  No PyTorch involvement: the
library links only the CUDA runtime.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libcvx.so")
DIAG_LIB = os.path.join(OUT_DIR, "libcvx_diag.so")  # include/cvx_diag.h: measurement helpers, not the ABI
DIAG_SOURCES = ["microbench.cu"]
SOURCES = ["surface.cu", "bricks.cu", "solid.cu", "api.cu", "dropin.cpp", "noalloc.cu", "server.cu", "clear.cu", "mesh.cu", "transcode.cu", "encode.cu"]
HEADERS = ["cvx_device.cuh", "surface.cuh", "engine.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    return os.path.join(home, "bin", "nvcc")


def cuda_lib_dir() -> str:
    home = os.path.dirname(os.path.dirname(os.path.realpath(nvcc_path())))
    for d in ("lib64", "lib"):
        if os.path.isdir(os.path.join(home, d)):
            return os.path.join(home, d)
    return os.path.join(home, "lib64")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                   "-I", os.path.join(ROOT, "include"), "-I", CSRC]


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


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target) or foreign_binary(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra_flags=None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = nvcc_path()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", h)
                                                         for h in ("cvx.h", "cvx_dropin.h", "cvx_diag.h")]
    objs, diag_objs = [], []
    jobs = []
    for src in SOURCES + DIAG_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src + ".o")
        (diag_objs if src in DIAG_SOURCES else objs).append(o)
        if _stale(o, [s, __file__] + hdrs):
            cmd = [nvcc] + _flags() + list(extra_flags or []) + ["-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES) + len(DIAG_SOURCES)) as ex:
        for err in ex.map(run, jobs):
            if verbose and err:
                print(err, file=sys.stderr)
    for lib, o in ((LIB, objs), (DIAG_LIB, diag_objs)):
        if jobs or _stale(lib, o):
            run([nvcc] + ARCH + ["-shared", "-cudart", "shared", "-Xlinker", "--no-undefined", "-o", lib] + o +
                ["-Xlinker", "-rpath," + cuda_lib_dir()])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
