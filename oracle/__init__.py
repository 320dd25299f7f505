"""The oracle: CPU restatement of the reference voxelizer and runners for the reference's own code.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline leg may import this package; the engine in ``cuda_voxelizer_gb300`` never does.

* :func:`voxelize` -- ``oracle/cvx_oracle.c``, a restatement of ``cpu_voxelize_mesh`` /
  ``cpu_voxelize_mesh_solid`` (src/cpu_voxelizer.cpp:35, :241), pinned bit for bit against the
  reference's own CPU build (tests/test_oracle.py, tests/golden/).
* :func:`ref_cpu_voxelize` -- the reference's own ``src/cpu_voxelizer.cpp`` built by
  ``oracle/build_ref.sh`` (only where that build ran: it is host code).
* :class:`RefGPU` -- the reference's own CUDA kernels (src/voxelize.cu, src/voxelize_solid.cu)
  built for sm_103a by ``oracle/build_ref.sh`` and launched by ``oracle/ref_gpu_runner.cu``.
"""
from __future__ import annotations

import contextlib
import ctypes
import os
import sys

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


class OvxMode(ctypes.Structure):
    """Fused-multiply-add pattern selection (see ``ovx_mode`` in cvx_oracle.c)."""

    _fields_ = [("cross", ctypes.c_int), ("dot3", ctypes.c_int), ("dot2", ctypes.c_int),
                ("plane", ctypes.c_int), ("edge_xy", ctypes.c_int), ("edge_yz", ctypes.c_int),
                ("edge_zx", ctypes.c_int), ("ccw", ctypes.c_int), ("pt", ctypes.c_int), ("getx", ctypes.c_int),
                ("clip", ctypes.c_int), ("inv_len", ctypes.POINTER(ctypes.c_float))]


def gpu_mode(morton: bool, inv_len: np.ndarray | None = None, clip: bool = True) -> OvxMode:
    """The reference CUDA kernels' arithmetic: the fused-multiply-add pattern nvcc gives their
    helper_math expressions on sm_103a (src/voxelize.cu:89-165, src/voxelize_solid.cu:24-64, with
    get_x_coordinate contracted one way in the kernel's linear-order code and the other way in its
    Morton-order code), their double-promoted solid arithmetic, and -- if given -- 1/|n| values taken
    from the device's own rsqrtf (see :func:`device_inv_len`).  ``clip`` keeps the solid writes inside
    the grid the way the CUDA engine does where the reference writes outside its table.  Keep the
    ``inv_len`` array alive while the mode is in use."""
    m = OvxMode(cross=1, dot3=1, dot2=2, plane=2, edge_xy=1, edge_yz=1, edge_zx=2, ccw=2, pt=1,
                getx=2 if morton else 1, clip=int(bool(clip)))
    if inv_len is not None:
        assert inv_len.dtype == np.float32 and inv_len.flags.c_contiguous
        m.inv_len = inv_len.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    return m


def len2(info: bytes, tris, mode: OvxMode | None = None) -> np.ndarray:
    """dot(c, c) of every triangle's cross product under ``mode``'s patterns (the rsqrtf argument
    of the reference kernels' normalize)."""
    t = _soup(tris, info)
    ib = ctypes.create_string_buffer(bytes(info), 64)
    out = np.zeros(t.shape[0], dtype=np.float32)
    lib().ovx_len2(ctypes.addressof(ib), _ptr(t), ctypes.addressof(mode) if mode is not None else None, _ptr(out))
    return out


_lib = None
_ref_cpu = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        L.ovx_voxelize.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_void_p]
        L.ovx_voxelize_omp.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int]
        L.ovx_morton_encode.argtypes = [ctypes.c_uint32] * 3
        L.ovx_morton_encode.restype = ctypes.c_uint64
        L.ovx_morton_lut.argtypes = [ctypes.c_int, ctypes.c_void_p]
        L.ovx_mesh_bbcube.argtypes = [ctypes.c_void_p] * 4
        L.ovx_info_init.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_uint64]
        L.ovx_max_threads.restype = ctypes.c_int
        L.ovx_len2.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.ovx_count_atomics.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.ovx_count_atomics.restype = ctypes.c_uint64
        L.ovx_binvox_payload.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64]
        L.ovx_binvox_payload.restype = ctypes.c_uint64
        L.ovx_vox_list.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64]
        L.ovx_vox_list.restype = ctypes.c_uint64
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def table_words(info: bytes) -> int:
    g = np.frombuffer(info, dtype=np.uint32, count=3, offset=24).astype(np.uint64)
    return int((int(g[0]) * int(g[1]) * int(g[2]) + 31) // 32)


def _soup(tris, info: bytes | None = None) -> np.ndarray:
    t = np.ascontiguousarray(np.asarray(tris, dtype=np.float32).reshape(-1, 9))
    if info is not None:
        n = int(np.frombuffer(info, dtype=np.uint64, count=1, offset=40)[0])
        if t.shape[0] < n:
            raise ValueError(f"voxinfo says {n} triangles but only {t.shape[0]} were given")
    return t


def with_count(info: bytes, n: int) -> bytes:
    """The same voxinfo with n_triangles replaced (e.g. for a sample of the mesh)."""
    b = bytearray(info)
    b[40:48] = int(n).to_bytes(8, "little")
    return bytes(b)


def voxelize(info: bytes, tris, morton: bool = False, solid: bool = False, mode: OvxMode | None = None,
             table: np.ndarray | None = None) -> np.ndarray:
    """Serial restatement; returns (or ORs/XORs into) a uint32 table of ceil(g^3/32) words."""
    assert len(info) == 64
    t = _soup(tris, info)
    ib = ctypes.create_string_buffer(bytes(info), 64)
    if table is None:
        table = np.zeros(table_words(info), dtype=np.uint32)
    lib().ovx_voxelize(ctypes.addressof(ib), _ptr(t), _ptr(table), int(morton), int(solid),
                       ctypes.addressof(mode) if mode is not None else None)
    return table


def voxelize_omp(info: bytes, tris, morton: bool = False, solid: bool = False, threads: int = 0) -> np.ndarray:
    """Restatement run like the reference's OpenMP CPU path (parallel for, critical per bit)."""
    t = _soup(tris, info)
    ib = ctypes.create_string_buffer(bytes(info), 64)
    table = np.zeros(table_words(info), dtype=np.uint32)
    lib().ovx_voxelize_omp(ctypes.addressof(ib), _ptr(t), _ptr(table), int(morton), int(solid), int(threads))
    return table


def count_atomics(info: bytes, tris, morton: bool = False, solid: bool = False) -> int:
    """Atomic term of the roofline: distinct table words per triangle summed (surface) or column
    hits (solid), counted by the restatement without writing a table."""
    t = _soup(tris, info)
    ib = ctypes.create_string_buffer(bytes(info), 64)
    return int(lib().ovx_count_atomics(ctypes.addressof(ib), _ptr(t), int(morton), int(solid)))


def binvox_payload(info: bytes, table: np.ndarray) -> bytes:
    """write_binvox's RLE data section for a linear-order table (restatement)."""
    ib = ctypes.create_string_buffer(bytes(info), 64)
    t = np.ascontiguousarray(table, dtype=np.uint32)
    n = int(lib().ovx_binvox_payload(ctypes.addressof(ib), _ptr(t), None, 0))
    out = np.zeros(max(n, 1), dtype=np.uint8)
    lib().ovx_binvox_payload(ctypes.addressof(ib), _ptr(t), _ptr(out), n)
    return out[:n].tobytes()


def vox_list(info: bytes, table: np.ndarray) -> np.ndarray:
    """The (x, gz - z, y) triples write_vox passes to AddVoxel, in order (restatement)."""
    ib = ctypes.create_string_buffer(bytes(info), 64)
    t = np.ascontiguousarray(table, dtype=np.uint32)
    n = int(lib().ovx_vox_list(ctypes.addressof(ib), _ptr(t), None, 0))
    out = np.zeros((max(n, 1), 3), dtype=np.int32)
    lib().ovx_vox_list(ctypes.addressof(ib), _ptr(t), _ptr(out), n)
    return out[:n]


def max_threads() -> int:
    return int(lib().ovx_max_threads())


def morton_encode(x: int, y: int, z: int) -> int:
    return int(lib().ovx_morton_encode(x, y, z))


def morton_lut(axis: int) -> np.ndarray:
    out = np.zeros(256, dtype=np.uint32)
    lib().ovx_morton_lut(axis, _ptr(out))
    return out


def mesh_bbcube(bmin, bmax):
    a = np.asarray(bmin, dtype=np.float32).copy()
    b = np.asarray(bmax, dtype=np.float32).copy()
    omin = np.zeros(3, np.float32)
    omax = np.zeros(3, np.float32)
    lib().ovx_mesh_bbcube(_ptr(a), _ptr(b), _ptr(omin), _ptr(omax))
    return omin, omax


def info_init(bmin, bmax, grid, n_tri) -> bytes:
    out = ctypes.create_string_buffer(64)
    a = np.asarray(bmin, dtype=np.float32).copy()
    b = np.asarray(bmax, dtype=np.float32).copy()
    g = np.asarray(grid, dtype=np.uint32).copy()
    lib().ovx_info_init(out, _ptr(a), _ptr(b), _ptr(g), int(n_tri))
    return bytes(out.raw)


# --- the reference's own CPU build (host code; present only where oracle/build_ref.sh ran) ------

def ref_cpu_lib():
    global _ref_cpu
    if _ref_cpu is None:
        path = os.path.join(REF_DIR, "libref_cpu.so")
        if not os.path.exists(path):
            return None
        if _build.foreign_binary(path):  # built on a machine of another architecture
            return None
        try:
            L = ctypes.CDLL(path)
        except OSError:
            return None
        L.ref_cpu_voxelize.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.ref_cpu_voxelize_solid.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.ref_create_mesh_bbcube.argtypes = [ctypes.c_void_p] * 4
        L.ref_voxinfo_init.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                       ctypes.c_void_p]
        L.ref_morton_lut.argtypes = [ctypes.c_int, ctypes.c_void_p]
        _ref_cpu = L
    return _ref_cpu


def ref_cpu_available() -> bool:
    return ref_cpu_lib() is not None


@contextlib.contextmanager
def _stdout_to_devnull():
    """Send file descriptor 1 to /dev/null for the duration (the reference CPU voxelizer prints
    "[Info] Using N threads" and "[Perf] CPU voxelization time" on stdout; the shim flushes C stdio
    before returning, so nothing of it reaches the real stdout afterwards)."""
    sys.stdout.flush()
    saved = os.dup(1)
    null = os.open(os.devnull, os.O_WRONLY)
    try:
        os.dup2(null, 1)
        yield
    finally:
        os.dup2(saved, 1)
        os.close(null)
        os.close(saved)


def ref_cpu_voxelize(info: bytes, tris, morton: bool = False, solid: bool = False,
                     quiet: bool = False) -> np.ndarray:
    """The reference's cpu_voxelize_mesh / cpu_voxelize_mesh_solid (src/cpu_voxelizer.cpp:35, :241)
    on a soup.  ``quiet`` drops the reference's own stdout lines (for callers whose stdout is a
    machine-read record, like the benchmark's JSON line)."""
    L = ref_cpu_lib()
    if L is None:
        raise RuntimeError("reference CPU build not available on this machine")
    t = _soup(tris, info)
    ib = ctypes.create_string_buffer(bytes(info), 64)
    # The reference's solid loop can run past its table for nearly x-parallel triangles near the
    # table's end (its float32 xmax exceeds the grid; the reference writes outside its buffer
    # there): a guard area as large as the table keeps those writes in memory this call owns.
    words = table_words(info)
    buf = np.zeros(2 * words + 1024, dtype=np.uint32)
    table = buf[:words]
    fn = L.ref_cpu_voxelize_solid if solid else L.ref_cpu_voxelize
    if quiet:
        with _stdout_to_devnull():
            fn(ctypes.addressof(ib), _ptr(t), _ptr(table), int(morton))
    else:
        fn(ctypes.addressof(ib), _ptr(t), _ptr(table), int(morton))
    return table


# --- the reference's own CUDA kernels ------------------------------------------------------------

class RefGPU:
    """Launch the reference kernels (compiled from its sources for sm_103a) on device buffers."""

    def __init__(self):
        path = _build.build_gpu_runner()
        if path is None:
            raise RuntimeError("nvcc not available to build the reference kernel runner")
        if not os.path.exists(os.path.join(REF_DIR, "ref_voxelize.cubin")):
            raise RuntimeError("reference cubins missing from oracle/_ref (run oracle/build_ref.sh)")
        L = ctypes.CDLL(path)
        L.refgpu_init.argtypes = [ctypes.c_char_p]
        L.refgpu_voxelize.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_void_p]
        L.refgpu_last_error.restype = ctypes.c_char_p
        L.refgpu_rsqrt.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
        if L.refgpu_init(REF_DIR.encode()) != 0:
            raise RuntimeError("refgpu_init: " + L.refgpu_last_error().decode())
        self.L = L

    def rsqrt(self, d_in: int, d_out: int, n: int, stream: int = 0):
        """d_out[i] = rsqrtf(d_in[i]) on the device (float32 device buffers of n values)."""
        if self.L.refgpu_rsqrt(d_in, d_out, n, stream) != 0:
            raise RuntimeError("refgpu_rsqrt: " + self.L.refgpu_last_error().decode())

    def voxelize(self, info: bytes, d_tris: int, d_table: int, morton: bool, solid: bool, stream: int = 0):
        ib = ctypes.create_string_buffer(bytes(info), 64)
        if self.L.refgpu_voxelize(ctypes.addressof(ib), d_tris, d_table, int(morton), int(solid), stream) != 0:
            raise RuntimeError("refgpu_voxelize: " + self.L.refgpu_last_error().decode())
