"""The reference's drop-in contract, run the way its main() runs it.

The reference's main() (src/main.cpp:61-80, :209-222) copies the triangles on the host into
cudaMallocManaged memory, allocates the table with cudaMallocManaged (not cleared: fresh managed
pages are zero), and calls the C++ functions

    void voxelize(const voxinfo& v, float* triangle_data, unsigned int* vtable, bool morton_code);
    void voxelize_solid(const voxinfo& v, float* triangle_data, unsigned int* vtable, bool morton_code);

(src/voxelize.cu:192, src/voxelize_solid.cu:147), which run on the default stream, synchronize the
device, print "[Perf] Voxelization GPU time" and exit the process on an error.  libcvx.so exports
both symbols with the same mangled names; these tests call them through ctypes on managed buffers,
read the table back on the host as main() does, and compare it bit for bit with the reference's own
kernels (oracle/_ref cubins) run on device copies of the same triangles.  The C ABI is run on the
same managed pointers too.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle  # noqa: E402
from cuda_voxelizer_gb300 import _lib  # noqa: E402
from cuda_voxelizer_gb300 import api as cv  # noqa: E402
from cuda_voxelizer_gb300 import meshgen  # noqa: E402
from oracle.ref_safety import safe_triangles  # noqa: E402

pytestmark = pytest.mark.gpu

SYM_SURFACE = "_Z8voxelizeRK7voxinfoPfPjb"
SYM_SOLID = "_Z14voxelize_solidRK7voxinfoPfPjb"
MODES = [(False, False), (True, False), (False, True), (True, True)]


def _cudart():
    """The CUDA runtime libcvx.so was linked against (already loaded by it, found by soname)."""
    for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
        except OSError:
            continue
        rt.cudaMallocManaged.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t, ctypes.c_uint]
        rt.cudaMallocManaged.restype = ctypes.c_int
        rt.cudaFree.argtypes = [ctypes.c_void_p]
        rt.cudaFree.restype = ctypes.c_int
        rt.cudaDeviceSynchronize.restype = ctypes.c_int
        return rt
    pytest.fail("CUDA runtime library not found")


def _symbol(name):
    f = getattr(_lib.lib, name)
    f.argtypes = [ctypes.POINTER(cv.VoxInfo), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_bool]
    f.restype = None
    return f


class Managed:
    """A cudaMallocManaged buffer (cudaMemAttachGlobal), freed on exit."""

    def __init__(self, rt, nbytes):
        self.rt = rt
        self.ptr = ctypes.c_void_p()
        assert rt.cudaMallocManaged(ctypes.byref(self.ptr), max(int(nbytes), 4), 1) == 0
        self.nbytes = int(nbytes)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        assert self.rt.cudaDeviceSynchronize() == 0
        assert self.rt.cudaFree(self.ptr) == 0

    def write(self, a: np.ndarray):
        """Host writes into the managed pages (main() copies triangle by triangle; one memmove here)."""
        a = np.ascontiguousarray(a)
        assert a.nbytes <= self.nbytes
        ctypes.memmove(self.ptr.value, a.ctypes.data, a.nbytes)

    def read_u32(self, words):
        return np.ctypeslib.as_array((ctypes.c_uint32 * words).from_address(self.ptr.value)).copy()


def _mesh(name):
    if name == "torus":
        return meshgen.torus(0), 64
    return meshgen.icosphere(3, level=6), 256


def _reference_table(ref, info, tris, morton, solid):
    t = torch.from_numpy(np.ascontiguousarray(tris).reshape(-1)).cuda()
    b = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    ref.voxelize(bytes(info), t.data_ptr(), b.data_ptr(), morton, solid, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return b.cpu().numpy().view(np.uint32)


@pytest.fixture(scope="module")
def ref():
    return oracle.RefGPU()


@pytest.mark.parametrize("name", ["torus", "ico6"])
@pytest.mark.parametrize("morton,solid", MODES)
def test_cxx_symbols_on_managed_memory(ref, capfd, name, morton, solid):
    rt = _cudart()
    tris, g = _mesh(name)
    info = cv.make_voxinfo(tris, g)
    if solid:
        # the reference solid kernel writes outside its table for some near-x-parallel triangles
        # (oracle/ref_safety.py); both sides get the mesh without them
        tris = np.ascontiguousarray(tris[safe_triangles(tris, bytes(info), morton)])
        info = cv.VoxInfo.from_buffer_copy(bytes(info))
        info.n_triangles = tris.shape[0]
    words = cv.table_words(info)
    want = _reference_table(ref, info, tris, morton, solid)
    capfd.readouterr()
    with Managed(rt, tris.nbytes) as mt, Managed(rt, 4 * words) as mv:
        mt.write(tris)
        _symbol(SYM_SOLID if solid else SYM_SURFACE)(ctypes.byref(info), mt.ptr, mv.ptr, morton)
        ctypes.CDLL(None).fflush(None)  # the [Perf] line is a buffered printf, as in the reference
        out = capfd.readouterr().out
        got = mv.read_u32(words)  # the call synchronized the device: host reads are safe
        assert "[Perf] Voxelization GPU time:" in out, out
        d = np.nonzero(got != want)[0]
        assert d.size == 0, f"{name} morton={morton} solid={solid}: {d.size} words differ, first {d[:8]}"
        # the C ABI on the same managed triangles, into a second managed table
        with Managed(rt, 4 * words) as mv2:
            ctypes.memset(mv2.ptr.value, 0, 4 * words)
            fn = _lib.lib.cvx_voxelize_solid if solid else _lib.lib.cvx_voxelize
            s = torch.cuda.current_stream().cuda_stream
            assert fn(ctypes.byref(info), mt.ptr.value, mv2.ptr.value, int(morton), s) == 0
            assert _lib.lib.cvx_device_status(s) == 0, _lib.lib.cvx_last_error_message()
            got2 = mv2.read_u32(words)
            assert np.array_equal(got2, want)


def test_cxx_symbol_exits_on_an_unsupported_request():
    """The reference exits the process on a CUDA error (checkCudaErrors, helper_cuda.h:567-579);
    the drop-in does the same, and also refuses Morton order on a grid it cannot address (the
    reference would write outside its table) before anything is launched."""
    code = f"""
import ctypes, sys
sys.path.insert(0, {os.path.dirname(os.path.dirname(os.path.abspath(__file__)))!r})
from cuda_voxelizer_gb300 import _lib, api as cv, meshgen
tris = meshgen.torus(0)
info = cv.make_voxinfo(tris, 100)
f = getattr(_lib.lib, {SYM_SURFACE!r})
f.argtypes = [ctypes.POINTER(cv.VoxInfo), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_bool]
f(ctypes.byref(info), ctypes.c_void_p(256), ctypes.c_void_p(256), True)
print("returned")
"""
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 1, (r.returncode, r.stdout, r.stderr)
    assert "returned" not in r.stdout
    assert "Morton order needs a cubic power-of-two grid" in r.stderr, r.stderr
