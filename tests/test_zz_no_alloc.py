"""cvx_voxelize_solid_noalloc: solid voxelization that allocates no device memory.

It exists for callers that must not allocate while voxelizing (per-frame code with a fixed GPU
memory budget, hosts whose allocator policy forbids driver allocations); its scratch is a fixed
4 MiB array inside libcvx.so, which limits the grid to 2^24 voxels.  These tests call it through the
C ABI and require the same bits as cvx_voxelize_solid, on two calls in a row (the second call runs
on the scratch the first one left behind).  The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from cuda_voxelizer_gb300 import _lib  # noqa: E402
from cuda_voxelizer_gb300 import api as cv  # noqa: E402
from cuda_voxelizer_gb300 import meshgen  # noqa: E402

pytestmark = pytest.mark.gpu


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _run(fn, info, t, morton):
    table = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    rc = fn(ctypes.byref(info), t.data_ptr(), table.data_ptr(), int(morton), _stream())
    assert rc == 0, _lib.lib.cvx_last_error_message().decode()
    # device-side checks of the call (bulk-copy timeouts, queue overflows): the no-alloc call keeps
    # its error word in the fixed array, and cvx_device_status reads it
    rc = _lib.lib.cvx_device_status(_stream())
    assert rc == 0, _lib.lib.cvx_last_error_message().decode()
    torch.cuda.synchronize()
    return table


# Grids: g < 32 (Morton resolved word by word), 32..1024 (Morton slabs), non-power-of-two (linear
# only).  "slice": exactly one full slice of the fixed triangle queue (65,536 triangles); "slice+1"
# needs a second slice.
@pytest.mark.parametrize("mesh,g", [("torus", 64), ("ico5", 128), ("soup", 256), ("ico4", 100), ("ico3", 8),
                                    ("ico4", 16), ("slice", 128), ("slice+1", 128)])
@pytest.mark.parametrize("morton", [False, True])
def test_noalloc_matches_solid_twice(mesh, g, morton):
    if morton and g & (g - 1):
        pytest.skip("Morton order needs a power-of-two grid")
    tris = {"torus": lambda: meshgen.torus(7), "ico5": lambda: meshgen.icosphere(8, level=5),
            "soup": lambda: meshgen.soup(9, n=100_000, lmin=0.5 / 256, lmax=0.3),
            "ico4": lambda: meshgen.icosphere(10, level=4), "ico3": lambda: meshgen.icosphere(12, level=3),
            "slice": lambda: meshgen.soup(13, n=65_536, lmin=0.5 / 128, lmax=0.2),
            "slice+1": lambda: meshgen.soup(14, n=65_537, lmin=0.5 / 128, lmax=0.2)}[mesh]()
    if mesh.startswith("slice"):
        assert tris.shape[0] == {"slice": 65_536, "slice+1": 65_537}[mesh]
    info = cv.make_voxinfo(tris, g)
    t = torch.from_numpy(tris.reshape(-1)).cuda()
    want = _run(_lib.lib.cvx_voxelize_solid, info, t, morton)
    for _ in range(2):
        got = _run(_lib.lib.cvx_voxelize_solid_noalloc, info, t, morton)
        assert torch.equal(got, want), f"{mesh}@{g} morton={morton}: {int((got != want).sum())} words differ"


def test_noalloc_rejects_grids_beyond_its_scratch():
    tris = meshgen.torus(11)
    info = cv.make_voxinfo(tris, 512)  # 2^27 voxels > 2^24
    t = torch.from_numpy(tris.reshape(-1)).cuda()
    table = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    rc = _lib.lib.cvx_voxelize_solid_noalloc(ctypes.byref(info), t.data_ptr(), table.data_ptr(), 0, _stream())
    assert rc == 1
    assert b"exceeds the fixed scratch" in _lib.lib.cvx_last_error_message()
    torch.cuda.synchronize()
    assert int(table.count_nonzero()) == 0


def test_noalloc_rejects_axes_beyond_2_22():
    """Same per-axis limit as cvx_voxelize_solid (the solid column arithmetic reproduces the
    reference only for indices below 2^22), although 2^23 x 2 x 1 fits the fixed scratch."""
    tris = meshgen.torus(11)
    info = cv.make_voxinfo(tris, 64)
    info.gridsize[0], info.gridsize[1], info.gridsize[2] = 1 << 23, 2, 1
    t = torch.from_numpy(tris.reshape(-1)).cuda()
    table = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    for fn in (_lib.lib.cvx_voxelize_solid_noalloc, _lib.lib.cvx_voxelize_solid):
        rc = fn(ctypes.byref(info), t.data_ptr(), table.data_ptr(), 0, _stream())
        assert rc == 2, _lib.lib.cvx_last_error_message()
        assert b"above 2^22" in _lib.lib.cvx_last_error_message()
    torch.cuda.synchronize()
    assert int(table.count_nonzero()) == 0
