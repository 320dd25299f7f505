"""The shared-memory brick rasterizer of surface jobs on grids of 2^29+ voxels (csrc/bricks.cu).

Its larger triangles are binned to 32^3 bricks of the table, rasterized brick by brick in shared
memory and flushed with one global atomicOr per word.  The tables must be bit-identical to the
reference kernel voxelize_triangle (src/voxelize.cu:58) with the full pair area (brick_pairs = 16),
with a pair area too small for the mesh (brick_pairs = 1: the triangles that do not fit fall back to
row-by-row global atomics, mixed with the ones that did), and with bricks switched off
(brick_pairs = 0), on cubic and non-cubic grids (rows not word-aligned), linear and Morton order.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle  # noqa: E402
from cuda_voxelizer_gb300 import api as cv  # noqa: E402
from cuda_voxelizer_gb300 import meshgen  # noqa: E402

pytestmark = pytest.mark.gpu

GUARD = 256


@pytest.fixture(scope="module")
def ref():
    return oracle.RefGPU()


def _case(name):
    if name == "soup1024":
        t = meshgen.soup(21, n=200_000)
        return t, cv.make_voxinfo(t, 1024)
    if name == "soup1024_big":
        t = meshgen.soup(22, n=30_000, lmin=8 / 1024, lmax=0.25)
        return t, cv.make_voxinfo(t, 1024)
    if name == "ico5_1024":
        t = meshgen.icosphere(23, level=5)  # 20,480 triangles of about 20 voxels
        return t, cv.make_voxinfo(t, 1024)
    t = meshgen.soup(24, n=60_000, lmin=2 / 1024, lmax=0.3)
    info = cv.make_voxinfo(t, 1024)
    dims = {"noncubic": (1000, 700, 800), "thin_x": (2048, 512, 512)}[name]
    for i in range(3):
        info.gridsize[i] = dims[i]
        info.unit[i] = np.float32((np.float32(info.bbox_max[i]) - np.float32(info.bbox_min[i])) / np.float32(dims[i]))
    return t, info


CASES = [("soup1024", False), ("soup1024", True), ("soup1024_big", False), ("soup1024_big", True),
         ("ico5_1024", True), ("noncubic", False), ("thin_x", False)]


@pytest.mark.parametrize("name,morton", CASES)
def test_bricks_match_reference_kernel(ref, name, morton):
    tris, info = _case(name)
    g = info.gridsize
    assert g[0] * g[1] * g[2] >= 1 << 29  # a grid the brick rasterizer serves
    d = torch.from_numpy(np.ascontiguousarray(tris).reshape(-1)).cuda()
    W = cv.table_words(info)
    want = torch.zeros(W + GUARD, dtype=torch.int32, device="cuda")
    ref.voxelize(bytes(info), d.data_ptr(), want.data_ptr(), morton, False, torch.cuda.current_stream().cuda_stream)
    before = cv.get_tuning(0)
    try:
        for pairs in (16, 1, 0):
            cv.set_tuning(0, brick_pairs=pairs)
            got = torch.zeros(W + GUARD, dtype=torch.int32, device="cuda")
            cv.voxelize(info, d, got, morton)
            torch.cuda.synchronize()
            cv.device_status()
            n = int((got != want).sum())
            assert n == 0, f"{name} morton={morton} brick_pairs={pairs}: {n} words differ"
    finally:
        cv.set_tuning(0, **before)
