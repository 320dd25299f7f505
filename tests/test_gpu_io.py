"""GPU ingest, layout and output kernels against the reference's writers and the oracle:

* cvx_encode_binvox == the reference's write_binvox payload (golden files from src/util_io.cpp);
* cvx_encode_voxel_list == the restated write_vox voxel loop;
* cvx_transcode: Morton <-> linear, pinned by the engine's own (reference-exact) Morton and linear
  tables of the same mesh, and by round trips of random tables;
* cvx_mesh_bbox_device / cvx_voxinfo_from_device == the host setup; cvx_gather_soup == indexing.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle  # noqa: E402
from cuda_voxelizer_gb300 import api as cv  # noqa: E402
from cuda_voxelizer_gb300 import meshgen  # noqa: E402
from cuda_voxelizer_gb300._lib import CvxVoxinfo  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_io.npz")


def _cases():
    g = np.load(GOLDEN)
    return sorted({k.rsplit("__", 1)[0] for k in g.files})


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def _dev(table):
    return torch.from_numpy(np.ascontiguousarray(table).view(np.int32)).cuda()


@pytest.mark.parametrize("name", _cases())
def test_binvox_payload_equals_reference_writer(golden, name):
    info = CvxVoxinfo.from_buffer_copy(golden[f"{name}__info"].tobytes())
    got = cv.encode_binvox(info, _dev(golden[f"{name}__table"]))
    assert got == golden[f"{name}__payload"].tobytes()


def test_binvox_of_engine_table_equals_reference_writer_restatement():
    tris = meshgen.icosphere(4, level=6)
    info = cv.make_voxinfo(tris, 256)
    tab = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    cv.voxelize_solid(info, torch.from_numpy(tris.reshape(-1)).cuda(), tab)
    host = tab.cpu().numpy().view(np.uint32)
    assert cv.encode_binvox(info, tab) == oracle.binvox_payload(bytes(info), host)


@pytest.mark.parametrize("name", ["torus_g64__linear__surface", "ico5_g128__linear__solid", "random_g32",
                                  "sparse_g128", "full_g64", "empty_g64", "ico3_g8__linear__surface"])
def test_voxel_list_equals_restated_writer(golden, name):
    info_b = golden[f"{name}__info"].tobytes()
    info = CvxVoxinfo.from_buffer_copy(info_b)
    table = golden[f"{name}__table"]
    got = cv.encode_voxel_list(info, _dev(table)).cpu().numpy()
    want = oracle.vox_list(info_b, table)
    assert got.shape == want.shape and np.array_equal(got, want)


def test_voxel_list_rejects_grids_with_y_unequal_z(golden):
    info = CvxVoxinfo.from_buffer_copy(golden["random_40x24x36__info"].tobytes())
    with pytest.raises(cv.CvxError) as e:
        cv.encode_voxel_list(info, _dev(golden["random_40x24x36__table"]))
    assert e.value.status == 2


@pytest.mark.parametrize("g", [8, 16, 64, 128, 512])
@pytest.mark.parametrize("solid", [False, True])
def test_transcode_matches_engine_morton_tables(g, solid):
    tris = meshgen.icosphere(5, level=6 if g >= 128 else 4)
    info = cv.make_voxinfo(tris, g)
    d = torch.from_numpy(tris.reshape(-1)).cuda()
    lin = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    mor = torch.zeros_like(lin)
    f = cv.voxelize_solid if solid else cv.voxelize
    f(info, d, lin, False)
    f(info, d, mor, True)
    assert torch.equal(cv.transcode(lin, g, True), mor)
    assert torch.equal(cv.transcode(mor, g, False), lin)


@pytest.mark.parametrize("g", [4, 32, 256])
def test_transcode_round_trip_random(g):
    gen = torch.Generator(device="cuda").manual_seed(g)
    t = torch.randint(-2 ** 31, 2 ** 31 - 1, (g ** 3 // 32,), dtype=torch.int32, device="cuda", generator=gen)
    m = cv.transcode(t, g, True)
    assert torch.equal(cv.transcode(m, g, False), t)
    # spot-check single bits against the oracle's Morton encoder
    host = t.cpu().numpy().view(np.uint32)
    mh = m.cpu().numpy().view(np.uint32)
    rng = np.random.default_rng(g)
    for _ in range(200):
        x, y, z = (int(v) for v in rng.integers(0, g, 3))
        li = x + g * (y + g * z)
        mi = oracle.morton_encode(x, y, z)
        assert ((host[li >> 5] >> (31 - (li & 31))) & 1) == ((mh[mi >> 5] >> (31 - (mi & 31))) & 1)


@pytest.mark.parametrize("mesh", ["torus", "ico", "soup"])
def test_device_bbox_and_voxinfo_equal_host_setup(mesh):
    tris = {"torus": lambda: meshgen.torus(3), "ico": lambda: meshgen.icosphere(1, level=7),
            "soup": lambda: meshgen.soup(2, n=300_000)}[mesh]()
    d = torch.from_numpy(tris.reshape(-1)).cuda()
    lo, hi = cv.mesh_bbox_device(d)
    hlo, hhi = cv.mesh_bbox(tris)
    assert np.array_equal(lo, hlo) and np.array_equal(hi, hhi)
    assert bytes(cv.voxinfo_from_device(d, 256)) == bytes(cv.make_voxinfo(tris, 256))


def test_gather_soup_matches_indexing_and_flags_bad_faces():
    rng = np.random.default_rng(9)
    verts = rng.normal(size=(5000, 3)).astype(np.float32)
    faces = rng.integers(0, 5000, size=(20000, 3)).astype(np.int32)
    soup, bad = cv.gather_soup(torch.from_numpy(verts).cuda(), torch.from_numpy(faces).cuda())
    assert bad == 0
    assert np.array_equal(soup.cpu().numpy().reshape(-1, 3, 3), verts[faces])
    faces[[3, 77], 1] = 5000
    soup, bad = cv.gather_soup(torch.from_numpy(verts).cuda(), torch.from_numpy(faces).cuda())
    s = soup.cpu().numpy().reshape(-1, 9)
    assert bad == 2 and np.isnan(s[[3, 77]]).all() and not np.isnan(np.delete(s, [3, 77], axis=0)).any()
