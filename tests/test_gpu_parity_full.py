"""GPU parity at the workloads' full sizes, including the triangles the reference kernel cannot run.

* The 2,000,000-triangle stress soup at 1024^3 (the size-stress workload, surface, linear order):
  the engine against the reference kernel voxelize_triangle (src/voxelize.cu:58), which clamps its
  bounding box to the grid and is safe on any input.
* The 256-mesh uneven mix (meshgen.batch_mix(0, 256): tori and displaced icospheres of 1k-500k
  triangles, grids 64-512, surface:solid 3:1, linear:Morton 1:1) as one clearing plan, every table
  against the reference kernels.
* Solid voxelization on the triangles oracle/ref_safety.py removes before the reference solid kernel
  may run (nearly x-parallel or nearly degenerate triangles, whose float32 xmax can leave the grid:
  the reference kernel then writes outside its table, and once faulted the GPU).  Those triangles
  are checked against the oracle in GPU-arithmetic mode instead -- the reference kernel's fused
  multiply-add pattern and double-promoted solid arithmetic restated on the CPU
  (oracle/cvx_oracle.c, src/voxelize_solid.cu:16-145), fed with 1/|n| from the device's own rsqrtf,
  with the engine's rule for writes outside the grid (the reference's are undefined) -- on the
  displaced icosphere at 512^3 and on a near-x-parallel soup at 1024^3, both orders.

Solid voxelization XORs a run of bits per column hit, so a mesh's table is the XOR of the tables of
any split of its triangles; surface voxelization ORs.  The full mesh's engine table must therefore
equal reference(kept) XOR oracle(removed), and this is asserted on the full, unfiltered meshes --
the same meshes the benchmark voxelizes.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle  # noqa: E402
from cuda_voxelizer_gb300 import api as cv  # noqa: E402
from cuda_voxelizer_gb300 import meshgen  # noqa: E402
from oracle.ref_safety import safe_triangles  # noqa: E402

pytestmark = pytest.mark.gpu

GUARD = 256  # zero words after every table: a write past the end shows up as a difference


@pytest.fixture(scope="module")
def ref():
    return oracle.RefGPU()


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _with_count(info, n):
    i = cv.VoxInfo.from_buffer_copy(bytes(info))
    i.n_triangles = int(n)
    return i


def _dev(tris):
    return torch.from_numpy(np.ascontiguousarray(tris, dtype=np.float32).reshape(-1)).cuda()


def engine_table(info, tris, morton, solid):
    t = _dev(tris)
    a = torch.zeros(cv.table_words(info) + GUARD, dtype=torch.int32, device="cuda")
    (cv.voxelize_solid if solid else cv.voxelize)(_with_count(info, tris.shape[0]), t, a, morton)
    torch.cuda.synchronize()
    cv.device_status()
    return a.cpu().numpy().view(np.uint32)


def reference_table(ref, info, tris, morton, solid):
    t = _dev(tris)
    b = torch.zeros(cv.table_words(info) + GUARD, dtype=torch.int32, device="cuda")
    ref.voxelize(bytes(_with_count(info, tris.shape[0])), t.data_ptr(), b.data_ptr(), morton, solid, _stream())
    torch.cuda.synchronize()
    return b.cpu().numpy().view(np.uint32)


def device_inv_len(ref, info, tris):
    """1/|n| per triangle as the reference kernels compute it: rsqrtf on the device, of dot(c, c)
    evaluated with the kernels' fused-multiply-add pattern."""
    l2 = oracle.len2(bytes(_with_count(info, tris.shape[0])), tris, oracle.gpu_mode(False))
    d_in = torch.from_numpy(l2).cuda()
    d_out = torch.empty_like(d_in)
    ref.rsqrt(d_in.data_ptr(), d_out.data_ptr(), l2.size, _stream())
    torch.cuda.synchronize()
    return np.ascontiguousarray(d_out.cpu().numpy())


def oracle_solid_gpu(ref, info, tris, morton):
    """The oracle in GPU-arithmetic mode with the engine's clip rule, as a table with guard words."""
    out = np.zeros(cv.table_words(info) + GUARD, dtype=np.uint32)
    if tris.shape[0] == 0:
        return out
    inv = device_inv_len(ref, info, tris)
    mode = oracle.gpu_mode(morton, inv_len=inv)
    oracle.voxelize(bytes(_with_count(info, tris.shape[0])), tris, morton, True, mode=mode,
                    table=out[:cv.table_words(info)])
    return out


def assert_same(a, b, what):
    d = np.nonzero(a != b)[0]
    pa = int(np.unpackbits(a.view(np.uint8)).sum())
    pb = int(np.unpackbits(b.view(np.uint8)).sum())
    assert d.size == 0, f"{what}: {d.size} words differ (engine {pa} bits, expected {pb} bits), first {d[:8]}"


def composed_solid(ref, info, tris, morton):
    """reference(kept) XOR oracle(removed): the expected table of the full mesh, and the removed
    triangles."""
    keep = safe_triangles(tris, bytes(info), morton)
    a = reference_table(ref, info, np.ascontiguousarray(tris[keep]), morton, True)
    removed = np.ascontiguousarray(tris[~keep])
    return a ^ oracle_solid_gpu(ref, info, removed, morton), removed


# ---- the size-stress soup at its full size -------------------------------------------------------

def test_soup_2m_1024_full_size(ref):
    tris = meshgen.soup(0, n=2_000_000)  # the benchmark's soup
    info = cv.make_voxinfo(tris, 1024)
    a = engine_table(info, tris, False, False)
    b = reference_table(ref, info, tris, False, False)
    assert_same(a, b, "soup 2M @1024^3")


# ---- solid: the triangles the reference kernel cannot run ----------------------------------------

@pytest.fixture(scope="module")
def ico8():
    return meshgen.icosphere(0, level=8)  # the benchmark's mesh


@pytest.mark.parametrize("morton", [False, True])
def test_icosphere512_solid_full_mesh(ref, ico8, morton):
    info = cv.make_voxinfo(ico8, 512)
    want, removed = composed_solid(ref, info, ico8, morton)
    assert removed.shape[0] > 1000  # about 1% of the mesh
    # the removed triangles alone, engine against the oracle
    assert_same(engine_table(info, removed, morton, True), oracle_solid_gpu(ref, info, removed, morton),
                f"ico8@512 removed triangles, morton={morton}")
    # the whole unfiltered mesh (the benchmark's solid tables)
    assert_same(engine_table(info, ico8, morton, True), want, f"ico8@512 full mesh, morton={morton}")


def near_x_parallel_soup(seed, n, g):
    """Triangles whose plane nearly contains the x axis (|n.x| log-uniform in [1e-7, 2e-2]): the
    solid xmax divides a cancelling sum by n.x.  Equilateral, edges log-uniform 0.5 to 32 voxels,
    centres uniform in the unit cube; mixed 1:1 with an ordinary soup of the same sizes."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3))
    s = np.exp(rng.uniform(np.log(1e-7), np.log(2e-2), n)) * rng.choice([-1.0, 1.0], n)
    a = rng.uniform(0, 2 * np.pi, n)
    nrm = np.stack([s, np.cos(a), np.sin(a)], 1)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    ex = np.array([1.0, 0.0, 0.0])
    u = ex - (nrm @ ex)[:, None] * nrm
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    w = np.cross(nrm, u)
    L = np.exp(rng.uniform(np.log(0.5 / g), np.log(32.0 / g), n))
    phi = rng.uniform(0, 2 * np.pi, n)
    verts = [c + (L / np.sqrt(3))[:, None] * (np.cos(phi + k * 2 * np.pi / 3)[:, None] * u +
                                              np.sin(phi + k * 2 * np.pi / 3)[:, None] * w) for k in range(3)]
    par = np.concatenate(verts, 1).astype(np.float32)
    other = meshgen.soup(seed + 1, n=n, lmin=0.5 / g, lmax=32.0 / g)
    return np.ascontiguousarray(np.concatenate([par, other]))


@pytest.mark.parametrize("morton", [False, True])
def test_near_x_parallel_soup_1024_solid(ref, morton):
    tris = near_x_parallel_soup(5, 20_000, 1024)
    info = cv.make_voxinfo(tris, 1024)
    want, removed = composed_solid(ref, info, tris, morton)
    assert removed.shape[0] > 15_000
    assert_same(engine_table(info, tris, morton, True), want, f"near-x-parallel soup @1024^3, morton={morton}")


# ---- the 256-mesh uneven mix as one plan ---------------------------------------------------------

def test_mix256_plan_vs_reference_kernels(ref):
    specs = meshgen.batch_mix(0, 256)  # the benchmark's mix
    meshes = [s.build() for s in specs]
    infos = [cv.make_voxinfo(m, s.gridsize) for s, m in zip(specs, meshes)]
    tris = [_dev(m) for m in meshes]
    tables = [torch.full((cv.table_words(i) + GUARD,), 0x5A5A5A5A, dtype=torch.int32, device="cuda")
              for i in infos]
    for t, i in zip(tables, infos):
        t[cv.table_words(i):] = 0
    jobs = [cv.Job(i, t, tb, s.morton, s.solid) for s, i, t, tb in zip(specs, infos, tris, tables)]
    plan = cv.Plan(jobs, clear_tables=True)  # clears the dirty tables inside the graph
    plan.launch()
    torch.cuda.synchronize()
    cv.device_status()
    n_removed = 0
    for k, (s, m, i, tb) in enumerate(zip(specs, meshes, infos, tables)):
        got = tb.cpu().numpy().view(np.uint32)
        if s.solid:
            want, removed = composed_solid(ref, i, m, s.morton)
            n_removed += removed.shape[0]
        else:
            want = reference_table(ref, i, m, s.morton, False)
        assert_same(got, want, f"mix mesh {k} ({s.kind}, {m.shape[0]} tris, g={s.gridsize}, "
                               f"solid={s.solid}, morton={s.morton})")
    del plan
