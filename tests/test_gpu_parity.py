"""GPU parity: the engine against the reference's own CUDA kernels and its CPU voxelizer.

* Bit-exact against the reference kernels voxelize_triangle / voxelize_triangle_solid
  (src/voxelize.cu:58, src/voxelize_solid.cu:73), compiled from the reference sources for sm_103a
  (oracle/build_ref.sh) and run by oracle/ref_gpu_runner.cu on the same device buffers: the
  golden meshes, the 64^3 torus, the 512^3 displaced icosphere (surface and solid, linear and
  Morton), triangle-size-stress soups at 1024^3, and edge cases (degenerate, grid-aligned,
  axis-aligned and out-of-bbox triangles, tiny / odd / non-cubic grids, empty meshes).
* Against the reference CPU voxelizer (the golden fixtures): every differing bit is counted and
  traced to a boundary tie (tests/tie_trace.py).  Tolerance: a difference is a tie when a predicate
  is within 1e-4 voxel (surface) / 1e-3 (solid column decision) of its boundary in float64.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle  # noqa: E402
from cuda_voxelizer_gb300 import api as cv  # noqa: E402
from cuda_voxelizer_gb300 import meshgen  # noqa: E402
from golden_data import arrays, manifest, mesh, table_keys  # noqa: E402
import tie_trace  # noqa: E402
from oracle.ref_safety import safe_triangles  # noqa: E402

pytestmark = pytest.mark.gpu

MODES = [(False, False), (True, False), (False, True), (True, True)]


@pytest.fixture(scope="module")
def ref():
    return oracle.RefGPU()


def _stream():
    return torch.cuda.current_stream().cuda_stream


GUARD = 256  # zero words after every table: a write past the end shows up as a difference


def run_engine(info, t_dev, morton, solid):
    table = torch.zeros(cv.table_words(info) + GUARD, dtype=torch.int32, device="cuda")
    (cv.voxelize_solid if solid else cv.voxelize)(info, t_dev, table, morton)
    return table


def run_ref(ref, info, t_dev, morton, solid):
    table = torch.zeros(cv.table_words(info) + GUARD, dtype=torch.int32, device="cuda")
    ref.voxelize(bytes(info), t_dev.data_ptr(), table.data_ptr(), morton, solid, _stream())
    return table


_SAFE = {}


def for_reference(tris, info, morton, solid):
    """The reference solid kernel writes outside its table for some near-x-parallel triangles
    (oracle/ref_safety.py); both implementations get the mesh without them."""
    if not solid:
        return tris, info
    import hashlib
    key = (hashlib.sha1(np.ascontiguousarray(tris).tobytes()).hexdigest(), bytes(info), bool(morton))
    if key not in _SAFE:
        _SAFE[key] = safe_triangles(tris, bytes(info), morton)
    keep = _SAFE[key]
    tris = np.ascontiguousarray(np.asarray(tris, dtype=np.float32).reshape(-1, 9)[keep])
    info = cv.VoxInfo.from_buffer_copy(bytes(info))
    info.n_triangles = int(tris.shape[0])
    return tris, info


def compare(ref, tris, info, morton, solid):
    tris, info = for_reference(tris, info, morton, solid)
    t = torch.from_numpy(np.ascontiguousarray(tris, dtype=np.float32).reshape(-1)).cuda()
    a = run_engine(info, t, morton, solid)
    b = run_ref(ref, info, t, morton, solid)
    torch.cuda.synchronize()
    cv.device_status()
    a = a.cpu().numpy().view(np.uint32)
    b = b.cpu().numpy().view(np.uint32)
    return a, b


def assert_same(a, b, what):
    d = np.nonzero(a != b)[0]
    pa = int(np.unpackbits(a.view(np.uint8)).sum())
    pb = int(np.unpackbits(b.view(np.uint8)).sum())
    assert d.size == 0, f"{what}: {d.size} words differ (engine {pa} bits, reference {pb} bits), first {d[:8]}"


def info_of(tris, g):
    return cv.make_voxinfo(tris, g)


# ---- bit-exact against the reference kernels ----------------------------------------------------

@pytest.mark.parametrize("name,key,morton,solid", table_keys())
def test_golden_meshes_vs_reference_kernels(ref, name, key, morton, solid):
    c = manifest()["cases"][name]
    info = cv.VoxInfo.from_buffer_copy(bytes.fromhex(c["voxinfo_hex"]))
    a, b = compare(ref, mesh(name), info, morton, solid)
    assert_same(a, b, key)


@pytest.mark.parametrize("morton,solid", MODES)
def test_torus_64(ref, morton, solid):
    t = meshgen.torus(0)
    a, b = compare(ref, t, info_of(t, 64), morton, solid)
    assert_same(a, b, "torus64")


@pytest.fixture(scope="module")
def ico8():
    return meshgen.icosphere(0, level=8)


@pytest.mark.parametrize("morton,solid", MODES)
def test_icosphere_512(ref, ico8, morton, solid):
    a, b = compare(ref, ico8, info_of(ico8, 512), morton, solid)
    assert_same(a, b, "ico8@512")


@pytest.mark.parametrize("seed,n", [(1, 20_000), (2, 200_000)])
def test_soup_1024(ref, seed, n):
    t = meshgen.soup(seed, n=n)
    a, b = compare(ref, t, info_of(t, 1024), False, False)
    assert_same(a, b, f"soup{n}@1024")


@pytest.mark.parametrize("solid", [False, True])
def test_soup_dense_512_solid_and_surface(ref, solid):
    t = meshgen.soup(3, n=30_000, lmin=0.5 / 512, lmax=0.2)
    a, b = compare(ref, t, info_of(t, 512), False, solid)
    assert_same(a, b, "soup30k@512")


def _adversarial(seed, g):
    rng = np.random.default_rng(seed)
    parts = []
    s = meshgen.soup(seed, n=3000, lmin=0.3 / g, lmax=0.4)
    parts.append(s)
    q = s[:500].copy()
    q = np.round(q * g * 2) / (g * 2)                  # vertices on voxel faces and centres
    parts.append(q)
    a = s[500:900].copy().reshape(-1, 3, 3)
    a[:, :, rng.integers(0, 3)] = a[:, :1, rng.integers(0, 3)]  # axis-aligned planes
    parts.append(a.reshape(-1, 9))
    d = s[900:1000].copy().reshape(-1, 3, 3)
    d[:50, 1] = d[:50, 0]                               # zero-area: repeated vertex
    d[50:, 2] = 0.5 * (d[50:, 0] + d[50:, 1])           # collinear
    parts.append(d.reshape(-1, 9))
    return np.concatenate(parts).astype(np.float32)


@pytest.mark.parametrize("g", [8, 37, 64, 100, 256])
@pytest.mark.parametrize("morton,solid", MODES)
def test_adversarial_vs_reference_kernels(ref, g, morton, solid):
    if morton and g & (g - 1):
        pytest.skip("Morton order needs a power-of-two grid")
    t = _adversarial(g, g)
    a, b = compare(ref, t, info_of(t, g), morton, solid)
    assert_same(a, b, f"adversarial g={g}")


def _random_case(seed):
    """One seeded random configuration: grid (cubic or not, 8 to 1024), mode, soup size and
    triangle-size range."""
    rng = np.random.default_rng(seed)
    cubic = rng.random() < 0.7
    g = int(rng.choice([8, 16, 32, 37, 64, 100, 128, 256, 512, 1024])) if cubic else None
    dims = (g, g, g) if cubic else tuple(int(x) for x in rng.integers(5, 300, 3))
    morton = bool(cubic and (g & (g - 1)) == 0 and rng.random() < 0.5)
    solid = bool(rng.random() < 0.5)
    gm = max(dims)
    t = meshgen.soup(int(rng.integers(1 << 30)), n=int(rng.integers(1, 40000)), lmin=0.3 / gm,
                     lmax=float(rng.choice([2, 8, 40, 200])) / gm).astype(np.float32)
    info = info_of(t, dims[0])
    for i in range(3):
        info.gridsize[i] = dims[i]
        info.unit[i] = np.float32((np.float32(info.bbox_max[i]) - np.float32(info.bbox_min[i])) / np.float32(dims[i]))
    return t, info, morton, solid


@pytest.mark.parametrize("seed", range(24))
def test_randomized_vs_reference_kernels(ref, seed):
    """Seeded random soups, grids and modes: per call and as a clearing plan over a dirty table,
    against the reference kernels (a sweep like this found the per-order contraction of
    get_x_coordinate)."""
    t, info, morton, solid = _random_case(1000 + seed)
    t, info = for_reference(t, info, morton, solid)
    d = torch.from_numpy(np.ascontiguousarray(t).reshape(-1)).cuda()
    W = cv.table_words(info)
    a = run_engine(info, d, morton, solid)
    b = run_ref(ref, info, d, morton, solid)
    c = torch.full((W + GUARD,), 0x5A5A5A5A, dtype=torch.int32, device="cuda")
    c[W:] = 0
    plan = cv.Plan([cv.Job(info, d, c, morton, solid)], clear_tables=True)
    plan.launch()
    torch.cuda.synchronize()
    cv.device_status()
    plan.close()
    dims = tuple(info.gridsize)
    assert torch.equal(a, b), f"{dims} morton={morton} solid={solid}: {int((a != b).sum())} words differ (call)"
    assert torch.equal(c, b), f"{dims} morton={morton} solid={solid}: {int((c != b).sum())} words differ (plan)"


@pytest.mark.parametrize("solid", [False, True])
def test_non_cubic_grid(ref, solid):
    t = meshgen.icosphere(4, level=4)
    info = cv.make_voxinfo(t, 64)
    info.gridsize[0], info.gridsize[1], info.gridsize[2] = 96, 64, 40
    for i, gdim in enumerate((96, 64, 40)):
        info.unit[i] = np.float32((np.float32(info.bbox_max[i]) - np.float32(info.bbox_min[i])) / np.float32(gdim))
    a, b = compare(ref, t, info, False, solid)
    assert_same(a, b, "non-cubic")


def _compare_on_device(ref, t, info, morton):
    """Engine vs reference kernel on tables too large to copy to the host: compared on the GPU."""
    d = torch.from_numpy(np.ascontiguousarray(t, dtype=np.float32).reshape(-1)).cuda()
    a = run_engine(info, d, morton, False)
    b = run_ref(ref, info, d, morton, False)
    torch.cuda.synchronize()
    cv.device_status()
    differ, set_words = int((a != b).sum()), int(a.count_nonzero())
    del a, b
    torch.cuda.empty_cache()
    return differ, set_words


@pytest.mark.parametrize("morton", [False, True])
def test_grid_2048_indices_above_32_bits(ref, morton):
    """At 2048^3 Morton codes and linear indices exceed 32 bits: the engine's 64-bit write path
    (grids up to 2^32 voxels and Morton grids up to 1024 use 32-bit index arithmetic)."""
    t = np.concatenate([meshgen.soup(7, n=30_000, lmin=0.3 / 2048, lmax=8 / 2048),
                        meshgen.soup(8, n=200, lmin=8 / 2048, lmax=40 / 2048)]).astype(np.float32)
    differ, set_words = _compare_on_device(ref, t, info_of(t, 2048), morton)
    assert differ == 0 and set_words > 0, f"{differ} words differ"


@pytest.mark.parametrize("morton", [False, True])
def test_solid_1024_large_triangles_both_orders(ref, morton):
    """A 1024^3 soup of large triangles, solid, in both orders.  The reference kernel contracts
    get_x_coordinate differently in its linear and Morton code (fma on the n.y term, on the n.z
    term), so on a few columns of this mesh its xmax differs by one voxel between the two orders;
    the engine follows each order."""
    t = meshgen.soup(616136667, n=35380, lmin=0.3 / 1024, lmax=200 / 1024).astype(np.float32)
    info = info_of(t, 1024)
    t, info = for_reference(t, info, morton, True)
    d = torch.from_numpy(np.ascontiguousarray(t).reshape(-1)).cuda()
    a = run_engine(info, d, morton, True)
    b = run_ref(ref, info, d, morton, True)
    torch.cuda.synchronize()
    cv.device_status()
    differ, set_words = int((a != b).sum()), int(a.count_nonzero())
    del a, b
    torch.cuda.empty_cache()
    assert differ == 0 and set_words > 0, f"{differ} words differ"


def _near_x_parallel(seed, n, g):
    """Triangles whose planes are nearly parallel to x (|n.x| log-uniform in [1e-5, 1e-2]), every
    vertex in z <= 0.45 of a unit-cube grid box."""
    rng = np.random.default_rng(seed)
    c = np.stack([rng.uniform(0.05, 0.95, n), rng.uniform(0.05, 0.95, n), rng.uniform(0.05, 0.40, n)], 1)
    size = np.exp(rng.uniform(np.log(0.5 / g), np.log(40 / g), n))
    nx = np.exp(rng.uniform(np.log(1e-5), np.log(1e-2), n)) * rng.choice([-1, 1], n)
    phi = rng.uniform(0, 2 * np.pi, n)
    nrm = np.stack([nx, np.sqrt(1 - nx * nx) * np.cos(phi), np.sqrt(1 - nx * nx) * np.sin(phi)], 1)
    a = np.cross(nrm, np.array([1.0, 0, 0]))
    a /= np.linalg.norm(a, axis=1)[:, None]
    b = np.cross(nrm, a)
    ang = rng.uniform(0, 2 * np.pi, (n, 3)) + np.array([0, 2.1, 4.2])
    v = c[:, None, :] + size[:, None, None] * (np.cos(ang)[..., None] * a[:, None, :] + np.sin(ang)[..., None] * b[:, None, :])
    v[..., 2] = np.clip(v[..., 2], 0.0, 0.45)
    v[..., :2] = np.clip(v[..., :2], 0.0, 1.0)
    return v.reshape(n, 9).astype(np.float32)


@pytest.mark.parametrize("g", [512, 1024])
def test_near_x_parallel_solid_linear(ref, g):
    """Solid voxelization where xmax is most sensitive to float32 rounding (|n.x| down to 1e-5,
    which the reference-safety filter drops elsewhere).  Safe for the reference kernel by
    construction: every triangle lies in z <= 0.45 of the grid, so a run past x = gx continues
    into following rows of the same table (more than g^2 / 2 rows follow any hit column)."""
    t = _near_x_parallel(100 * g, 20000, g)
    info = cv.make_info((0, 0, 0), (1, 1, 1), g, t.shape[0])
    d = torch.from_numpy(t.reshape(-1).copy()).cuda()
    a = run_engine(info, d, False, True)
    b = run_ref(ref, info, d, False, True)
    torch.cuda.synchronize()
    cv.device_status()
    differ = int((a != b).sum())
    del a, b
    torch.cuda.empty_cache()
    assert differ == 0, f"{differ} words differ"


def test_linear_grid_of_exactly_2_to_32_voxels(ref):
    """2048 x 2048 x 1024: the largest linear index is 2^32 - 1, the edge of the 32-bit path."""
    t = np.concatenate([meshgen.soup(9, n=30_000, lmin=0.3 / 2048, lmax=8 / 2048),
                        meshgen.soup(10, n=200, lmin=8 / 2048, lmax=40 / 2048)]).astype(np.float32)
    info = info_of(t, 2048)
    info.gridsize[2] = 1024
    info.unit[2] = np.float32((np.float32(info.bbox_max[2]) - np.float32(info.bbox_min[2])) / np.float32(1024))
    differ, set_words = _compare_on_device(ref, t, info, False)
    assert differ == 0 and set_words > 0, f"{differ} words differ"


@pytest.mark.parametrize("solid", [False, True])
def test_triangles_outside_bbox(ref, solid):
    """The caller's bbox covers only part of the mesh: surface clamps to the grid; solid columns
    whose row range runs past x = gx continue into the next rows, exactly as in the reference."""
    t = meshgen.icosphere(5, level=4)
    info = cv.make_voxinfo(t, 64)
    for i in range(3):  # shrink the box towards its low corner: many vertices beyond bbox_max
        info.bbox_max[i] = np.float32(info.bbox_min[i] + 0.7 * (info.bbox_max[i] - info.bbox_min[i]))
        info.unit[i] = np.float32((np.float32(info.bbox_max[i]) - np.float32(info.bbox_min[i])) / np.float32(64))
    # Solid: keep triangles whose columns lie in rows y, z <= 0.9 g, so that a row range running past
    # x = gx continues into a following row inside the table (past the table's end, and for columns
    # outside the grid, the reference writes out of bounds).
    lim = np.array(info.bbox_min[1:], np.float32) + 0.9 * (np.array(info.bbox_max[1:], np.float32) -
                                                            np.array(info.bbox_min[1:], np.float32))
    keep = np.all(t.reshape(-1, 3, 3)[:, :, 1:] >= np.array(info.bbox_min[1:], np.float32), axis=(1, 2))
    keep &= np.all(t.reshape(-1, 3, 3)[:, :, 1:] <= lim, axis=(1, 2))
    t = np.ascontiguousarray(t[keep]) if solid else t
    info.n_triangles = t.shape[0]
    a, b = compare(ref, t, info, False, solid)
    assert_same(a, b, "outside-bbox")


def test_empty_mesh():
    info = cv.make_info((0, 0, 0), (1, 1, 1), 32, 0)
    table = torch.zeros(cv.table_words(info) + GUARD, dtype=torch.int32, device="cuda")
    cv.voxelize(info, torch.zeros(9, device="cuda"), table)
    cv.voxelize_solid(info, torch.zeros(9, device="cuda"), table)
    torch.cuda.synchronize()
    assert int(table.abs().sum()) == 0


def test_accumulates_into_existing_table(ref):
    """Surface ORs into the caller's table and solid XORs into it, like the reference."""
    t0 = meshgen.torus(3)
    info0 = info_of(t0, 64)
    td0 = torch.from_numpy(t0.reshape(-1)).cuda()
    init = torch.randint(-2 ** 31, 2 ** 31 - 1, (cv.table_words(info0) + GUARD,), dtype=torch.int32, device="cuda")
    for solid in (False, True):
        t, info = for_reference(t0, info0, False, solid)
        td = torch.from_numpy(t.reshape(-1)).cuda() if solid else td0
        a = init.clone()
        b = init.clone()
        (cv.voxelize_solid if solid else cv.voxelize)(info, td, a, False)
        ref.voxelize(bytes(info), td.data_ptr(), b.data_ptr(), False, solid, _stream())
        torch.cuda.synchronize()
        assert torch.equal(a, b)


# ---- against the reference CPU voxelizer: differences are ties --------------------------------

@pytest.mark.parametrize("name,key,morton,solid", [k for k in table_keys() if not k[2]])
def test_cpu_differences_are_ties(name, key, morton, solid):
    c = manifest()["cases"][name]
    info = cv.VoxInfo.from_buffer_copy(bytes.fromhex(c["voxinfo_hex"]))
    tris = mesh(name)
    got = cv.voxelize_host(info, tris, morton=False, solid=solid)
    want = arrays()[key]
    bits = tie_trace.diff_bits(got, want)
    if bits.size == 0:
        return
    grid = np.frombuffer(bytes(info), np.uint32, 3, 24)
    x, y, z = tie_trace.linear_to_xyz(bits, grid, False)
    if not solid:
        m = tie_trace.surface_margin(tris, bytes(info), np.stack([x, y, z], 1))
        assert np.all(m < 1e-4), f"{key}: {bits.size} differing bits, untraced margins {np.sort(m)[-5:]}"
    else:
        rows = sorted(set(zip(y.tolist(), z.tolist())))
        m = tie_trace.solid_row_margin(tris, bytes(info), rows)
        assert np.all(m < 1e-3), f"{key}: {bits.size} differing bits in {len(rows)} rows, untraced {np.sort(m)[-5:]}"


# ---- batch, plan and caller-owned scratch give the same bits --------------------------------------

def _mixed_jobs():
    specs = [(meshgen.torus(10), 64, False, False), (meshgen.icosphere(11, 5), 128, True, False),
             (meshgen.icosphere(12, 4), 64, False, True), (meshgen.torus(13, nu=40, nv=20), 128, True, True),
             (meshgen.soup(14, n=5000, lmin=0.01, lmax=0.3), 256, False, False),
             (meshgen.icosphere(15, 6), 100, False, True)]
    jobs = []
    for t, g, morton, solid in specs:
        info = info_of(t, g)
        td = torch.from_numpy(t.reshape(-1)).cuda()
        jobs.append(cv.Job(info, td, torch.zeros(cv.table_words(info) + GUARD, dtype=torch.int32, device="cuda"),
                           morton, solid))
    return jobs


def test_batch_equals_single_calls():
    jobs = _mixed_jobs()
    cv.voxelize_batch(jobs)
    torch.cuda.synchronize()
    cv.device_status()
    for j in jobs:
        single = run_engine(j.info, j.triangles, j.morton, j.solid)
        torch.cuda.synchronize()
        assert torch.equal(single, j.table)


def test_plan_equals_single_calls_and_replays():
    """A clearing plan starts every table from zero whatever it held: surface tables are zeroed by
    their lane, solid tables are overwritten word by word by their resolve (the guard words after
    each table must stay zero)."""
    jobs = _mixed_jobs()
    for j in jobs:
        j.table[:cv.table_words(j.info)] = 0x5A5A5A5A  # dirty tables
    plan = cv.Plan(jobs, clear_tables=True)
    for _ in range(3):
        plan.launch()
    torch.cuda.synchronize()
    for j in jobs:
        single = run_engine(j.info, j.triangles, j.morton, j.solid)
        torch.cuda.synchronize()
        assert torch.equal(single, j.table)
    plan.close()


def test_plan_kernel_nodes():
    """cvx_plan_kernel_nodes counts the graph's kernel launches: a clearing plan of one surface job
    is its lane's clear, classify and rows kernels; one linear solid job (its table overwritten, not
    cleared) is classify, columns and resolve; both together run as two lanes of three each."""
    t = meshgen.torus(40)
    info = info_of(t, 64)
    td = torch.from_numpy(t.reshape(-1)).cuda()
    a = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    b = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    for jobs, want in (([cv.Job(info, td, a, False, False)], 3), ([cv.Job(info, td, b, False, True)], 3),
                       ([cv.Job(info, td, a, False, False), cv.Job(info, td, b, False, True)], 6)):
        plan = cv.Plan(jobs, clear_tables=True)
        assert plan.kernel_nodes() == want
        plan.launch()
        torch.cuda.synchronize()
        plan.close()
    assert torch.equal(a, run_engine(info, td, False, False)[:cv.table_words(info)])
    assert torch.equal(b, run_engine(info, td, False, True)[:cv.table_words(info)])


def test_plan_jobs_sharing_a_table_accumulate():
    """Jobs whose tables share words accumulate into them as repeated reference calls would: a
    clearing plan zeroes the shared table once, the surface job ORs, the solid job XORs (the plan
    runs such jobs one after another instead of on concurrent lanes)."""
    t1, t2 = meshgen.torus(30), meshgen.icosphere(31, 5)
    info1, info2 = info_of(t1, 64), info_of(t2, 64)
    d1, d2 = torch.from_numpy(t1.reshape(-1)).cuda(), torch.from_numpy(t2.reshape(-1)).cuda()
    W = cv.table_words(info1)
    shared = torch.full((W + GUARD,), 0x5A5A5A5A, dtype=torch.int32, device="cuda")
    shared[W:] = 0
    other = torch.full((W + GUARD,), 0x5A5A5A5A, dtype=torch.int32, device="cuda")
    other[W:] = 0
    jobs = [cv.Job(info1, d1, shared, False, False), cv.Job(info2, d2, shared, False, True),
            cv.Job(info2, d2, other, False, True)]
    plan = cv.Plan(jobs, clear_tables=True)
    for _ in range(2):
        plan.launch()
    torch.cuda.synchronize()
    cv.device_status()
    surf = run_engine(info1, d1, False, False)
    solid = run_engine(info2, d2, False, True)
    torch.cuda.synchronize()
    assert torch.equal(shared, surf ^ solid)
    assert torch.equal(other, solid)
    plan.close()


@pytest.mark.parametrize("solid", [False, True])
def test_stream_release_frees_scratch_and_calls_still_work(solid):
    """cvx_stream_release frees a stream's scratch; later calls on the stream allocate it afresh
    and give the same table."""
    t = meshgen.icosphere(21, level=5)
    info = info_of(t, 128)
    td = torch.from_numpy(t.reshape(-1)).cuda()
    s = torch.cuda.Stream()
    tables = []
    for _ in range(2):
        tab = torch.zeros(cv.table_words(info) + GUARD, dtype=torch.int32, device="cuda")
        with torch.cuda.stream(s):
            (cv.voxelize_solid if solid else cv.voxelize)(info, td, tab, True, stream=s)
        cv.stream_release(s)  # synchronizes the stream, then frees
        tables.append(tab)
    assert torch.equal(tables[0], tables[1]) and int(tables[0].count_nonzero()) > 0
    cv.stream_release(torch.cuda.Stream())  # a stream the library never used


def test_plan_without_clearing_keeps_xor_semantics():
    """A plan that does not clear its tables ORs (surface) and XORs (solid) into them like plain
    calls: launched twice, surface tables are unchanged and solid tables return to zero."""
    jobs = _mixed_jobs()
    for j in jobs:
        j.table.zero_()
    plan = cv.Plan(jobs, clear_tables=False)
    plan.launch()
    torch.cuda.synchronize()
    once = [j.table.clone() for j in jobs]
    for j, t in zip(jobs, once):
        assert torch.equal(t, run_engine(j.info, j.triangles, j.morton, j.solid))
    plan.launch()
    torch.cuda.synchronize()
    for j, t in zip(jobs, once):
        if j.solid:
            assert int(j.table.count_nonzero()) == 0
        else:
            assert torch.equal(j.table, t)
    plan.close()


@pytest.mark.parametrize("solid", [False, True])
def test_caller_workspace_equals_internal(solid):
    t = meshgen.soup(20, n=20000, lmin=0.002, lmax=0.3)
    info = info_of(t, 256)
    td = torch.from_numpy(t.reshape(-1)).cuda()
    ws = torch.empty(cv.workspace_size(info, solid), dtype=torch.uint8, device="cuda")
    a = torch.zeros(cv.table_words(info) + GUARD, dtype=torch.int32, device="cuda")
    cv.voxelize_ws(info, td, a, ws, morton_code=False, solid=solid)
    b = run_engine(info, td, False, solid)
    torch.cuda.synchronize()
    assert torch.equal(a, b)


def test_repeated_calls_are_identical():
    t = meshgen.icosphere(21, 6)
    info = info_of(t, 256)
    td = torch.from_numpy(t.reshape(-1)).cuda()
    for morton in (False, True):
        for solid in (False, True):
            outs = [run_engine(info, td, morton, solid) for _ in range(3)]
            torch.cuda.synchronize()
            assert torch.equal(outs[0], outs[1]) and torch.equal(outs[0], outs[2])


@pytest.mark.parametrize("solid", [False, True])
def test_mesh_above_one_launch_is_split_exactly(solid):
    """A mesh of more than 2^24 - 1 triangles runs as several launch groups on one table; by
    linearity (surface ORs, solid XORs per triangle) it must equal the OR / XOR of its halves."""
    rng = np.random.default_rng(21)
    n = (1 << 24) + 12_345
    base = meshgen.icosphere(8, level=7)  # 327,680 triangles
    reps = n // base.shape[0] + 1
    tris = np.concatenate([base + np.tile(rng.normal(0, 0.02, 3), 3).astype(np.float32) for _ in range(reps)])[:n]
    info = cv.make_voxinfo(tris, 256)
    d = torch.from_numpy(tris.reshape(-1)).cuda()
    f = cv.voxelize_solid if solid else cv.voxelize
    whole = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    f(info, d, whole)
    halves = []
    h = n // 2
    for a, b in ((0, h), (h, n)):
        ic = cv.VoxInfo.from_buffer_copy(bytes(info))
        ic.n_triangles = b - a
        t = torch.zeros_like(whole)
        f(ic, d[9 * a:9 * b], t)
        halves.append(t)
    want = (halves[0] ^ halves[1]) if solid else (halves[0] | halves[1])
    torch.cuda.synchronize()
    assert torch.equal(whole, want)
    assert int(whole.count_nonzero()) > 0


@pytest.mark.parametrize("morton", [False, True])
def test_non_finite_vertices_vs_reference_kernel(ref, morton):
    """Triangles with NaN or infinite vertices, mixed into a normal mesh: the reference kernel's
    conversions (NaN -> 0, +-inf saturated, then clamped to the grid) and its predicates on NaN
    (every comparison false) decide which voxels are set; the engine must set the same ones.
    Surface only: the reference solid kernel writes outside its table for such input."""
    t = meshgen.icosphere(7, level=3).copy()
    info = info_of(t, 64)
    bad = t[:12].copy().reshape(-1, 3, 3)
    bad[0, 0, 0] = np.nan
    bad[1, 1, :] = np.nan
    bad[2, :, :] = np.nan
    bad[3, 2, 1] = np.inf
    bad[4, 0, 2] = -np.inf
    bad[5, 1, 0] = np.inf
    bad[5, 2, 0] = -np.inf
    bad[6, 0, :] = np.inf
    t2 = np.concatenate([t, bad.reshape(-1, 9)[:7]]).astype(np.float32)
    info.n_triangles = t2.shape[0]
    a, b = compare(ref, t2, info, morton, False)
    assert_same(a, b, "non-finite")
