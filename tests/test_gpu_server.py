"""The voxelization server (cvx_server_*): continuous batching under a device-memory budget.

Every result the server returns must be bit-identical to the same request run alone through
cvx_voxelize / cvx_voxelize_solid (which the parity tests pin to the reference kernels), whatever
batch it landed in and whatever ran beside it.  Admission must keep the arena within its budget and
refuse requests that could never fit.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from cuda_voxelizer_gb300 import api as cv  # noqa: E402
from cuda_voxelizer_gb300 import meshgen  # noqa: E402

pytestmark = pytest.mark.gpu

GARBAGE = 0x5A5A5A5A  # output buffers start dirty: the server must clear each table itself


def _mesh_requests(n, seed, max_tris):
    out = []
    for spec in meshgen.batch_mix(seed, 16 * n):
        if spec.n_triangles <= max_tris:
            out.append(spec)
        if len(out) == n:
            break
    return out


def _host(spec):
    tris = spec.build()
    info = cv.make_voxinfo(tris, spec.gridsize)
    h_tris = torch.from_numpy(tris.reshape(-1).copy()).pin_memory()
    table = torch.full((cv.table_words(info),), GARBAGE, dtype=torch.int32).pin_memory()
    return info, h_tris, table


def _alone(info, h_tris, morton, solid):
    t = h_tris.cuda()
    table = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    (cv.voxelize_solid if solid else cv.voxelize)(info, t, table, morton)
    torch.cuda.synchronize()
    return table.cpu()


def test_server_results_identical_alone_and_in_the_mix():
    specs = _mesh_requests(32, seed=3, max_tris=60_000)
    assert {s.solid for s in specs} == {False, True} and {s.morton for s in specs} == {False, True}
    host = [_host(s) for s in specs]
    with cv.Server(memory_budget_bytes=1 << 30, max_batch=8, max_inflight=3) as srv:
        ids = [srv.submit(info, t, tab, s.morton, s.solid) for s, (info, t, tab) in zip(specs, host)]
        lat = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st["completed"] == len(specs) and st["pending"] == 0 and st["memory_used"] == 0
    assert st["memory_peak"] <= st["memory_budget"]
    assert all(x > 0 for x in lat)
    for s, (info, t, tab) in zip(specs, host):
        want = _alone(info, t, s.morton, s.solid)
        assert torch.equal(tab, want), f"{s}: {int((tab != want).sum())} words differ from the request run alone"


def test_server_admission_keeps_the_budget():
    # 512^3 tables are 16 MiB each; a 40 MiB budget holds two such requests (with records) at a time.
    specs = [meshgen.MeshSpec("torus", 20 + i, 24, 512, bool(i % 3 == 0), bool(i % 2)) for i in range(8)]
    host = [_host(s) for s in specs]
    budget = 40 << 20
    with cv.Server(memory_budget_bytes=budget, max_batch=64, max_inflight=4) as srv:
        ids = [srv.submit(info, t, tab, s.morton, s.solid) for s, (info, t, tab) in zip(specs, host)]
        for i in ids:
            srv.wait(i)
        st = srv.stats()
    assert st["memory_peak"] <= budget
    assert st["batches"] >= 4, st  # memory, not max_batch, limited the batches
    for s, (info, t, tab) in zip(specs, host):
        assert torch.equal(tab, _alone(info, t, s.morton, s.solid)), s


def test_server_refuses_a_request_larger_than_the_budget():
    info, t, tab = _host(meshgen.MeshSpec("torus", 1, 16, 512, False, False))
    with cv.Server(memory_budget_bytes=8 << 20, max_batch=4, max_inflight=1) as srv:
        with pytest.raises(cv.CvxError) as e:
            srv.submit(info, t, tab)
        assert e.value.status == 3
        assert srv.stats()["completed"] == 0


def test_server_replay_stops_at_a_refused_request():
    """A replay whose third request cannot fit the budget returns its error after the two it had
    submitted completed (their latencies are written, the call does not hang), and the server
    serves the next call normally."""
    ok_info, ok_t, ok_tab = _host(meshgen.MeshSpec("torus", 1, 16, 64, False, False))
    big_info, big_t, big_tab = _host(meshgen.MeshSpec("torus", 1, 16, 512, False, False))
    pool = [cv.Server.request(ok_info, ok_t, ok_tab, False, False),
            cv.Server.request(big_info, big_t, big_tab, False, False)]
    with cv.Server(memory_budget_bytes=8 << 20, max_batch=4, max_inflight=1) as srv:
        with pytest.raises(cv.CvxError) as e:
            srv.replay(pool, np.array([0, 0, 1, 0]), np.zeros(4))
        assert e.value.status == 3
        assert srv.stats()["completed"] == 2
        lat = srv.replay(pool, np.array([0, 0]), np.zeros(2))
        assert np.all(lat > 0) and srv.stats()["completed"] == 4
    assert torch.equal(ok_tab, _alone(ok_info, ok_t, False, False))


def test_server_empty_mesh_returns_a_cleared_table():
    tris = np.zeros((0, 9), dtype=np.float32)
    info = cv.make_info((0, 0, 0), (1, 1, 1), 64, 0)
    tab = torch.full((cv.table_words(info),), GARBAGE, dtype=torch.int32).pin_memory()
    with cv.Server(memory_budget_bytes=16 << 20, max_batch=4, max_inflight=2) as srv:
        srv.wait(srv.submit(info, torch.from_numpy(tris.reshape(-1)), tab, False, True))
    assert int(tab.count_nonzero()) == 0


def test_server_open_loop_replay():
    specs = _mesh_requests(6, seed=5, max_tris=40_000)
    host = [_host(s) for s in specs]
    pool = [cv.Server.request(info, t, tab, s.morton, s.solid) for s, (info, t, tab) in zip(specs, host)]
    arrivals = meshgen.poisson_arrivals(3000.0, 0.03, seed=1)
    index = np.random.default_rng(2).integers(0, len(pool), size=len(arrivals))
    with cv.Server(memory_budget_bytes=1 << 30, max_batch=16, max_inflight=2) as srv:
        lat = srv.replay(pool, index, arrivals)
        st = srv.stats()
    assert len(lat) == len(arrivals) > 20 and np.all(lat > 0) and np.all(np.isfinite(lat))
    assert st["completed"] == len(arrivals)
    # the queue wait is part of the latency; the generator's own lateness is reported beside it
    assert 0 <= st["queue_p99_ms"] <= st["max_ms"]
    assert 0 <= st["replay_late_p99_ms"] <= st["replay_late_max_ms"]
    assert 0 < st["service_p50_ms"] <= st["service_p99_ms"] <= st["max_ms"]
    assert st["issue_p50_us"] > 0
    for s, (info, t, tab) in zip(specs, host):
        if np.any(index == specs.index(s)):
            assert torch.equal(tab, _alone(info, t, s.morton, s.solid)), s


def _read_device_words(ptr, words):
    """Copy `words` uint32 from a raw device address into a host tensor (through the CUDA runtime
    the library itself links)."""
    import ctypes
    rt = ctypes.CDLL("libcudart.so.13")
    out = torch.empty(words, dtype=torch.int32)
    rc = rt.cudaMemcpy(ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(ptr), ctypes.c_size_t(4 * words),
                       ctypes.c_int(2))  # cudaMemcpyDeviceToHost
    assert rc == 0
    return out


def test_server_device_resident_requests():
    """Triangles already on the device are read in place; a request without a host table keeps
    its table resident (inside the budget) until it is released."""
    specs = _mesh_requests(12, seed=8, max_tris=50_000)
    budget = 512 << 20
    with cv.Server(memory_budget_bytes=budget, max_batch=8, max_inflight=2) as srv:
        meshes = []
        for s in specs:
            tris = s.build()
            meshes.append((s, cv.make_voxinfo(tris, s.gridsize), torch.from_numpy(tris.reshape(-1)).cuda()))
        torch.cuda.synchronize()  # the server's streams do not order after torch's
        reqs = [(s, info, d, srv.submit(info, d, None, s.morton, s.solid)) for s, info, d in meshes]
        for s, info, d, rid in reqs:
            srv.wait(rid)
        used = srv.stats()["memory_used"]
        assert used >= sum(4 * cv.table_words(info) for _, info, _, _ in reqs)  # tables still held
        for s, info, d, rid in reqs:
            got = _read_device_words(srv.table(rid), cv.table_words(info))
            want = _alone(info, d.cpu(), s.morton, s.solid)
            assert torch.equal(got, want), s
            srv.release(rid)
        assert srv.stats()["memory_used"] == 0
        with pytest.raises(cv.CvxError):
            srv.table(reqs[0][3])  # released
