"""Host-buffer plans (cvx_plan_create_host): the round trip of the reference's main() -- triangles
up from host memory, voxelize, table back (src/main.cpp:209-222) -- as one graph, with the
triangles uploaded in chunks that are voxelized as they land.

Every table a plan copies back must be bit-identical to the same job run alone through
cvx_voxelize / cvx_voxelize_solid (which the parity tests pin to the reference kernels), for any
chunk count, on every replay, with tables that start dirty.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from cuda_voxelizer_gb300 import api as cv  # noqa: E402
from cuda_voxelizer_gb300 import meshgen  # noqa: E402

pytestmark = pytest.mark.gpu

MODES = [(False, False), (True, False), (False, True), (True, True)]  # (morton, solid)
GARBAGE = 0x5A5A5A5A


def _alone(info, tris, morton, solid):
    t = torch.from_numpy(np.ascontiguousarray(tris, dtype=np.float32).reshape(-1)).cuda()
    table = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    (cv.voxelize_solid if solid else cv.voxelize)(info, t, table, morton)
    torch.cuda.synchronize()
    return table.cpu()


def _shared_upload_jobs(tris, g):
    """The four modes over one mesh: one upload serves every job."""
    info = cv.make_voxinfo(tris, g)
    h_tris = torch.from_numpy(tris.reshape(-1).copy()).pin_memory()
    d_tris = torch.empty(h_tris.numel(), dtype=torch.float32, device="cuda")
    jobs = []
    for morton, solid in MODES:
        W = cv.table_words(info)
        jobs.append(cv.HostJob(info, h_tris, d_tris,
                               torch.full((W,), GARBAGE, dtype=torch.int32).pin_memory(),
                               torch.full((W,), GARBAGE, dtype=torch.int32, device="cuda"), morton, solid))
    return info, jobs


@pytest.mark.parametrize("n_chunks", [0, 1, 2, 3, 4, 64])
def test_four_modes_one_upload_match_plain_calls(n_chunks):
    tris = meshgen.icosphere(2, level=6)  # 81,920 triangles: 640 tiles, ragged over 3 and 64 chunks
    info, jobs = _shared_upload_jobs(tris, 256)
    plan = cv.HostPlan(jobs, n_chunks=n_chunks)
    # every chunk's surface launches (classify + rows per job) and the two solid jobs' passes
    assert plan.kernel_nodes() >= 2 * n_chunks + 3
    for _ in range(2):  # replays: each launch clears and recomputes every table
        plan.launch()
        torch.cuda.synchronize()
        for (morton, solid), j in zip(MODES, jobs):
            want = _alone(info, tris, morton, solid)
            assert torch.equal(j.h_table, want), f"morton={morton} solid={solid}: {int((j.h_table != want).sum())} words"
    plan.close()


def test_small_mesh_with_more_chunks_than_tiles():
    tris = meshgen.torus(5)  # 9,216 triangles = 36 tiles; 64 chunks leave most chunks empty
    info, jobs = _shared_upload_jobs(tris, 64)
    with_plan = cv.HostPlan(jobs, n_chunks=64)
    with_plan.launch()
    torch.cuda.synchronize()
    for (morton, solid), j in zip(MODES, jobs):
        assert torch.equal(j.h_table, _alone(info, tris, morton, solid))


def test_many_meshes_each_its_own_upload():
    specs = [s for s in meshgen.batch_mix(11, 64) if s.n_triangles <= 80_000][:10]
    assert {s.solid for s in specs} == {False, True}
    jobs, meshes = [], []
    for s in specs:
        tris = s.build()
        info = cv.make_voxinfo(tris, s.gridsize)
        W = cv.table_words(info)
        h = torch.from_numpy(tris.reshape(-1).copy()).pin_memory()
        jobs.append(cv.HostJob(info, h, torch.empty(h.numel(), dtype=torch.float32, device="cuda"),
                               torch.full((W,), GARBAGE, dtype=torch.int32).pin_memory(),
                               torch.full((W,), GARBAGE, dtype=torch.int32, device="cuda"), s.morton, s.solid))
        meshes.append(tris)
    plan = cv.HostPlan(jobs, n_chunks=4)
    plan.launch()
    torch.cuda.synchronize()
    for s, j, tris in zip(specs, jobs, meshes):
        assert torch.equal(j.h_table, _alone(j.info, tris, s.morton, s.solid)), str(s)


def test_replay_reads_the_host_triangles_again():
    a = meshgen.icosphere(3, level=5)
    b = meshgen.icosphere(4, level=5)
    lo = np.minimum(a.reshape(-1, 3).min(0), b.reshape(-1, 3).min(0))
    hi = np.maximum(a.reshape(-1, 3).max(0), b.reshape(-1, 3).max(0))
    clo, chi = cv.create_mesh_bbox_cube(lo, hi)
    info = cv.make_info(clo, chi, 128, a.shape[0])
    h_tris = torch.from_numpy(a.reshape(-1).copy()).pin_memory()
    d_tris = torch.empty(h_tris.numel(), dtype=torch.float32, device="cuda")
    W = cv.table_words(info)
    jobs = [cv.HostJob(info, h_tris, d_tris, torch.zeros(W, dtype=torch.int32).pin_memory(),
                       torch.zeros(W, dtype=torch.int32, device="cuda"), m, s) for m, s in MODES]
    plan = cv.HostPlan(jobs)
    plan.launch()
    torch.cuda.synchronize()
    h_tris.copy_(torch.from_numpy(b.reshape(-1)))
    plan.launch()
    torch.cuda.synchronize()
    for (morton, solid), j in zip(MODES, jobs):
        assert torch.equal(j.h_table, _alone(info, b, morton, solid))


def test_empty_mesh_gives_a_zero_table():
    info = cv.make_info((0, 0, 0), (1, 1, 1), 64, 0)
    W = cv.table_words(info)
    jobs = [cv.HostJob(info, None, None, torch.full((W,), GARBAGE, dtype=torch.int32).pin_memory(),
                       torch.full((W,), GARBAGE, dtype=torch.int32, device="cuda"), m, s) for m, s in MODES]
    plan = cv.HostPlan(jobs)
    plan.launch()
    torch.cuda.synchronize()
    for j in jobs:
        assert int(j.h_table.count_nonzero()) == 0


def test_rejects_pageable_host_memory_and_conflicting_uploads():
    tris = meshgen.torus(1)
    info = cv.make_voxinfo(tris, 64)
    W = cv.table_words(info)
    d_tris = torch.empty(tris.size, dtype=torch.float32, device="cuda")
    d_tab = torch.zeros(W, dtype=torch.int32, device="cuda")
    pinned = torch.from_numpy(tris.reshape(-1).copy()).pin_memory()
    with pytest.raises(cv.CvxError, match="page-locked"):
        cv.HostPlan([cv.HostJob(info, np.ascontiguousarray(tris.reshape(-1)), d_tris,
                                torch.zeros(W, dtype=torch.int32).pin_memory(), d_tab)])
    with pytest.raises(cv.CvxError, match="page-locked"):
        cv.HostPlan([cv.HostJob(info, pinned, d_tris, np.zeros(W, np.uint32), d_tab)])
    other = torch.from_numpy(tris.reshape(-1).copy()).pin_memory()
    d_tab2 = torch.zeros(W, dtype=torch.int32, device="cuda")
    with pytest.raises(cv.CvxError, match="different upload"):
        cv.HostPlan([cv.HostJob(info, pinned, d_tris, torch.zeros(W, dtype=torch.int32).pin_memory(), d_tab),
                     cv.HostJob(info, other, d_tris, torch.zeros(W, dtype=torch.int32).pin_memory(), d_tab2)])


def test_two_plans_in_flight_on_two_streams():
    """Back-to-back steps on two host plans launched on their own streams in turn (the e2e form of
    the benchmark): each plan owns its counters, queues and flip tables, so the two round trips may
    overlap and each must still return its own tables exactly.  Different meshes and grids per plan
    make any shared state show."""
    slots = []
    for seed, level, g in ((3, 5, 128), (4, 6, 256)):
        tris = meshgen.icosphere(seed, level=level)
        info, jobs = _shared_upload_jobs(tris, g)
        slots.append((tris, info, jobs, cv.HostPlan(jobs, n_chunks=2), torch.cuda.Stream()))
    main = torch.cuda.current_stream()
    start = torch.cuda.Event()
    start.record(main)
    for *_, s in slots:
        s.wait_event(start)
    for k in range(8):
        plan, s = slots[k % 2][3:]
        plan.launch(s)
    for *_, s in slots:
        main.wait_stream(s)
    torch.cuda.synchronize()
    for tris, info, jobs, plan, _ in slots:
        for (morton, solid), j in zip(MODES, jobs):
            want = _alone(info, tris, morton, solid)
            assert torch.equal(j.h_table, want), f"morton={morton} solid={solid}: {int((j.h_table != want).sum())} words"
        plan.close()


def test_host_pipeline_slot_results_as_they_complete():
    """cv.HostPipeline: submit() rotates over the slots; after wait(slot) that slot's host tables
    hold its round trip's result while the other slots' round trips may still run."""
    meshes, slot_jobs = [], []
    for seed, level, g in ((5, 5, 64), (6, 6, 128), (7, 5, 256)):
        tris = meshgen.icosphere(seed, level=level)
        info, jobs = _shared_upload_jobs(tris, g)
        meshes.append((tris, info))
        slot_jobs.append(jobs)
    pipe = cv.HostPipeline(slot_jobs, n_chunks=2)
    assert pipe.slots == 3 and pipe.kernel_nodes() >= 2 * 2 + 3
    want = [[_alone(info, tris, m, s) for m, s in MODES] for tris, info in meshes]
    pipe.begin()
    order = [pipe.submit() for _ in range(3)]
    assert order == [0, 1, 2]
    for k in range(9):
        slot = k % 3
        pipe.wait(slot)
        for (morton, solid), j, w in zip(MODES, slot_jobs[slot], want[slot]):
            assert torch.equal(j.h_table, w), f"slot {slot} morton={morton} solid={solid}"
            j.h_table.fill_(GARBAGE)  # consumed: the next round trip must write it all again
        assert pipe.submit() == slot
    pipe.end()
    torch.cuda.synchronize()
    pipe.close()
