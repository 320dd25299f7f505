"""Named workloads for kernel profiling: ``python -m cuda_voxelizer_gb300.profile_cases <case>``.

Each case builds its seeded synthetic input, runs the engine once to warm up and then ``--reps``
more times, synchronising after each, so that a profiler can skip the warm-up launches and capture
the ones after.  Cases:

  ico8        displaced icosphere, 8 subdivisions (1,310,720 triangles) at 512^3, four calls:
              surface linear, surface Morton, solid linear, solid Morton
  soup        2,000,000-triangle soup (edges log-uniform in [0.25, 512] voxels) at 1024^3, surface
  batch       the 256-mesh uneven mix (triangle counts 1k-500k, grids 64-512, 3:1 surface:solid,
              1:1 linear:Morton) as one cvx_voxelize_batch
  batch_g512  the surface meshes of that mix gridded at 512^3, as one batch
  io          a random 1024^3 table transcoded linear -> Morton -> linear, then the 512^3 solid
              icosphere's binvox payload and voxel list
"""
from __future__ import annotations

import argparse

import torch

from . import api as cv
from . import meshgen

MODES = [(False, False), (True, False), (False, True), (True, True)]  # (morton, solid)


def _table(info):
    return torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")


def case_ico8():
    tris = meshgen.icosphere(0, level=8)
    info = cv.make_voxinfo(tris, 512)
    d = torch.from_numpy(tris.reshape(-1)).cuda()
    tabs = [_table(info) for _ in MODES]

    def run():
        for (morton, solid), tab in zip(MODES, tabs):
            tab.zero_()
            (cv.voxelize_solid if solid else cv.voxelize)(info, d, tab, morton)
    return run


def case_soup():
    tris = meshgen.soup(0, n=2_000_000)
    info = cv.make_voxinfo(tris, 1024)
    d = torch.from_numpy(tris.reshape(-1)).cuda()
    tab = _table(info)

    def run():
        tab.zero_()
        cv.voxelize(info, d, tab)
    return run


def _mix_jobs(select):
    jobs = []
    for s in meshgen.batch_mix(0, 256):
        if not select(s):
            continue
        t = s.build()
        info = cv.make_voxinfo(t, s.gridsize)
        jobs.append(cv.Job(info, torch.from_numpy(t.reshape(-1)).cuda(), _table(info), s.morton, s.solid))
    return jobs


def case_batch():
    jobs = _mix_jobs(lambda s: True)

    def run():
        for j in jobs:
            j.table.zero_()
        cv.voxelize_batch(jobs)
    return run


def case_batch_g512():
    jobs = _mix_jobs(lambda s: not s.solid and s.gridsize == 512)

    def run():
        for j in jobs:
            j.table.zero_()
        cv.voxelize_batch(jobs)
    return run


def case_io():
    gen = torch.Generator(device="cuda").manual_seed(1)
    tab = torch.randint(-2 ** 31, 2 ** 31 - 1, (1024 ** 3 // 32,), dtype=torch.int32, device="cuda", generator=gen)
    tris = meshgen.icosphere(0, level=8)
    info = cv.make_voxinfo(tris, 512)
    t512 = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    cv.voxelize_solid(info, torch.from_numpy(tris.reshape(-1)).cuda(), t512)

    def run():
        m = cv.transcode(tab, 1024, True)
        cv.transcode(m, 1024, False)
        cv.encode_binvox(info, t512)
        cv.encode_voxel_list(info, t512)
    return run


CASES = {"ico8": case_ico8, "soup": case_soup, "batch": case_batch, "batch_g512": case_batch_g512, "io": case_io}


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("case", choices=sorted(CASES))
    p.add_argument("--reps", type=int, default=1)
    a = p.parse_args(argv)
    run = CASES[a.case]()
    for _ in range(1 + a.reps):
        run()
        torch.cuda.synchronize()
    cv.device_status()
    print(f"{a.case}: {1 + a.reps} runs done")


if __name__ == "__main__":
    main()
