"""Autotuner for the engine's bin thresholds (cvx_tuning), with a per-device cache.

The thresholds decide which triangles a classify kernel finishes inside its CTA and which it
queues for the cooperative kernels: ``small_vox`` (surface: triangles whose grid bounding box
holds at most this many voxels are tested voxel by voxel in the classify kernel) and
``small_cols`` (solid: triangles with at most this many voxel-centre columns).  Results never
depend on them; only the time does.  ``autotune()`` times a fixed set of seeded workloads (sub-voxel
and few-voxel triangles at several grids, surface and solid, linear and Morton) for every candidate
pair, keeps the fastest, applies it with cvx_set_tuning and stores it in a JSON cache keyed by the
device name; ``load_cached()`` applies a cached choice without timing anything.

    python -m cuda_voxelizer_gb300.autotune            # tune device 0, print and cache the result
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

from . import api as cv
from . import meshgen

SMALL_VOX = (16, 32, 64, 128, 255)
SMALL_COLS = (4, 8, 16)
DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "cuda_voxelizer_gb300", "tuning.json")


def _device_key(device: int) -> str:
    import torch
    p = torch.cuda.get_device_properties(device)
    return f"{p.name} sm_{p.major}{p.minor} {p.multi_processor_count}SM"


def _workloads(torch):
    """(name, info, device triangles, solid, morton) of the tuning set."""
    out = []
    for name, tris, g in (("ico7_g256", meshgen.icosphere(11, level=7), 256),
                          ("ico6_g512", meshgen.icosphere(12, level=6), 512),
                          ("torus_g128", meshgen.torus(13, nu=384, nv=192), 128)):
        info = cv.make_voxinfo(tris, g)
        d = torch.from_numpy(tris.reshape(-1)).cuda()
        for solid in (False, True):
            for morton in (False, True):
                out.append((f"{name}_{'solid' if solid else 'surf'}_{'mor' if morton else 'lin'}", info, d, solid,
                            morton))
    return out


def _time_all(torch, work, tables, reps):
    stream = torch.cuda.current_stream()
    total = 0.0
    for (name, info, d, solid, morton), tab in zip(work, tables):
        f = cv.voxelize_solid if solid else cv.voxelize
        tab.zero_()
        f(info, d, tab, morton)
        best = float("inf")
        for _ in range(reps):
            tab.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            f(info, d, tab, morton)
            b.record(stream)
            b.synchronize()
            best = min(best, a.elapsed_time(b))
        total += best
    return total


def autotune(device: int = 0, cache_path: str | None = DEFAULT_CACHE, reps: int = 5, verbose: bool = False) -> dict:
    """Times every (small_vox, small_cols) candidate, applies and caches the fastest."""
    import torch
    torch.cuda.set_device(device)
    work = _workloads(torch)
    tables = [torch.empty(cv.table_words(info), dtype=torch.int32, device="cuda") for _, info, _, _, _ in work]
    before = cv.get_tuning(device)
    results = []
    t0 = time.perf_counter()
    for sv in SMALL_VOX:
        for sc in SMALL_COLS:
            cv.set_tuning(device, small_vox=sv, small_cols=sc)
            ms = _time_all(torch, work, tables, reps)
            results.append({"small_vox": sv, "small_cols": sc, "ms": ms})
            if verbose:
                print(f"small_vox={sv:3d} small_cols={sc:2d}: {ms:.3f} ms", flush=True)
    best = min(results, key=lambda r: r["ms"])
    cv.set_tuning(device, small_vox=best["small_vox"], small_cols=best["small_cols"])
    out = {"device": _device_key(device), "small_vox": best["small_vox"], "small_cols": best["small_cols"],
           "ms": best["ms"], "default": before, "default_ms": next(
               (r["ms"] for r in results if r["small_vox"] == before["small_vox"] and r["small_cols"] ==
                before["small_cols"]), None), "candidates": results, "seconds": time.perf_counter() - t0}
    if cache_path:
        cache = {}
        if os.path.exists(cache_path):
            try:
                with open(cache_path) as f:
                    cache = json.load(f)
            except (OSError, ValueError):
                cache = {}
        cache[out["device"]] = {"small_vox": out["small_vox"], "small_cols": out["small_cols"]}
        os.makedirs(os.path.dirname(cache_path), exist_ok=True)
        with open(cache_path, "w") as f:
            json.dump(cache, f, indent=1)
    return out


def load_cached(device: int = 0, cache_path: str = DEFAULT_CACHE) -> dict | None:
    """Applies this device's cached thresholds, if any; returns them (None when not cached)."""
    try:
        with open(cache_path) as f:
            entry = json.load(f).get(_device_key(device))
    except (OSError, ValueError):
        return None
    if not entry:
        return None
    cv.set_tuning(device, small_vox=int(entry["small_vox"]), small_cols=int(entry["small_cols"]))
    return entry


if __name__ == "__main__":
    r = autotune(verbose=True)
    print(json.dumps({k: v for k, v in r.items() if k != "candidates"}))
