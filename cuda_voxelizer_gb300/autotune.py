"""Autotuner for the engine's tuning knobs (cvx_tuning), with a per-device cache.

The knobs decide where a triangle's work goes; results never depend on them, only the time does:
``small_vox`` (surface: triangles whose grid bounding box holds at most this many voxels are tested
voxel by voxel in the classify kernel), ``small_cols`` (solid: triangles with at most this many
voxel-centre columns stay in the classify kernel) and ``brick_pairs`` (surface, grids of 2^29+
voxels: (brick, triangle) pairs per triangle the shared-memory brick rasterizer may use; 0 sends
every larger triangle to the row-by-row path with global atomics).  ``autotune()`` times a fixed set
of seeded workloads -- sub-voxel and few-voxel triangles at several grids, surface and solid, linear
and Morton, and a soup of large triangles at 1024^3 -- for every candidate, keeps the fastest,
applies it with cvx_set_tuning and stores it in a JSON cache keyed by the device; ``load_cached()``
applies a cached choice without timing anything.  The package applies the cache once per device
the first time a Plan or Server is made (``apply_cached_once``).

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
BRICK_PAIRS = (0, 16)
KNOBS = ("small_vox", "small_cols", "brick_pairs")
# A candidate replaces the thresholds in effect only when it is at least this much faster on the
# tuning set: smaller gains are within run-to-run noise, and a choice picked by noise was measured
# slower on other workloads (small_vox 16 instead of 64: 2% faster here, 2.4% slower on the 256-mesh mix).
MIN_GAIN = 0.03
DEFAULT_CACHE = os.environ.get("CVX_TUNING_CACHE") or os.path.join(os.path.expanduser("~"), ".cache",
                                                                     "cuda_voxelizer_gb300", "tuning.json")


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
    soup = meshgen.soup(14, n=200_000)
    out.append(("soup200k_g1024_surf_lin", cv.make_voxinfo(soup, 1024), torch.from_numpy(soup.reshape(-1)).cuda(),
                False, False))
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


def _write_cache(cache_path: str, key: str, choice: dict) -> None:
    cache = {}
    if os.path.exists(cache_path):
        try:
            with open(cache_path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    cache[key] = choice
    os.makedirs(os.path.dirname(cache_path), exist_ok=True)
    with open(cache_path, "w") as f:
        json.dump(cache, f, indent=1)


def autotune(device: int = 0, cache_path: str | None = DEFAULT_CACHE, reps: int = 5, verbose: bool = False,
             min_gain: float = MIN_GAIN) -> dict:
    """Times every (small_vox, small_cols, brick_pairs) candidate, applies and caches the fastest --
    unless it beats the thresholds in effect by less than `min_gain`, in which case they stay."""
    import torch
    torch.cuda.set_device(device)
    work = _workloads(torch)
    tables = [torch.empty(cv.table_words(info), dtype=torch.int32, device="cuda") for _, info, _, _, _ in work]
    before = cv.get_tuning(device)
    results = []
    t0 = time.perf_counter()
    for sv in SMALL_VOX:
        for sc in SMALL_COLS:
            for bp in BRICK_PAIRS:
                cv.set_tuning(device, small_vox=sv, small_cols=sc, brick_pairs=bp)
                ms = _time_all(torch, work, tables, reps)
                results.append({"small_vox": sv, "small_cols": sc, "brick_pairs": bp, "ms": ms})
                if verbose:
                    print(f"small_vox={sv:3d} small_cols={sc:2d} brick_pairs={bp}: {ms:.3f} ms", flush=True)
    best = min(results, key=lambda r: r["ms"])
    current = next((r for r in results if all(r[k] == before[k] for k in KNOBS)), None)
    if current is not None and best["ms"] > current["ms"] * (1.0 - min_gain):
        best = current
    choice = {k: best[k] for k in KNOBS}
    cv.set_tuning(device, **choice)
    out = {"device": _device_key(device), **choice, "ms": best["ms"], "default": before,
           "default_ms": current["ms"] if current else None, "min_gain": min_gain,
           "candidates": results, "seconds": time.perf_counter() - t0}
    if cache_path:
        _write_cache(cache_path, out["device"], choice)
    return out


def load_cached(device: int = 0, cache_path: str = DEFAULT_CACHE) -> dict | None:
    """Applies this device's cached choice, if any; returns it (None when not cached).  Knobs the
    cache does not name keep their current values."""
    try:
        with open(cache_path) as f:
            entry = json.load(f).get(_device_key(device))
    except (OSError, ValueError):
        return None
    if not entry:
        return None
    choice = {k: int(entry[k]) for k in KNOBS if k in entry}
    cv.set_tuning(device, **choice)
    return choice


_applied: set = set()


def apply_cached_once(device: int = 0) -> dict | None:
    """load_cached(device) the first time it is called for `device` in this process."""
    if device in _applied:
        return None
    _applied.add(device)
    return load_cached(device)


if __name__ == "__main__":
    r = autotune(verbose=True)
    print(json.dumps({k: v for k, v in r.items() if k != "candidates"}))
