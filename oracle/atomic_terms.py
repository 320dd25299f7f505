"""Atomic term A of the roofline for the benchmark workloads, counted exactly by the oracle.

    python oracle/atomic_terms.py        # writes profiles/atomic_terms.json

A (per voxelization call) is, for surface voxelization, the number of distinct 32-bit table words
each triangle sets a bit in, summed over the triangles; for solid voxelization, the number of
column hits.  bench.py divides it by the measured scattered atomicOr rate to get the atomic part of
the roofline time.  TEST INFRASTRUCTURE: runs the oracle on the host, never on the product path.
"""
from __future__ import annotations

import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from cuda_voxelizer_gb300 import meshgen  # noqa: E402

MODES = [("surface_linear", False, False), ("surface_morton", True, False), ("solid_linear", False, True),
         ("solid_morton", True, True)]


def icosphere512():
    tris = meshgen.icosphere(0, level=8)
    pts = tris.reshape(-1, 3)
    lo, hi = oracle.mesh_bbcube(pts.min(0), pts.max(0))
    info = oracle.info_init(lo, hi, (512, 512, 512), tris.shape[0])
    out = {"workload": "icosphere level 8 (1,310,720 triangles) at 512^3", "triangles": int(tris.shape[0])}
    for name, morton, solid in MODES:
        t0 = time.perf_counter()
        out[name] = oracle.count_atomics(info, tris, morton=morton, solid=solid)
        print(f"{name}: {out[name]} ({time.perf_counter() - t0:.1f} s)", flush=True)
    return out


def main():
    path = os.path.join(ROOT, "profiles", "atomic_terms.json")
    os.makedirs(os.path.dirname(path), exist_ok=True)
    try:
        with open(path) as f:
            res = json.load(f)  # keep entries measured elsewhere (the soup's, from ncu)
    except (OSError, ValueError):
        res = {}
    res["definition"] = "surface: sum over triangles of distinct table words set; solid: column hits"
    res["icosphere_l8_512"] = icosphere512()
    with open(path, "w") as f:
        json.dump(res, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
