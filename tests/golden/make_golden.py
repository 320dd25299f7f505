"""Generate the golden fixtures of tests/golden/ by running the REFERENCE'S OWN CPU voxelizer.

The reference (Forceflow/cuda_voxelizer) ships no tests, golden vectors or known answers, so its
own code is the source of truth: oracle/build_ref.sh compiles src/cpu_voxelizer.cpp unmodified
into oracle/_ref/libref_cpu.so, and this script runs it on seeded synthetic meshes
(cuda_voxelizer_gb300.meshgen) and stores the resulting bit tables.  It also records the
reference's Morton tables (src/morton_LUTs.h), createMeshBBCube (src/util.h:80-110) and voxinfo
(src/util.h:56-61) outputs.

Run on the development machine only (it needs the reference tree):
    python tests/golden/make_golden.py
The fixtures are committed; tests compare against them anywhere.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from cuda_voxelizer_gb300 import meshgen  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def info_for(tris: np.ndarray, g) -> bytes:
    """main()'s setup (src/main.cpp:179-186) through the reference's own functions."""
    L = oracle.ref_cpu_lib()
    import ctypes
    v = tris.reshape(-1, 3)
    lo = v.min(0).astype(np.float32)
    hi = v.max(0).astype(np.float32)
    omin = np.zeros(3, np.float32)
    omax = np.zeros(3, np.float32)
    L.ref_create_mesh_bbcube(lo.ctypes.data, hi.ctypes.data, omin.ctypes.data, omax.ctypes.data)
    grid = np.asarray(g if not np.isscalar(g) else (g, g, g), dtype=np.uint32)
    out = ctypes.create_string_buffer(64)
    L.ref_voxinfo_init(omin.ctypes.data, omax.ctypes.data, grid.ctypes.data, tris.shape[0], out)
    b = bytearray(out.raw)
    b[36:40] = b"\0\0\0\0"  # padding
    b[60:64] = b"\0\0\0\0"
    return bytes(b)


# name -> (mesh builder, grid)
CASES = {
    "torus_g64": (lambda: meshgen.torus(0), 64),
    "torus_g128": (lambda: meshgen.torus(1), 128),
    "ico4_g64": (lambda: meshgen.icosphere(2, level=4), 64),
    "ico5_g128": (lambda: meshgen.icosphere(3, level=5), 128),
    "soup2k_g64": (lambda: meshgen.soup(4, n=2000, lmin=0.25 / 64, lmax=0.5), 64),
    "soup500_g100": (lambda: meshgen.soup(5, n=500, lmin=0.5 / 100, lmax=0.3), 100),
    "ico3_g8": (lambda: meshgen.icosphere(6, level=3), 8),
}
MODES = [(False, False), (True, False), (False, True), (True, True)]  # (morton, solid)


def main() -> None:
    if not oracle.ref_cpu_available():
        raise SystemExit("oracle/_ref/libref_cpu.so missing: run oracle/build_ref.sh first")
    L = oracle.ref_cpu_lib()
    manifest = {"cases": {}}
    arrays = {}
    for name, (build, g) in CASES.items():
        tris = build()
        info = info_for(tris, g)
        manifest["cases"][name] = {"grid": g, "n_triangles": int(tris.shape[0]), "input_sha256": sha(tris),
                                   "voxinfo_hex": info.hex(), "tables": {}}
        for morton, solid in MODES:
            if morton and (g & (g - 1)):
                continue  # Morton needs a power-of-two grid
            table = oracle.ref_cpu_voxelize(info, tris, morton=morton, solid=solid)
            key = f"{name}__{'morton' if morton else 'linear'}__{'solid' if solid else 'surface'}"
            arrays[key] = table
            manifest["cases"][name]["tables"][key] = {"popcount": int(np.unpackbits(table.view(np.uint8)).sum()),
                                                      "sha256": sha(table)}
            print(key, manifest["cases"][name]["tables"][key]["popcount"], file=sys.stderr)
    # Morton LUTs of src/morton_LUTs.h
    for axis, nm in enumerate("xyz"):
        out = np.zeros(256, np.uint32)
        L.ref_morton_lut(axis, out.ctypes.data)
        arrays[f"lut_{nm}"] = out
    # createMeshBBCube / voxinfo on assorted boxes
    rng = np.random.default_rng(7)
    boxes = []
    for _ in range(64):
        lo = rng.normal(0, 10, 3).astype(np.float32)
        hi = (lo + np.abs(rng.normal(0, 5, 3)) * (rng.random(3) < 0.8)).astype(np.float32)
        omin = np.zeros(3, np.float32)
        omax = np.zeros(3, np.float32)
        L.ref_create_mesh_bbcube(lo.ctypes.data, hi.ctypes.data, omin.ctypes.data, omax.ctypes.data)
        boxes.append(np.concatenate([lo, hi, omin, omax]))
    arrays["bbcube"] = np.stack(boxes)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
