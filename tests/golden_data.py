"""Loader for the committed golden fixtures (made by tests/golden/make_golden.py from the
reference's own CPU voxelizer)."""
import json
import os

import numpy as np

from cuda_voxelizer_gb300 import meshgen

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_MESHES = {
    "torus_g64": lambda: meshgen.torus(0),
    "torus_g128": lambda: meshgen.torus(1),
    "ico4_g64": lambda: meshgen.icosphere(2, level=4),
    "ico5_g128": lambda: meshgen.icosphere(3, level=5),
    "soup2k_g64": lambda: meshgen.soup(4, n=2000, lmin=0.25 / 64, lmax=0.5),
    "soup500_g100": lambda: meshgen.soup(5, n=500, lmin=0.5 / 100, lmax=0.3),
    "ico3_g8": lambda: meshgen.icosphere(6, level=3),
}


def manifest():
    with open(os.path.join(HERE, "golden.json")) as f:
        return json.load(f)


def arrays():
    return np.load(os.path.join(HERE, "golden.npz"))


def mesh(name):
    return _MESHES[name]()


def table_keys():
    m = manifest()
    out = []
    for name, c in m["cases"].items():
        for key in c["tables"]:
            _, order, mode = key.split("__")
            out.append((name, key, order == "morton", mode == "solid"))
    return out
