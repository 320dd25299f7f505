"""Generate tests/golden/golden_io.npz by running the REFERENCE'S OWN binvox writer.

oracle/build_ref.sh compiles src/util_io.cpp (with its vendored MagicaVoxel writer) unmodified into
oracle/_ref/libref_io.so; this script feeds it linear-order tables -- the reference CPU
voxelizer's golden tables of golden.npz plus a few synthetic ones (empty, full, random,
non-cubic) -- and stores each .binvox file it writes, split into header and run-length payload.

Run on the development machine only (it needs the reference tree):
    python tests/golden/make_golden_io.py
"""
from __future__ import annotations

import ctypes
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402


def info_bytes(grid, bmin=(0.0, 0.0, 0.0), bmax=(1.0, 1.0, 1.0), n=0) -> bytes:
    return oracle.info_init(np.asarray(bmin, np.float32), np.asarray(bmax, np.float32), grid, n)


def synthetic():
    rng = np.random.default_rng(11)
    out = {}
    g = (64, 64, 64)
    out["empty_g64"] = (info_bytes(g), np.zeros(64 ** 3 // 32, np.uint32))
    out["full_g64"] = (info_bytes(g, (-1.0, -2.0, 0.5), (3.0, 2.5, 1.5)), np.full(64 ** 3 // 32, 0xFFFFFFFF, np.uint32))
    out["random_g32"] = (info_bytes((32, 32, 32)), rng.integers(0, 2 ** 32, 32 ** 3 // 32, dtype=np.uint64).astype(np.uint32))
    # sparse runs of every length, long zero runs (split at 255)
    sp = np.zeros(128 ** 3 // 32, np.uint32)
    idx = rng.choice(sp.size, 3000, replace=False)
    sp[idx] = rng.integers(0, 2 ** 32, idx.size, dtype=np.uint64).astype(np.uint32)
    out["sparse_g128"] = (info_bytes((128, 128, 128)), sp)
    nc = (40, 24, 36)
    words = (40 * 24 * 36 + 31) // 32
    out["random_40x24x36"] = (info_bytes(nc, (0.0, 0.0, 0.0), (4.0, 2.4, 3.6)),
                              rng.integers(0, 2 ** 32, words, dtype=np.uint64).astype(np.uint32))
    return out


def main() -> None:
    lib_path = os.path.join(ROOT, "oracle", "_ref", "libref_io.so")
    if not os.path.exists(lib_path):
        raise SystemExit("oracle/_ref/libref_io.so missing: run oracle/build_ref.sh first")
    L = ctypes.CDLL(lib_path)
    L.ref_write_binvox.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p]
    g = np.load(os.path.join(HERE, "golden.npz"))
    import json
    manifest = json.load(open(os.path.join(HERE, "golden.json")))
    cases = {}
    for name, c in manifest["cases"].items():
        key = f"{name}__linear__surface"
        if key in g.files:
            cases[key] = (bytes.fromhex(c["voxinfo_hex"]), g[key])
        key = f"{name}__linear__solid"
        if key in g.files:
            cases[key] = (bytes.fromhex(c["voxinfo_hex"]), g[key])
    cases.update(synthetic())
    arrays = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, (info, table) in cases.items():
            base = os.path.join(tmp, name)
            t = np.ascontiguousarray(table, np.uint32)
            ib = ctypes.create_string_buffer(info, 64)
            L.ref_write_binvox(t.ctypes.data, ctypes.addressof(ib), base.encode())
            gx = int(np.frombuffer(info[24:28], np.uint32)[0])
            data = open(f"{base}_{gx}.binvox", "rb").read()
            cut = data.index(b"data\n") + len(b"data\n")
            arrays[f"{name}__info"] = np.frombuffer(info, np.uint8)
            arrays[f"{name}__table"] = t
            arrays[f"{name}__header"] = np.frombuffer(data[:cut], np.uint8)
            arrays[f"{name}__payload"] = np.frombuffer(data[cut:], np.uint8)
            print(name, len(data) - cut, "payload bytes", file=sys.stderr)
    np.savez_compressed(os.path.join(HERE, "golden_io.npz"), **arrays)


if __name__ == "__main__":
    main()
