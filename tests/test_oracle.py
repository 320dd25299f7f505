"""CPU tests: the oracle and the host-side setup, pinned to the reference's own code.

* the C restatement (oracle/cvx_oracle.c) reproduces the reference CPU voxelizer bit for bit on
  every golden fixture (tests/golden/, generated by the reference's src/cpu_voxelizer.cpp);
* the engine's host functions (cvx_bbox_cube, cvx_voxinfo_init) reproduce createMeshBBCube and
  the voxinfo constructor of src/util.h exactly;
* the synthetic meshes are the ones the fixtures were made from (input hashes);
* the Morton tables equal src/morton_LUTs.h.
When the reference build is present (development machine), the restatement is also compared with
it live on fresh random inputs.
"""
import hashlib

import numpy as np
import pytest

import oracle
from cuda_voxelizer_gb300 import api as cv
from cuda_voxelizer_gb300 import meshgen
from golden_data import arrays, manifest, mesh, table_keys


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", list(manifest()["cases"].keys()))
def test_mesh_generator_matches_fixture_inputs(name):
    c = manifest()["cases"][name]
    t = mesh(name)
    assert t.shape == (c["n_triangles"], 9)
    assert sha(t) == c["input_sha256"]


@pytest.mark.parametrize("name,key,morton,solid", table_keys())
def test_oracle_matches_reference_golden(name, key, morton, solid):
    c = manifest()["cases"][name]
    info = bytes.fromhex(c["voxinfo_hex"])
    got = oracle.voxelize(info, mesh(name), morton=morton, solid=solid)
    want = arrays()[key]
    assert got.shape == want.shape
    diff = np.nonzero(got != want)[0]
    assert diff.size == 0, f"{key}: {diff.size} words differ, first at {diff[:5]}"


def test_oracle_omp_matches_serial():
    name = "ico4_g64"
    info = bytes.fromhex(manifest()["cases"][name]["voxinfo_hex"])
    t = mesh(name)
    for solid in (False, True):
        a = oracle.voxelize(info, t, solid=solid)
        b = oracle.voxelize_omp(info, t, solid=solid, threads=4)
        assert np.array_equal(a, b)


def test_morton_luts_match_reference():
    a = arrays()
    for axis, nm in enumerate("xyz"):
        assert np.array_equal(oracle.morton_lut(axis), a[f"lut_{nm}"])


def test_morton_encode_spreads_bits():
    rng = np.random.default_rng(0)
    for _ in range(200):
        x, y, z = (int(v) for v in rng.integers(0, 1 << 16, 3))
        want = 0
        for i in range(16):
            want |= ((x >> i) & 1) << (3 * i) | ((y >> i) & 1) << (3 * i + 1) | ((z >> i) & 1) << (3 * i + 2)
        assert oracle.morton_encode(x, y, z) == want


def test_bbcube_matches_reference():
    rows = arrays()["bbcube"]
    for r in rows:
        lo, hi, want_lo, want_hi = r[0:3], r[3:6], r[6:9], r[9:12]
        got_lo, got_hi = cv.create_mesh_bbox_cube(lo, hi)
        assert np.array_equal(got_lo.view(np.uint32), want_lo.astype(np.float32).view(np.uint32))
        assert np.array_equal(got_hi.view(np.uint32), want_hi.astype(np.float32).view(np.uint32))
        o_lo, o_hi = oracle.mesh_bbcube(lo, hi)
        assert np.array_equal(o_lo, want_lo.astype(np.float32)) and np.array_equal(o_hi, want_hi.astype(np.float32))


@pytest.mark.parametrize("name", list(manifest()["cases"].keys()))
def test_host_voxinfo_matches_reference(name):
    c = manifest()["cases"][name]
    info = cv.make_voxinfo(mesh(name), c["grid"])
    want = bytes.fromhex(c["voxinfo_hex"])
    assert bytes(info) == want


def test_table_words():
    for g in (8, 64, 100, 1024):
        info = cv.make_info((0, 0, 0), (1, 1, 1), g, 1)
        assert cv.table_words(info) == (g ** 3 + 31) // 32
    info = cv.make_info((0, 0, 0), (1, 1, 1), (3, 5, 7), 1)
    assert cv.table_words(info) == (105 + 31) // 32


@pytest.mark.skipif(not oracle.ref_cpu_available(), reason="reference CPU build not present on this machine")
@pytest.mark.parametrize("seed", range(4))
def test_oracle_matches_reference_live(seed):
    """Fresh random inputs, including triangles poking out of the bbox and degenerate ones."""
    rng = np.random.default_rng(100 + seed)
    g = int(rng.choice([16, 32, 64, 50]))
    t = meshgen.soup(seed, n=300, lmin=0.3 / g, lmax=0.6).reshape(-1, 9)
    t[:10, 3:6] = t[:10, 0:3]          # degenerate: two equal vertices
    t[10:20] = np.round(t[10:20] * g) / g  # grid-aligned vertices
    info = cv.make_voxinfo(t, g)
    raw = bytearray(bytes(info))
    for morton in (False, True):
        if morton and g & (g - 1):
            continue
        for solid in (False, True):
            a = oracle.voxelize(bytes(raw), t, morton=morton, solid=solid)
            b = oracle.ref_cpu_voxelize(bytes(raw), t, morton=morton, solid=solid)
            assert np.array_equal(a, b), (g, morton, solid)


@pytest.mark.skipif(not oracle.ref_cpu_available(), reason="reference CPU build not present on this machine")
def test_reference_cpu_quiet_keeps_stdout_clean(capfd):
    """The benchmark prints one JSON line on stdout; the reference CPU voxelizer's own "[Info]" and
    "[Perf]" lines must not reach it when the benchmark times that build."""
    t = meshgen.torus(0, nu=16, nv=8)
    info = bytes(cv.make_voxinfo(t, 32))
    capfd.readouterr()
    loud = oracle.ref_cpu_voxelize(info, t)
    assert "[Perf]" in capfd.readouterr().out
    quiet = oracle.ref_cpu_voxelize(info, t, quiet=True)
    print("after")
    assert capfd.readouterr().out == "after\n"
    assert np.array_equal(loud, quiet)


@pytest.mark.parametrize("solid", [False, True])
@pytest.mark.parametrize("morton", [False, True])
def test_count_atomics_matches_per_triangle_tables(morton, solid):
    """The roofline's atomic term: one triangle at a time, the surface count is the number of
    nonzero table words and the solid count the number of rows it flips (one hit per column)."""
    from cuda_voxelizer_gb300 import meshgen
    tris = meshgen.torus(3, nu=12, nv=6)
    info = oracle.info_init(*oracle.mesh_bbcube(tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)), (32, 32, 32),
                            tris.shape[0])
    want = 0
    for t in tris:
        one = oracle.with_count(info, 1)
        tab = oracle.voxelize(one, t.reshape(1, 9), morton=morton, solid=solid)
        if not solid:
            want += int(np.count_nonzero(tab))
        else:
            lin = tab if not morton else oracle.voxelize(one, t.reshape(1, 9), solid=True)
            bits = np.unpackbits(lin.view(np.uint8).reshape(-1, 4)[:, ::-1].reshape(-1)).reshape(32 * 32, 32)
            want += int(np.count_nonzero(bits.any(axis=1)))
    assert oracle.count_atomics(info, tris, morton=morton, solid=solid) == want
