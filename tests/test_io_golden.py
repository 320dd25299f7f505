"""Output writers on the host side: the oracle's restatement of write_binvox against the reference's
own binvox files (tests/golden/golden_io.npz, made by tests/golden/make_golden_io.py from
src/util_io.cpp), the header formatting, and the restated write_vox voxel list."""
import os

import numpy as np
import pytest

import oracle
from cuda_voxelizer_gb300 import api as cv
from cuda_voxelizer_gb300._lib import CvxVoxinfo

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_io.npz")


def _cases():
    g = np.load(GOLDEN)
    return sorted({k.rsplit("__", 1)[0] for k in g.files})


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("name", _cases())
def test_oracle_binvox_payload_matches_reference_writer(golden, name):
    info = golden[f"{name}__info"].tobytes()
    got = oracle.binvox_payload(info, golden[f"{name}__table"])
    assert got == golden[f"{name}__payload"].tobytes()


@pytest.mark.parametrize("name", _cases())
def test_binvox_header_matches_reference_writer(golden, name):
    info = CvxVoxinfo.from_buffer_copy(golden[f"{name}__info"].tobytes())
    assert cv.binvox_header(info) == golden[f"{name}__header"].tobytes()


def test_vox_list_restatement_counts_and_order(golden):
    info = golden["torus_g64__linear__surface__info"].tobytes()
    table = golden["torus_g64__linear__surface__table"]
    lst = oracle.vox_list(info, table)
    bits = np.unpackbits(table.view(np.uint8).reshape(-1, 4)[:, ::-1].reshape(-1)).reshape(64, 64, 64)  # [z][y][x]
    assert len(lst) == int(bits.sum())
    x, zz, y = lst[:, 0], 64 - lst[:, 1], lst[:, 2]
    assert np.all(bits[zz, y, x] == 1)
    key = (x.astype(np.int64) * 64 + y) * 64 + zz  # traversal order: x, then y, then z
    assert np.all(np.diff(key) > 0)
