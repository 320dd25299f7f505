"""The bin-threshold autotuner: every candidate gives the same bits (results never depend on the
tuning), the tuner applies and caches its choice, and the cache is re-applied by load_cached."""
import json

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from cuda_voxelizer_gb300 import api as cv  # noqa: E402
from cuda_voxelizer_gb300 import autotune as at  # noqa: E402
from cuda_voxelizer_gb300 import meshgen  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("solid", [False, True])
@pytest.mark.parametrize("morton", [False, True])
def test_results_do_not_depend_on_the_thresholds(solid, morton):
    tris = np.concatenate([meshgen.icosphere(3, level=6), meshgen.soup(4, n=20_000, lmin=0.5 / 256, lmax=0.05)])
    info = cv.make_voxinfo(tris, 256)
    d = torch.from_numpy(tris.reshape(-1)).cuda()
    before = cv.get_tuning(0)
    ref = None
    try:
        for sv in at.SMALL_VOX + (0, 1):
            for sc in at.SMALL_COLS + (0, 1):
                cv.set_tuning(0, small_vox=sv, small_cols=sc)
                t = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
                (cv.voxelize_solid if solid else cv.voxelize)(info, d, t, morton)
                if ref is None:
                    ref = t
                assert torch.equal(t, ref), (sv, sc)
    finally:
        cv.set_tuning(0, **before)


def test_autotune_keeps_thresholds_unless_clearly_faster(tmp_path):
    """With a required gain no candidate can reach, the thresholds in effect stay."""
    before = cv.get_tuning(0)
    try:
        r = at.autotune(0, cache_path=str(tmp_path / "t.json"), reps=1, min_gain=0.99)
        assert {k: r[k] for k in at.KNOBS} == before == cv.get_tuning(0)
        assert r["ms"] == r["default_ms"]
    finally:
        cv.set_tuning(0, **before)


def test_autotune_applies_and_caches(tmp_path):
    before = cv.get_tuning(0)
    path = str(tmp_path / "tuning.json")
    try:
        r = at.autotune(0, cache_path=path, reps=2, min_gain=0.0)
        choice = {k: r[k] for k in at.KNOBS}
        assert cv.get_tuning(0) == choice
        assert r["ms"] <= min(c["ms"] for c in r["candidates"]) + 1e-9
        with open(path) as f:
            assert json.load(f)[r["device"]] == choice
        cv.set_tuning(0, **before)
        assert at.load_cached(0, path) == choice
        assert cv.get_tuning(0) == choice
    finally:
        cv.set_tuning(0, **before)
