"""bench.py's output contract: stdout is exactly one JSON line with the keys the benchmark record
needs.  The reference arm runs on the CPU (the reference's own CPU voxelizer where it was built on
this machine, else the oracle port) and is checked here without a GPU; the engine arm needs one."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BASE_KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
             "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}


def _run(args, timeout):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                       timeout=timeout, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, f"stdout must be one JSON line, got {len(lines)}: {r.stdout[:500]}"
    return json.loads(lines[0])


def test_reference_arm_prints_one_json_line():
    line = _run(["--impl", "reference", "--steps", "1", "--warmup", "0", "--no-extras"], timeout=600)
    assert line["impl"] == "reference"
    assert BASE_KEYS <= set(line)
    assert line["value"] > 0 and line["unit"] == "Mtris/s"
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


@pytest.mark.gpu
def test_engine_arm_prints_one_json_line():
    line = _run(["--steps", "3", "--warmup", "3", "--no-extras"], timeout=1200)
    assert BASE_KEYS | {"roofline", "clocks", "gpu_launches", "tuning"} <= set(line)
    assert line["value"] > 0 and line["gpu_launches"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] > 0 and line["e2e"]["d2h_bytes_per_step"] > 0
    # the link bounds both forms (the bounds come from copy rates measured beside the steps, so a
    # fraction a little above 1 is measurement noise; far above would mean bytes were not moved)
    e2e = line["e2e"]
    assert 0 < e2e["frac_of_copy_bound"] < 1.2 and 0 < e2e["single_step"]["frac_of_copy_bound"] < 1.2
    assert e2e["ms_per_step"] < e2e["single_step"]["ms_per_step"]
    r = line["roofline"]
    assert {"bound", "achieved", "peak", "unit", "frac", "traffic"} <= set(r)
    assert line["clocks"]["sm_mhz"] is not None


def test_cpu_leg_sizing():
    """The CPU legs run the whole workload when the run fits its budget, else the largest
    power-of-two share that does (at most 1/32)."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench.cpu_fraction(4.0, 25, 120.0) == 1
    assert bench.cpu_fraction(4.5, 410, 120.0) == 16
    assert bench.cpu_fraction(1e9, 10, 1.0) == bench.SAMPLE_FRACTION


def test_cpu_work_drops_only_unsafe_solid_triangles():
    sys.path.insert(0, ROOT)
    import bench
    import oracle
    meshgen = bench.load_meshgen()
    tris = meshgen.icosphere(0, level=5)
    info = bench.reference_voxinfo(tris, 128)
    work = bench.cpu_work(info, tris)
    assert work[0].shape == tris.shape and work[1].shape == tris.shape  # surface modes: every triangle
    for w, (morton, solid) in zip(work, bench.MODES):
        if solid:
            from oracle.ref_safety import safe_triangles
            assert w.shape[0] == int(safe_triangles(tris, oracle.with_count(info, tris.shape[0]), morton).sum())


def test_smoke_resolves_its_imports_without_a_gpu():
    """smoke() imports the package, the oracle and the triangle filter before it asks for cuda:0;
    on a machine without a GPU it must get that far and stop at its own check."""
    code = ("import torch, __graft_entry__ as g\n"
            "assert not torch.cuda.is_available()\n"
            "try:\n    g.smoke()\nexcept AssertionError as e:\n    print('stopped:', e)\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "stopped: smoke() needs cuda:0" in r.stdout


def test_link_bound():
    """Both directions at once while both have bytes left, then the longer one alone; one after the
    other when running them together is no faster."""
    sys.path.insert(0, ROOT)
    import bench
    r = {"h2d_gbs": 200.0, "d2h_gbs": 200.0, "h2d_with_d2h_gbs": 150.0, "d2h_with_h2d_gbs": 150.0}
    # 150 MB each way together in 1 ms, then 50 MB down alone in 0.25 ms
    assert abs(bench.link_bound_s(150e6, 200e6, r) - 1.25e-3) < 1e-12
    assert abs(bench.link_bound_s(200e6, 150e6, r) - 1.25e-3) < 1e-12
    slow = dict(r, h2d_with_d2h_gbs=80.0, d2h_with_h2d_gbs=80.0)
    assert abs(bench.link_bound_s(150e6, 200e6, slow) - 1.75e-3) < 1e-12
