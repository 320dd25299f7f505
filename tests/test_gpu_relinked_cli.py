"""The reference's own command-line program relinked against libcvx.so.

oracle/build_ref.sh builds the reference's src/main.cpp (with its I/O and CUDA-init helpers,
unmodified, and a small Trimesh stand-in that reads OBJ files) against libcvx.so in place of
src/voxelize.cu and src/voxelize_solid.cu, exactly the relink INTEGRATION.md describes.  Run on a
mesh file, it must go through the engine (its "[Perf] Voxelization GPU time" line is printed by
libcvx.so's voxelize / voxelize_solid) and write the same files as this repository's own CLI
(cuda_voxelizer_gb300.cli): binvox surface and solid tables and the raw Morton table.
"""
import os
import subprocess

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from cuda_voxelizer_gb300 import cli  # noqa: E402
from cuda_voxelizer_gb300 import meshgen  # noqa: E402

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RELINKED = os.path.join(ROOT, "oracle", "_ref", "cuda_voxelizer_relinked")


def _write_obj(path, tris):
    t = np.asarray(tris, dtype=np.float32).reshape(-1, 3, 3)
    with open(path, "w") as f:
        for tri in t:
            for v in tri:
                f.write("v %.9g %.9g %.9g\n" % (v[0], v[1], v[2]))  # float32 round-trips at 9 digits
        for i in range(t.shape[0]):
            f.write("f %d %d %d\n" % (3 * i + 1, 3 * i + 2, 3 * i + 3))


@pytest.fixture(scope="module")
def meshes(tmp_path_factory):
    if not os.path.exists(RELINKED):
        pytest.skip("the reference's command-line program was not built here (no reference sources)")
    base = tmp_path_factory.mktemp("relinked")
    out = {}
    for name, tris in (("torus", meshgen.torus(0)), ("ico5", meshgen.icosphere(7, level=5))):
        for side in ("ref", "own"):
            os.makedirs(base / side, exist_ok=True)
            _write_obj(str(base / side / f"{name}.obj"), tris)
        out[name] = base
    return out


@pytest.mark.parametrize("name", ["torus", "ico5"])
@pytest.mark.parametrize("args,suffix", [(["-o", "binvox"], "_64.binvox"), (["-o", "binvox", "-solid"], "_64.binvox"),
                                         (["-o", "morton"], ".bin")])
def test_relinked_reference_cli_writes_the_engines_files(meshes, name, args, suffix):
    base = meshes[name]
    ref_obj = str(base / "ref" / f"{name}.obj")
    own_obj = str(base / "own" / f"{name}.obj")
    for p in (ref_obj + suffix, own_obj + suffix):
        if os.path.exists(p):
            os.remove(p)
    r = subprocess.run([RELINKED, "-f", ref_obj, "-s", "64"] + args, capture_output=True, text=True, timeout=300,
                       cwd=str(base / "ref"))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "[Perf] Voxelization GPU time" in r.stdout, r.stdout[-2000:]
    assert "CPU VOXELISATION" not in r.stdout
    cli.run(["-f", own_obj, "-s", "64"] + args)
    with open(ref_obj + suffix, "rb") as f:
        ref_bytes = f.read()
    with open(own_obj + suffix, "rb") as f:
        own_bytes = f.read()
    assert len(ref_bytes) == len(own_bytes) and ref_bytes == own_bytes
