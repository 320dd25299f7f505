"""The command-line voxelizer: mesh readers on the CPU, and the whole pipeline (upload, GPU gather,
device bbox / voxinfo, voxelize, encode, files named as the reference names them) on the GPU."""
import os
import struct

import numpy as np
import pytest

import oracle
from cuda_voxelizer_gb300 import cli
from cuda_voxelizer_gb300 import meshgen


def _write_obj(path, verts, faces, quads=False):
    with open(path, "w") as f:
        for v in verts:
            f.write(f"v {float(v[0])!r} {float(v[1])!r} {float(v[2])!r}\n")
        for t in faces:
            f.write("f " + " ".join(f"{i + 1}/{i + 1}" for i in t) + "\n")


def test_obj_reader_fans_polygons_and_negative_indices(tmp_path):
    p = tmp_path / "q.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3 4\nf -4 -2 -1\n")
    v, f = cli.read_obj(str(p))
    assert v.shape == (4, 3) and f.tolist() == [[0, 1, 2], [0, 2, 3], [0, 2, 3]]


@pytest.mark.parametrize("binary", [False, True])
def test_ply_reader(tmp_path, binary):
    verts = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0.5]], np.float32)
    p = tmp_path / "m.ply"
    head = (f"ply\nformat {'binary_little_endian' if binary else 'ascii'} 1.0\nelement vertex 4\n"
            "property float x\nproperty float y\nproperty float z\nelement face 1\n"
            "property list uchar int vertex_indices\nend_header\n").encode()
    if binary:
        body = verts.tobytes() + struct.pack("<B4i", 4, 0, 1, 2, 3)
    else:
        body = ("".join(f"{a} {b} {c}\n" for a, b, c in verts) + "4 0 1 2 3\n").encode()
    p.write_bytes(head + body)
    v, f = cli.read_ply(str(p))
    assert np.array_equal(v, verts) and f.tolist() == [[0, 1, 2], [0, 2, 3]]


def test_argument_rules():
    o = cli.parse(["-f", "a.obj", "-s", "128", "-o", "BINVOX", "-solid"])
    assert o == {"file": "a.obj", "gridsize": 128, "output": "binvox", "cpu": False, "solid": True}
    with pytest.raises(SystemExit):
        cli.parse(["-f", "a.obj", "-o", "stl"])


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", ["binvox", "morton", "obj_points"])
@pytest.mark.parametrize("solid", [False, True])
def test_cli_pipeline_matches_api(tmp_path, fmt, solid):
    torch = pytest.importorskip("torch")
    from cuda_voxelizer_gb300 import api as cv
    tris = meshgen.torus(5)
    verts = tris.reshape(-1, 3)
    faces = np.arange(verts.shape[0]).reshape(-1, 3)
    path = str(tmp_path / "torus.obj")
    _write_obj(path, verts, faces)
    r = cli.run(["-f", path, "-s", "64", "-o", fmt] + (["-solid"] if solid else []))
    info = cv.make_voxinfo(tris, 64)
    assert bytes(r["info"]) == bytes(info)
    t = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    (cv.voxelize_solid if solid else cv.voxelize)(info, torch.from_numpy(tris.reshape(-1)).cuda(), t, fmt == "morton")
    host = t.cpu().numpy().view(np.uint32)
    data = open(r["path"], "rb").read()
    if fmt == "morton":
        assert r["path"] == path + ".bin" and data == host.tobytes()
    elif fmt == "binvox":
        assert r["path"] == f"{path}_64.binvox"
        assert data == cv.binvox_header(info) + oracle.binvox_payload(bytes(info), host)
    else:
        assert r["path"] == f"{path}_64_pointcloud.obj"
        lines = data.decode().splitlines()
        bits = np.unpackbits(host.view(np.uint8).reshape(-1, 4)[:, ::-1].reshape(-1)).reshape(64, 64, 64)
        assert len(lines) == int(bits.sum())
        x, y, z = (float(s) - 0.5 for s in lines[0].split()[1:])
        assert bits[int(z), int(y), int(x)] == 1
