"""Command-line voxelizer with the reference program's flags (src/main.cpp:109-155), on the engine.

    python -m cuda_voxelizer_gb300.cli -f model.obj -s 256 -o binvox [-solid]

Flags as in the reference: -f <mesh file> (required), -s <gridsize> (default 256), -o <output
format>, -solid, -cpu, -h.  The pipeline is the reference main()'s (src/main.cpp:159-261) with
every stage after mesh reading on the GPU: vertices and faces are uploaded once, expanded to the
triangle soup by cvx_gather_soup, the bounding box / createMeshBBCube / voxinfo come from
cvx_voxinfo_from_device, the table from voxelize / voxelize_solid (Morton order for -o morton), and
the output from the GPU encoders.  Output files are named as the reference names them:
<file>.bin (morton, the raw table), <file>_<g>.binvox, <file>_<g>_pointcloud.obj.

Differences, stated: mesh files are read by a small OBJ / PLY reader of this package (the reference
uses Trimesh2, which also reads 3DS and other formats; polygons are split into fans as Trimesh2
does); -o vox (MagicaVoxel scene file) and -o obj (cube mesh through Trimesh2) are not written -- the
GPU produces the voxel list the MagicaVoxel writer consumes (cvx_encode_voxel_list); -cpu is
refused: this engine has no CPU path.
"""
from __future__ import annotations

import os
import struct
import sys
import time

import numpy as np

FORMATS = ("binvox", "morton", "obj", "obj_points", "vox")


def _fan(poly):
    return [(poly[0], poly[i], poly[i + 1]) for i in range(1, len(poly) - 1)]


def read_obj(path: str):
    """Vertices (V, 3) float32 and triangle faces (F, 3) int64 of a Wavefront OBJ file."""
    verts, faces = [], []
    with open(path, "r", errors="replace") as f:
        for line in f:
            p = line.split()
            if not p:
                continue
            if p[0] == "v" and len(p) >= 4:
                verts.append((float(p[1]), float(p[2]), float(p[3])))
            elif p[0] == "f" and len(p) >= 4:
                idx = []
                for tok in p[1:]:
                    i = int(tok.split("/")[0])
                    idx.append(i - 1 if i > 0 else len(verts) + i)  # 1-based; negative = relative
                faces.extend(_fan(idx))
    return np.asarray(verts, dtype=np.float32).reshape(-1, 3), np.asarray(faces, dtype=np.int64).reshape(-1, 3)


_PLY_TYPES = {"char": "b", "int8": "b", "uchar": "B", "uint8": "B", "short": "h", "int16": "h", "ushort": "H",
              "uint16": "H", "int": "i", "int32": "i", "uint": "I", "uint32": "I", "float": "f", "float32": "f",
              "double": "d", "float64": "d"}


def read_ply(path: str):
    """Vertices and triangle faces of an ASCII or binary PLY file (x, y, z vertex properties and a
    vertex_indices / vertex_index face list)."""
    with open(path, "rb") as f:
        if f.readline().strip() != b"ply":
            raise ValueError(f"{path}: not a PLY file")
        fmt, elements = None, []
        while True:
            line = f.readline()
            if not line:
                raise ValueError(f"{path}: truncated header")
            p = line.decode("ascii", "replace").split()
            if not p:
                continue
            if p[0] == "format":
                fmt = p[1]
            elif p[0] == "element":
                elements.append([p[1], int(p[2]), []])
            elif p[0] == "property":
                elements[-1][2].append(p[1:])
            elif p[0] == "end_header":
                break
        if fmt not in ("ascii", "binary_little_endian", "binary_big_endian"):
            raise ValueError(f"{path}: unsupported PLY format {fmt}")
        end = "<" if fmt == "binary_little_endian" else ">"
        verts, faces = None, []
        body = f.read()
    pos = 0
    tokens = body.split() if fmt == "ascii" else None
    ti = 0
    for name, count, props in elements:
        rows = []
        for _ in range(count):
            row = {}
            for prop in props:
                if prop[0] == "list":
                    ct, it, pname = prop[1], prop[2], prop[3]
                    if tokens is not None:
                        n = int(tokens[ti]); ti += 1
                        vals = [int(tokens[ti + k]) for k in range(n)]
                        ti += n
                    else:
                        (n,) = struct.unpack_from(end + _PLY_TYPES[ct], body, pos)
                        pos += struct.calcsize(_PLY_TYPES[ct])
                        fmt_i = end + _PLY_TYPES[it] * n
                        vals = list(struct.unpack_from(fmt_i, body, pos))
                        pos += struct.calcsize(fmt_i)
                    row[pname] = vals
                else:
                    t, pname = prop[0], prop[1]
                    if tokens is not None:
                        v = float(tokens[ti]); ti += 1
                    else:
                        (v,) = struct.unpack_from(end + _PLY_TYPES[t], body, pos)
                        pos += struct.calcsize(_PLY_TYPES[t])
                    row[pname] = v
            rows.append(row)
        if name == "vertex":
            verts = np.asarray([(r["x"], r["y"], r["z"]) for r in rows], dtype=np.float32).reshape(-1, 3)
        elif name == "face":
            for r in rows:
                idx = r.get("vertex_indices", r.get("vertex_index"))
                faces.extend(_fan([int(i) for i in idx]))
    if verts is None:
        raise ValueError(f"{path}: no vertex element")
    return verts, np.asarray(faces, dtype=np.int64).reshape(-1, 3)


def read_mesh(path: str):
    ext = os.path.splitext(path)[1].lower()
    if ext == ".obj":
        return read_obj(path)
    if ext == ".ply":
        return read_ply(path)
    raise ValueError(f"unsupported mesh format {ext} (this reader knows .obj and .ply)")


def parse(argv):
    """The reference's argument rules (src/main.cpp:109-155)."""
    opts = {"file": None, "gridsize": 256, "output": "vox", "cpu": False, "solid": False}
    i = 0
    while i < len(argv):
        a = argv[i]
        if a == "-f":
            opts["file"] = argv[i + 1]
            i += 1
        elif a == "-s":
            opts["gridsize"] = int(argv[i + 1])
            i += 1
        elif a == "-h":
            opts["help"] = True
        elif a == "-o":
            out = argv[i + 1].lower()
            if out not in FORMATS:
                raise SystemExit(f"[Err] Unrecognized output format: {out}, valid options are binvox, morton, obj, "
                                 "obj_points or vox")
            opts["output"] = out
            i += 1
        elif a == "-cpu":
            opts["cpu"] = True
        elif a == "-solid":
            opts["solid"] = True
        i += 1
    return opts


def run(argv) -> dict:
    import torch

    from . import api as cv
    t_all = time.perf_counter()
    o = parse(argv)
    if o.get("help"):
        print(__doc__)
        return {}
    if not o["file"]:
        raise SystemExit("[Err] You didn't specify a file using -f (path). This is required. Exiting.")
    if not os.path.exists(o["file"]):
        raise SystemExit(f"[Err] File does not exist / cannot access: {o['file']}")
    if o["cpu"]:
        raise SystemExit("[Err] -cpu: this engine has no CPU voxelizer (GPU only)")
    if o["output"] in ("vox", "obj"):
        raise SystemExit(f"[Err] -o {o['output']}: not written by this CLI (use binvox, morton or obj_points; "
                         "the GPU voxel list for MagicaVoxel is cvx_encode_voxel_list)")
    fn, g = o["file"], o["gridsize"]
    print(f"[Info] Filename: {fn}\n[Info] Grid size: {g}\n[Info] Output format: {o['output']}\n"
          f"[Info] Using Solid Voxelization: {'Yes' if o['solid'] else 'No'}")
    verts, faces = read_mesh(fn)
    print(f"[Mesh] Number of triangles: {faces.shape[0]}\n[Mesh] Number of vertices: {verts.shape[0]}")
    d_verts = torch.from_numpy(verts.reshape(-1)).cuda()
    d_faces = torch.from_numpy(faces.astype(np.int32).reshape(-1)).cuda()
    soup, bad = cv.gather_soup(d_verts, d_faces)
    if bad:
        raise SystemExit(f"[Err] {bad} faces reference vertices that do not exist")
    info = cv.voxinfo_from_device(soup, g)
    morton = o["output"] == "morton"
    table = torch.zeros(cv.table_words(info), dtype=torch.int32, device="cuda")
    t0 = time.perf_counter()
    (cv.voxelize_solid if o["solid"] else cv.voxelize)(info, soup, table, morton)
    torch.cuda.synchronize()
    print(f"[Perf] Voxelization GPU time: {(time.perf_counter() - t0) * 1e3:.1f} ms")
    if o["output"] == "morton":
        path = fn + ".bin"  # write_binary(vtable, vtable_size, filename) (src/main.cpp:240)
        with open(path, "wb") as f:
            f.write(table.cpu().numpy().tobytes())
    elif o["output"] == "binvox":
        path = f"{fn}_{g}.binvox"
        with open(path, "wb") as f:
            f.write(cv.binvox_header(info) + cv.encode_binvox(info, table))
    else:  # obj_points: x, then y, then z; "v x+0.5 y+0.5 z+0.5" (src/util_io.cpp:168-180)
        path = f"{fn}_{g}_pointcloud.obj"
        lst = cv.encode_voxel_list(info, table).cpu().numpy().astype(np.int64)
        gz = int(info.gridsize[2])
        pts = np.stack([lst[:, 0], lst[:, 2], gz - lst[:, 1]], axis=1) + 0.5
        with open(path, "w") as f:
            f.writelines(f"v {p[0]:g} {p[1]:g} {p[2]:g}\n" for p in pts)
    print(f"[I/O] Wrote {path}\n[Perf] Total runtime: {(time.perf_counter() - t_all) * 1e3:.1f} ms")
    return {"path": path, "info": info, "table": table}


def main():
    run(sys.argv[1:])


if __name__ == "__main__":
    main()
