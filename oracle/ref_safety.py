"""Keep the reference's solid code inside its table (test infrastructure: the checker, never the
product).

The reference kernel voxelize_triangle_solid (src/voxelize_solid.cu:73-145) never clips x: it XORs
bits x = 0..xmax of each hit column, with xmax = int(get_x_coordinate(...) / unit.x - 0.5)
(:123).  For triangles nearly parallel to the x axis (|n.x| just above its 1e-6 cut-off) or nearly
degenerate, get_x_coordinate divides a cancelling float32 sum by a tiny n.x and xmax can land far
beyond the grid (xmax = 549 at g = 512 on one column of the displaced icosphere; up to 3396 in a
random soup).  In Morton order every x >= g encodes past the end of the table, so the reference
kernel writes outside its buffer; on the GPU this corrupted other allocations and once raised a
memory fault (Xid 31).  In linear order the run continues into the following rows and only leaves
the table from its last rows.

Before the reference kernel runs in a test, `safe_triangles` removes every triangle that could
produce such a write, using float64 geometry with generous margins:
  * triangles whose float32 cross product is exactly zero (the reference's normal is NaN, so it
    only ever writes x = 0) are kept;
  * other triangles are dropped when nearly degenerate (sine of the corner angle < 1e-3) or nearly
    parallel to x (|n.x| < 1e-2), where float32 xmax is not predictable from float64 (at
    |n.x| = 0.0017 a random soup at 1024^3 gave a float32 xmax of 1056 where float64 put the plane
    inside the grid, and the reference wrote past its table);
  * the rest are dropped if, at any column centre the reference can count as a hit (inside the
    triangle's yz projection or within 1e-3 world units of an edge: the reference's 1e-6 tolerance
    on an edge's cross product), the plane's x (plus a 16-voxel margin) reaches g - 1 (Morton) or the run
    x + y*gx + z*gx*gy (plus margin) reaches the end of the table (linear).
The reference's CPU solid loop (src/cpu_voxelizer.cpp:293-296) has the same xmax and one more
hazard: it stores int(...) into an unsigned int, so a negative xmax becomes a loop of about 2^32
iterations writing far outside the table (the displaced icosphere has such a triangle, n.x = -7.6e-5).
The triangles kept here are far from both (the filter drops every |n.x| < 1e-2, and elsewhere the
plane's x at a counted column is inside the mesh's bbox), so the benchmark's CPU legs run the
reference's solid code on them.

The engine itself clips these writes (x to the grid in Morton order, the run to the table in linear
order), so it needs no such filter.
"""
from __future__ import annotations

import numpy as np


def _cross32_zero(t32: np.ndarray) -> np.ndarray:
    v = t32.reshape(-1, 3, 3)
    e0 = v[:, 1] - v[:, 0]
    e1 = v[:, 2] - v[:, 1]
    c = np.cross(e0, e1)  # float32 arithmetic; only its exact zeros are used
    return np.all(c == 0, axis=1)


def safe_triangles(tris: np.ndarray, info_bytes: bytes, morton: bool) -> np.ndarray:
    """Boolean mask of triangles the reference solid kernel can process without writing outside
    its table."""
    t32 = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
    bmin = np.frombuffer(info_bytes, np.float32, 3, 0).astype(np.float64)
    unit = np.frombuffer(info_bytes, np.float32, 3, 48).astype(np.float64)
    g = np.frombuffer(info_bytes, np.uint32, 3, 24).astype(np.int64)
    total = int(g[0] * g[1] * g[2])
    t = t32.reshape(-1, 3, 3).astype(np.float64) - bmin
    v0, v1, v2 = t[:, 0], t[:, 1], t[:, 2]
    e0, e1 = v1 - v0, v2 - v1
    c = np.cross(e0, e1)
    cn = np.linalg.norm(c, axis=1)
    sin = cn / np.maximum(np.linalg.norm(e0, axis=1) * np.linalg.norm(e1, axis=1), 1e-300)
    n = c / np.maximum(cn, 1e-300)[:, None]
    zero = _cross32_zero(t32)
    keep = zero | ((sin >= 1e-3) & (np.abs(n[:, 0]) >= 1e-2))
    cand = np.nonzero(keep & ~zero)[0]
    # column ranges (voxel-centre columns of the yz bbox, widened by one)
    lo = np.minimum(np.minimum(v0, v1), v2)[:, 1:]
    hi = np.maximum(np.maximum(v0, v1), v2)[:, 1:]
    y0 = np.ceil(lo[:, 0] / unit[1] - 0.5).astype(np.int64) - 1
    y1 = np.floor(hi[:, 0] / unit[1] - 0.5).astype(np.int64) + 1
    z0 = np.ceil(lo[:, 1] / unit[2] - 0.5).astype(np.int64) - 1
    z1 = np.floor(hi[:, 1] / unit[2] - 0.5).astype(np.int64) + 1
    ny_cols = np.maximum(y1 - y0 + 1, 0)
    nz_cols = np.maximum(z1 - z0 + 1, 0)
    # The reference accepts a column "on" an edge when |cross(PA, PB)| < 1e-6 (world units squared)
    # and the column centre lies within the edge's bounding box: up to min(L, 1e-6 / L) <= 1e-3
    # world units from an edge of length L.  Columns that close to the projection count as hits.
    tol = max(1e-3 * float(min(unit[1], unit[2])), 1e-3)
    bad = np.zeros(t.shape[0], dtype=bool)
    # process triangles in groups of equal column-count bound to stay vectorised
    cols = ny_cols * nz_cols
    order = cand[np.argsort(cols[cand])]
    start = 0
    while start < order.size:
        k = int(cols[order[start]])
        stop = start
        while stop < order.size and cols[order[stop]] <= max(k, 1) * 2:
            stop += 1
        idx = order[start:stop]
        start = stop
        K = int(cols[idx].max()) if idx.size else 0
        if K == 0:
            continue
        j = np.arange(K)[None, :]
        nzc = np.maximum(nz_cols[idx], 1)[:, None]
        valid = j < cols[idx][:, None]
        yy = y0[idx][:, None] + j // nzc
        zz = z0[idx][:, None] + j % nzc
        py = (yy + 0.5) * unit[1]
        pz = (zz + 0.5) * unit[2]
        a, b, cc = v0[idx][:, None, 1:], v1[idx][:, None, 1:], v2[idx][:, None, 1:]
        p = np.stack([py, pz], -1)

        def seg_dist(p, q, r):
            d = r - q
            L2 = np.maximum(np.sum(d * d, -1), 1e-300)
            s = np.clip(np.sum((p - q) * d, -1) / L2, 0, 1)
            return np.linalg.norm(p - (q + s[..., None] * d), axis=-1)

        def side(p, q, r):
            return (r[..., 0] - q[..., 0]) * (p[..., 1] - q[..., 1]) - (r[..., 1] - q[..., 1]) * (p[..., 0] - q[..., 0])

        s1, s2, s3 = side(p, a, b), side(p, b, cc), side(p, cc, a)
        inside = ((s1 >= 0) & (s2 >= 0) & (s3 >= 0)) | ((s1 <= 0) & (s2 <= 0) & (s3 <= 0))
        near = np.minimum(np.minimum(seg_dist(p, a, b), seg_dist(p, b, cc)), seg_dist(p, cc, a)) <= tol
        hit = valid & (inside | near)
        nn = n[idx]
        xh = -(nn[:, 1:2] * (py - v0[idx][:, 1:2]) + nn[:, 2:3] * (pz - v0[idx][:, 2:3])) / nn[:, 0:1] + v0[idx][:, 0:1]
        xmax = xh / unit[0] - 0.5 + 16.0
        if morton:
            over = hit & (xmax >= g[0] - 1)
        else:
            lin = xmax + yy * g[0] + zz * g[0] * g[1]
            over = hit & ((lin >= total - 1) | (yy < 0) | (zz < 0) | (yy >= g[1]) | (zz >= g[2]))
        bad[idx] = np.any(over, axis=1)
    return keep & ~bad
