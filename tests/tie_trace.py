"""Trace differing voxels to boundary ties (test infrastructure).

The reference GPU kernels and the reference CPU voxelizer evaluate the same predicates with
different fp32 arithmetic (the GPU contracts a*b+c into fused multiply-adds and uses the
approximate rsqrtf; the CPU rounds every product and uses 1/sqrtf), so their bit tables may differ
where a predicate is within rounding of zero.  These helpers re-evaluate the predicates in float64
and report, for each differing voxel (surface) or row (solid), the smallest normalised margin of any
triangle there; a difference is "traced to a tie" when that margin is below the tolerance.

Surface (src/voxelize.cu:71-165): margins in voxel units of the plane test and the nine edge tests.
Solid (src/voxelize_solid.cu:83-123): margin of the point-in-triangle test (distance of the column
centre to the nearest edge, and of |t| to the 1e-6 edge tolerance) and of xmax (distance of
x_hit / unit.x - 0.5 to the nearest integer).
"""
from __future__ import annotations

import numpy as np


def _setup(tris: np.ndarray, info: bytes):
    bmin = np.frombuffer(info, np.float32, 3, 0).astype(np.float64)
    unit = np.frombuffer(info, np.float32, 3, 48).astype(np.float64)
    grid = np.frombuffer(info, np.uint32, 3, 24).astype(np.int64)
    t = tris.reshape(-1, 3, 3).astype(np.float64) - bmin
    return t, unit, grid


def linear_to_xyz(bits: np.ndarray, grid, morton: bool):
    if morton:
        def compact(v):
            out = np.zeros_like(v)
            for i in range(21):
                out |= ((v >> (3 * i)) & 1) << i
            return out
        return compact(bits), compact(bits >> 1), compact(bits >> 2)
    gx, gy = int(grid[0]), int(grid[1])
    return bits % gx, (bits // gx) % gy, bits // (gx * gy)


def diff_bits(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Indices (MSB-first bit order) of differing bits of two uint32 tables."""
    x = (a.view(np.uint32) ^ b.view(np.uint32))
    w = np.nonzero(x)[0]
    out = []
    for wi in w:
        v = int(x[wi])
        for k in range(32):
            if v & (0x80000000 >> k):
                out.append(int(wi) * 32 + k)
    return np.array(out, dtype=np.int64)


def surface_margin(tris: np.ndarray, info: bytes, vox: np.ndarray) -> np.ndarray:
    """For each voxel (x, y, z) the smallest |margin| (voxel units) over triangles whose grid bbox
    holds it and which pass every test at it within that margin."""
    t, unit, grid = _setup(tris, info)
    v0, v1, v2 = t[:, 0], t[:, 1], t[:, 2]
    e = [v1 - v0, v2 - v1, v0 - v2]
    n = np.cross(e[0], e[1])
    nn = np.linalg.norm(n, axis=1, keepdims=True)
    nn[nn == 0] = 1
    n = n / nn
    lo = np.clip(np.floor(np.minimum(np.minimum(v0, v1), v2) / unit), 0, grid - 1)
    hi = np.clip(np.floor(np.maximum(np.maximum(v0, v1), v2) / unit), 0, grid - 1)
    c = np.where(n > 0, unit, 0.0)
    d1 = np.sum(n * (c - v0), axis=1)
    d2 = np.sum(n * ((unit - c) - v0), axis=1)
    vs = [v0, v1, v2]
    res = np.full(len(vox), np.inf)
    for k, p in enumerate(vox):
        inb = np.all((lo <= p) & (p <= hi), axis=1)
        idx = np.nonzero(inb)[0]
        if idx.size == 0:
            continue
        pw = p * unit
        margins = []
        s = n[idx] @ pw
        scale_p = np.abs(n[idx]) @ unit + 1e-300
        margins.append(np.minimum(s + d1[idx], -(s + d2[idx])) / scale_p)
        for (a, b, sgn_axis) in ((0, 1, 2), (1, 2, 0), (2, 0, 1)):
            sgn = np.where(n[idx, sgn_axis] < 0, -1.0, 1.0)
            for i in range(3):
                ne = np.stack([-e[i][idx, b], e[i][idx, a]], 1) * sgn[:, None]
                d = -(ne[:, 0] * vs[i][idx, a] + ne[:, 1] * vs[i][idx, b]) + np.maximum(0, unit[a] * ne[:, 0]) + \
                    np.maximum(0, unit[b] * ne[:, 1])
                val = ne[:, 0] * pw[a] + ne[:, 1] * pw[b] + d
                scale = np.abs(ne[:, 0]) * unit[a] + np.abs(ne[:, 1]) * unit[b] + 1e-300
                margins.append(val / scale)
        m = np.min(np.stack(margins, 1), axis=1)  # >= 0: inside in exact arithmetic
        res[k] = np.min(np.abs(m))
    return res


def solid_row_margin(tris: np.ndarray, info: bytes, rows) -> np.ndarray:
    """For each row (y, z): the smallest margin over triangles whose column test or xmax at the
    row's column centre is near a decision boundary (absolute units: voxels for xmax and edge
    distance, and the distance of |t| to the 1e-6 tolerance relative to |t| scale)."""
    t, unit, grid = _setup(tris, info)
    v0, v1, v2 = t[:, 0], t[:, 1], t[:, 2]
    n = np.cross(v1 - v0, v2 - v1)
    nn = np.linalg.norm(n, axis=1, keepdims=True)
    nn[nn == 0] = 1
    n = n / nn
    out = np.full(len(rows), np.inf)
    P = [t[:, i, 1:3] for i in range(3)]
    for k, (y, z) in enumerate(rows):
        pt = np.array([(y + 0.5) * unit[1], (z + 0.5) * unit[2]])
        lo = np.minimum(np.minimum(P[0], P[1]), P[2])
        hi = np.maximum(np.maximum(P[0], P[1]), P[2])
        near = np.all((lo - unit[1:] <= pt) & (pt <= hi + unit[1:]), axis=1)
        idx = np.nonzero(near)[0]
        best = np.inf
        for i in idx:
            a, b, c = P[0][i], P[1][i], P[2][i]
            ms = []
            for (p, q) in ((a, b), (b, c), (c, a)):
                ev = q - p
                L = np.hypot(*ev) + 1e-300
                cr = (pt[0] - p[0]) * (pt[1] - q[1]) - (pt[1] - p[1]) * (pt[0] - q[0])
                ms.append(abs(cr) / L / unit[1])                     # distance to the edge line, voxels
                ms.append(abs(abs(cr) - 1e-6) / (L * unit[1] + 1e-300))  # distance to the 1e-6 tolerance
            if abs(n[i, 0]) > 0:
                xh = -(n[i, 1] * (pt[0] - v0[i, 1]) + n[i, 2] * (pt[1] - v0[i, 2])) / n[i, 0] + v0[i, 0]
                q = xh / unit[0] - 0.5
                ms.append(abs(q - np.round(q)))
                ms.append(abs(abs(n[i, 0]) - 1e-6) / 1e-6)
            best = min(best, min(ms))
        out[k] = best
    return out
