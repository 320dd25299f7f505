"""Seeded synthetic meshes for the benchmark workloads and the parity tests.

No dataset is involved: every mesh is generated from a seed with numpy's PCG64 generator, in
float64, and returned as a float32 triangle soup of shape (n, 9) -- v0.xyz, v1.xyz, v2.xyz per
triangle, the layout the reference uploads (src/main.cpp:61-80).

* :func:`torus`            watertight torus, R = 1.0, r = 0.35, 96 x 48 quads (9,216 triangles),
                           vertices jittered by N(0, 0.002) and randomly rotated.
* :func:`icosphere`        icosahedron subdivided `level` times (20 * 4^level triangles), radially
                           displaced by r = 1 + 0.15 * (sum of 6 sinusoids: 3 in theta, 3 in phi)
                           with integer frequencies in [1, 12] and uniform phases from the seed.
* :func:`soup`             independent equilateral triangles, centres uniform in the unit cube,
                           edge length log-uniform in [0.25/1024, 0.5] (0.25 voxel to half the grid
                           extent of a unit cube at 1024^3), uniformly random orientation.
* :func:`batch_mix`        256 meshes (torus or icosphere) with triangle counts log-uniform in
                           [1k, 500k], grid in {64, 128, 256, 512}, surface:solid = 3:1,
                           linear:Morton = 1:1.
* :func:`poisson_arrivals` arrival times of a Poisson request stream.
"""
from __future__ import annotations

from dataclasses import dataclass
from functools import lru_cache

import numpy as np


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniform random rotation matrix (Shoemake's uniform quaternion)."""
    u1, u2, u3 = rng.random(3)
    q = np.array([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)])
    return _quat_to_mat(q[None, :])[0]


def _quat_to_mat(q: np.ndarray) -> np.ndarray:
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], -2)


def _soup(verts: np.ndarray, faces: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(verts[faces].reshape(-1, 9), dtype=np.float32)


def torus(seed: int = 0, nu: int = 96, nv: int = 48, R: float = 1.0, r: float = 0.35, jitter: float = 0.002,
          rotate: bool = True) -> np.ndarray:
    """Watertight torus: nu x nv quads, two triangles each, shared vertices jittered once."""
    rng = np.random.default_rng(seed)
    u = 2 * np.pi * np.arange(nu) / nu
    v = 2 * np.pi * np.arange(nv) / nv
    uu, vv = np.meshgrid(u, v, indexing="ij")
    verts = np.stack([(R + r * np.cos(vv)) * np.cos(uu), (R + r * np.cos(vv)) * np.sin(uu), r * np.sin(vv)],
                     -1).reshape(-1, 3)
    verts = verts + rng.normal(0.0, jitter, verts.shape)
    if rotate:
        verts = verts @ random_rotation(rng).T
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    a = (i * nv + j).ravel()
    b = (((i + 1) % nu) * nv + j).ravel()
    c = (((i + 1) % nu) * nv + (j + 1) % nv).ravel()
    d = (i * nv + (j + 1) % nv).ravel()
    faces = np.empty((2 * a.size, 3), dtype=np.int64)
    faces[0::2] = np.stack([a, b, c], -1)
    faces[1::2] = np.stack([a, c, d], -1)
    return _soup(verts, faces)


@lru_cache(maxsize=None)
def _icosphere_base(level: int):
    """Unit icosphere (vertices on the sphere, consistently wound faces) after `level` subdivisions."""
    t = (1.0 + 5 ** 0.5) / 2.0
    verts = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t],
                      [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    verts /= np.linalg.norm(verts, axis=1, keepdims=True)
    faces = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                      [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                      [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(level):
        nvert = verts.shape[0]
        e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]], 0)
        key = np.minimum(e[:, 0], e[:, 1]) * nvert + np.maximum(e[:, 0], e[:, 1])
        uniq, inv = np.unique(key, return_inverse=True)
        lo, hi = uniq // nvert, uniq % nvert
        mid = verts[lo] + verts[hi]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        verts = np.concatenate([verts, mid], 0)
        nf = faces.shape[0]
        m01, m12, m20 = (nvert + inv[:nf], nvert + inv[nf:2 * nf], nvert + inv[2 * nf:])
        a, b, c = faces[:, 0], faces[:, 1], faces[:, 2]
        faces = np.concatenate([np.stack([a, m01, m20], -1), np.stack([b, m12, m01], -1),
                                np.stack([c, m20, m12], -1), np.stack([m01, m12, m20], -1)], 0)
    verts.setflags(write=False)
    faces.setflags(write=False)
    return verts, faces


def icosphere(seed: int = 0, level: int = 8, amplitude: float = 0.15) -> np.ndarray:
    """Icosphere subdivided `level` times, radially displaced by 6 seeded sinusoids."""
    rng = np.random.default_rng(seed)
    verts, faces = _icosphere_base(level)
    theta = np.arccos(np.clip(verts[:, 2], -1.0, 1.0))
    phi = np.arctan2(verts[:, 1], verts[:, 0])
    k = rng.integers(1, 13, size=6)
    ph = rng.uniform(0.0, 2 * np.pi, size=6)
    s = np.zeros(verts.shape[0])
    for i in range(6):
        ang = theta if i < 3 else phi
        s += np.sin(k[i] * ang + ph[i])
    r = 1.0 + amplitude * s
    return _soup(verts * r[:, None], faces)


def soup(seed: int = 0, n: int = 2_000_000, lmin: float = 0.25 / 1024, lmax: float = 0.5) -> np.ndarray:
    """Independent equilateral triangles with log-uniform edge length and random orientation."""
    rng = np.random.default_rng(seed)
    centers = rng.random((n, 3))
    L = np.exp(rng.uniform(np.log(lmin), np.log(lmax), size=n))
    ang = np.array([np.pi / 2, np.pi / 2 + 2 * np.pi / 3, np.pi / 2 + 4 * np.pi / 3])
    tmpl = np.stack([np.cos(ang), np.sin(ang), np.zeros(3)], -1) / np.sqrt(3.0)  # circumradius L/sqrt(3)
    u = rng.random((n, 3))
    q = np.stack([np.sqrt(1 - u[:, 0]) * np.sin(2 * np.pi * u[:, 1]), np.sqrt(1 - u[:, 0]) * np.cos(2 * np.pi * u[:, 1]),
                  np.sqrt(u[:, 0]) * np.sin(2 * np.pi * u[:, 2]), np.sqrt(u[:, 0]) * np.cos(2 * np.pi * u[:, 2])], -1)
    out = np.empty((n, 9), dtype=np.float32)
    step = 1 << 20
    for s0 in range(0, n, step):
        s1 = min(n, s0 + step)
        R = _quat_to_mat(q[s0:s1])
        v = np.einsum("nij,kj->nki", R, tmpl) * L[s0:s1, None, None] + centers[s0:s1, None, :]
        out[s0:s1] = v.reshape(-1, 9)
    return out


@dataclass
class MeshSpec:
    kind: str          # "torus" or "icosphere"
    seed: int
    size: int          # torus: nv (nu = 2 nv); icosphere: subdivision level
    gridsize: int
    solid: bool
    morton: bool

    def build(self) -> np.ndarray:
        if self.kind == "torus":
            return torus(self.seed, nu=2 * self.size, nv=self.size)
        return icosphere(self.seed, level=self.size)

    @property
    def n_triangles(self) -> int:
        return 4 * self.size * self.size if self.kind == "torus" else 20 * 4 ** self.size


def draw_spec(rng: np.random.Generator, seed: int) -> MeshSpec:
    """One request of the batched / served distribution."""
    count = float(np.exp(rng.uniform(np.log(1_000), np.log(500_000))))
    kind = "torus" if rng.random() < 0.5 else "icosphere"
    if kind == "torus":
        size = max(8, int(round(np.sqrt(count / 4.0))))           # 2 * (2 nv) * nv triangles
    else:
        size = int(np.clip(np.round(np.log(count / 20.0) / np.log(4.0)), 3, 7))  # nearest level in log
    g = int(rng.choice([64, 128, 256, 512]))
    solid = bool(rng.random() < 0.25)
    morton = bool(rng.random() < 0.5)
    return MeshSpec(kind, seed, size, g, solid, morton)


def batch_mix(seed: int = 0, n: int = 256) -> list[MeshSpec]:
    rng = np.random.default_rng(seed)
    return [draw_spec(rng, seed * 100_003 + i) for i in range(n)]


def poisson_arrivals(rate_per_s: float, duration_s: float, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    n = int(rate_per_s * duration_s * 1.5) + 16
    t = np.cumsum(rng.exponential(1.0 / rate_per_s, size=n))
    return t[t < duration_s]
