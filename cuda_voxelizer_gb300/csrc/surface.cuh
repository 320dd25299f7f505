// surface.cuh -- exact surface-voxelization predicates (Schwarz-Seidel triangle/box overlap) and
// the row-interval search built on them.
//
// Reference: voxelize_triangle, src/voxelize.cu:58-190.  Per triangle the reference computes a
// plane test (:89-95) and nine 2D edge functions (:97-133) once, then tests every voxel of the
// triangle's grid bbox (:136-181).  Here the per-triangle part is SurfTri/surf_setup; the per-voxel
// part is fail_bits + yz_pass, which evaluate the very same fp32 expressions for a voxel (x, y, z).
//
// Row intervals.  For a fixed row (y, z) every test depends on x only through p.x = x * unit.x,
// and each test value is a composition of correctly rounded, monotone operations of p.x.  So each
// edge test passes on a prefix or a suffix of x, and so does each side of the plane test (see
// fail_bits).  The voxels of a row that pass all tests therefore form one interval [xl, xh].
// row_interval finds it: a real-valued estimate of every test's crossing picks the candidate
// ends, then exact evaluations at the candidates (and a walk if an estimate was off) pin them.
// The result is identical to testing every voxel of the row; only the number of evaluations
// changes.
#pragma once
#include "cvx_device.cuh"

namespace cvx {

struct SurfTri {
	float nx, ny, nz, d1, d2;
	float exy[3][2], eyz[3][2], ezx[3][2];   // edge normals n_xy_ei, n_yz_ei, n_zx_ei after the flips
	float dxy[3], dyz[3], dzx[3];
	int bx0, by0, bz0, bx1, by1, bz1;        // clamped grid bbox
};

// dot(n_e, v) of the setup, a.x*v.x + a.y*v.y, where n_e = (-e.?, e.?) may have been negated
// (flip < 0).  Pattern 3: second product fused unless flipped, then the first; 4: the opposite.
template <int P>
__device__ __forceinline__ float setup_dot(float ax, float vx, float ay, float vy, float flip) {
	if constexpr (P == 3) return flip < 0.0f ? mul_add<1>(ax, vx, ay, vy) : mul_add<2>(ax, vx, ay, vy);
	else if constexpr (P == 4) return flip < 0.0f ? mul_add<2>(ax, vx, ay, vy) : mul_add<1>(ax, vx, ay, vy);
	else return mul_add<P>(ax, vx, ay, vy);
}

// Triangle setup, src/voxelize.cu:71-133.  `t` holds v0.xyz, v1.xyz, v2.xyz in world space.
template <class P>
__device__ __forceinline__ void surf_setup(const float* t, const float* bmin, const float* unit, const float* inv,
                                           const uint32_t* grid, SurfTri& S) {
	const float v0x = __fsub_rn(t[0], bmin[0]), v0y = __fsub_rn(t[1], bmin[1]), v0z = __fsub_rn(t[2], bmin[2]);
	const float v1x = __fsub_rn(t[3], bmin[0]), v1y = __fsub_rn(t[4], bmin[1]), v1z = __fsub_rn(t[5], bmin[2]);
	const float v2x = __fsub_rn(t[6], bmin[0]), v2y = __fsub_rn(t[7], bmin[1]), v2z = __fsub_rn(t[8], bmin[2]);
	const float e0x = __fsub_rn(v1x, v0x), e0y = __fsub_rn(v1y, v0y), e0z = __fsub_rn(v1z, v0z);
	const float e1x = __fsub_rn(v2x, v1x), e1y = __fsub_rn(v2y, v1y), e1z = __fsub_rn(v2z, v1z);
	const float e2x = __fsub_rn(v0x, v2x), e2y = __fsub_rn(v0y, v2y), e2z = __fsub_rn(v0z, v2z);
	// n = normalize(cross(e0, e1))  (helper_math cross / normalize: v * rsqrtf(dot(v, v)))
	const float cx = mul_sub<P::cross>(e0y, e1z, e0z, e1y);
	const float cy = mul_sub<P::cross>(e0z, e1x, e0x, e1z);
	const float cz = mul_sub<P::cross>(e0x, e1y, e0y, e1x);
	const float rlen = rsqrtf(dot3<P::dot3>(cx, cy, cz, cx, cy, cz));
	S.nx = __fmul_rn(cx, rlen);
	S.ny = __fmul_rn(cy, rlen);
	S.nz = __fmul_rn(cz, rlen);

	// grid bbox: clamp(int(min(v) / unit), 0, g - 1)  (:83-87)
	const int gmx = (int)grid[0] - 1, gmy = (int)grid[1] - 1, gmz = (int)grid[2] - 1;
	S.bx0 = min(max(div_trunc(fminf(v0x, fminf(v1x, v2x)), unit[0], inv[0]), 0), gmx);
	S.by0 = min(max(div_trunc(fminf(v0y, fminf(v1y, v2y)), unit[1], inv[1]), 0), gmy);
	S.bz0 = min(max(div_trunc(fminf(v0z, fminf(v1z, v2z)), unit[2], inv[2]), 0), gmz);
	S.bx1 = min(max(div_trunc(fmaxf(v0x, fmaxf(v1x, v2x)), unit[0], inv[0]), 0), gmx);
	S.by1 = min(max(div_trunc(fmaxf(v0y, fmaxf(v1y, v2y)), unit[1], inv[1]), 0), gmy);
	S.bz1 = min(max(div_trunc(fmaxf(v0z, fmaxf(v1z, v2z)), unit[2], inv[2]), 0), gmz);

	// plane test: critical point c and d1, d2  (:90-95)
	const float cxp = S.nx > 0.0f ? unit[0] : 0.0f;
	const float cyp = S.ny > 0.0f ? unit[1] : 0.0f;
	const float czp = S.nz > 0.0f ? unit[2] : 0.0f;
	S.d1 = dot3<P::dot3d>(S.nx, S.ny, S.nz, __fsub_rn(cxp, v0x), __fsub_rn(cyp, v0y), __fsub_rn(czp, v0z));
	S.d2 = dot3<P::dot3d>(S.nx, S.ny, S.nz, __fsub_rn(__fsub_rn(unit[0], cxp), v0x),
	                     __fsub_rn(__fsub_rn(unit[1], cyp), v0y), __fsub_rn(__fsub_rn(unit[2], czp), v0z));

	// projection tests (:97-133).  n_xy_e = (-e.y, e.x), negated when n.z < 0; d = -dot(n_e, v) +
	// max(0, u.a * n_e.x) + max(0, u.b * n_e.y).
	const float ex[3] = {e0x, e1x, e2x}, ey[3] = {e0y, e1y, e2y}, ez[3] = {e0z, e1z, e2z};
	const float vx[3] = {v0x, v1x, v2x}, vy[3] = {v0y, v1y, v2y}, vz[3] = {v0z, v1z, v2z};
	const float sxy = S.nz < 0.0f ? -1.0f : 1.0f;
	const float syz = S.nx < 0.0f ? -1.0f : 1.0f;
	const float szx = S.ny < 0.0f ? -1.0f : 1.0f;
#pragma unroll
	for (int i = 0; i < 3; i++) {
		// -1.0f * e.y and the sign flips are exact negations
		const float axy = sxy * -ey[i], bxy = sxy * ex[i];
		const float ayz = syz * -ez[i], byz = syz * ey[i];
		const float azx = szx * -ex[i], bzx = szx * ez[i];
		S.exy[i][0] = axy; S.exy[i][1] = bxy;
		S.eyz[i][0] = ayz; S.eyz[i][1] = byz;
		S.ezx[i][0] = azx; S.ezx[i][1] = bzx;
		S.dxy[i] = __fadd_rn(__fadd_rn(-setup_dot<P::dot2_xy>(axy, vx[i], bxy, vy[i], sxy), fmaxf(0.0f, __fmul_rn(unit[0], axy))),
		                     fmaxf(0.0f, __fmul_rn(unit[1], bxy)));
		S.dyz[i] = __fadd_rn(__fadd_rn(-setup_dot<P::dot2_yz>(ayz, vy[i], byz, vz[i], syz), fmaxf(0.0f, __fmul_rn(unit[1], ayz))),
		                     fmaxf(0.0f, __fmul_rn(unit[2], byz)));
		S.dzx[i] = __fadd_rn(__fadd_rn(-setup_dot<P::dot2_zx>(azx, vz[i], bzx, vx[i], szx), fmaxf(0.0f, __fmul_rn(unit[0], azx))),
		                     fmaxf(0.0f, __fmul_rn(unit[2], bzx)));
	}
}

// Per-row constants of the x-dependent tests (products that do not involve p.x).
struct RowK {
	float py, pz;
	float kpl;       // plane: ny*py (pattern 1) / the partial sum the pattern keeps fixed
	float kpl2;      // plane: nz*pz (pattern 2)
	float kxy[3];    // XY edge i: n_xy.y * p.y (pattern 1)
	float kzx[3];    // ZX edge i: n_zx.x * p.z (pattern 2)
};

template <class P>
__device__ __forceinline__ void row_consts(const SurfTri& S, float py, float pz, RowK& K) {
	K.py = py;
	K.pz = pz;
	K.kpl = __fmul_rn(S.ny, py);
	K.kpl2 = __fmul_rn(S.nz, pz);
#pragma unroll
	for (int i = 0; i < 3; i++) {
		K.kxy[i] = __fmul_rn(S.exy[i][1], py);
		K.kzx[i] = __fmul_rn(S.ezx[i][0], pz);
	}
}

// Bit i set = x-dependent test i fails at voxel x of the row.
//   bit 0: plane test fails with both (s+d1), (s+d2) < 0   ("below" the slab)
//   bit 1: plane test fails with both > 0                  ("above")
//   bits 2-4: XY edge tests, bits 5-7: ZX edge tests.
// The reference fails the plane test iff (s+d1)*(s+d2) > 0 (:146); a positive product needs equal
// signs, so bit0|bit1 is exactly that condition.  As x grows, s moves monotonically; "below"
// holds on one end of the row and "above" on the other, so each bit flips at most once.
template <class P>
__device__ __forceinline__ uint32_t fail_bits(const SurfTri& S, const RowK& K, float ux, int x) {
	const float px = __fmul_rn(__int2float_rn(x), ux);
	float s;
	if constexpr (P::plane == 1) s = __fmaf_rn(S.nz, K.pz, __fmaf_rn(S.nx, px, K.kpl));
	else if constexpr (P::plane == 2) s = __fadd_rn(__fmaf_rn(S.nx, px, K.kpl), K.kpl2);
	else if constexpr (P::plane == 3) s = __fmaf_rn(S.nz, K.pz, __fmaf_rn(S.ny, K.py, __fmul_rn(S.nx, px)));
	else s = __fadd_rn(__fadd_rn(__fmul_rn(S.nx, px), K.kpl), K.kpl2);
	const float a = __fadd_rn(s, S.d1), b = __fadd_rn(s, S.d2);
	const bool pf = __fmul_rn(a, b) > 0.0f;
	uint32_t f = (pf && a < 0.0f ? 1u : 0u) | (pf && a > 0.0f ? 2u : 0u);
#pragma unroll
	for (int i = 0; i < 3; i++) {
		float v;
		if constexpr (P::edge_xy == 1) v = __fmaf_rn(S.exy[i][0], px, K.kxy[i]);
		else v = mul_add<P::edge_xy>(S.exy[i][0], px, S.exy[i][1], K.py);
		f |= (__fadd_rn(v, S.dxy[i]) < 0.0f ? 1u : 0u) << (2 + i);
	}
#pragma unroll
	for (int i = 0; i < 3; i++) {
		float v;
		if constexpr (P::edge_zx == 2) v = __fmaf_rn(S.ezx[i][1], px, K.kzx[i]);
		else v = mul_add<P::edge_zx>(S.ezx[i][0], K.pz, S.ezx[i][1], px);
		f |= (__fadd_rn(v, S.dzx[i]) < 0.0f ? 1u : 0u) << (5 + i);
	}
	return f;
}

// All x-dependent tests at once, as one pass/fail (the small-triangle path needs no more).
template <class P>
__device__ __forceinline__ bool voxel_pass(const SurfTri& S, const RowK& K, float ux, int x) {
	const float px = __fmul_rn(__int2float_rn(x), ux);
	float s;
	if constexpr (P::plane == 1) s = __fmaf_rn(S.nz, K.pz, __fmaf_rn(S.nx, px, K.kpl));
	else if constexpr (P::plane == 2) s = __fadd_rn(__fmaf_rn(S.nx, px, K.kpl), K.kpl2);
	else if constexpr (P::plane == 3) s = __fmaf_rn(S.nz, K.pz, __fmaf_rn(S.ny, K.py, __fmul_rn(S.nx, px)));
	else s = __fadd_rn(__fadd_rn(__fmul_rn(S.nx, px), K.kpl), K.kpl2);
	bool ok = !(__fmul_rn(__fadd_rn(s, S.d1), __fadd_rn(s, S.d2)) > 0.0f);
#pragma unroll
	for (int i = 0; i < 3; i++) {
		float v;
		if constexpr (P::edge_xy == 1) v = __fmaf_rn(S.exy[i][0], px, K.kxy[i]);
		else v = mul_add<P::edge_xy>(S.exy[i][0], px, S.exy[i][1], K.py);
		ok = ok && !(__fadd_rn(v, S.dxy[i]) < 0.0f);
	}
#pragma unroll
	for (int i = 0; i < 3; i++) {
		float v;
		if constexpr (P::edge_zx == 2) v = __fmaf_rn(S.ezx[i][1], px, K.kzx[i]);
		else v = mul_add<P::edge_zx>(S.ezx[i][0], K.pz, S.ezx[i][1], px);
		ok = ok && !(__fadd_rn(v, S.dzx[i]) < 0.0f);
	}
	return ok;
}

// A small triangle's setup parked in shared memory between the two phases of the classify kernel
// (36 words): SurfTri without the bbox maxima, which are packed as extents (each below 256).
struct SmallTri {
	float v[32];           // nx ny nz d1 d2, exy[3][2], eyz[3][2], ezx[3][2], dxy[3], dyz[3], dzx[3]
	int bx0, by0, bz0;
	uint32_t ext;          // (bx1-bx0) | (by1-by0) << 8 | (bz1-bz0) << 16
};

__device__ __forceinline__ void pack_small(const SurfTri& S, SmallTri& o) {
	o.v[0] = S.nx; o.v[1] = S.ny; o.v[2] = S.nz; o.v[3] = S.d1; o.v[4] = S.d2;
#pragma unroll
	for (int i = 0; i < 3; i++) {
		o.v[5 + 2 * i] = S.exy[i][0]; o.v[6 + 2 * i] = S.exy[i][1];
		o.v[11 + 2 * i] = S.eyz[i][0]; o.v[12 + 2 * i] = S.eyz[i][1];
		o.v[17 + 2 * i] = S.ezx[i][0]; o.v[18 + 2 * i] = S.ezx[i][1];
		o.v[23 + i] = S.dxy[i]; o.v[26 + i] = S.dyz[i]; o.v[29 + i] = S.dzx[i];
	}
	o.bx0 = S.bx0; o.by0 = S.by0; o.bz0 = S.bz0;
	o.ext = (uint32_t)(S.bx1 - S.bx0) | ((uint32_t)(S.by1 - S.by0) << 8) | ((uint32_t)(S.bz1 - S.bz0) << 16);
}

__device__ __forceinline__ void unpack_small(const SmallTri& o, SurfTri& S) {
	S.nx = o.v[0]; S.ny = o.v[1]; S.nz = o.v[2]; S.d1 = o.v[3]; S.d2 = o.v[4];
#pragma unroll
	for (int i = 0; i < 3; i++) {
		S.exy[i][0] = o.v[5 + 2 * i]; S.exy[i][1] = o.v[6 + 2 * i];
		S.eyz[i][0] = o.v[11 + 2 * i]; S.eyz[i][1] = o.v[12 + 2 * i];
		S.ezx[i][0] = o.v[17 + 2 * i]; S.ezx[i][1] = o.v[18 + 2 * i];
		S.dxy[i] = o.v[23 + i]; S.dyz[i] = o.v[26 + i]; S.dzx[i] = o.v[29 + i];
	}
	S.bx0 = o.bx0; S.by0 = o.by0; S.bz0 = o.bz0;
	S.bx1 = o.bx0 + (int)(o.ext & 0xFFu);
	S.by1 = o.by0 + (int)((o.ext >> 8) & 0xFFu);
	S.bz1 = o.bz0 + (int)((o.ext >> 16) & 0xFFu);
}

// YZ edge tests for row (y, z): independent of x.  Bit i set = YZ edge i fails.
template <class P>
__device__ __forceinline__ uint32_t yz_fail_bits(const SurfTri& S, float py, float pz) {
	uint32_t f = 0;
#pragma unroll
	for (int i = 0; i < 3; i++) {
		const float v = mul_add<P::edge_yz>(S.eyz[i][0], py, S.eyz[i][1], pz);
		f |= (__fadd_rn(v, S.dyz[i]) < 0.0f ? 1u : 0u) << i;
	}
	return f;
}

// Direction of every x-dependent test for this triangle: lo = passes on a suffix of x (a lower
// bound), hi = passes on a prefix (an upper bound); tests in neither mask do not depend on x.
// The reciprocals only steer where the exact walk of row_interval starts, so the fast
// approximate division is enough (an infinite or NaN estimate falls back to the bbox end).
struct RowDirs {
	uint32_t lo, hi;
	float inv[8];    // -1 / (coefficient of x in the test, in voxels): x* = (row term + d) * inv
};

__device__ __forceinline__ void row_dirs(const SurfTri& S, float ux, RowDirs& D) {
	D.lo = 0; D.hi = 0;
	// plane: s increases with x when n.x > 0. "below" (bit 0) then holds on a prefix -> lower bound.
	if (S.nx > 0.0f) { D.lo |= 1u; D.hi |= 2u; }
	else if (S.nx < 0.0f) { D.lo |= 2u; D.hi |= 1u; }
	const float ipl = __fdividef(-1.0f, S.nx * ux);
	D.inv[0] = ipl; D.inv[1] = ipl;
#pragma unroll
	for (int i = 0; i < 3; i++) {
		const float cxy = S.exy[i][0], czx = S.ezx[i][1];
		if (cxy > 0.0f) D.lo |= 1u << (2 + i); else if (cxy < 0.0f) D.hi |= 1u << (2 + i);
		if (czx > 0.0f) D.lo |= 1u << (5 + i); else if (czx < 0.0f) D.hi |= 1u << (5 + i);
		D.inv[2 + i] = __fdividef(-1.0f, cxy * ux);
		D.inv[5 + i] = __fdividef(-1.0f, czx * ux);
	}
}

// Real-valued crossing of test i (in voxel x units) for the row.
__device__ __forceinline__ float crossing(const SurfTri& S, const RowDirs& D, float py, float pz, int i) {
	if (i == 0) return (S.ny * py + S.nz * pz + S.d1) * D.inv[0];
	if (i == 1) return (S.ny * py + S.nz * pz + S.d2) * D.inv[1];
	if (i < 5) return (S.exy[i - 2][1] * py + S.dxy[i - 2]) * D.inv[i];
	return (S.ezx[i - 5][0] * pz + S.dzx[i - 5]) * D.inv[i];
}

// Exact pass interval of row (y, z) within [bx0, bx1] (a sub-range of the triangle's bbox: each
// test is monotone on any range).  Returns false if the row is empty.  Correct for any estimate
// quality: the estimates only choose where the exact walk starts.
template <class P>
__device__ __forceinline__ bool row_interval_in(const SurfTri& S, const RowDirs& D, const RowK& K, float ux, int bx0,
                                                int bx1, int& xl, int& xh) {
	const uint32_t cmask = ~(D.lo | D.hi) & 0xFFu;
	// tests that do not depend on x: evaluate once
	if (cmask && (fail_bits<P>(S, K, ux, bx0) & cmask)) return false;
	// candidate ends from the real-valued crossings
	float elo = (float)bx0, ehi = (float)bx1;
#pragma unroll
	for (int i = 0; i < 8; i++) {
		const uint32_t bit = 1u << i;
		if ((D.lo | D.hi) & bit) {
			const float c = crossing(S, D, K.py, K.pz, i);
			if (D.lo & bit) elo = fmaxf(elo, ceilf(c));
			else ehi = fminf(ehi, floorf(c));
		}
	}
	// lower end: first x with every lower-bound test passing
	int e = (int)fminf(fmaxf(elo, (float)bx0), (float)bx1);
	if (!(fail_bits<P>(S, K, ux, e) & D.lo)) {
		while (e > bx0 && !(fail_bits<P>(S, K, ux, e - 1) & D.lo)) e--;
	} else {
		do { e++; } while (e <= bx1 && (fail_bits<P>(S, K, ux, e) & D.lo));
		if (e > bx1) return false;
	}
	xl = e;
	// upper end: last x >= xl with every upper-bound test passing
	int f = (int)fminf(fmaxf(ehi, (float)xl), (float)bx1);
	if (!(fail_bits<P>(S, K, ux, f) & D.hi)) {
		while (f < bx1 && !(fail_bits<P>(S, K, ux, f + 1) & D.hi)) f++;
	} else {
		do { f--; } while (f >= xl && (fail_bits<P>(S, K, ux, f) & D.hi));
		if (f < xl) return false;
	}
	xh = f;
	return true;
}

// The x-dependent tests selected by `mask` at voxel x (bit i set = test i fails; bit layout of
// fail_bits): the tests outside the mask are not evaluated.
template <class P>
__device__ __forceinline__ uint32_t fail_bits_masked(const SurfTri& S, const RowK& K, float ux, int x, uint32_t mask) {
	const float px = __fmul_rn(__int2float_rn(x), ux);
	uint32_t f = 0;
	if (mask & 3u) {
		float s;
		if constexpr (P::plane == 1) s = __fmaf_rn(S.nz, K.pz, __fmaf_rn(S.nx, px, K.kpl));
		else if constexpr (P::plane == 2) s = __fadd_rn(__fmaf_rn(S.nx, px, K.kpl), K.kpl2);
		else if constexpr (P::plane == 3) s = __fmaf_rn(S.nz, K.pz, __fmaf_rn(S.ny, K.py, __fmul_rn(S.nx, px)));
		else s = __fadd_rn(__fadd_rn(__fmul_rn(S.nx, px), K.kpl), K.kpl2);
		const float a = __fadd_rn(s, S.d1), b = __fadd_rn(s, S.d2);
		const bool pf = __fmul_rn(a, b) > 0.0f;
		f = (pf && a < 0.0f ? 1u : 0u) | (pf && a > 0.0f ? 2u : 0u);
	}
#pragma unroll
	for (int i = 0; i < 3; i++) {
		if (mask & (4u << i)) {
			float v;
			if constexpr (P::edge_xy == 1) v = __fmaf_rn(S.exy[i][0], px, K.kxy[i]);
			else v = mul_add<P::edge_xy>(S.exy[i][0], px, S.exy[i][1], K.py);
			f |= (__fadd_rn(v, S.dxy[i]) < 0.0f ? 4u : 0u) << i;
		}
	}
#pragma unroll
	for (int i = 0; i < 3; i++) {
		if (mask & (32u << i)) {
			float v;
			if constexpr (P::edge_zx == 2) v = __fmaf_rn(S.ezx[i][1], px, K.kzx[i]);
			else v = mul_add<P::edge_zx>(S.ezx[i][0], K.pz, S.ezx[i][1], px);
			f |= (__fadd_rn(v, S.dzx[i]) < 0.0f ? 32u : 0u) << i;
		}
	}
	return f & mask;
}

// Exact pass interval of row (y, z) within the triangle's bbox [S.bx0, S.bx1].
template <class P>
__device__ __forceinline__ bool row_interval(const SurfTri& S, const RowDirs& D, const RowK& K, float ux, int& xl,
                                             int& xh) {
	return row_interval_in<P>(S, D, K, ux, S.bx0, S.bx1, xl, xh);
}

// Certified x-interval of a row, without walking.
//
// Each x-dependent test i has the form "fails iff g(x) < 0" (or > 0 for the plane's "above" side)
// with g(x) = fl(fl(fl(fma(a, fl(x * ux), k1)) + k2) + d): a the test's coefficient of x, k1 and k2
// the row constants (k2 = 0 for the edge tests), d the triangle constant.  Its real counterpart
// G(x) = a*ux*x + k1 + k2 + d is linear with root x* = -(k1 + k2 + d) / (a * ux).  Rounding moves
// each intermediate by at most u = 2^-24 relative, and the last rounding preserves the sign, so
// sign(g(x)) = sign(G(x) + E) with |E| <= 3.01u (|a ux x| + |k1| + |k2|): the float test agrees with
// the real one at every integer x with |x - x*| > W = 3.01u (|x| + (|k1| + |k2|) / |a ux|).  The
// estimate xe = fl(fl(k1 + k2 + d) * inv), inv the fast reciprocal of -a * ux, is within
// 2.01u (|k1| + |k2| + |d|) |inv| + 5u |xe| of x*.  So with the band
//     B = 2^-20 (|xe| + (|k1| + |k2| + |d|) |inv| + 1)  >=  W + |xe - x*| + the rounding of xe +- B,
// every integer outside [xe - B, xe + B] is decided like the real test; when B < 1/4 the band holds
// at most one integer, and that one is decided by evaluating the float test there.  The plane's two
// sides use a = fl(s + d1) and b = fl(s + d2) with the same s: for d1 >= d2 rounding keeps b <= a,
// so "below" fails iff a < 0 and "above" iff b > 0, except when the product a * b underflows, which
// needs |a| < 2^-75 and cannot happen outside the band while |n.x * ux| >= 2^-40.  The lower end is
// the largest first-passing x of the tests that pass on a suffix, the upper end the smallest last-
// passing x of those that pass on a prefix.  Identical to row_interval_in wherever it answers; it
// declines (returns 2) for x-independent tests, d1 < d2, crossings beyond 2^22 voxels or bands of a
// quarter voxel and more, and the caller then uses row_interval_in.  Returns 1 with [xl, xh] set,
// or 0 for an empty row.
template <class P>
__device__ __forceinline__ int row_interval_cert(const SurfTri& S, const RowDirs& D, const RowK& K, float ux, int bx0,
                                                 int bx1, int& xl, int& xh) {
	static_assert(P::plane == 2 && P::edge_xy == 1 && P::edge_zx == 2,
	              "the certified row interval follows the pinned fused-multiply-add pattern");
	if (((D.lo | D.hi) & 0xFFu) != 0xFFu || !(S.d1 >= S.d2) || !(fabsf(D.inv[0]) <= 1e12f)) return 2;
	constexpr float kBand = 0x1p-20f;
	float lo = (float)bx0, hi = (float)bx1;
	bool ok = true;
	const float kp = __fadd_rn(K.kpl, K.kpl2), mp = fabsf(K.kpl) + fabsf(K.kpl2);
#pragma unroll
	for (int i = 0; i < 8; i++) {
		float t, m;
		if (i == 0) { t = __fadd_rn(kp, S.d1); m = mp + fabsf(S.d1); }
		else if (i == 1) { t = __fadd_rn(kp, S.d2); m = mp + fabsf(S.d2); }
		else if (i < 5) { t = __fadd_rn(K.kxy[i - 2], S.dxy[i - 2]); m = fabsf(K.kxy[i - 2]) + fabsf(S.dxy[i - 2]); }
		else { t = __fadd_rn(K.kzx[i - 5], S.dzx[i - 5]); m = fabsf(K.kzx[i - 5]) + fabsf(S.dzx[i - 5]); }
		const float inv = D.inv[i];
		const float xe = __fmul_rn(t, inv);
		const float B = kBand * (fabsf(xe) + m * fabsf(inv) + 1.0f);
		ok = ok && fabsf(xe) < 4194304.0f && B < 0.25f && inv != 0.0f;  // false for NaN too
		const bool is_lo = (D.lo >> i) & 1u;
		const float c = is_lo ? ceilf(xe - B) : floorf(xe + B);  // the one integer the band may hold
		float e = c;
		if (ok && (is_lo ? c < xe + B : c > xe - B)) {
			const bool fails = fail_bits_masked<P>(S, K, ux, (int)c, 1u << i) != 0u;
			e = is_lo ? (fails ? c + 1.0f : c) : (fails ? c - 1.0f : c);
		}
		if (is_lo) lo = fmaxf(lo, e); else hi = fminf(hi, e);
	}
	if (!ok) return 2;
	if (lo > hi) return 0;
	xl = (int)lo;
	xh = (int)hi;
	return 1;
}

// Exact x-interval of a row within [bx0, bx1]: the certified computation, or the walk where that
// declines.
template <class P>
__device__ __forceinline__ bool row_interval_fast(const SurfTri& S, const RowDirs& D, const RowK& K, float ux, int bx0,
                                                  int bx1, int& xl, int& xh) {
	const int r = row_interval_cert<P>(S, D, K, ux, bx0, bx1, xl, xh);
	if (r != 2) return r == 1;
	return row_interval_in<P>(S, D, K, ux, bx0, bx1, xl, xh);
}

// Pass interval of the YZ tests along y for a fixed z slice, within [by0, by1] (a sub-range of the
// triangle's bbox; same scheme: every YZ test is monotone in p.y).
template <class P>
__device__ __forceinline__ bool y_interval_in(const SurfTri& S, float uy, float pz, int by0, int by1, int& ya,
                                              int& yb) {
	uint32_t lo = 0, hi = 0;
	float elo = (float)by0, ehi = (float)by1;
#pragma unroll
	for (int i = 0; i < 3; i++) {
		const float a = S.eyz[i][0];
		if (a > 0.0f) lo |= 1u << i; else if (a < 0.0f) hi |= 1u << i;
		if (a != 0.0f) {
			const float c = __fdividef(-(S.eyz[i][1] * pz + S.dyz[i]), a * uy);
			if (a > 0.0f) elo = fmaxf(elo, ceilf(c)); else ehi = fminf(ehi, floorf(c));
		}
	}
	const uint32_t cmask = ~(lo | hi) & 7u;
	auto fails = [&](int y) { return yz_fail_bits<P>(S, __fmul_rn(__int2float_rn(y), uy), pz); };
	if (cmask && (fails(by0) & cmask)) return false;
	int e = (int)fminf(fmaxf(elo, (float)by0), (float)by1);
	if (!(fails(e) & lo)) {
		while (e > by0 && !(fails(e - 1) & lo)) e--;
	} else {
		do { e++; } while (e <= by1 && (fails(e) & lo));
		if (e > by1) return false;
	}
	ya = e;
	int f = (int)fminf(fmaxf(ehi, (float)ya), (float)by1);
	if (!(fails(f) & hi)) {
		while (f < by1 && !(fails(f + 1) & hi)) f++;
	} else {
		do { f--; } while (f >= ya && (fails(f) & hi));
		if (f < ya) return false;
	}
	yb = f;
	return true;
}

template <class P>
__device__ __forceinline__ bool y_interval(const SurfTri& S, float uy, float pz, int& ya, int& yb) {
	return y_interval_in<P>(S, uy, pz, S.by0, S.by1, ya, yb);
}

// The writers below come in two code types C: uint64_t in general, uint32_t for JOB_NARROW jobs
// (every index and Morton code below 2^32), which halves the index arithmetic; both give the same
// words.  The wrappers pick one per job.

// Write the bits of row (y, z), x in [xl, xh].  Linear index x + y*gx + z*gx*gy (:175-178).
template <class C>
__device__ __forceinline__ void write_row_t(uint32_t* table, bool morton, const uint32_t* grid, int y, int z, int xl,
                                            int xh) {
	if (morton) {
		or_span_morton<C>(table, xl, xh, (uint32_t)y, (uint32_t)z);
	} else {
		const C base = (C)y * grid[0] + (C)z * ((C)grid[1] * grid[0]);
		or_span<C>(table, base + (C)xl, base + (C)xh);
	}
}

// OR the voxels x0 + i of row (y, z) for the set bits i of `pm` (i < 16).  Linear: the run spans at
// most two words; the bit of voxel idx is 31 - idx % 32, so a word's bits are the bit-reversed mask
// shifted by the first voxel's offset.  Morton: one word per 4-voxel x-group (offsets {0, 1, 8, 9}
// from the group's code, as in or_span_morton).
template <class C>
__device__ __forceinline__ void write_row_mask_t(uint32_t* table, bool morton, const uint32_t* grid, int y, int z,
                                                 int x0, uint32_t pm) {
	if (morton) {
		const C yz = (spread3_t<C>((uint32_t)y) << 1) | (spread3_t<C>((uint32_t)z) << 2);
		const int x1 = x0 + 31 - __clz(pm);
		C xd = spread3_t<C>((uint32_t)(x0 & ~3));
		for (int k = x0 >> 2; k <= (x1 >> 2); k++) {
			const int sh = (k << 2) - x0;  // mask bit of x = 4k
			const uint32_t n = (sh >= 0 ? pm >> sh : pm << -sh) & 0xFu;
			if (n) {
				const C code = xd | yz;
				const uint32_t m = ((n & 1u) << 31) | ((n & 2u) << 29) | ((n & 4u) << 21) | ((n & 8u) << 19);
				atomicOr(table + (code >> 5), m >> (uint32_t)(code & 31u));
			}
			xd = morton_x_add_t<C>(xd, (C)kMortonX4);
		}
	} else {
		const C idx = (C)y * grid[0] + (C)z * ((C)grid[1] * grid[0]) + (C)x0;
		const C w = idx >> 5;
		const uint32_t off = (uint32_t)(idx & 31u);
		const uint32_t m0 = __brev(pm) >> off;
		if (m0) atomicOr(table + w, m0);
		if (off) {
			const uint32_t m1 = __brev(pm >> (32u - off));
			if (m1) atomicOr(table + w + 1, m1);
		}
	}
}

// write_row by a whole warp (every lane calls it with the same row): lane i takes words
// w0 + i, w0 + i + 32, ... of the linear span, or x groups k0 + i, ... of the Morton span.
template <class C>
__device__ __forceinline__ void write_row_warp_t(uint32_t* table, bool morton, const uint32_t* grid, int y, int z,
                                                 int xl, int xh, uint32_t lane) {
	if (morton) {
		const C yz = (spread3_t<C>((uint32_t)y) << 1) | (spread3_t<C>((uint32_t)z) << 2);
		for (int k = (xl >> 2) + (int)lane; k <= (xh >> 2); k += 32) {
			const C code = spread3_t<C>((uint32_t)(k << 2)) | yz;
			const int j0 = max(xl - (k << 2), 0), j1 = min(xh - (k << 2), 3);
			const uint32_t n = (0xFu << j0) & (0xFu >> (3 - j1));
			const uint32_t m = ((n & 1u) << 31) | ((n & 2u) << 29) | ((n & 4u) << 21) | ((n & 8u) << 19);
			atomicOr(table + (code >> 5), m >> (uint32_t)(code & 31u));
		}
	} else {
		const C base = (C)y * grid[0] + (C)z * ((C)grid[1] * grid[0]);
		const C lo = base + (C)xl, hi = base + (C)xh;
		const C w0 = lo >> 5, w1 = hi >> 5;
		for (C w = w0 + lane; w <= w1; w += 32) {
			const uint32_t a = (w == w0) ? (uint32_t)(lo & 31u) : 0u;
			const uint32_t b = (w == w1) ? (uint32_t)(hi & 31u) : 31u;
			atomicOr(table + w, span_mask(a, b));
		}
	}
}

__device__ __forceinline__ void write_row(uint32_t* table, bool morton, bool narrow, const uint32_t* grid, int y,
                                          int z, int xl, int xh) {
	if (narrow) write_row_t<uint32_t>(table, morton, grid, y, z, xl, xh);
	else write_row_t<uint64_t>(table, morton, grid, y, z, xl, xh);
}
__device__ __forceinline__ void write_row_mask(uint32_t* table, bool morton, bool narrow, const uint32_t* grid, int y,
                                               int z, int x0, uint32_t pm) {
	if (narrow) write_row_mask_t<uint32_t>(table, morton, grid, y, z, x0, pm);
	else write_row_mask_t<uint64_t>(table, morton, grid, y, z, x0, pm);
}
__device__ __forceinline__ void write_row_warp(uint32_t* table, bool morton, bool narrow, const uint32_t* grid, int y,
                                               int z, int xl, int xh, uint32_t lane) {
	if (narrow) write_row_warp_t<uint32_t>(table, morton, grid, y, z, xl, xh, lane);
	else write_row_warp_t<uint64_t>(table, morton, grid, y, z, xl, xh, lane);
}

}  // namespace cvx
