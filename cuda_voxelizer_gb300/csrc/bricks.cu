// bricks.cu -- surface rasterization of larger triangles in shared-memory bricks.
//
// The reference sets one bit per covered voxel with a global atomicOr (setBit, src/voxelize.cu:50-55,
// :171-179).  For meshes with larger triangles the same table word is then written by many triangles
// (on the 2M-triangle stress soup at 1024^3, about 100 times per word on average), and for a table
// larger than the L2 cache every one of those atomics is a read-modify-write of HBM.  For JOB_BRICKS
// jobs (surface, tables of 2^29+ voxels) the triangles that the classify kernel does not finish
// itself take this path instead:
//   brick_bin      one warp per queued triangle: the setup is computed once and cached (BrickTri);
//                  the 32^3 bricks of the table inside the triangle's grid bbox whose box, widened
//                  by one voxel, the triangle's plane crosses are counted per brick.  A triangle
//                  whose pairs do not fit the pair area is queued for surf_rows instead.
//   brick_scan     one CTA: exclusive prefix sums of the pair counts and of the raster work units
//                  (kPairsPerUnit pairs each) per brick.
//   brick_fill     one warp per binned triangle: the same bricks again, each pair written into its
//                  brick's slot range (counting sort).
//   brick_raster   persistent; each warp owns a 4 KiB brick in shared memory and takes work units
//                  (a brick's pairs, kPairsPerUnit at a time) from a ticket counter: it clears its
//                  brick, rasterizes each pair's triangle into it -- lanes on the z-slices for the
//                  y-intervals, then on the rows for the exact x-intervals, all clipped to the brick
//                  -- and ORs the brick into the table with one global atomicOr per nonzero word.
// The table words are identical to the per-voxel tests of the reference: every voxel is decided by
// the same exact predicates; only where the bits are accumulated changes.  A voxel the reference
// sets lies inside the triangle's grid bbox and within one voxel of its plane, so its brick is
// always among the triangle's pairs.
//
// Brick layout in shared memory: linear tables keep one word per brick row (word z * 32 + y, MSB
// first), flushed row by row at the table's bit alignment; Morton tables keep the brick in Morton
// order (a 32^3 brick of a power-of-two grid is a contiguous run of 1024 table words).
#include "engine.h"
#include "surface.cuh"

namespace cvx {

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr uint32_t kBinThreads = 256;
constexpr uint32_t kScanThreads = 1024;
constexpr uint32_t kRasterWarps = kRowsThreads / 32;

// Bricks per axis of a job's grid.
__device__ __forceinline__ uint32_t bricks_along(uint32_t g) { return (g + kBrick - 1) >> kBrickShift; }

// Job owning brick b of the launch.  brick_begin is the running count of bricks over the jobs before
// (jobs without bricks take the next job's value), so the last job whose brick_begin <= b is the
// JOB_BRICKS job that owns it.
__device__ __forceinline__ uint32_t job_of_brick(const LaunchDesc& L, uint32_t b) {
	return job_search(L, b, [](const JobDesc& J) { return (uint64_t)J.brick_begin; });
}

// The cached setup of a queued triangle (BrickTri layout), written by lane 0.
__device__ __forceinline__ void store_setup(BrickTri* rec, const SurfTri& S, const float* v0, uint32_t binned) {
	float f[44];
	f[0] = S.nx; f[1] = S.ny; f[2] = S.nz; f[3] = S.d1; f[4] = S.d2;
#pragma unroll
	for (int i = 0; i < 3; i++) {
		f[5 + 2 * i] = S.exy[i][0]; f[6 + 2 * i] = S.exy[i][1];
		f[11 + 2 * i] = S.eyz[i][0]; f[12 + 2 * i] = S.eyz[i][1];
		f[17 + 2 * i] = S.ezx[i][0]; f[18 + 2 * i] = S.ezx[i][1];
		f[23 + i] = S.dxy[i]; f[26 + i] = S.dyz[i]; f[29 + i] = S.dzx[i]; f[32 + i] = v0[i];
	}
	f[35] = __int_as_float(S.bx0); f[36] = __int_as_float(S.by0); f[37] = __int_as_float(S.bz0);
	f[38] = __int_as_float(S.bx1); f[39] = __int_as_float(S.by1); f[40] = __int_as_float(S.bz1);
	f[41] = __uint_as_float(binned); f[42] = 0.0f; f[43] = 0.0f;
	float4* p = reinterpret_cast<float4*>(rec);
#pragma unroll
	for (int k = 0; k < 11; k++) p[k] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
}

// Read a cached setup (every lane of the warp reads the same 176 bytes: broadcast loads).
__device__ __forceinline__ uint32_t load_setup(const BrickTri* rec, SurfTri& S, float* v0) {
	const float4* p = reinterpret_cast<const float4*>(rec);
	float f[44];
#pragma unroll
	for (int k = 0; k < 11; k++) {
		const float4 q = p[k];
		f[4 * k] = q.x; f[4 * k + 1] = q.y; f[4 * k + 2] = q.z; f[4 * k + 3] = q.w;
	}
	S.nx = f[0]; S.ny = f[1]; S.nz = f[2]; S.d1 = f[3]; S.d2 = f[4];
#pragma unroll
	for (int i = 0; i < 3; i++) {
		S.exy[i][0] = f[5 + 2 * i]; S.exy[i][1] = f[6 + 2 * i];
		S.eyz[i][0] = f[11 + 2 * i]; S.eyz[i][1] = f[12 + 2 * i];
		S.ezx[i][0] = f[17 + 2 * i]; S.ezx[i][1] = f[18 + 2 * i];
		S.dxy[i] = f[23 + i]; S.dyz[i] = f[26 + i]; S.dzx[i] = f[29 + i]; v0[i] = f[32 + i];
	}
	S.bx0 = __float_as_int(f[35]); S.by0 = __float_as_int(f[36]); S.bz0 = __float_as_int(f[37]);
	S.bx1 = __float_as_int(f[38]); S.by1 = __float_as_int(f[39]); S.bz1 = __float_as_int(f[40]);
	return __float_as_uint(f[41]);
}

// Does the triangle's plane cross brick (bx, by, bz), restricted to the triangle's grid bbox and
// widened by one voxel on every side?  Conservative: float error is far below the one-voxel margin.
// Every operation is explicitly rounded, so brick_bin and brick_fill get the same answers.
__device__ __forceinline__ bool plane_hits_brick(const SurfTri& S, const float* v0, const float* unit, int bx, int by,
                                                 int bz) {
	const int x0 = max(bx << kBrickShift, S.bx0) - 1, x1 = min((bx << kBrickShift) + (int)kBrick - 1, S.bx1) + 2;
	const int y0 = max(by << kBrickShift, S.by0) - 1, y1 = min((by << kBrickShift) + (int)kBrick - 1, S.by1) + 2;
	const int z0 = max(bz << kBrickShift, S.bz0) - 1, z1 = min((bz << kBrickShift) + (int)kBrick - 1, S.bz1) + 2;
	const float hx = __fmul_rn(0.5f * (float)(x1 - x0), unit[0]), cx = __fmul_rn(0.5f * (float)(x0 + x1), unit[0]);
	const float hy = __fmul_rn(0.5f * (float)(y1 - y0), unit[1]), cy = __fmul_rn(0.5f * (float)(y0 + y1), unit[1]);
	const float hz = __fmul_rn(0.5f * (float)(z1 - z0), unit[2]), cz = __fmul_rn(0.5f * (float)(z0 + z1), unit[2]);
	const float d = __fadd_rn(__fadd_rn(__fmul_rn(S.nx, __fsub_rn(cx, v0[0])), __fmul_rn(S.ny, __fsub_rn(cy, v0[1]))),
	                          __fmul_rn(S.nz, __fsub_rn(cz, v0[2])));
	const float r = __fadd_rn(__fadd_rn(__fmul_rn(fabsf(S.nx), hx), __fmul_rn(fabsf(S.ny), hy)), __fmul_rn(fabsf(S.nz), hz));
	return !(fabsf(d) > r);  // NaN normals (degenerate triangles) keep every brick of the bbox
}

// Candidate bricks of a triangle: its grid bbox in brick units.
struct BrickBox {
	int bx, by, bz;
	uint32_t nx, ny, ncand;
	__device__ explicit BrickBox(const SurfTri& S) {
		bx = S.bx0 >> kBrickShift;
		by = S.by0 >> kBrickShift;
		bz = S.bz0 >> kBrickShift;
		nx = (uint32_t)((S.bx1 >> kBrickShift) - bx + 1);
		ny = (uint32_t)((S.by1 >> kBrickShift) - by + 1);
		ncand = nx * ny * (uint32_t)((S.bz1 >> kBrickShift) - bz + 1);
	}
};

// Queue a triangle for surf_rows (one item per kZch z-slices).
__device__ __forceinline__ void queue_for_rows(const LaunchDesc& L, uint32_t job, uint32_t tri, const SurfTri& S) {
	const uint32_t items = (uint32_t)(S.bz1 - S.bz0) / kZch + 1u;
	const unsigned long long old = atomicAdd(&L.scr.ctr->big, (1ull << kBigShift) | (unsigned long long)items);
	const uint32_t r = (uint32_t)(old >> kBigShift);
	const uint64_t first = old & kBigItemMask;
	if (r < L.scr.cap && first + items <= kBigItemMask)
		L.scr.big[r] = BigRec{first, job, tri, items, 0u};
	else
		set_error(L, kErrQueueOverflow);
}

template <class P>
__global__ void __launch_bounds__(kBinThreads) brick_bin(const __grid_constant__ LaunchDesc L) {
	const uint32_t lane = threadIdx.x & 31u;
	Counters* C = L.scr.ctr;
	__shared__ unsigned s_n;
	if (threadIdx.x == 0) s_n = *reinterpret_cast<volatile unsigned*>(&C->bq);
	__syncthreads();
	const uint32_t n = min(s_n, L.scr.cap);
	if ((uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5) >= n) return;
	WarpTickets wt(n, gridDim.x * (blockDim.x >> 5));
	for (;;) {
		unsigned long long tk = 0;
		if (!wt.take(&C->bticket, n, lane, tk)) break;
		const MidRec rec = L.scr.bq[tk];
		if (rec.job >= L.n_jobs || rec.tri >= job_at(L, rec.job).n_tri) {  // never follow a malformed record
			if (lane == 0) L.scr.tri[tk].binned = 0u;
			continue;
		}
		const JobDesc& J = job_at(L, rec.job);
		const float tv = lane < 9 ? J.tris[(uint64_t)rec.tri * 9 + lane] : 0.0f;
		float t[9];
#pragma unroll
		for (int k = 0; k < 9; k++) t[k] = __shfl_sync(FULL, tv, k);
		const float unit[3] = {J.unit[0], J.unit[1], J.unit[2]};
		const uint32_t grid[3] = {J.grid[0], J.grid[1], J.grid[2]};
		SurfTri S;
		surf_setup<P>(t, J.bmin, unit, J.inv_unit, grid, S);
		const float v0[3] = {__fsub_rn(t[0], J.bmin[0]), __fsub_rn(t[1], J.bmin[1]), __fsub_rn(t[2], J.bmin[2])};
		const BrickBox B(S);
		uint32_t cnt = 0;
		for (uint32_t c = lane; c < B.ncand; c += 32) {
			const uint32_t cx = c % B.nx, cy = (c / B.nx) % B.ny, cz = c / (B.nx * B.ny);
			cnt += plane_hits_brick(S, v0, unit, B.bx + (int)cx, B.by + (int)cy, B.bz + (int)cz) ? 1u : 0u;
		}
#pragma unroll
		for (int d = 16; d >= 1; d >>= 1) cnt += __shfl_xor_sync(FULL, cnt, d);
		unsigned long long base = 0;
		if (lane == 0) base = atomicAdd(&C->pairs, (unsigned long long)cnt);
		base = __shfl_sync(FULL, base, 0);
		const bool fits = base + cnt <= L.scr.pair_cap;
		if (lane == 0) {
			store_setup(L.scr.tri + tk, S, v0, fits ? 1u : 0u);
			if (!fits) queue_for_rows(L, rec.job, rec.tri, S);
		}
		if (!fits) continue;
		const uint32_t nbx = bricks_along(J.grid[0]), nby = bricks_along(J.grid[1]);
		for (uint32_t c = lane; c < B.ncand; c += 32) {
			const uint32_t cx = c % B.nx, cy = (c / B.nx) % B.ny, cz = c / (B.nx * B.ny);
			const int bx = B.bx + (int)cx, by = B.by + (int)cy, bz = B.bz + (int)cz;
			const uint32_t b = J.brick_begin + (uint32_t)bx + nbx * ((uint32_t)by + nby * (uint32_t)bz);
			if (b < L.n_bricks && plane_hits_brick(S, v0, unit, bx, by, bz)) atomicAdd(&L.scr.brick_cnt[b], 1u);
		}
	}
}

// Exclusive prefix sums over the launch's bricks: pair offsets and raster work units.  The counts
// are cleared for the next launch sequence.
__global__ void __launch_bounds__(kScanThreads) brick_scan(const __grid_constant__ LaunchDesc L) {
	__shared__ uint32_t s_c[kScanThreads / 32], s_u[kScanThreads / 32];
	const uint32_t n = L.n_bricks, lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	const uint32_t per = (n + kScanThreads - 1) / kScanThreads;
	const uint32_t b0 = min(threadIdx.x * per, n), b1 = min(b0 + per, n);
	uint32_t c = 0, u = 0;
	for (uint32_t b = b0; b < b1; b++) {
		const uint32_t k = L.scr.brick_cnt[b];
		c += k;
		u += (k + kPairsPerUnit - 1) / kPairsPerUnit;
	}
	uint32_t ic = c, iu = u;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		const uint32_t vc = __shfl_up_sync(FULL, ic, d), vu = __shfl_up_sync(FULL, iu, d);
		if (lane >= (uint32_t)d) { ic += vc; iu += vu; }
	}
	if (lane == 31) { s_c[warp] = ic; s_u[warp] = iu; }
	__syncthreads();
	if (warp == 0) {
		uint32_t wc = s_c[lane], wu = s_u[lane];
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			const uint32_t vc = __shfl_up_sync(FULL, wc, d), vu = __shfl_up_sync(FULL, wu, d);
			if (lane >= (uint32_t)d) { wc += vc; wu += vu; }
		}
		s_c[lane] = wc;
		s_u[lane] = wu;
	}
	__syncthreads();
	uint32_t oc = (warp ? s_c[warp - 1] : 0u) + ic - c, ou = (warp ? s_u[warp - 1] : 0u) + iu - u;
	for (uint32_t b = b0; b < b1; b++) {
		const uint32_t k = L.scr.brick_cnt[b];
		L.scr.brick_cnt[b] = 0;  // zero again for the next launch sequence
		L.scr.brick_off[b] = oc;
		L.scr.unit_begin[b] = ou;
		L.scr.brick_cur[b] = 0;
		oc += k;
		ou += (k + kPairsPerUnit - 1) / kPairsPerUnit;
	}
	if (threadIdx.x == kScanThreads - 1) {
		L.scr.brick_off[n] = s_c[kScanThreads / 32 - 1];
		L.scr.unit_begin[n] = s_u[kScanThreads / 32 - 1];
		L.scr.ctr->units = s_u[kScanThreads / 32 - 1];
	}
}

// The binned triangles' pairs into their bricks' slot ranges (same candidates and tests as brick_bin,
// from the cached setup).
__global__ void __launch_bounds__(kBinThreads) brick_fill(const __grid_constant__ LaunchDesc L) {
	const uint32_t lane = threadIdx.x & 31u;
	Counters* C = L.scr.ctr;
	__shared__ unsigned s_n;
	if (threadIdx.x == 0) s_n = *reinterpret_cast<volatile unsigned*>(&C->bq);
	__syncthreads();
	const uint32_t n = min(s_n, L.scr.cap);
	if ((uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5) >= n) return;
	WarpTickets wt(n, gridDim.x * (blockDim.x >> 5));
	for (;;) {
		unsigned long long tk = 0;
		if (!wt.take(&C->fticket, n, lane, tk)) break;
		SurfTri S;
		float v0[3];
		if (!load_setup(L.scr.tri + tk, S, v0)) continue;  // queued for surf_rows
		const MidRec rec = L.scr.bq[tk];
		if (rec.job >= L.n_jobs) continue;
		const JobDesc& J = job_at(L, rec.job);
		const float unit[3] = {J.unit[0], J.unit[1], J.unit[2]};
		const uint32_t nbx = bricks_along(J.grid[0]), nby = bricks_along(J.grid[1]);
		const BrickBox B(S);
		for (uint32_t c = lane; c < B.ncand; c += 32) {
			const uint32_t cx = c % B.nx, cy = (c / B.nx) % B.ny, cz = c / (B.nx * B.ny);
			const int bx = B.bx + (int)cx, by = B.by + (int)cy, bz = B.bz + (int)cz;
			if (!plane_hits_brick(S, v0, unit, bx, by, bz)) continue;
			const uint32_t b = J.brick_begin + (uint32_t)bx + nbx * ((uint32_t)by + nby * (uint32_t)bz);
			if (b >= L.n_bricks) continue;  // never: bricks of the job's grid
			const uint32_t pos = L.scr.brick_off[b] + atomicAdd(&L.scr.brick_cur[b], 1u);
			if (pos < L.scr.brick_off[b + 1]) L.scr.pair_sorted[pos] = (uint32_t)tk;
		}
	}
}

// OR local x in [a, b] (0 <= a <= b < 32) of brick row (ly, lz) into the warp's brick.  Linear: the
// row is one word and the warp's lanes hold distinct rows, so a plain read-modify-write suffices.
__device__ __forceinline__ void brick_row_or(uint32_t* s, bool morton, int a, int b, uint32_t ly, uint32_t lz) {
	if (!morton) {
		s[(lz << kBrickShift) + ly] |= span_mask((uint32_t)a, (uint32_t)b);
		return;
	}
	const uint32_t yz = (spread3_narrow(ly) << 1) | (spread3_narrow(lz) << 2);
	uint32_t xd = spread3_narrow((uint32_t)(a & ~3));
	for (int k = a >> 2; k <= (b >> 2); k++) {
		const uint32_t code = xd | yz;
		const int j0 = max(a - (k << 2), 0), j1 = min(b - (k << 2), 3);
		const uint32_t nb = (0xFu << j0) & (0xFu >> (3 - j1));
		const uint32_t m = ((nb & 1u) << 31) | ((nb & 2u) << 29) | ((nb & 4u) << 21) | ((nb & 8u) << 19);
		atomicOr(s + (code >> 5), m >> (code & 31u));  // rows 4 apart in y share Morton words
		xd = morton_x_add_t<uint32_t>(xd, (uint32_t)kMortonX4);
	}
}

// Rasterize the cached triangle into the warp's brick (bx, by, bz): lanes on the z-slices
// (y-intervals), then on the rows (x-intervals), both clipped to the brick.
// Rows y of z-slice z whose voxels in x in [xlo, xhi] the triangle's plane can reach: the plane
// crosses the box [xlo, xhi + 1] x [y, y + 1] x [z, z + 1] (in voxels) only for y in one interval.
// The rows it removes are those whose x-interval lies in another brick.  Widened by 1e-4 of the
// magnitudes involved (float32 error of this estimate and of the plane test itself is below 1e-6 of
// them) and by a hundredth of a row, so no row the exact tests would set is dropped.
__device__ __forceinline__ void plane_rows(const SurfTri& S, const float* v0, const float* unit, int xlo, int xhi, int z,
                                           int& ya, int& yb) {
	const float hx = 0.5f * (float)(xhi + 1 - xlo) * unit[0], cx = 0.5f * (float)(xlo + xhi + 1) * unit[0];
	const float hy = 0.5f * unit[1], hz = 0.5f * unit[2], cz = ((float)z + 0.5f) * unit[2];
	const float ax = S.nx * (cx - v0[0]), az = S.nz * (cz - v0[2]), ay = S.ny * (hy - v0[1]);
	const float A = ax + az + ay;
	const float r = fabsf(S.nx) * hx + fabsf(S.ny) * hy + fabsf(S.nz) * hz;
	const float slack = r + 1e-4f * (r + fabsf(ax) + fabsf(az) + fabsf(ay) +
	                                 fabsf(S.ny * unit[1]) * (float)max(abs(ya), abs(yb)));
	const float k = S.ny * unit[1];
	if (!(fabsf(k) > 0.0f)) {  // rows do not move the plane across the box (or a NaN normal): keep all
		if (!(fabsf(A) > slack)) return;
		ya = 1;
		yb = 0;
		return;
	}
	const float t0 = (-slack - A) / k, t1 = (slack - A) / k;
	float lo = fminf(t0, t1), hi = fmaxf(t0, t1);
	lo -= 0.01f + 1e-5f * fabsf(lo);
	hi += 0.01f + 1e-5f * fabsf(hi);
	if (lo > (float)ya) ya = lo > (float)yb ? yb + 1 : (int)ceilf(lo);
	if (hi < (float)yb) yb = hi < (float)ya ? ya - 1 : (int)floorf(hi);
}

template <class P>
__device__ __forceinline__ void raster_pair(const SurfTri& S, const float* v0, const float* unit, int bx, int by, int bz,
                                            uint32_t* s, bool morton, uint32_t lane) {
	const int ox = bx << kBrickShift, oy = by << kBrickShift, oz = bz << kBrickShift;
	const int xlo = max(S.bx0, ox), xhi = min(S.bx1, ox + (int)kBrick - 1);
	const int ylo = max(S.by0, oy), yhi = min(S.by1, oy + (int)kBrick - 1);
	const int zlo = max(S.bz0, oz), zhi = min(S.bz1, oz + (int)kBrick - 1);
	if (xlo > xhi || ylo > yhi || zlo > zhi) return;
	RowDirs D;
	row_dirs(S, unit[0], D);
	const int zl = zlo + (int)lane;
	int ya = 0, yb = -1;
	if (zl <= zhi) {
		int pa = ylo, pb = yhi;
		plane_rows(S, v0, unit, xlo, xhi, zl, pa, pb);
		const float pz = __fmul_rn(__int2float_rn(zl), unit[2]);
		if (pa > pb || !y_interval_in<P>(S, unit[1], pz, pa, pb, ya, yb)) { ya = 0; yb = -1; }
	}
	const int cnt = yb - ya + 1;
	int incl = cnt;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		const int v = __shfl_up_sync(FULL, incl, d);
		if (lane >= (uint32_t)d) incl += v;
	}
	const int R = __shfl_sync(FULL, incl, 31);
	for (int base = 0; base < R; base += 32) {
		const int k = base + (int)lane;
		int sl = 0;
#pragma unroll
		for (int step = 16; step >= 1; step >>= 1) {
			const int v = __shfl_sync(FULL, incl, sl + step - 1);
			if (v <= k) sl += step;
		}
		sl = min(sl, 31);
		const int incl_s = __shfl_sync(FULL, incl, sl);
		const int cnt_s = __shfl_sync(FULL, cnt, sl);
		const int ya_s = __shfl_sync(FULL, ya, sl);
		if (k < R) {
			const int y = ya_s + (k - (incl_s - cnt_s));
			const int z = zlo + sl;
			RowK K;
			row_consts<P>(S, __fmul_rn(__int2float_rn(y), unit[1]), __fmul_rn(__int2float_rn(z), unit[2]), K);
			int xl, xh;
			if (row_interval_fast<P>(S, D, K, unit[0], xlo, xhi, xl, xh))
				brick_row_or(s, morton, xl - ox, xh - ox, (uint32_t)(y - oy), (uint32_t)(z - oz));
		}
		__syncwarp();  // the next round's rows may share Morton words with this one's
	}
}

template <class P>
__global__ void __launch_bounds__(kRowsThreads, 3) brick_raster(const __grid_constant__ LaunchDesc L) {
	__shared__ __align__(16) uint32_t s_bricks[kRasterWarps][kBrickWords];
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	uint32_t* s = s_bricks[warp];
	Counters* C = L.scr.ctr;
	const uint32_t units = *reinterpret_cast<volatile unsigned*>(&C->units);
	if ((uint64_t)blockIdx.x * kRasterWarps + warp >= units) return;
	WarpTickets wt(units, gridDim.x * kRasterWarps);
	for (;;) {
		unsigned long long tk = 0;
		if (!wt.take(&C->rticket, units, lane, tk)) break;
		const uint32_t u = (uint32_t)tk;
		// the unit's brick: last brick whose first unit is <= u
		uint32_t lo = 0, hi = L.n_bricks - 1;
		while (lo < hi) {
			const uint32_t m = (lo + hi + 1) >> 1;
			if (L.scr.unit_begin[m] <= u) lo = m; else hi = m - 1;
		}
		const uint32_t b = lo;
		const JobDesc& J = job_at(L, job_of_brick(L, b));
		const bool morton = (J.flags & JOB_MORTON) != 0;
		const float unit[3] = {J.unit[0], J.unit[1], J.unit[2]};
		const uint32_t nbx = bricks_along(J.grid[0]), nby = bricks_along(J.grid[1]);
		const uint32_t lb = b - J.brick_begin;
		const int bx = (int)(lb % nbx), by = (int)((lb / nbx) % nby), bz = (int)(lb / (nbx * nby));
		const uint32_t p0 = L.scr.brick_off[b] + (u - L.scr.unit_begin[b]) * kPairsPerUnit;
		const uint32_t p1 = min(p0 + kPairsPerUnit, L.scr.brick_off[b + 1]);
#pragma unroll
		for (uint32_t i = 0; i < kBrickWords / 128; i++)
			reinterpret_cast<uint4*>(s)[i * 32 + lane] = make_uint4(0u, 0u, 0u, 0u);
		__syncwarp();
		for (uint32_t p = p0; p < p1; p++) {
			const uint32_t q = L.scr.pair_sorted[p];
			if (q >= L.scr.cap) continue;  // never follow a malformed pair
			SurfTri S;
			float v0[3];
			load_setup(L.scr.tri + q, S, v0);
			raster_pair<P>(S, v0, unit, bx, by, bz, s, morton, lane);
		}
		__syncwarp();
		// flush: one global atomicOr per nonzero word
		uint32_t* table = J.table;
		if (morton) {
			const uint64_t base = morton3((uint32_t)bx << kBrickShift, (uint32_t)by << kBrickShift,
			                              (uint32_t)bz << kBrickShift) >> 5;
			for (uint32_t w = lane; w < kBrickWords; w += 32) {
				const uint32_t v = s[w];
				if (v) atomicOr(table + base + w, v);
			}
		} else {
			const uint64_t gx = J.grid[0], gy = J.grid[1];
			for (uint32_t r = lane; r < kBrickWords; r += 32) {
				const uint32_t v = s[r];
				if (!v) continue;
				const uint64_t y = (uint64_t)(by << kBrickShift) + (r & (kBrick - 1));
				const uint64_t z = (uint64_t)(bz << kBrickShift) + (r >> kBrickShift);
				const uint64_t bit = (uint64_t)(bx << kBrickShift) + y * gx + z * gx * gy;
				uint32_t* t = table + (bit >> 5);
				const uint32_t off = (uint32_t)(bit & 31u);
				if (off == 0) {
					atomicOr(t, v);
				} else {
					const uint32_t g0 = v >> off, g1 = v << (32u - off);
					if (g0) atomicOr(t, g0);
					if (g1) atomicOr(t + 1, g1);
				}
			}
		}
		__syncwarp();  // the brick is read before the next unit clears it
	}
}

}  // namespace

// ---- host-side launchers ------------------------------------------------------------------------

template <class P>
static cudaError_t launch_bricks_t(const LaunchDesc& L, int grid, int raster_grid, cudaStream_t s, const Prof* prof) {
	cudaError_t e = launch_k(brick_bin<P>, (unsigned)grid, kBinThreads, 0, s, L);
	if (e != cudaSuccess) return e;
	if (prof) (*prof)("brick_bin", s);
	e = launch_k(brick_scan, 1u, kScanThreads, 0, s, L);
	if (e != cudaSuccess) return e;
	if (prof) (*prof)("brick_scan", s);
	e = launch_k(brick_fill, (unsigned)grid, kBinThreads, 0, s, L);
	if (e != cudaSuccess) return e;
	if (prof) (*prof)("brick_fill", s);
	e = launch_k(brick_raster<P>, (unsigned)raster_grid, kRowsThreads, 0, s, L);
	if (e != cudaSuccess) return e;
	if (prof) (*prof)("brick_raster", s);
	return cudaGetLastError();
}

cudaError_t launch_bricks(const LaunchDesc& L, int grid, int raster_grid, cudaStream_t s, const Prof* prof) {
	return launch_bricks_t<RefFma>(L, grid, raster_grid, s, prof);
}

int brick_raster_blocks_per_sm() {
	int n = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, brick_raster<RefFma>, kRowsThreads, 0);
	return n > 0 ? n : 1;
}

}  // namespace cvx
