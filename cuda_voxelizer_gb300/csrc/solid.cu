// solid.cu -- solid voxelization kernels (reference: voxelize_triangle_solid,
// src/voxelize_solid.cu:16-145).
//
// The reference casts, for every voxel-centre column (y, z) inside a triangle's YZ projection, the
// column onto the triangle's plane and XORs every voxel x in [0, xmax] (:115-135): O(g) single-bit
// atomics per column hit, and parity along +x yields the solid.  The engine computes the same
// column hits with the same arithmetic, but records each hit as two toggles in a linear-order flip
// table (the start of the row and xmax + 1), then resolves all rows with one prefix-XOR pass and
// XORs the resolved bits into the caller's table (or scatters them into Morton order).  The XOR of
// any set of [0, xmax] ranges is exactly what this produces.
//
// Kernels, in launch order:
//   solid_classify      one CTA per kTile-triangle tile (TMA bulk staging as in surface.cu); the
//                       columns of triangles with at most `small_cols` columns are dealt over the
//                       CTA, the other triangles queued.
//   solid_cols          persistent; each warp takes items of up to kColsPerItem columns.
//   solid_resolve       linear jobs: one thread per row run (whole rows; 16-byte words where rows
//                       are aligned): prefix XOR along x, XORed into the linear table (every word
//                       stored, for JOB_TABLE_OVERWRITE jobs), flip table cleared.
//   solid_morton_slab   Morton jobs with 32 <= g <= 1024: a CTA resolves a 16 x 16-row slab in
//                       shared memory and writes it as 16^3 Morton blocks (128 contiguous words).
//   solid_morton_brick  Morton jobs with g > 1024: groups of x-adjacent 32^3 bricks.
//   solid_morton_small  Morton jobs with g < 32 (one word at a time), then solid_zero clears the
//                       flip table.
#include "engine.h"

namespace cvx {

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr double kFloatError = 0.000001;  // src/voxelize_solid.cu:13 (a double literal)
// For a float f, (double)f < 0.000001 exactly when f <= 0x1.0c6f7ap-20f, the largest float below the
// double 1e-6 (floats are exact in double, and 0x1.0c6f7ap-20 < 1e-6 < its successor).
constexpr float kFloatErrorBelow = 0x1.0c6f7ap-20f;
static_assert((double)kFloatErrorBelow < kFloatError && (double)0x1.0c6f7cp-20f >= kFloatError,
              "kFloatErrorBelow is the largest float below the reference's float_error");

// floor((double)q - 0.5) and ceil(...) for a float q: q - 0.5f is exact in float when |q| < 2^22
// (its ulp is at most 0.5 there), so float floor/ceil give the double result; else use double.
__device__ __forceinline__ float floor_half(float q) {
	return fabsf(q) < 4194304.0f ? floorf(__fsub_rn(q, 0.5f)) : (float)floor((double)q - 0.5);
}
__device__ __forceinline__ float ceil_half(float q) {
	return fabsf(q) < 4194304.0f ? ceilf(__fsub_rn(q, 0.5f)) : (float)ceil((double)q - 0.5);
}
// floor_half / ceil_half of fl(a / u), using the reciprocal shortcut when the approximate
// quotient is clearly away from the decision boundary (the half-integers), as div_trunc does.
__device__ __forceinline__ float div_floor_half(float a, float u, float inv) {
	const float q = __fmul_rn(a, inv);
	const float h = __fsub_rn(q, 0.5f);
	const float f = floorf(h);
	const float room = 4.0f * __fmul_rn(fabsf(q), 1.1920929e-07f) + 1.0e-30f;
	if (fabsf(q) < 4194304.0f && h - f > room && (f + 1.0f) - h > room) return f;
	return floor_half(__fdiv_rn(a, u));
}
__device__ __forceinline__ float div_ceil_half(float a, float u, float inv) {
	const float q = __fmul_rn(a, inv);
	const float h = __fsub_rn(q, 0.5f);
	const float f = floorf(h);
	const float room = 4.0f * __fmul_rn(fabsf(q), 1.1920929e-07f) + 1.0e-30f;
	if (fabsf(q) < 4194304.0f && h - f > room && (f + 1.0f) - h > room) return f + 1.0f;
	return ceil_half(__fdiv_rn(a, u));
}

// int((double)q - 0.5) (truncation, saturating as cvt.rzi.s32.f64 does)
__device__ __forceinline__ int trunc_half(float q) {
	return fabsf(q) < 4194304.0f ? __float2int_rz(__fsub_rn(q, 0.5f)) : __double2int_rz((double)q - 0.5);
}

struct SolidTri {
	float nx, ny, nz;
	float v0x, v0y, v0z;
	float ax, ay, bx, by, cx, cy;  // v0_yz, v1_yz, v2_yz after the counter-clockwise swap
	int y0, y1, z0, z1;            // column range, clipped to the grid
	bool skip;
};

// Triangle setup, src/voxelize_solid.cu:83-119.
template <class P>
__device__ __forceinline__ void solid_setup(const float* t, const float* bmin, const float* unit, const float* inv,
                                            const uint32_t* grid, SolidTri& S) {
	const float v0x = __fsub_rn(t[0], bmin[0]), v0y = __fsub_rn(t[1], bmin[1]), v0z = __fsub_rn(t[2], bmin[2]);
	const float v1x = __fsub_rn(t[3], bmin[0]), v1y = __fsub_rn(t[4], bmin[1]), v1z = __fsub_rn(t[5], bmin[2]);
	const float v2x = __fsub_rn(t[6], bmin[0]), v2y = __fsub_rn(t[7], bmin[1]), v2z = __fsub_rn(t[8], bmin[2]);
	const float e0x = __fsub_rn(v1x, v0x), e0y = __fsub_rn(v1y, v0y), e0z = __fsub_rn(v1z, v0z);
	const float e1x = __fsub_rn(v2x, v1x), e1y = __fsub_rn(v2y, v1y), e1z = __fsub_rn(v2z, v1z);
	const float cx = mul_sub<P::cross>(e0y, e1z, e0z, e1y);
	const float cy = mul_sub<P::cross>(e0z, e1x, e0x, e1z);
	const float cz = mul_sub<P::cross>(e0x, e1y, e0y, e1x);
	const float rlen = rsqrtf(dot3<P::dot3>(cx, cy, cz, cx, cy, cz));
	S.nx = __fmul_rn(cx, rlen);
	S.ny = __fmul_rn(cy, rlen);
	S.nz = __fmul_rn(cz, rlen);
	S.v0x = v0x; S.v0y = v0y; S.v0z = v0z;
	S.skip = fabsf(S.nx) <= kFloatErrorBelow;  // :92, (double)|n.x| < 1e-6 (the thread returns)
	// YZ projection, made counter-clockwise (:95-105; checkCCW :55-64)
	float ax = v0y, ay = v0z, bx = v1y, by = v1z, qx = v2y, qy = v2z;
	const float ccw = mul_sub<P::ccw>(__fsub_rn(bx, ax), __fsub_rn(qy, ay), __fsub_rn(qx, ax), __fsub_rn(by, ay));
	if (!(ccw > 0.0f)) {
		float tx = bx, ty = by;
		bx = qx; by = qy; qx = tx; qy = ty;
	}
	S.ax = ax; S.ay = ay; S.bx = bx; S.by = by; S.cx = qx; S.cy = qy;
	// column range (:109-119): floor/ceil(q - 0.5) evaluated in double, loop y from (int)min while
	// (float)y <= max.  Columns outside the grid are dropped (the reference writes them outside the
	// table or into neighbouring rows).
	const float mxy = fmaxf(ax, fmaxf(bx, qx)), mxz = fmaxf(ay, fmaxf(by, qy));
	const float mny = fminf(ax, fminf(bx, qx)), mnz = fminf(ay, fminf(by, qy));
	const float gmaxy = div_floor_half(mxy, unit[1], inv[1]);
	const float gmaxz = div_floor_half(mxz, unit[2], inv[2]);
	const float gminy = div_ceil_half(mny, unit[1], inv[1]);
	const float gminz = div_ceil_half(mnz, unit[2], inv[2]);
	int y0 = __float2int_rz(gminy), z0 = __float2int_rz(gminz);
	// last integer y with (float)y <= gmax (gmax holds an integer value, or is not finite)
	int y1 = gmaxy >= 2147483520.0f ? 2147483647 : (gmaxy >= -2147483648.0f ? (int)gmaxy : (-2147483647 - 1));
	int z1 = gmaxz >= 2147483520.0f ? 2147483647 : (gmaxz >= -2147483648.0f ? (int)gmaxz : (-2147483647 - 1));
	if (!(gmaxy == gmaxy)) y1 = y0 - 1;  // NaN bound: the loop never runs
	if (!(gmaxz == gmaxz)) z1 = z0 - 1;
	S.y0 = max(y0, 0); S.z0 = max(z0, 0);
	S.y1 = min(y1, (int)grid[1] - 1); S.z1 = min(z1, (int)grid[2] - 1);
}

__device__ __forceinline__ bool top_left(float v0x, float v0y, float v1x, float v1y) {
	return (v1y < v0y) || (v1y == v0y && v0x > v1x);  // :67-70
}

// Column test for voxel-centre column (y, z): returns true and xmax on a hit (:119-123).  `morton`
// selects the contraction of get_x_coordinate the reference uses for that table order.
template <class P>
__device__ __forceinline__ bool column_hit(const SolidTri& S, const float* unit, int y, int z, bool morton, int& xmax) {
	// ((y + 0.5) * unit.y) in double then rounded to float == the float product of the exact y+0.5f
	// for |y| < 2^22 (the double product is exact, so both round the same real number once).
	const float px = __fmul_rn(__int2float_rn(y) + 0.5f, unit[1]);
	const float py = __fmul_rn(__int2float_rn(z) + 0.5f, unit[2]);
	// check_point_triangle (:24-46)
	const float PAx = __fsub_rn(px, S.ax), PAy = __fsub_rn(py, S.ay);
	const float PBx = __fsub_rn(px, S.bx), PBy = __fsub_rn(py, S.by);
	const float PCx = __fsub_rn(px, S.cx), PCy = __fsub_rn(py, S.cy);
	int check;
	const float t1 = mul_sub<P::pt>(PAx, PBy, PAy, PBx);
	const float t2 = mul_sub<P::pt>(PBx, PCy, PBy, PCx);
	const float t3 = mul_sub<P::pt>(PCx, PAy, PCy, PAx);
	if (fabsf(t1) <= kFloatErrorBelow && __fmul_rn(PAx, PBx) <= 0.0f && __fmul_rn(PAy, PBy) <= 0.0f) check = 1;
	else if (fabsf(t2) <= kFloatErrorBelow && __fmul_rn(PBx, PCx) <= 0.0f && __fmul_rn(PBy, PCy) <= 0.0f) check = 2;
	else if (fabsf(t3) <= kFloatErrorBelow && __fmul_rn(PCx, PAx) <= 0.0f && __fmul_rn(PCy, PAy) <= 0.0f) check = 3;
	else if (__fmul_rn(t1, t2) > 0.0f && __fmul_rn(t1, t3) > 0.0f) check = 0;
	else check = -1;
	const bool in = (check == 1 && top_left(S.ax, S.ay, S.bx, S.by)) || (check == 2 && top_left(S.bx, S.by, S.cx, S.cy)) ||
	                (check == 3 && top_left(S.cx, S.cy, S.ax, S.ay)) || (check == 0);
	if (!in) return false;
	// get_x_coordinate (:49-52): -(n.y*(p.x - v0.y) + n.z*(p.y - v0.z)) / n.x + v0.x
	const float A = __fsub_rn(px, S.v0y), B = __fsub_rn(py, S.v0z);
	const float m = morton ? mul_add<P::getx_morton>(S.ny, A, S.nz, B) : mul_add<P::getx>(S.ny, A, S.nz, B);
	const float xh = __fadd_rn(__fdiv_rn(-m, S.nx), S.v0x);
	xmax = trunc_half(__fdiv_rn(xh, unit[0]));  // int(... / unit.x - 0.5), the 0.5 a double
	return true;
}

__device__ __forceinline__ void toggle(uint32_t* flips, uint64_t bit) { atomicXor(flips + (bit >> 5), bit_of(bit)); }

// Record column hit (y, z, xmax): the reference flips bits [0, xmax] of the column's row, i.e. the
// linear bit range [r*gx, r*gx + xmax]; a range longer than the row continues into the following
// rows (:124-135).  Morton order has no such continuation (x is encoded on its own), the range is
// clipped at the row end there (beyond it the reference writes outside the table).
__device__ __forceinline__ void record_hit(uint32_t* flips, const uint32_t* grid, bool morton, int y, int z, int xmax) {
	if (xmax < 0) return;
	const uint64_t gx = grid[0];
	const uint64_t rows = (uint64_t)grid[1] * grid[2];
	const uint64_t row = (uint64_t)y + (uint64_t)z * grid[1];
	const uint64_t len = (uint64_t)xmax + 1;
	if (morton || len <= gx) {
		toggle(flips, row * gx);
		const uint64_t e = len < gx ? len : gx;
		if (e < gx) toggle(flips, row * gx + e);
		return;
	}
	const uint64_t q = len / gx, rem = len % gx;
	for (uint64_t k = 0; k < q && row + k < rows; k++) toggle(flips, (row + k) * gx);
	if (rem && row + q < rows) {
		toggle(flips, (row + q) * gx);
		toggle(flips, (row + q) * gx + rem);
	}
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
	for (uint32_t it = 0; it < (1u << 24); it++) {
		uint32_t ok;
		asm volatile(
		    "{\n\t.reg .pred p;\n\t"
		    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		    "selp.u32 %0, 1, 0, p;\n\t}"
		    : "=r"(ok)
		    : "r"(bar), "r"(parity)
		    : "memory");
		if (ok) return true;
	}
	return false;
}

// Stage `cnt` triangles (9 floats each) from global memory into shared memory.  A full, aligned
// tile of plain device memory goes through one bulk copy completing on an mbarrier; anything else
// (a partial or unaligned tile, managed or host memory: `plain`) is loaded cooperatively.
// Returns false (in every thread) if the bulk copy did not complete within the bounded wait: the
// error word is set, the CTA waits once more (again bounded) for the copy still in flight, and the
// caller skips the tile without touching the shared memory the copy may still write.
__device__ __forceinline__ bool stage_tile(const LaunchDesc& L, const float* src, uint32_t cnt, float* s_tri,
                                           uint64_t* s_bar, bool plain) {
	const uint32_t bytes = cnt * 36u;
	const bool bulk = cnt == kTile && ((reinterpret_cast<uintptr_t>(src) & 15u) == 0) && !plain;
	if (bulk) {
		const uint32_t bar = (uint32_t)__cvta_generic_to_shared(s_bar);
		const uint32_t dst = (uint32_t)__cvta_generic_to_shared(s_tri);
		if (threadIdx.x == 0) {
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
			asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
			asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
			asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
			             "l"(src), "r"(bytes), "r"(bar)
			             : "memory");
		}
		__syncthreads();  // barrier initialised before anyone waits on it
		const bool late = !mbar_wait(bar, 0);
		if (__syncthreads_or(late)) {
			if (threadIdx.x == 0) set_error(L, kErrBulkTimeout);
			mbar_wait(bar, 0);
			return false;
		}
		return true;
	}
	for (uint32_t i = threadIdx.x; i < cnt * 9u; i += blockDim.x) s_tri[i] = src[i];
	__syncthreads();
	return true;
}

// A small triangle's solid setup parked in shared memory between the classify phases.  15 words
// padded to 20: records stay 16-byte aligned for vector access, and the 8 lanes of a quarter warp
// touching 8 records start on banks 0, 20, 8, 28, 16, 4, 24, 12 -- no conflicts (at 16 words, 4-way).
struct __align__(16) SmallSolid {
	float nx, ny, nz, v0x, v0y, v0z, ax, ay, bx, by, cx, cy;
	int y0, z0;
	uint32_t ext;  // (y1 - y0) | (z1 - z0) << 16
	uint32_t pad[5];
};
static_assert(sizeof(SmallSolid) == 80, "SmallSolid stride");

__device__ __forceinline__ uint32_t block_scan(uint32_t v, uint32_t* s_warp, uint32_t* total) {
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	uint32_t incl = v;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		const uint32_t u = __shfl_up_sync(FULL, incl, d);
		if (lane >= (uint32_t)d) incl += u;
	}
	if (lane == 31) s_warp[warp] = incl;
	__syncthreads();
	if (warp == 0) {
		uint32_t w = lane < kTile / 32 ? s_warp[lane] : 0u;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			const uint32_t u = __shfl_up_sync(FULL, w, d);
			if (lane >= (uint32_t)d) w += u;
		}
		if (lane < kTile / 32) s_warp[lane] = w;
	}
	__syncthreads();
	*total = s_warp[kTile / 32 - 1];
	return (warp ? s_warp[warp - 1] : 0u) + incl - v;
}

// Phase 1: one thread per triangle (setup, classify, queue the big ones, park the small ones).
// Phase 2: the columns of all small triangles of the tile, one (triangle, column) item per thread.
template <class P>
__global__ void __launch_bounds__(kTile) solid_classify(const __grid_constant__ LaunchDesc L, const uint32_t small_cols) {
	__shared__ __align__(16) union {
		float tri[kTile * 9];
		SmallSolid small[kTile];
	} sm;
	__shared__ uint32_t s_items[kTile * kSmallCols];  // (triangle | dy << 8 | dz << 16) per column
	__shared__ uint32_t s_warp[kTile / 32];
	__shared__ __align__(8) uint64_t s_bar;
	const uint32_t tile = blockIdx.x;
	const uint32_t j = job_of_tile(L, tile);
	const JobDesc& J = job_at(L, j);
	const uint64_t n = J.n_tri;
	const bool morton = (J.flags & JOB_MORTON) != 0;
	const float bmin[3] = {J.bmin[0], J.bmin[1], J.bmin[2]};
	const float unit[3] = {J.unit[0], J.unit[1], J.unit[2]};
	const float inv[3] = {J.inv_unit[0], J.inv_unit[1], J.inv_unit[2]};
	const uint32_t grid[3] = {J.grid[0], J.grid[1], J.grid[2]};
	uint32_t* flips = J.flips;
	const uint64_t t0 = (uint64_t)(tile - J.tile_begin) * kTile;
	const uint32_t cnt = (uint32_t)umin64((uint64_t)kTile, n - t0);
	if (!stage_tile(L, J.tris + t0 * 9, cnt, sm.tri, &s_bar, (J.flags & JOB_PLAIN_LOADS) != 0)) return;  // tile not staged: error word set

	const uint32_t lane = threadIdx.x & 31u;
	const bool valid = threadIdx.x < cnt;
	float t[9];
#pragma unroll
	for (int k = 0; k < 9; k++) t[k] = valid ? sm.tri[threadIdx.x * 9 + k] : 0.0f;
	__syncthreads();

	bool is_mid = false, is_big = false;
	uint32_t n_items = 0, n_cols = 0;
	if (valid) {
		SolidTri S;
		solid_setup<P>(t, bmin, unit, inv, grid, S);
		if (!S.skip && S.y0 <= S.y1 && S.z0 <= S.z1) {
			const uint64_t ncols = (uint64_t)(S.y1 - S.y0 + 1) * (uint64_t)(S.z1 - S.z0 + 1);
			if (ncols <= small_cols && ncols <= kSmallCols) {
				SmallSolid& o = sm.small[threadIdx.x];
				o.nx = S.nx; o.ny = S.ny; o.nz = S.nz; o.v0x = S.v0x; o.v0y = S.v0y; o.v0z = S.v0z;
				o.ax = S.ax; o.ay = S.ay; o.bx = S.bx; o.by = S.by; o.cx = S.cx; o.cy = S.cy;
				o.y0 = S.y0; o.z0 = S.z0;
				o.ext = (uint32_t)(S.y1 - S.y0) | ((uint32_t)(S.z1 - S.z0) << 16);
				n_cols = (uint32_t)ncols;
			} else {
				const uint64_t it = (ncols + kColsPerItem - 1) / kColsPerItem;
				n_items = (uint32_t)umin64(it, 0xFFFFFFu);
				is_mid = n_items == 1;
				is_big = n_items > 1;
			}
		}
	}
	const uint32_t lt = (1u << lane) - 1u;
	const uint32_t mid_ballot = __ballot_sync(FULL, is_mid);
	if (mid_ballot) {
		uint32_t base = 0;
		const uint32_t leader = __ffs(mid_ballot) - 1;
		if (lane == leader) base = atomicAdd(&L.scr.ctr->mid, (unsigned)__popc(mid_ballot));
		base = __shfl_sync(FULL, base, leader);
		const uint32_t slot = base + __popc(mid_ballot & lt);
		if (is_mid) {
			if (slot < L.scr.cap) L.scr.mid[slot] = MidRec{j, (uint32_t)(t0 + threadIdx.x)};
			else set_error(L, kErrQueueOverflow);
		}
	}
	const uint32_t big_ballot = __ballot_sync(FULL, is_big);
	if (big_ballot) {
		uint32_t incl = is_big ? n_items : 0u;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			const uint32_t v = __shfl_up_sync(FULL, incl, d);
			if (lane >= (uint32_t)d) incl += v;
		}
		const uint32_t total = __shfl_sync(FULL, incl, 31);
		unsigned long long old = 0;
		if (lane == 0)
			old = atomicAdd(&L.scr.ctr->big, ((unsigned long long)__popc(big_ballot) << kBigShift) | (unsigned long long)total);
		old = __shfl_sync(FULL, old, 0);
		if (is_big) {
			const uint32_t rec = (uint32_t)(old >> kBigShift) + __popc(big_ballot & lt);
			const uint64_t first = (old & kBigItemMask) + incl - n_items;
			if (rec < L.scr.cap && first + n_items <= kBigItemMask)
				L.scr.big[rec] = BigRec{first, j, (uint32_t)(t0 + threadIdx.x), n_items, 0u};
			else
				set_error(L, kErrQueueOverflow);
		}
	}

	// Phase 2: columns of the small triangles (src/voxelize_solid.cu:115-139).
	uint32_t total_cols = 0;
	const uint32_t off = block_scan(n_cols, s_warp, &total_cols);
	if (n_cols) {
		const uint32_t ext = sm.small[threadIdx.x].ext;
		const uint32_t nyc = (ext & 0xFFFFu) + 1u, nzc = (ext >> 16) + 1u;
		uint32_t c = off;
		for (uint32_t dy = 0; dy < nyc; dy++)
			for (uint32_t dz = 0; dz < nzc; dz++) s_items[c++] = threadIdx.x | (dy << 8) | (dz << 16);
	}
	__syncthreads();
	for (uint32_t k = threadIdx.x; k < total_cols; k += kTile) {
		const uint32_t it = s_items[k];
		const SmallSolid& o = sm.small[it & 0xFFu];
		SolidTri S;
		S.nx = o.nx; S.ny = o.ny; S.nz = o.nz; S.v0x = o.v0x; S.v0y = o.v0y; S.v0z = o.v0z;
		S.ax = o.ax; S.ay = o.ay; S.bx = o.bx; S.by = o.by; S.cx = o.cx; S.cy = o.cy;
		const int y = o.y0 + (int)((it >> 8) & 0xFFu), z = o.z0 + (int)(it >> 16);
		int xmax;
		if (column_hit<P>(S, unit, y, z, morton, xmax)) record_hit(flips, grid, morton, y, z, xmax);
	}
}

template <class P>
__global__ void __launch_bounds__(kRowsThreads) solid_cols(const __grid_constant__ LaunchDesc L) {
	const uint32_t lane = threadIdx.x & 31u;
	Counters* C = L.scr.ctr;
	__shared__ unsigned long long s_bigc;  // read once per CTA (see surf_rows)
	__shared__ unsigned s_mid;
	if (threadIdx.x == 0) {
		s_bigc = *reinterpret_cast<volatile unsigned long long*>(&C->big);
		s_mid = *reinterpret_cast<volatile unsigned*>(&C->mid);
	}
	__syncthreads();
	const unsigned long long bigc = s_bigc;
	const uint32_t n_big = min((uint32_t)(bigc >> kBigShift), L.scr.cap);
	const uint64_t n_big_items = bigc & kBigItemMask;
	const uint32_t n_mid = min(s_mid, L.scr.cap);
	const uint64_t total = n_big_items + n_mid;
	// Warps beyond the number of queued items have nothing to claim: they leave without touching
	// the ticket counter (all of them do when only small triangles were queued).
	if ((uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5) >= total) return;
	WarpTickets wt(total, gridDim.x * (blockDim.x >> 5));
	for (;;) {
		unsigned long long tk = 0;
		if (!wt.take(&C->ticket, total, lane, tk)) break;
		uint32_t job = 0, tri = 0, chunk = 0, ok = 0;
		if (lane == 0) {
			if (tk < n_big_items) {
				if (n_big > 0) {
					uint32_t lo = 0, hi = n_big - 1;
					while (lo < hi) {
						const uint32_t m = (lo + hi + 1) >> 1;
						if (L.scr.big[m].item_begin <= tk) lo = m; else hi = m - 1;
					}
					const BigRec r = L.scr.big[lo];
					job = r.job; tri = r.tri; chunk = (uint32_t)(tk - r.item_begin);
					ok = tk >= r.item_begin && chunk < r.n_items;
				}
			} else {
				const MidRec r = L.scr.mid[tk - n_big_items];
				job = r.job; tri = r.tri;
				ok = 1;
			}
			// never follow a malformed record (only possible after a queue overflow)
			if (ok && (job >= L.n_jobs || tri >= job_at(L, job).n_tri)) ok = 0;
		}
		ok = __shfl_sync(FULL, ok, 0);
		if (!ok) continue;
		job = __shfl_sync(FULL, job, 0);
		tri = __shfl_sync(FULL, tri, 0);
		chunk = __shfl_sync(FULL, chunk, 0);
		const JobDesc& J = job_at(L, job);
		const float unit[3] = {J.unit[0], J.unit[1], J.unit[2]};
		const uint32_t grid[3] = {J.grid[0], J.grid[1], J.grid[2]};
		const bool morton = (J.flags & JOB_MORTON) != 0;
		float tv = lane < 9 ? J.tris[(uint64_t)tri * 9 + lane] : 0.0f;
		float t[9];
#pragma unroll
		for (int k = 0; k < 9; k++) t[k] = __shfl_sync(FULL, tv, k);
		SolidTri S;
		solid_setup<P>(t, J.bmin, unit, J.inv_unit, grid, S);
		const uint64_t nzc = (uint64_t)(S.z1 - S.z0 + 1);
		const uint64_t ncols = (uint64_t)(S.y1 - S.y0 + 1) * nzc;
		const uint64_t c0 = (uint64_t)chunk * kColsPerItem;
		const uint64_t c1 = umin64(ncols, c0 + kColsPerItem);
		// column c is (y0 + c / nzc, z0 + c % nzc): one division for the lane's first column, then
		// steps of 32 columns (dy rows and dz slices, carrying z into y)
		const uint64_t cf = c0 + lane;
		if (cf < c1) {  // (no lane enters when the range is empty: nzc may be 0 then)
			int y = S.y0 + (int)(cf / nzc), z = S.z0 + (int)(cf % nzc);
			const int dy = (int)(32u / nzc), dz = (int)(32u % nzc);
			for (uint64_t c = cf; c < c1; c += 32) {
				int xmax;
				if (column_hit<P>(S, unit, y, z, morton, xmax)) record_hit(J.flips, grid, morton, y, z, xmax);
				y += dy;
				z += dz;
				if (z > S.z1) {
					z -= (int)nzc;
					y++;
				}
			}
		}
	}
}

__device__ __forceinline__ uint32_t prefix_xor_msb(uint32_t t) {
	t ^= t >> 1;
	t ^= t >> 2;
	t ^= t >> 4;
	t ^= t >> 8;
	t ^= t >> 16;
	return t;
}

// Morton grids resolved and transcoded in one pass by solid_morton_slab (cubic powers of two).
__host__ __device__ __forceinline__ bool slab_grid(uint64_t g) { return g >= 32 && g <= 1024; }

// Resolve one word: toggles t (MSB first) plus the parity carried in from the row's earlier words.
__device__ __forceinline__ uint32_t resolve_word(uint32_t t, uint32_t& carry) {
	const uint32_t res = prefix_xor_msb(t) ^ (carry ? 0xFFFFFFFFu : 0u);
	carry = res & 1u;  // the row's parity after this word's last bit
	return res;
}

// Linear jobs: table ^= resolved, toggles cleared.  Morton jobs: toggles replaced by the resolved
// bits for solid_morton_* to gather.
// XOR a resolved word into the table (the reference's semantics: the caller's table is XORed), or
// store it, zero or not, when the engine owns the table's content (JOB_TABLE_OVERWRITE).
__device__ __forceinline__ void xor_out(uint32_t* dest, uint64_t w, uint32_t v, bool overwrite) {
	if (overwrite) dest[w] = v;
	else if (v) dest[w] ^= v;
}

__device__ __forceinline__ void resolve_store(uint32_t* flips, uint32_t* dest, uint64_t w, uint32_t t, uint32_t res,
                                              bool morton, bool overwrite) {
	if (morton) {
		if (res != t) flips[w] = res;
	} else {
		xor_out(dest, w, res, overwrite);
		if (t) flips[w] = 0u;
	}
}

// One thread per resolve unit.  gx a multiple of 32: a unit is one row (whole words; 16-byte
// loads when the row and both tables are 16-byte aligned).  Other gx: the shortest run of rows
// that starts and ends on word boundaries, walked bit by bit (odd grid sizes only).
__global__ void __launch_bounds__(256) solid_resolve(const __grid_constant__ LaunchDesc L) {
	const uint32_t unit_id = blockIdx.x * blockDim.x + threadIdx.x;
	if (unit_id >= L.n_units) return;
	const uint32_t j = job_search(L, unit_id, [](const JobDesc& d) { return (uint64_t)d.unit_begin; });
	const JobDesc& J = job_at(L, j);
	const uint64_t gx = J.grid[0];
	const uint64_t rows = (uint64_t)J.grid[1] * J.grid[2];
	const bool morton = (J.flags & JOB_MORTON) != 0;
	const bool overwrite = (J.flags & JOB_TABLE_OVERWRITE) != 0 && !morton;  // Morton words: written below
	uint32_t* flips = J.flips;
	uint32_t* dest = J.table;
	const uint64_t u = unit_id - J.unit_begin;
	if (morton && slab_grid(gx)) return;  // solid_morton_slab resolves these jobs itself
	if (gx % 32 == 0) {
		const uint32_t wpr = (uint32_t)(gx >> 5);
		const uint64_t w0 = u * wpr;
		uint32_t carry = 0;
		const bool vec = (wpr & 3u) == 0 && ((reinterpret_cast<uintptr_t>(flips + w0) | reinterpret_cast<uintptr_t>(dest + w0)) & 15u) == 0;
		if (vec) {
			for (uint32_t i = 0; i < wpr; i += 4) {
				const uint4 t = *reinterpret_cast<const uint4*>(flips + w0 + i);
				if ((t.x | t.y | t.z | t.w) == 0u && carry == 0u) {  // outside the solid
					if (overwrite) *reinterpret_cast<uint4*>(dest + w0 + i) = make_uint4(0u, 0u, 0u, 0u);
					continue;
				}
				const uint32_t r0 = resolve_word(t.x, carry), r1 = resolve_word(t.y, carry);
				const uint32_t r2 = resolve_word(t.z, carry), r3 = resolve_word(t.w, carry);
				if (morton) {
					*reinterpret_cast<uint4*>(flips + w0 + i) = make_uint4(r0, r1, r2, r3);
				} else if (overwrite) {
					*reinterpret_cast<uint4*>(dest + w0 + i) = make_uint4(r0, r1, r2, r3);
					if (t.x | t.y | t.z | t.w) *reinterpret_cast<uint4*>(flips + w0 + i) = make_uint4(0u, 0u, 0u, 0u);
				} else {
					uint4 d = *reinterpret_cast<const uint4*>(dest + w0 + i);
					d.x ^= r0; d.y ^= r1; d.z ^= r2; d.w ^= r3;
					*reinterpret_cast<uint4*>(dest + w0 + i) = d;
					if (t.x | t.y | t.z | t.w) *reinterpret_cast<uint4*>(flips + w0 + i) = make_uint4(0u, 0u, 0u, 0u);
				}
			}
		} else {
			for (uint32_t i = 0; i < wpr; i++) {
				const uint32_t t = flips[w0 + i];
				if (t == 0u && carry == 0u) {
					if (overwrite) dest[w0 + i] = 0u;
					continue;
				}
				resolve_store(flips, dest, w0 + i, t, resolve_word(t, carry), morton, overwrite);
			}
		}
	} else {
		const uint64_t g = gx;
		uint64_t a = g, bb = 32;
		while (bb) { const uint64_t r = a % bb; a = bb; bb = r; }
		const uint64_t p = 32 / a;  // rows per unit: lcm(gx, 32) / gx
		const uint64_t r0 = u * p, r1 = umin64(rows, r0 + p);
		const uint64_t b0 = r0 * g, b1 = r1 * g;
		uint32_t carry = 0;
		uint64_t next_row = b0;  // bit index of the next row start
		for (uint64_t w = b0 >> 5; (w << 5) < b1; w++) {
			const uint32_t t = flips[w];
			uint32_t res = 0;
			for (uint32_t k = 0; k < 32; k++) {
				const uint64_t bit = (w << 5) + k;
				if (bit >= b1) break;
				if (bit == next_row) {
					carry = 0;
					next_row += g;
				}
				carry ^= (t >> (31 - k)) & 1u;
				res |= carry << (31 - k);
			}
			resolve_store(flips, dest, w, t, res, morton, overwrite);
		}
	}
}



// Morton jobs with g >= 32: one CTA per group of W = min(4, g/32) x-adjacent Morton-aligned 32^3
// bricks.  Each brick is 1,024 consecutive Morton words; the group's 32 x 32 rows of W*32 x-bits are
// staged in shared memory (16-byte accesses when W = 4) and cleared in the flip table (this CTA is
// their only reader), then each Morton word is assembled from eight 4-bit row nibbles and XORed into
// the table with coalesced accesses.
__global__ void __launch_bounds__(256) solid_morton_brick(const __grid_constant__ LaunchDesc L) {
	__shared__ __align__(16) uint32_t s_rows[32 * 32 * 4];  // [z][y][W] words of x-bits
	const uint64_t group = blockIdx.x;
	const uint32_t j = job_search(L, group, [](const JobDesc& d) { return d.mbrick_begin; });
	const JobDesc& J = job_at(L, j);
	const uint64_t g = J.grid[0];
	const uint32_t W = g >= 128 ? 4u : (uint32_t)(g >> 5);       // bricks per group
	const uint64_t gi = group - J.mbrick_begin;                  // group index within the job
	// groups are numbered x-fastest over (g/32/W) x (g/32) x (g/32); group gi covers the bricks
	// (W*Bx + k, by, bz), k < W (g is a power of two: the divisions are shifts)
	const uint32_t lg_nb = 31u - __clz((uint32_t)(g >> 5));      // log2(bricks per axis)
	const uint32_t lg_w = W == 4 ? 2u : (W == 2 ? 1u : 0u);
	const uint64_t Bx = gi & ((1ull << (lg_nb - lg_w)) - 1ull);
	const uint64_t by = (gi >> (lg_nb - lg_w)) & ((1ull << lg_nb) - 1ull);
	const uint64_t bz = gi >> (2 * lg_nb - lg_w);
	const uint64_t bx = Bx * W;
	uint32_t* flips = J.flips;
	const uint64_t wpr = g >> 5;
	for (uint32_t i = threadIdx.x; i < 1024; i += 256) {
		const uint64_t z = bz * 32 + (i >> 5), y = by * 32 + (i & 31);
		const uint64_t w = (z * g + y) * wpr + bx;
		if (W == 4 && ((reinterpret_cast<uintptr_t>(flips + w) & 15u) == 0)) {
			const uint4 v = *reinterpret_cast<const uint4*>(flips + w);
			*reinterpret_cast<uint4*>(s_rows + i * 4) = v;
			if (v.x | v.y | v.z | v.w) *reinterpret_cast<uint4*>(flips + w) = make_uint4(0u, 0u, 0u, 0u);
		} else {
			for (uint32_t k = 0; k < W; k++) {
				const uint32_t v = flips[w + k];
				s_rows[i * 4 + k] = v;
				if (v) flips[w + k] = 0u;
			}
		}
	}
	__syncthreads();
	for (uint32_t xk = 0; xk < W; xk++) {
		// brick (bx + xk, by, bz): its Morton words are the 1,024 starting at its Morton index * 1024
		const uint64_t brick = spread3((uint32_t)(bx + xk)) | (spread3((uint32_t)by) << 1) | (spread3((uint32_t)bz) << 2);
		uint32_t* dest = J.table + (brick << 10);
		for (uint32_t m = threadIdx.x; m < 1024; m += 256) {
			const uint32_t X = compact3(m >> 1), Y = compact3(m >> 2), Z = compact3(m);
			uint32_t out = 0;
#pragma unroll
			for (uint32_t dz = 0; dz < 2; dz++)
#pragma unroll
				for (uint32_t dy = 0; dy < 4; dy++) {
					const uint32_t row = s_rows[((2 * Z + dz) * 32 + 4 * Y + dy) * 4 + xk];
					const uint32_t nib = (row >> (28u - 4u * X)) & 0xFu;
					out |= nibble_mask(nib) >> (2u * (dy & 1u) + 4u * dz + 16u * (dy >> 1));
				}
			xor_out(dest, m, out, (J.flags & JOB_TABLE_OVERWRITE) != 0);
		}
	}
}

// Morton jobs with 32 <= g <= 1024: resolve, transcode and clear in one pass.  One CTA per slab of
// 16 x 16 rows (y block by, z block bz, 16 each): for each of its 16 z-slices the slab's 16 rows are
// contiguous in the flip table, so they are loaded with coalesced 16-byte accesses into shared
// memory (rows padded to an odd word count: no bank conflicts below) and cleared; each thread
// resolves one whole row (prefix XOR along x); then every 16^3 block along x -- 128 consecutive
// Morton words -- is gathered from 4-bit row nibbles and XORed into the table.
__global__ void __launch_bounds__(256) solid_morton_slab(const __grid_constant__ LaunchDesc L) {
	extern __shared__ __align__(16) uint32_t s_slab[];  // row zi*16 + yi at slab_row(row, stride)
	const uint64_t slab = blockIdx.x;
	const uint32_t j = job_search(L, slab, [](const JobDesc& d) { return d.mslab_begin; });
	const JobDesc& J = job_at(L, j);
	const uint64_t g = J.grid[0];
	const uint32_t wpr = (uint32_t)(g >> 5);           // words per row
	const uint32_t stride = wpr | 1u;
	const uint32_t lgw = 31u - __clz(wpr);
	const uint32_t nb = (uint32_t)(g >> 4);            // 16-blocks per axis
	const uint32_t lgb = 31u - __clz(nb);
	const uint64_t si = slab - J.mslab_begin;
	const uint64_t by = si & (nb - 1u), bz = si >> lgb;
	uint32_t* flips = J.flips;
	const uint32_t chunk = 16u * wpr;                   // words of the slab in one z-slice
	for (uint32_t i = threadIdx.x; i < 16u * (chunk / 4u); i += 256) {
		const uint32_t zi = i / (chunk / 4u), q = i % (chunk / 4u);
		uint4* src = reinterpret_cast<uint4*>(flips + ((bz * 16 + zi) * g + by * 16) * wpr) + q;
		const uint4 v = *src;
		const uint32_t vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
		for (int k = 0; k < 4; k++) {
			const uint32_t idx = 4 * q + k;
			s_slab[slab_row(zi * 16 + (idx >> lgw), stride) + (idx & (wpr - 1u))] = vv[k];
		}
		if (v.x | v.y | v.z | v.w) *src = make_uint4(0u, 0u, 0u, 0u);
	}
	__syncthreads();
	{
		uint32_t* row = s_slab + slab_row(threadIdx.x, stride);  // 256 rows, one per thread
		uint32_t carry = 0;
		for (uint32_t w = 0; w < wpr; w++) {
			const uint32_t t = row[w];
			if (t == 0u && carry == 0u) continue;
			row[w] = resolve_word(t, carry);
		}
	}
	__syncthreads();
	// 16^3 blocks along x: two per pass (128 Morton words each, one per thread)
	const uint32_t half = threadIdx.x >> 7, m = threadIdx.x & 127u;
	const uint32_t X = compact3(m >> 1), Y = compact3(m >> 2), Z = compact3(m);  // 2, 2, 3 bits
	for (uint32_t bx = half; bx < nb; bx += 2) {
		const uint64_t blk = spread3(bx) | (spread3((uint32_t)by) << 1) | (spread3((uint32_t)bz) << 2);
		const uint32_t wsel = bx >> 1, xoff = (bx & 1u) * 16u + 4u * X;  // word, first x bit in it
		uint32_t out = 0;
#pragma unroll
		for (uint32_t dz = 0; dz < 2; dz++)
#pragma unroll
			for (uint32_t dy = 0; dy < 4; dy++) {
				const uint32_t rw = s_slab[slab_row((2 * Z + dz) * 16 + 4 * Y + dy, stride) + wsel];
				const uint32_t nib = (rw >> (28u - xoff)) & 0xFu;
				out |= nibble_mask(nib) >> (2u * (dy & 1u) + 4u * dz + 16u * (dy >> 1));
			}
		xor_out(J.table, (blk << 7) + m, out, (J.flags & JOB_TABLE_OVERWRITE) != 0);
	}
}

// Morton jobs with g < 32: one Morton word per thread, 32 codes decoded one by one.
__global__ void __launch_bounds__(256) solid_morton_small(const __grid_constant__ LaunchDesc L) {
	const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (idx >= L.n_mwords) return;
	const uint32_t j = job_search(L, idx, [](const JobDesc& d) { return d.mword_begin; });
	const JobDesc& J = job_at(L, j);
	const uint64_t m = idx - J.mword_begin;
	const uint64_t g = J.grid[0];
	const uint32_t* flips = J.flips;
	uint32_t out = 0;
	const uint64_t total = g * g * g;
	for (uint32_t i = 0; i < 32; i++) {
		const uint64_t c = m * 32 + i;
		if (c >= total) break;
		const uint64_t x = compact3(c), y = compact3(c >> 1), z = compact3(c >> 2);
		const uint64_t lin = x + g * (y + g * z);
		out |= ((flips[lin >> 5] >> (31u - (uint32_t)(lin & 31u))) & 1u) << (31u - i);
	}
	xor_out(J.table, m, out, (J.flags & JOB_TABLE_OVERWRITE) != 0);
}

// Morton jobs with g < 32: clear the resolved flip table, one thread per resolve unit (the larger
// grids' bricks clear their own words).
__global__ void __launch_bounds__(256) solid_zero(const __grid_constant__ LaunchDesc L) {
	const uint32_t unit_id = blockIdx.x * blockDim.x + threadIdx.x;
	if (unit_id >= L.n_units) return;
	const uint32_t j = job_search(L, unit_id, [](const JobDesc& d) { return (uint64_t)d.unit_begin; });
	const JobDesc& J = job_at(L, j);
	if (!(J.flags & JOB_MORTON) || J.grid[0] >= 32) return;
	const uint64_t gx = J.grid[0];
	const uint64_t rows = (uint64_t)J.grid[1] * J.grid[2];
	uint64_t a = gx, bb = 32;
	while (bb) { const uint64_t r = a % bb; a = bb; bb = r; }
	const uint64_t p = (gx % 32 == 0) ? 1 : 32 / a;
	const uint64_t u = unit_id - J.unit_begin;
	const uint64_t r0 = u * p, r1 = umin64(rows, r0 + p);
	for (uint64_t w = (r0 * gx) >> 5; w < ((r1 * gx + 31) >> 5); w++) J.flips[w] = 0u;
}

}  // namespace

SolidUnits solid_units(const uint32_t grid[3]) {
	const uint64_t gx = grid[0];
	const uint64_t rows = (uint64_t)grid[1] * grid[2];
	SolidUnits s;
	s.aligned = gx % 32 == 0;
	if (s.aligned) {
		s.rows_per_unit = 1;  // one row per resolve thread
	} else {
		uint64_t a = gx, b = 32;
		while (b) { uint64_t r = a % b; a = b; b = r; }
		s.rows_per_unit = 32 / a;
	}
	s.units = (rows + s.rows_per_unit - 1) / s.rows_per_unit;
	return s;
}

template <class P>
static cudaError_t launch_solid_t(const LaunchDesc& L, const Tune& tune, int cols_grid, cudaStream_t s, unsigned phases,
                                  const Prof* prof) {
	cudaError_t e = cudaSuccess;
	if (prof) (*prof)(nullptr, s);
	if ((phases & kSolidToggles) && L.n_tiles) {
		solid_classify<P><<<L.n_tiles, kTile, 0, s>>>(L, tune.small_cols);
		if ((e = cudaGetLastError()) != cudaSuccess) return e;
		if (prof) (*prof)("solid_classify", s);
		if ((e = launch_k(solid_cols<P>, (unsigned)cols_grid, kRowsThreads, 0, s, L)) != cudaSuccess) return e;
		if (prof) (*prof)("solid_cols", s);
	}
	if (phases & kSolidResolve) {
		if (L.n_units) {
			if ((e = launch_k(solid_resolve, (L.n_units + 255) / 256, 256, 0, s, L)) != cudaSuccess) return e;
			if (prof) (*prof)("solid_resolve", s);
		}
		if (L.n_mslabs) {
			static int attr_set[64] = {};
			int dev = 0;
			cudaGetDevice(&dev);
			if (dev >= 0 && dev < 64 && !attr_set[dev]) {
				if ((e = cudaFuncSetAttribute(solid_morton_slab, cudaFuncAttributeMaxDynamicSharedMemorySize,
				                              (256 * (32 + 1) + kSlabSkewWords) * 4)) != cudaSuccess)
					return e;
				attr_set[dev] = 1;
			}
			if ((e = launch_k(solid_morton_slab, (unsigned)L.n_mslabs, 256, L.slab_smem, s, L)) != cudaSuccess) return e;
			if (prof) (*prof)("solid_morton_slab", s);
		}
		if (L.n_mbricks) {
			if ((e = launch_k(solid_morton_brick, (unsigned)L.n_mbricks, 256, 0, s, L)) != cudaSuccess) return e;
			if (prof) (*prof)("solid_morton", s);
		}
		if (L.n_mwords) {
			if ((e = launch_k(solid_morton_small, (unsigned)((L.n_mwords + 255) / 256), 256, 0, s, L)) != cudaSuccess)
				return e;
			if ((e = launch_k(solid_zero, (L.n_units + 255) / 256, 256, 0, s, L)) != cudaSuccess) return e;
			if (prof) (*prof)("solid_morton_small", s);
		}
	}
	return cudaSuccess;
}

cudaError_t launch_solid(const LaunchDesc& L, const Tune& tune, int cols_grid, cudaStream_t s, unsigned phases,
                         const Prof* prof) {
	return launch_solid_t<RefFma>(L, tune, cols_grid, s, phases, prof);
}

int solid_cols_blocks_per_sm() {
	int n = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, solid_cols<RefFma>, kRowsThreads, 0);
	return n > 0 ? n : 1;
}

}  // namespace cvx
