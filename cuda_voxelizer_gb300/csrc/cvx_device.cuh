// cvx_device.cuh -- device-side building blocks shared by the surface and solid engines.
//
// Exactness contract.  Every predicate of the reference kernels (src/voxelize.cu:58-190,
// src/voxelize_solid.cu:16-145) is re-evaluated here with the same operands, the same operation
// order and the same rounding: each multiply, add and fused multiply-add is written as an explicit
// __fmul_rn / __fadd_rn / __fmaf_rn, so the compiler cannot contract or reorder them, and the
// fused-multiply-add pattern is the one nvcc produces for the reference's helper_math expressions
// on sm_103a (class RefFma below).  rsqrtf, IEEE division (__fdiv_rn), fminf/fmaxf and the
// float->int conversions are the same device operations the reference compiles to.  Any
// re-organisation the engine does (row intervals, column queues, parity flips) only changes
// *which* voxels are evaluated and in what order, never the value of a predicate at a voxel.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace cvx {

// ------------------------------------------------------------------------------------------------
// Fused-multiply-add pattern of the reference kernels as nvcc (--fmad=true) compiles them for
// sm_103a.  Values: 0 = no fusion, a*b and c*d rounded separately; 1 = the first product is fused,
// fma(a, b, c*d); 2 = the second, fma(c, d, a*b) (for a*b - c*d: fma(a,b,-(c*d)) / fma(-c,d,a*b)).
// Pinned empirically against the reference kernels compiled from their own sources (bit-exact
// tables on millions of near-tie voxels; source level reasons in parentheses):
struct RefFma {
	static constexpr int cross = 1;    // helper_math cross() in normalize(cross(e0, e1))
	static constexpr int dot3 = 1;     // dot(c, c) inside normalize: fma(z,z',fma(x,x',y*y'))
	static constexpr int dot3d = 1;    // d1, d2 = dot(n, c - v0), dot(n, delta_p - c - v0)
	static constexpr int dot2_xy = 2;  // setup dot(n_xy_e, v.xy): n_xy_e.x = -1.0f*e.y is a negation,
	static constexpr int dot2_yz = 2;  //   so its product is not the one fused; same for n_yz_e,
	static constexpr int dot2_zx = 2;  //   n_zx_e (src/voxelize.cu:99-133)
	static constexpr int plane = 2;    // per-voxel dot(n,p): fma(nx,px,ny*py) + nz*pz (the y and z
	                                   //   products are hoisted out of the x loop before fusion)
	static constexpr int edge_xy = 1;  // per-voxel dot(n_xy_e, p_xy): fma(a.x, px, a.y*py)
	static constexpr int edge_yz = 1;  // per-voxel dot(n_yz_e, p_yz): fma(a.x, py, a.y*pz)
	static constexpr int edge_zx = 2;  // per-voxel dot(n_zx_e, p_zx): fma(a.y, px, a.x*pz) (pz term hoisted)
	static constexpr int ccw = 2;      // solid checkCCW: e0.x*e1.y - e1.x*e0.y -> fma(-e1.x, e0.y, e0.x*e1.y)
	static constexpr int pt = 1;       // solid check_point_triangle t1..t3: fma(a, b, -(c*d))
	static constexpr int getx = 1;     // solid get_x_coordinate: fma(n.y, A, n.z*B) for linear tables,
	static constexpr int getx_morton = 2;  // fma(n.z, B, n.y*A) for Morton tables: the reference
	                                   //   kernel tests its morton_order argument inside the x loop,
	                                   //   and its compiled Morton copy contracts the sum the other
	                                   //   way (xmax then differs by one voxel on a few columns, e.g.
	                                   //   16 of ~700k on a 1024^3 soup)
};

template <int P>
__device__ __forceinline__ float mul_sub(float a, float b, float c, float d) {
	if constexpr (P == 1) return __fmaf_rn(a, b, -__fmul_rn(c, d));
	else if constexpr (P == 2) return __fmaf_rn(-c, d, __fmul_rn(a, b));
	else return __fsub_rn(__fmul_rn(a, b), __fmul_rn(c, d));
}
template <int P>
__device__ __forceinline__ float mul_add(float a, float b, float c, float d) {
	if constexpr (P == 1) return __fmaf_rn(a, b, __fmul_rn(c, d));
	else if constexpr (P == 2) return __fmaf_rn(c, d, __fmul_rn(a, b));
	else return __fadd_rn(__fmul_rn(a, b), __fmul_rn(c, d));
}
template <int P>
__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
	if constexpr (P == 1) return __fmaf_rn(az, bz, __fmaf_rn(ax, bx, __fmul_rn(ay, by)));
	else if constexpr (P == 2) return __fmaf_rn(az, bz, __fmaf_rn(ay, by, __fmul_rn(ax, bx)));
	else return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// ------------------------------------------------------------------------------------------------
// Job and launch descriptors.

// JOB_NARROW: every voxel index of the job fits 32 bits (linear: gx*gy*gz <= 2^32; Morton: a cubic
// grid of at most 1024), so the surface writes compute indices and Morton codes in 32-bit
// arithmetic.  Set by the host; a hint only (the 64-bit path gives the same words).
// JOB_TABLE_OVERWRITE (solid jobs): the engine owns the table's content in this launch sequence
// (plans that clear their tables, host plans, server batches): the resolve passes store every word
// of the table, zeros included, instead of XOR-ing into it.  The table need not be zeroed first:
// the result equals XOR-ing into a zeroed table, with one write per word and no read.
// JOB_PLAIN_LOADS: the job's triangles are not plain device memory (managed, host-registered or
// system memory -- the reference's main() passes cudaMallocManaged buffers): the classify kernels
// read them with ordinary loads instead of bulk copies.
// JOB_BRICKS: a surface job whose queued (larger) triangles are rasterized brick by brick in shared
// memory (bricks.cu) instead of by per-row global atomics.
enum : uint32_t { JOB_MORTON = 1u, JOB_SOLID = 2u, JOB_NARROW = 4u, JOB_TABLE_OVERWRITE = 8u, JOB_PLAIN_LOADS = 16u,
                  JOB_BRICKS = 32u };

// One mesh voxelization.  Plain data, uploaded as an array for batches or passed by value for a
// single mesh.
struct JobDesc {
	const float* tris;     // 9 floats per triangle (v0.xyz, v1.xyz, v2.xyz), device memory
	uint32_t* table;       // destination bit table, ceil(gx*gy*gz/32) words, OR (surface) / XOR (solid)
	uint32_t* flips;       // solid only: linear-order toggle table, zero on entry and left zero
	uint64_t n_tri;
	float bmin[3];
	float unit[3];
	float inv_unit[3];     // 1.0f / unit, correctly rounded (host); only used for the exactly checked div_trunc
	uint32_t grid[3];
	uint32_t flags;        // JOB_MORTON | JOB_SOLID | JOB_NARROW | JOB_TABLE_OVERWRITE | ...
	uint32_t tile_begin;   // first triangle tile of this job in the launch's tile space
	uint32_t unit_begin;   // solid: first resolve unit of this job in the launch's unit space
	uint64_t mword_begin;  // solid Morton, g < 32: first Morton word in the launch's word space
	uint64_t mbrick_begin; // solid Morton, g > 1024: first group of x-adjacent 32^3 bricks in the launch
	uint64_t mslab_begin;  // solid Morton, 32 <= g <= 1024: first 16x16-row slab in the launch
	uint32_t brick_begin;  // JOB_BRICKS: first 32^3 brick of this job in the launch's brick space
	uint32_t pad;
};

// Work-queue records written by the classify kernels and consumed by the cooperative kernels.
struct BigRec {            // triangle whose work is split into several items
	uint64_t item_begin;
	uint32_t job, tri, n_items, pad;
};
struct MidRec {            // triangle handled as a single item
	uint32_t job, tri;
};

// Device counters; zeroed before every launch sequence.
// `big` packs (number of BigRec << 40) | (number of big items) so that one 64-bit atomic hands a
// warp both its record slots and its item range; records are then sorted by item_begin, which
// the consumer's binary search relies on.  A launch holds fewer than 2^24 triangles (the host
// splits larger ones), so neither field can overflow into the other.
constexpr int kBigShift = 40;
constexpr unsigned long long kBigItemMask = (1ull << kBigShift) - 1ull;
struct Counters {
	unsigned long long big;
	unsigned long long ticket;   // next work ticket of the cooperative kernel
	unsigned long long pairs;    // (brick, triangle) pairs reserved by brick_bin
	unsigned long long bticket;  // next triangle of the brick queue for brick_bin
	unsigned long long fticket;  // next triangle of the brick queue for brick_fill
	unsigned long long rticket;  // next raster work unit for brick_raster
	unsigned int mid;            // number of MidRec
	unsigned int bq;             // number of triangles in the brick queue
	unsigned int units;          // raster work units (written by brick_scan)
	unsigned int error;          // nonzero: a device-side check failed (value says which)
	unsigned int pad[2];
};
// Everything before `error` is reset before every launch sequence; `error` persists until read.
constexpr size_t kCountersResetBytes = offsetof(Counters, error);

// Work tickets of the cooperative kernels, claimed by a warp K at a time: one atomic on the shared
// counter per K items instead of per item (a single hot address serialises in its L2 slice when
// hundreds of thousands of small items are queued).  K grows with the items per warp, up to 16,
// so the tail left when the counter runs out stays short.
struct WarpTickets {
	unsigned long long next = 0, end = 0;
	uint32_t K;
	__device__ WarpTickets(uint64_t total, uint32_t n_warps) {
		const uint64_t per = total / ((uint64_t)n_warps * 8u);
		K = (uint32_t)(per < 1 ? 1 : (per > 16 ? 16 : per));
	}
	// Next ticket of this warp (the same in every lane); false once every ticket is claimed.
	__device__ __forceinline__ bool take(unsigned long long* ctr, uint64_t total, uint32_t lane,
	                                     unsigned long long& tk) {
		if (next >= end) {
			unsigned long long b = 0;
			if (lane == 0) b = atomicAdd(ctr, (unsigned long long)K);
			b = __shfl_sync(0xFFFFFFFFu, b, 0);
			next = b;
			end = b + K;
		}
		if (next >= total) return false;
		tk = next++;
		return true;
	}
};

// Brick rasterization (JOB_BRICKS jobs, bricks.cu): the queued triangles of those jobs are binned to
// the 32^3 bricks of their tables that their planes cross, the (brick, triangle) pairs are grouped
// by brick with a counting sort, and each warp rasterizes a brick's pairs into a brick of its own in
// shared memory, then ORs it into the table with one global atomic per nonzero word.
constexpr uint32_t kBrickShift = 5;
constexpr uint32_t kBrick = 1u << kBrickShift;                       // voxels per brick edge
constexpr uint32_t kBrickWords = kBrick * kBrick * kBrick / 32u;      // 1024 words = 4 KiB per warp
constexpr uint32_t kPairsPerUnit = 256;                                // pairs per raster work unit

// A queued triangle's setup, cached by brick_bin for brick_fill and brick_raster (176 bytes).
struct __align__(16) BrickTri {
	float f[35];      // nx ny nz d1 d2, exy[3][2] eyz[3][2] ezx[3][2], dxy[3] dyz[3] dzx[3], v0.xyz
	int bb[6];        // bx0 by0 bz0 bx1 by1 bz1
	uint32_t binned;  // 1: its pairs are in the pair area; 0: surf_rows rasterizes it
	uint32_t pad[2];
};
static_assert(sizeof(BrickTri) == 176, "BrickTri is eleven 16-byte vectors");

struct Scratch {
	Counters* ctr;
	BigRec* big;
	MidRec* mid;
	uint32_t cap;          // capacity of big[], mid[], bq[] and tri[] (>= triangles in the launch)
	uint32_t pair_cap;     // capacity of pair_sorted (0: no pair area, every triangle goes to surf_rows)
	MidRec* bq;            // triangles of JOB_BRICKS jobs queued by the classify kernel
	BrickTri* tri;         // their setups, in queue order
	uint32_t* brick_cnt;   // pairs per brick (zero between launch sequences: brick_scan clears what it read)
	uint32_t* brick_off;   // n_bricks + 1: first sorted pair of each brick
	uint32_t* brick_cur;   // fill cursors
	uint32_t* unit_begin;  // n_bricks + 1: first raster work unit of each brick
	uint32_t* pair_sorted; // queue index of each pair's triangle, grouped by brick
};

struct LaunchDesc {
	const JobDesc* jobs;   // device array of n_jobs descriptors (n_jobs > 1)
	JobDesc single;        // the descriptor itself when n_jobs == 1
	uint32_t n_jobs;
	uint32_t n_tiles;      // total triangle tiles over all jobs
	uint32_t n_units;      // solid resolve units over all jobs
	uint64_t n_mwords;     // Morton words of solid Morton jobs with g < 32
	uint64_t n_mbricks;    // groups of x-adjacent 32^3 bricks of solid Morton jobs with g > 1024
	uint64_t n_mslabs;     // 16x16-row slabs of solid Morton jobs with 32 <= g <= 1024
	uint32_t slab_smem;    // dynamic shared memory of the slab kernel (largest slab of the launch)
	uint32_t n_bricks;     // 32^3 bricks of the launch's JOB_BRICKS jobs
	Scratch scr;
};

__device__ __forceinline__ const JobDesc& job_at(const LaunchDesc& L, uint32_t j) {
	return L.n_jobs == 1 ? L.single : L.jobs[j];
}

// Job owning triangle tile `tile` (jobs are sorted by tile_begin).
__device__ __forceinline__ uint32_t job_of_tile(const LaunchDesc& L, uint32_t tile) {
	if (L.n_jobs == 1) return 0;
	uint32_t lo = 0, hi = L.n_jobs - 1;
	while (lo < hi) {
		uint32_t mid = (lo + hi + 1) >> 1;
		if (L.jobs[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
	}
	return lo;
}

// ------------------------------------------------------------------------------------------------
// Morton order.  The reference encodes through three 256-entry LUTs (src/voxelize.cuh:20-34) whose
// values are the 3-way bit spread of the byte (x -> bits 0,3,6,..; y -> 1,4,..; z -> 2,5,..).  For
// coordinates below 2^16 (every grid whose table fits in memory) that equals the bit spread below.

__device__ __forceinline__ uint64_t spread3(uint32_t v) {
	uint64_t x = v & 0xFFFFu;
	x = (x | (x << 16)) & 0x0000FF0000FFull;
	x = (x | (x << 8)) & 0x00F00F00F00Full;
	x = (x | (x << 4)) & 0x0C30C30C30C3ull;
	x = (x | (x << 2)) & 0x249249249249ull;
	return x;
}
// spread3 of v < 1024 in 32-bit arithmetic (bit i of v to bit 3i, i < 10).
__device__ __forceinline__ uint32_t spread3_narrow(uint32_t v) {
	uint32_t x = v & 0x3FFu;
	x = (x | (x << 16)) & 0xFF0000FFu;
	x = (x | (x << 8)) & 0x0300F00Fu;
	x = (x | (x << 4)) & 0x030C30C3u;
	x = (x | (x << 2)) & 0x09249249u;
	return x;
}
// spread3 in the code type of a write path: uint32_t (JOB_NARROW) or uint64_t.
template <class C>
__device__ __forceinline__ C spread3_t(uint32_t v) {
	if constexpr (sizeof(C) == 4) return spread3_narrow(v);
	else return spread3(v);
}
__device__ __forceinline__ uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
	return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}

__device__ __forceinline__ uint64_t umin64(uint64_t a, uint64_t b) { return a < b ? a : b; }

// Shared-memory slab of 256 rows (16 z-slices x 16 rows) of `stride` (odd) words: row r starts at
// r * stride + r / 32.  The odd stride spreads consecutive rows over the banks; the skew of one word
// per 32 rows does the same for rows 32 apart, which a Morton gather reads together (a word of a
// 16^3 block touches rows (2Z + dz) * 16 + 4Y + dy).
__host__ __device__ __forceinline__ uint32_t slab_row(uint32_t r, uint32_t stride) { return r * stride + (r >> 5); }
constexpr uint32_t kSlabSkewWords = 256 / 32;  // extra words of a 256-row slab

// Inverse of spread3: the bits at positions 0, 3, 6, ... of v, packed.
__device__ __forceinline__ uint32_t compact3(uint64_t v) {
	v &= 0x249249249249ull;
	v = (v ^ (v >> 2)) & 0x0C30C30C30C3ull;
	v = (v ^ (v >> 4)) & 0x00F00F00F00Full;
	v = (v ^ (v >> 8)) & 0x0000FF0000FFull;
	v = (v ^ (v >> 16)) & 0xFFFFull;
	return (uint32_t)v;
}

// Morton bit mask of a 4-bit row nibble (x = 4X'..4X'+3 in MSB-first order: nibble bit 3 is dx = 0)
// for dy = dz = 0.  In a Morton word the code offset of (dx, dy, dz) is
// (dx&1) | (dy&1)<<1 | dz<<2 | (dx>>1)<<3 | (dy>>1)<<4, and bits are MSB first, so other (dy, dz)
// shift the mask right by 2*(dy&1) + 4*dz + 16*(dy>>1).
__device__ __forceinline__ uint32_t nibble_mask(uint32_t nib) {
	// dx = 0, 1 (nibble bits 3, 2) -> offsets 0, 1 (bits 31, 30); dx = 2, 3 (bits 1, 0) -> offsets 8, 9
	return ((nib & 0xCu) << 28) | ((nib & 0x3u) << 22);
}


// (int)__fdiv_rn(a, u) (truncation of the correctly rounded quotient, as float3_to_int3 of
// `a / unit` in the reference, src/util.h:20-22), computed with the per-axis reciprocal inv ~ 1/u.
// fl(a * inv) is within 2 ulp of fl(a / u); truncation can only differ when the quotient is within
// that distance of an integer, and there the exact division decides.
__device__ __forceinline__ int div_trunc(float a, float u, float inv) {
	const float q = __fmul_rn(a, inv);
	const float t = truncf(q);
	const float room = 4.0f * __fmul_rn(fabsf(q), 1.1920929e-07f) + 1.0e-30f;  // 4 ulp-ish, never 0
	if (fabsf(q) < 8388608.0f && q - t > room && (t + 1.0f) - q > room && fabsf(q) > room)
		return (int)t;
	return __float2int_rz(__fdiv_rn(a, u));
}

// Bit layout (src/voxelize.cu:50-55): word = idx / 32, bit = 31 - idx % 32 (MSB first).
__device__ __forceinline__ uint32_t bit_of(uint64_t idx) { return 0x80000000u >> (uint32_t)(idx & 31u); }

// Mask of bit positions [a, b] (0 <= a <= b <= 31, counted MSB first) within one word.
__device__ __forceinline__ uint32_t span_mask(uint32_t a, uint32_t b) {
	return (0xFFFFFFFFu >> a) & (0xFFFFFFFFu << (31u - b));
}

// OR bits [lo, hi] of the linear bit stream into the table, one atomic per word.
template <class C = uint64_t>
__device__ __forceinline__ void or_span(uint32_t* table, C lo, C hi) {
	C w0 = lo >> 5, w1 = hi >> 5;
	for (C w = w0; w <= w1; w++) {
		uint32_t a = (w == w0) ? (uint32_t)(lo & 31u) : 0u;
		uint32_t b = (w == w1) ? (uint32_t)(hi & 31u) : 31u;
		atomicOr(table + w, span_mask(a, b));
	}
}

// Dilated-integer step of the x bits of a Morton code (x at bit positions 0, 3, 6, ...):
// code(x + d) from code(x) for d = 1 (kMortonX1) or d = 4 (kMortonX4), without re-spreading x.
constexpr uint64_t kMortonXMask = 0x249249249249ull;
constexpr uint64_t kMortonX1 = 1ull, kMortonX4 = 64ull;
__device__ __forceinline__ uint64_t morton_x_add(uint64_t xd, uint64_t step) {
	return ((xd | ~kMortonXMask) + step) & kMortonXMask;
}
// The same in the code type of a write path (the 32-bit mask covers x < 1024).
template <class C>
__device__ __forceinline__ C morton_x_add_t(C xd, C step) {
	if constexpr (sizeof(C) == 4) return ((xd | ~0x09249249u) + step) & 0x09249249u;
	else return morton_x_add(xd, step);
}

// OR the Morton-ordered bits of row (y, z), x in [xl, xh], one atomic per touched word.  Within a
// Morton word (32 consecutive codes) x varies in its two low bits only: codes of x = 4k..4k+3 sit at
// offsets {0, 1, 8, 9} from the code of x = 4k, i.e. MSB-first bits 31, 30, 23, 22 shifted right
// by that code's offset in its word.
template <class C = uint64_t>
__device__ __forceinline__ void or_span_morton(uint32_t* table, int xl, int xh, uint32_t y, uint32_t z) {
	const C yz = (spread3_t<C>(y) << 1) | (spread3_t<C>(z) << 2);
	const int k1 = xh >> 2;
	C xd = spread3_t<C>((uint32_t)(xl & ~3));
	for (int k = xl >> 2; k <= k1; k++) {
		const C code = xd | yz;
		const int j0 = max(xl - (k << 2), 0), j1 = min(xh - (k << 2), 3);
		const uint32_t n = (0xFu << j0) & (0xFu >> (3 - j1));  // x offsets j0..j1 of the group
		const uint32_t m = ((n & 1u) << 31) | ((n & 2u) << 29) | ((n & 4u) << 21) | ((n & 8u) << 19);
		atomicOr(table + (code >> 5), m >> (uint32_t)(code & 31u));
		xd = morton_x_add_t<C>(xd, (C)kMortonX4);
	}
}

// Last job whose range [begin, ...) starts at or before idx, for any monotone per-job begin field.
template <class F>
__device__ __forceinline__ uint32_t job_search(const LaunchDesc& L, uint64_t idx, F begin_of) {
	if (L.n_jobs == 1) return 0;
	uint32_t lo = 0, hi = L.n_jobs - 1;
	while (lo < hi) {
		uint32_t mid = (lo + hi + 1) >> 1;
		if (begin_of(L.jobs[mid]) <= idx) lo = mid; else hi = mid - 1;
	}
	return lo;
}

__device__ __forceinline__ void set_error(const LaunchDesc& L, unsigned code) {
	atomicCAS(&L.scr.ctr->error, 0u, code);
}

}  // namespace cvx
