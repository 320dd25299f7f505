// surface.cu -- surface voxelization kernels (reference: voxelize_triangle, src/voxelize.cu:58-190).
//
// Two kernels per launch sequence, both over a job table so that one mesh and a batch of meshes
// run through the same code:
//   surf_classify  one CTA per tile of kTile triangles of one job.  The tile is staged into shared
//                  memory with one cp.async.bulk (TMA bulk copy) when it is full and 16-byte
//                  aligned.  Each thread sets up its triangle; triangles whose grid bbox holds at
//                  most `small_vox` voxels (every voxel tested, like the reference) or at most
//                  kLocalRows rows (rows of up to kMaskRowVoxels voxels tested voxel by voxel,
//                  longer rows by row intervals) are finished by the CTA, their rows dealt over
//                  its threads; the others are queued, one record per triangle, as one item
//                  ("mid") or as one item per 32 z-slices ("big").
//   surf_rows      persistent CTAs of kRowsCtaThreads threads, seven per SM; each warp takes
//                  work tickets (big items first, then mid triangles), finds the y-interval of every z-slice of the item (one lane per slice),
//                  flattens the (y, z) rows and gives one row per lane; each lane finds the exact
//                  x-interval of its row and ORs it into the table one word at a time (the whole
//                  warp for long rows).  Jobs whose indices fit 32 bits (JOB_NARROW) write with
//                  32-bit index arithmetic.
#include "engine.h"
#include "surface.cuh"

namespace cvx {

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;

// Bounded wait on an mbarrier phase.  Returns false if the phase did not complete in time.
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

// Exclusive prefix sum over the CTA (kTile threads); returns this thread's offset, total in *total.
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
		if (lane < kTile / 32) s_warp[lane] = w;  // inclusive warp prefix
	}
	__syncthreads();
	*total = s_warp[kTile / 32 - 1];
	return (warp ? s_warp[warp - 1] : 0u) + incl - v;
}

// Phase 1: one thread per triangle: setup, then one of three bins.  Small triangles (a few voxels)
// and local ones (at most kLocalRows rows, extents below 256) park their setup in shared memory;
// the rest are queued for surf_rows.  Phase 2: the rows of the tile's small and local triangles
// are dealt out evenly over the CTA, one (triangle, row) item per thread at a time, so that no
// thread idles while another walks a larger bounding box.  A small triangle's row tests every
// voxel like the reference; a local triangle's row is found with row_interval.
// Registers (48) allow 10 CTAs of 128 threads per SM, shared memory (22.5 KB) 9.
template <class P>
__global__ void __launch_bounds__(kTile, 10) surf_classify(const __grid_constant__ LaunchDesc L, const uint32_t small_vox) {
	__shared__ __align__(16) union {
		float tri[kTile * 9];
		SmallTri small[kTile];
	} sm;
	// per row: small triangle | dy << 8 | dz << 12, or local triangle | row << 8
	__shared__ uint16_t s_items[kTile * kSmallRows];
	__shared__ uint32_t s_warp[kTile / 32];
	__shared__ uint32_t s_fit;  // end of the item list: the first local triangle that did not fit
	__shared__ __align__(8) uint64_t s_bar;
	const uint32_t tile = blockIdx.x;
	const uint32_t j = job_of_tile(L, tile);
	const JobDesc& J = job_at(L, j);
	const float* tris = J.tris;
	uint32_t* table = J.table;
	const uint64_t n = J.n_tri;
	const uint32_t jflags = J.flags;
	const float bmin[3] = {J.bmin[0], J.bmin[1], J.bmin[2]};
	const float unit[3] = {J.unit[0], J.unit[1], J.unit[2]};
	const float inv[3] = {J.inv_unit[0], J.inv_unit[1], J.inv_unit[2]};
	const uint32_t grid[3] = {J.grid[0], J.grid[1], J.grid[2]};
	const uint64_t t0 = (uint64_t)(tile - J.tile_begin) * kTile;
	const uint32_t cnt = (uint32_t)umin64((uint64_t)kTile, n - t0);
	if (!stage_tile(L, tris + t0 * 9, cnt, sm.tri, &s_bar, (jflags & JOB_PLAIN_LOADS) != 0)) return;  // tile not staged: error word set

	const uint32_t lane = threadIdx.x & 31u;
	const bool valid = threadIdx.x < cnt;
	float t[9];
#pragma unroll
	for (int k = 0; k < 9; k++) t[k] = valid ? sm.tri[threadIdx.x * 9 + k] : 0.0f;
	__syncthreads();  // the tile is consumed; its shared memory now holds SmallTri records

	bool is_mid = false, is_big = false;
	uint32_t n_items = 0, n_small = 0, n_local = 0;
	if (valid) {
		SurfTri S;
		surf_setup<P>(t, bmin, unit, inv, grid, S);
		const uint32_t ex = (uint32_t)(S.bx1 - S.bx0), ey = (uint32_t)(S.by1 - S.by0), ez = (uint32_t)(S.bz1 - S.bz0);
		const uint64_t rows = (uint64_t)(ey + 1) * (uint64_t)(ez + 1);
		const uint64_t nvox = (uint64_t)(ex + 1) * rows;
		if (nvox <= small_vox && nvox <= 255 && rows <= kSmallRows && ey < 16 && ez < 16) {
			pack_small(S, sm.small[threadIdx.x]);
			n_small = (uint32_t)rows;
		} else {
			n_items = (ez + kZch) / kZch;
			if (rows <= kLocalRows && ex < 256 && ey < 256 && ez < 256) {
				pack_small(S, sm.small[threadIdx.x]);
				n_local = (uint32_t)rows;
			}
		}
	}
	// One item list for the tile: the rows of the small triangles, then those of the local ones.
	// A local triangle whose rows no longer fit is queued like the larger ones.
	if (threadIdx.x == 0) s_fit = 0xFFFFFFFFu;  // ordered before the atomics by the scan's barriers
	uint32_t totals = 0;
	const uint32_t offs = block_scan(n_small | (n_local << 16), s_warp, &totals);
	const uint32_t total_small = totals & 0xFFFFu;
	const uint32_t loff = total_small + (offs >> 16);
	if (n_local && loff + n_local > kTile * kSmallRows) {
		atomicMin(&s_fit, loff);
		n_local = 0;
	}
	bool is_brick = false;
	if (n_items && !n_local) {
		if (jflags & JOB_BRICKS) {
			is_brick = true;  // rasterized in shared-memory bricks (bricks.cu)
		} else {
			is_mid = n_items == 1;
			is_big = n_items > 1;
		}
	}
	// Queue the other triangles: warp-aggregated appends.
	const uint32_t lt = (1u << lane) - 1u;
	const uint32_t brick_ballot = __ballot_sync(FULL, is_brick);
	if (brick_ballot) {
		uint32_t base = 0;
		const uint32_t leader = __ffs(brick_ballot) - 1;
		if (lane == leader) base = atomicAdd(&L.scr.ctr->bq, (unsigned)__popc(brick_ballot));
		base = __shfl_sync(FULL, base, leader);
		const uint32_t slot = base + __popc(brick_ballot & lt);
		if (is_brick) {
			if (slot < L.scr.cap) L.scr.bq[slot] = MidRec{j, (uint32_t)(t0 + threadIdx.x)};
			else set_error(L, kErrQueueOverflow);
		}
	}
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

	// Phase 2: the rows of the tile's small and local triangles, dealt evenly over the CTA.
	if (n_small) {
		const SmallTri& o = sm.small[threadIdx.x];
		const uint32_t ny = ((o.ext >> 8) & 0xFFu) + 1u, nz = ((o.ext >> 16) & 0xFFu) + 1u;
		uint32_t c = offs & 0xFFFFu;
		for (uint32_t dz = 0; dz < nz; dz++)
			for (uint32_t dy = 0; dy < ny; dy++) s_items[c++] = (uint16_t)(threadIdx.x | (dy << 8) | (dz << 12));
	}
	for (uint32_t r = 0; r < n_local; r++) s_items[loff + r] = (uint16_t)(threadIdx.x | (r << 8));
	__syncthreads();
	const uint32_t total_items = min(total_small + (totals >> 16), s_fit);
	for (uint32_t k = threadIdx.x; k < total_items; k += kTile) {
		const uint32_t it = s_items[k];
		SurfTri S;
		unpack_small(sm.small[it & 0xFFu], S);
		const bool small = k < total_small;
		int y, z;
		if (small) {
			y = S.by0 + (int)((it >> 8) & 0xFu);
			z = S.bz0 + (int)(it >> 12);
		} else {
			// row r of a local triangle: r = dy + dz * ny with r < kLocalRows and ny < 256, so the
			// approximate quotient is more than 1e-3 away from the next integer and truncates exactly
			const uint32_t r = it >> 8, ny = (uint32_t)(S.by1 - S.by0) + 1u;
			const uint32_t dz = (uint32_t)__fdividef((float)r + 0.5f, (float)ny);
			y = S.by0 + (int)(r - dz * ny);
			z = S.bz0 + (int)dz;
		}
		const float py = __fmul_rn(__int2float_rn(y), unit[1]);
		const float pz = __fmul_rn(__int2float_rn(z), unit[2]);
		if (yz_fail_bits<P>(S, py, pz)) continue;
		RowK K;
		row_consts<P>(S, py, pz, K);
		// Rows of at most kMaskRowVoxels voxels test every voxel (a local triangle's short rows too):
		// cheaper than setting up the crossing estimates of an exact interval search.
		if (small || S.bx1 - S.bx0 < (int)kMaskRowVoxels) {
			// src/voxelize.cu:136-183: every voxel of the row (at most 16), as a pass mask
			uint32_t pm = 0;
			for (int i = 0; i <= S.bx1 - S.bx0; i++) pm |= (uint32_t)voxel_pass<P>(S, K, unit[0], S.bx0 + i) << i;
			if (pm) write_row_mask(table, (jflags & JOB_MORTON) != 0, (jflags & JOB_NARROW) != 0, grid, y, z, S.bx0, pm);
		} else {
			RowDirs D;
			row_dirs(S, unit[0], D);
			int xl, xh;
			if (row_interval<P>(S, D, K, unit[0], xl, xh))
				write_row(table, (jflags & JOB_MORTON) != 0, (jflags & JOB_NARROW) != 0, grid, y, z, xl, xh);
		}
	}
}

// 128-thread CTAs at 72 registers: seven per SM (28 warps) instead of three 256-thread CTAs at 80
// registers (24 warps); measured 1% faster on the 256-mesh mix and the 1024^3 soup.
constexpr uint32_t kRowsCtaThreads = 128;

template <class P>
__global__ void __launch_bounds__(kRowsCtaThreads, 7) surf_rows(const __grid_constant__ LaunchDesc L) {
	const uint32_t lane = threadIdx.x & 31u;
	Counters* C = L.scr.ctr;
	// One thread per CTA reads the queue counters (thousands of warps reading one line would
	// serialise on its L2 slice), the CTA shares them through shared memory.
	__shared__ unsigned long long s_bigc;
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
		const bool narrow = (J.flags & JOB_NARROW) != 0;
		uint32_t* table = J.table;
		float tv = lane < 9 ? J.tris[(uint64_t)tri * 9 + lane] : 0.0f;
		float t[9];
#pragma unroll
		for (int k = 0; k < 9; k++) t[k] = __shfl_sync(FULL, tv, k);
		SurfTri S;
		surf_setup<P>(t, J.bmin, unit, J.inv_unit, grid, S);
		RowDirs D;
		row_dirs(S, unit[0], D);

		// y-interval of this lane's z-slice
		const int z0 = S.bz0 + (int)(chunk * kZch);
		const int zl = z0 + (int)lane;
		int ya = 0, yb = -1;
		if (zl <= S.bz1) {
			const float pz = __fmul_rn(__int2float_rn(zl), unit[2]);
			if (!y_interval<P>(S, unit[1], pz, ya, yb)) { ya = 0; yb = -1; }
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
			// slice s = first lane whose inclusive count exceeds k
			int s = 0;
#pragma unroll
			for (int step = 16; step >= 1; step >>= 1) {
				const int v = __shfl_sync(FULL, incl, s + step - 1);
				if (v <= k) s += step;
			}
			s = min(s, 31);
			const int incl_s = __shfl_sync(FULL, incl, s);
			const int cnt_s = __shfl_sync(FULL, cnt, s);
			const int ya_s = __shfl_sync(FULL, ya, s);
			int y = 0, z = 0, xl = 0, xh = -1;
			if (k < R) {
				y = ya_s + (k - (incl_s - cnt_s));
				z = z0 + s;
				const float py = __fmul_rn(__int2float_rn(y), unit[1]);
				const float pz = __fmul_rn(__int2float_rn(z), unit[2]);
				RowK K;
				row_consts<P>(S, py, pz, K);
				if (!row_interval_fast<P>(S, D, K, unit[0], S.bx0, S.bx1, xl, xh)) xh = -1;
			}
			// Short rows are written by their own lane.  Long rows are written by the whole warp, one
			// row at a time with the lanes on consecutive words (linear) or x groups (Morton): a
			// scattered atomic costs an L2 transaction of its own, a warp's atomics on one row
			// share a few lines.
			const bool has = xh >= xl;
			const bool wide = has && (morton ? (xh >> 2) - (xl >> 2) >= 4 : (xh >> 5) - (xl >> 5) >= 2);
			if (has && !wide) write_row(table, morton, narrow, grid, y, z, xl, xh);
			uint32_t todo = __ballot_sync(FULL, wide);
			while (todo) {
				const int src = __ffs(todo) - 1;
				todo &= todo - 1u;
				const int ry = __shfl_sync(FULL, y, src), rz = __shfl_sync(FULL, z, src);
				const int rl = __shfl_sync(FULL, xl, src), rh = __shfl_sync(FULL, xh, src);
				write_row_warp(table, morton, narrow, grid, ry, rz, rl, rh, lane);
			}
		}
	}
}

}  // namespace

// ---- host-side launchers ------------------------------------------------------------------------

template <class P>
static cudaError_t launch_surface_t(const LaunchDesc& L, const Tune& tune, int rows_grid, int raster_grid,
                                    cudaStream_t s, const Prof* prof) {
	if (L.n_tiles == 0) return cudaSuccess;
	if (prof) (*prof)(nullptr, s);
	surf_classify<P><<<L.n_tiles, kTile, 0, s>>>(L, tune.small_vox);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	if (prof) (*prof)("surf_classify", s);
	if (L.n_bricks) {  // with no pair area (pair_cap 0) brick_bin queues every triangle for surf_rows
		e = launch_bricks(L, rows_grid, raster_grid, s, prof);
		if (e != cudaSuccess) return e;
	}
	e = launch_k(surf_rows<P>, (unsigned)rows_grid, kRowsCtaThreads, 0, s, L);
	if (e != cudaSuccess) return e;
	if (prof) (*prof)("surf_rows", s);
	return cudaGetLastError();
}

cudaError_t launch_surface(const LaunchDesc& L, const Tune& tune, int rows_grid, int raster_grid, cudaStream_t s,
                           const Prof* prof) {
	return launch_surface_t<RefFma>(L, tune, rows_grid, raster_grid, s, prof);
}

int surf_rows_blocks_per_sm() {
	int n = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, surf_rows<RefFma>, kRowsCtaThreads, 0);
	return n > 0 ? n : 1;
}

}  // namespace cvx
