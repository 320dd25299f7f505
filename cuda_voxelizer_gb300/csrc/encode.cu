// encode.cu -- output encoders on the GPU: the binvox run-length payload and the .vox voxel list.
//
// Reference: write_binvox (src/util_io.cpp:202-246) walks the voxels with x outermost, then z, then
// y, and writes (value, count) byte pairs, a run ending where the value changes or after 255
// voxels; write_vox (src/util_io.cpp:249-285) walks x, then y over [0, gz), then z over [0, gy) and
// hands every set voxel to VoxWriter::AddVoxel as (x, gz - z, y).  Both read the table in linear
// order through checkVoxel (src/util.h:25-38).
//
// Here both start from the same step: the table is re-read in the writer's traversal order into a
// bit stream (a warp-ballot 32 x 32 bit transpose where the grid allows, a per-word gather
// otherwise).  binvox then marks run starts (a bit differs from its predecessor), compacts them
// with a prefix sum, splits runs longer than 255 and emits the pairs; the voxel list compacts the
// set bits.  The prefix sums are a plain three-pass block scan.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "cvx.h"
#include "engine.h"

namespace cvx {
namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr uint32_t kScanThreads = 256, kScanItems = 8, kScanTile = kScanThreads * kScanItems;

// ---- exclusive prefix sum of uint64 counts ------------------------------------------------------

__device__ __forceinline__ uint64_t block_exclusive(uint64_t v, uint64_t* s_warp, uint64_t* total) {
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	uint64_t incl = v;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		const uint64_t u = __shfl_up_sync(FULL, incl, d);
		if (lane >= (uint32_t)d) incl += u;
	}
	if (lane == 31) s_warp[warp] = incl;
	__syncthreads();
	if (warp == 0) {
		uint64_t w = lane < kScanThreads / 32 ? s_warp[lane] : 0ull;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			const uint64_t u = __shfl_up_sync(FULL, w, d);
			if (lane >= (uint32_t)d) w += u;
		}
		if (lane < kScanThreads / 32) s_warp[lane] = w;
	}
	__syncthreads();
	*total = s_warp[kScanThreads / 32 - 1];
	const uint64_t r = (warp ? s_warp[warp - 1] : 0ull) + incl - v;
	__syncthreads();  // s_warp is reused by the caller's next scan
	return r;
}

__global__ void __launch_bounds__(kScanThreads) scan_tiles(const uint64_t* in, uint64_t n, uint64_t* sums) {
	__shared__ uint64_t s_warp[kScanThreads / 32];
	const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
	uint64_t t = 0;
	for (uint32_t i = 0; i < kScanItems; i++)
		if (base + i < n) t += in[base + i];
	uint64_t total;
	block_exclusive(t, s_warp, &total);
	if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_apply(const uint64_t* in, uint64_t n, const uint64_t* offsets,
                                                           uint64_t* out) {
	__shared__ uint64_t s_warp[kScanThreads / 32];
	const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
	uint64_t v[kScanItems], t = 0;
	for (uint32_t i = 0; i < kScanItems; i++) {
		v[i] = base + i < n ? in[base + i] : 0ull;
		t += v[i];
	}
	uint64_t total;
	uint64_t run = block_exclusive(t, s_warp, &total) + (offsets ? offsets[blockIdx.x] : 0ull);
	for (uint32_t i = 0; i < kScanItems; i++) {
		if (base + i < n) out[base + i] = run;
		run += v[i];
	}
}

// out[i] = sum of in[0..i) for i < n, out[n] = the total (out holds n + 1 entries; may alias in).
cudaError_t exclusive_scan(const uint64_t* in, uint64_t n, uint64_t* out, cudaStream_t s) {
	const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
	if (tiles <= 1) {
		uint64_t* sums = nullptr;
		cudaError_t e = cudaMallocAsync((void**)&sums, sizeof(uint64_t), s);
		if (e != cudaSuccess) return e;
		scan_tiles<<<1, kScanThreads, 0, s>>>(in, n, sums);
		scan_apply<<<1, kScanThreads, 0, s>>>(in, n, nullptr, out);
		cudaMemcpyAsync(out + n, sums, sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
		cudaFreeAsync(sums, s);
		return cudaGetLastError();
	}
	uint64_t* sums = nullptr;
	cudaError_t e = cudaMallocAsync((void**)&sums, (tiles + 1) * sizeof(uint64_t), s);
	if (e != cudaSuccess) return e;
	scan_tiles<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, sums);
	e = exclusive_scan(sums, tiles, sums, s);  // in place: tile offsets, total at sums[tiles]
	if (e == cudaSuccess) {
		scan_apply<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, sums, out);
		e = cudaMemcpyAsync(out + n, sums + tiles, sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
	}
	cudaFreeAsync(sums, s);
	return e != cudaSuccess ? e : cudaGetLastError();
}

// ---- the table in a writer's traversal order -------------------------------------------------
// Stream bit o = ((x * A) + a) * B + b for voxel (x, y, z), where (a, b) = (z, y) for binvox
// (A = gz, B = gy) and (y, z) for the voxel list (A = gz, B = gy, y < gz, z < gy on cubic grids).
// `inner_is_y` selects the first.

__device__ __forceinline__ uint32_t voxel_bit(const uint32_t* table, uint64_t idx) {
	return (table[idx >> 5] >> (31u - (uint32_t)(idx & 31u))) & 1u;
}

// General grids: one thread per stream word, 32 gathered bits.
__global__ void __launch_bounds__(256) order_gather(const uint32_t* __restrict__ table, uint32_t* __restrict__ out,
                                                    uint64_t n_bits, uint32_t gx, uint32_t gy, uint32_t gz,
                                                    bool inner_is_y) {
	const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if ((w << 5) >= n_bits) return;
	const uint64_t B = gy, A = gz;  // inner and outer extents of both orders
	uint32_t word = 0;
	for (uint32_t i = 0; i < 32; i++) {
		const uint64_t o = (w << 5) + i;
		if (o >= n_bits) break;
		const uint64_t b = o % B, rest = o / B, a = rest % A, x = rest / A;
		const uint64_t y = inner_is_y ? b : a, z = inner_is_y ? a : b;
		const uint64_t idx = x + y * gx + z * (uint64_t)gx * gy;
		word |= voxel_bit(table, idx) << (31u - i);
	}
	out[w] = word;
}

// gx and the inner extent multiples of 32: a warp transposes a 32 x 32 bit block (32 x values of
// 32 consecutive inner coordinates) with ballots.  Warp id -> (x block, outer a, inner block).
__global__ void __launch_bounds__(256) order_transpose(const uint32_t* __restrict__ table, uint32_t* __restrict__ out,
                                                       uint32_t gx, uint32_t gy, uint32_t gz, bool inner_is_y) {
	const uint64_t warp_id = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t nxb = gx >> 5;
	const uint32_t B = gy, A = gz;  // inner extent, outer extent
	const uint32_t nib = B >> 5;
	const uint64_t n_warps = (uint64_t)nxb * A * nib;
	if (warp_id >= n_warps) return;
	const uint32_t ib = (uint32_t)(warp_id % nib);
	const uint64_t r = warp_id / nib;
	const uint32_t a = (uint32_t)(r % A), xb = (uint32_t)(r / A);
	const uint32_t inner = (ib << 5) + lane;
	const uint64_t y = inner_is_y ? inner : a, z = inner_is_y ? a : inner;
	const uint32_t w = table[((y * gx + z * (uint64_t)gx * gy) >> 5) + xb];
	uint32_t mine = 0;
#pragma unroll
	for (uint32_t k = 0; k < 32; k++) {
		const uint32_t b = __ballot_sync(FULL, (w >> (31u - k)) & 1u);
		if (lane == k) mine = __brev(b);
	}
	const uint64_t x = ((uint64_t)xb << 5) + lane;
	out[(x * A + a) * nib + ib] = mine;
}

cudaError_t traversal_stream(const cvx_voxinfo& v, const uint32_t* table, uint32_t* stream_words, bool inner_is_y,
                             cudaStream_t s) {
	const uint32_t gx = v.gridsize[0], gy = v.gridsize[1], gz = v.gridsize[2];
	const uint64_t n_bits = (uint64_t)gx * gy * gz;
	if (gx % 32 == 0 && gy % 32 == 0) {
		const uint64_t warps = (uint64_t)(gx >> 5) * gz * (gy >> 5);
		order_transpose<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(table, stream_words, gx, gy, gz, inner_is_y);
	} else {
		const uint64_t words = (n_bits + 31) / 32;
		order_gather<<<(unsigned)((words + 255) / 256), 256, 0, s>>>(table, stream_words, n_bits, gx, gy, gz, inner_is_y);
	}
	return cudaGetLastError();
}

// ---- binvox runs ---------------------------------------------------------------------------------

// Run starts: bit i of the stream starts a run if it differs from bit i - 1 (bit 0 always does).
__global__ void __launch_bounds__(256) run_starts(const uint32_t* __restrict__ st, uint64_t n_bits, uint32_t* diff,
                                                  uint64_t* counts) {
	const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
	const uint64_t words = (n_bits + 31) / 32;
	if (w >= words) return;
	const uint32_t cur = st[w];
	const uint32_t prev = w ? (st[w - 1] & 1u) : (~cur >> 31);  // bit 0: compare with its complement
	uint32_t d = cur ^ ((cur >> 1) | (prev << 31));
	const uint64_t valid = n_bits - (w << 5);
	if (valid < 32) d &= ~0u << (32 - valid);
	diff[w] = d;
	counts[w] = __popc(d);
}

__global__ void __launch_bounds__(256) run_positions(const uint32_t* __restrict__ diff, const uint64_t* __restrict__ roff,
                                                     uint64_t words, uint64_t* starts) {
	const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (w >= words) return;
	uint32_t d = diff[w];
	uint64_t r = roff[w];
	while (d) {
		const uint32_t i = __clz(d);  // MSB-first offset
		starts[r++] = (w << 5) + i;
		d &= ~(0x80000000u >> i);
	}
}

__global__ void __launch_bounds__(256) run_pieces(const uint64_t* __restrict__ starts, uint64_t n_runs, uint64_t n_bits,
                                                  uint64_t* pieces) {
	const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= n_runs) return;
	const uint64_t len = (r + 1 < n_runs ? starts[r + 1] : n_bits) - starts[r];
	pieces[r] = (len + 254) / 255;
}

__global__ void __launch_bounds__(256) run_emit(const uint32_t* __restrict__ st, const uint64_t* __restrict__ starts,
                                                const uint64_t* __restrict__ poff, uint64_t n_runs, uint64_t n_bits,
                                                uint8_t* out) {
	const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= n_runs) return;
	const uint64_t s0 = starts[r];
	const uint64_t len = (r + 1 < n_runs ? starts[r + 1] : n_bits) - s0;
	const uint8_t value = (uint8_t)((st[s0 >> 5] >> (31u - (uint32_t)(s0 & 31u))) & 1u);
	uint64_t p = poff[r];
	for (uint64_t done = 0; done < len; done += 255, p++) {
		const uint64_t c = len - done < 255 ? len - done : 255;
		out[2 * p] = value;
		out[2 * p + 1] = (uint8_t)c;
	}
}

// ---- voxel list ----------------------------------------------------------------------------------

__global__ void __launch_bounds__(256) bit_counts(const uint32_t* __restrict__ st, uint64_t words, uint64_t* counts) {
	const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (w < words) counts[w] = __popc(st[w]);
}

__global__ void __launch_bounds__(256) voxel_emit(const uint32_t* __restrict__ st, const uint64_t* __restrict__ off,
                                                  uint64_t words, uint32_t gy, uint32_t gz, int32_t* xyz) {
	const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (w >= words) return;
	uint32_t d = st[w];
	uint64_t k = off[w];
	while (d) {
		const uint32_t i = __clz(d);
		d &= ~(0x80000000u >> i);
		const uint64_t o = (w << 5) + i;
		const uint64_t z = o % gy, rest = o / gy, y = rest % gz, x = rest / gz;
		xyz[3 * k] = (int32_t)x;                    // AddVoxel(x, -z + gz, y)
		xyz[3 * k + 1] = (int32_t)gz - (int32_t)z;
		xyz[3 * k + 2] = (int32_t)y;
		k++;
	}
}

struct DevBuf {
	void* p = nullptr;
	cudaStream_t s;
	explicit DevBuf(cudaStream_t st) : s(st) {}
	cudaError_t alloc(size_t bytes) { return cudaMallocAsync(&p, bytes ? bytes : 16, s); }
	~DevBuf() {
		if (p) cudaFreeAsync(p, s);
	}
	template <class T> T* as() const { return static_cast<T*>(p); }
};

cvx_status cuda_status(cudaError_t e, const char* what) {
	if (e == cudaSuccess) return CVX_OK;
	set_message(std::string(what) + ": " + cudaGetErrorString(e));
	return CVX_ERR_CUDA;
}

cvx_status check_info(const cvx_voxinfo* info, const void* table, const char* fn) {
	if (!info || !table) {
		set_message(std::string(fn) + ": null argument");
		return CVX_ERR_INVALID_VALUE;
	}
	for (int i = 0; i < 3; i++)
		if (info->gridsize[i] == 0) {
			set_message(std::string(fn) + ": gridsize has a zero dimension");
			return CVX_ERR_INVALID_VALUE;
		}
	return CVX_OK;
}

#define CVX_TRY(expr, what)                                           \
	do {                                                              \
		const cvx_status st_ = cuda_status((expr), (what));           \
		if (st_ != CVX_OK) return st_;                                \
	} while (0)

}  // namespace
}  // namespace cvx

using namespace cvx;

extern "C" {

cvx_status cvx_encode_binvox(const cvx_voxinfo* info, const uint32_t* d_table, uint8_t* d_out, uint64_t out_capacity,
                             uint64_t* out_bytes, cvx_stream_t stream) {
	cvx_status st = check_info(info, d_table, "cvx_encode_binvox");
	if (st != CVX_OK) return st;
	if (!out_bytes) {
		set_message("cvx_encode_binvox: out_bytes is null");
		return CVX_ERR_INVALID_VALUE;
	}
	cudaStream_t s = (cudaStream_t)stream;
	const uint64_t n_bits = (uint64_t)info->gridsize[0] * info->gridsize[1] * info->gridsize[2];
	const uint64_t words = (n_bits + 31) / 32;
	const unsigned wb = (unsigned)((words + 255) / 256);
	DevBuf sbits(s), diff(s), counts(s);
	CVX_TRY(sbits.alloc(words * 4), "cudaMallocAsync");
	CVX_TRY(diff.alloc(words * 4), "cudaMallocAsync");
	CVX_TRY(counts.alloc((words + 1) * 8), "cudaMallocAsync");
	CVX_TRY(traversal_stream(*info, d_table, sbits.as<uint32_t>(), true, s), "binvox order");
	run_starts<<<wb, 256, 0, s>>>(sbits.as<uint32_t>(), n_bits, diff.as<uint32_t>(), counts.as<uint64_t>());
	CVX_TRY(cudaGetLastError(), "run_starts");
	CVX_TRY(exclusive_scan(counts.as<uint64_t>(), words, counts.as<uint64_t>(), s), "scan");
	uint64_t n_runs = 0;
	CVX_TRY(cudaMemcpyAsync(&n_runs, counts.as<uint64_t>() + words, 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
	CVX_TRY(cudaStreamSynchronize(s), "cudaStreamSynchronize");
	DevBuf starts(s), pieces(s);
	CVX_TRY(starts.alloc(n_runs * 8), "cudaMallocAsync");
	CVX_TRY(pieces.alloc((n_runs + 1) * 8), "cudaMallocAsync");
	run_positions<<<wb, 256, 0, s>>>(diff.as<uint32_t>(), counts.as<uint64_t>(), words, starts.as<uint64_t>());
	const unsigned rb = (unsigned)((n_runs + 255) / 256);
	run_pieces<<<rb, 256, 0, s>>>(starts.as<uint64_t>(), n_runs, n_bits, pieces.as<uint64_t>());
	CVX_TRY(cudaGetLastError(), "run_pieces");
	CVX_TRY(exclusive_scan(pieces.as<uint64_t>(), n_runs, pieces.as<uint64_t>(), s), "scan");
	uint64_t n_pairs = 0;
	CVX_TRY(cudaMemcpyAsync(&n_pairs, pieces.as<uint64_t>() + n_runs, 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
	CVX_TRY(cudaStreamSynchronize(s), "cudaStreamSynchronize");
	*out_bytes = 2 * n_pairs;
	if (!d_out) return CVX_OK;  // size query
	if (out_capacity < 2 * n_pairs) {
		set_message("cvx_encode_binvox: output buffer too small (see out_bytes)");
		return CVX_ERR_INVALID_VALUE;
	}
	run_emit<<<rb, 256, 0, s>>>(sbits.as<uint32_t>(), starts.as<uint64_t>(), pieces.as<uint64_t>(), n_runs, n_bits, d_out);
	CVX_TRY(cudaGetLastError(), "run_emit");
	CVX_TRY(cudaStreamSynchronize(s), "cudaStreamSynchronize");
	return CVX_OK;
}

cvx_status cvx_encode_voxel_list(const cvx_voxinfo* info, const uint32_t* d_table, int32_t* d_xyz, uint64_t capacity,
                                 uint64_t* out_count, cvx_stream_t stream) {
	cvx_status st = check_info(info, d_table, "cvx_encode_voxel_list");
	if (st != CVX_OK) return st;
	if (!out_count) {
		set_message("cvx_encode_voxel_list: out_count is null");
		return CVX_ERR_INVALID_VALUE;
	}
	if (info->gridsize[1] != info->gridsize[2]) {
		// the reference's loops run y to gz and z to gy through checkVoxel's (x, y, z): only
		// grids with gy == gz stay inside the table
		set_message("cvx_encode_voxel_list: needs gridsize y == z");
		return CVX_ERR_UNSUPPORTED;
	}
	cudaStream_t s = (cudaStream_t)stream;
	const uint64_t n_bits = (uint64_t)info->gridsize[0] * info->gridsize[1] * info->gridsize[2];
	const uint64_t words = (n_bits + 31) / 32;
	const unsigned wb = (unsigned)((words + 255) / 256);
	DevBuf sbits(s), counts(s);
	CVX_TRY(sbits.alloc(words * 4), "cudaMallocAsync");
	CVX_TRY(counts.alloc((words + 1) * 8), "cudaMallocAsync");
	CVX_TRY(traversal_stream(*info, d_table, sbits.as<uint32_t>(), false, s), "vox order");
	bit_counts<<<wb, 256, 0, s>>>(sbits.as<uint32_t>(), words, counts.as<uint64_t>());
	CVX_TRY(cudaGetLastError(), "bit_counts");
	CVX_TRY(exclusive_scan(counts.as<uint64_t>(), words, counts.as<uint64_t>(), s), "scan");
	uint64_t n = 0;
	CVX_TRY(cudaMemcpyAsync(&n, counts.as<uint64_t>() + words, 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
	CVX_TRY(cudaStreamSynchronize(s), "cudaStreamSynchronize");
	*out_count = n;
	if (!d_xyz) return CVX_OK;
	if (capacity < n) {
		set_message("cvx_encode_voxel_list: output buffer too small (see out_count)");
		return CVX_ERR_INVALID_VALUE;
	}
	voxel_emit<<<wb, 256, 0, s>>>(sbits.as<uint32_t>(), counts.as<uint64_t>(), words, info->gridsize[1],
	                               info->gridsize[2], d_xyz);
	CVX_TRY(cudaGetLastError(), "voxel_emit");
	CVX_TRY(cudaStreamSynchronize(s), "cudaStreamSynchronize");
	return CVX_OK;
}

}  // extern "C"
