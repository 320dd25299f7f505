// clear.cu -- zero many tables of different sizes with one launch.
//
// A batch of meshes needs every table zeroed before the kernels OR / XOR into it.  One
// cudaMemset per table costs a graph node or an API call each and runs the small tables at launch
// latency; this kernel clears a list of ranges in fixed chunks, one CTA per chunk, with 16-byte
// stores where the range allows them.
#include "engine.h"

namespace cvx {

namespace {

constexpr uint32_t kClearThreads = 256;

__global__ void __launch_bounds__(kClearThreads) clear_ranges(const ClearRange* __restrict__ r, uint32_t n) {
	// range of this chunk: the last one whose chunk_begin <= blockIdx.x
	uint32_t lo = 0, hi = n - 1;
	while (lo < hi) {
		const uint32_t m = (lo + hi + 1) >> 1;
		if (r[m].chunk_begin <= blockIdx.x) lo = m; else hi = m - 1;
	}
	const ClearRange c = r[lo];
	const uint64_t w0 = (uint64_t)(blockIdx.x - c.chunk_begin) * kClearChunkWords;
	if (w0 >= c.words) return;
	const uint64_t w1 = umin64(c.words, w0 + kClearChunkWords);
	uint32_t* p = c.ptr;
	if ((reinterpret_cast<uintptr_t>(p) & 15u) == 0) {
		const uint64_t v0 = w0 / 4, v1 = w1 / 4;  // w0 is a multiple of 4
		uint4* q = reinterpret_cast<uint4*>(p);
		for (uint64_t i = v0 + threadIdx.x; i < v1; i += kClearThreads) q[i] = make_uint4(0u, 0u, 0u, 0u);
		for (uint64_t i = v1 * 4 + threadIdx.x; i < w1; i += kClearThreads) p[i] = 0u;
	} else {
		for (uint64_t i = w0 + threadIdx.x; i < w1; i += kClearThreads) p[i] = 0u;
	}
}

}  // namespace

uint32_t clear_chunks(uint64_t words) { return (uint32_t)((words + kClearChunkWords - 1) / kClearChunkWords); }

cudaError_t launch_clear(const ClearRange* d_ranges, uint32_t n, uint32_t total_chunks, cudaStream_t s) {
	if (n == 0 || total_chunks == 0) return cudaSuccess;
	clear_ranges<<<total_chunks, kClearThreads, 0, s>>>(d_ranges, n);
	return cudaGetLastError();
}

}  // namespace cvx
