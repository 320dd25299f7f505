// microbench.cu -- device peak measurements the roofline needs and MEASURED_PEAKS.json lacks:
// the rate of 32-bit global atomicOr into a large table (L2 atomic throughput), for the access
// patterns the voxelizer produces.  Built into its own library, libcvx_diag.so (include/cvx_diag.h),
// apart from the voxelization library; used by bench.py.
//
//   pattern 0: every lane hits a pseudo-random word of the table (scattered, distinct lines)
//   pattern 1: each warp hits 32 consecutive words (one 128-byte line per warp instruction)
//   pattern 2: each lane hits a pseudo-random word, 8 consecutive words per lane (row spans)
#include <cuda_runtime.h>
#include <cstdint>

#include "cvx_diag.h"

namespace {

__device__ __forceinline__ uint32_t mix(uint32_t x) {
	x ^= x >> 16;
	x *= 0x7feb352du;
	x ^= x >> 15;
	x *= 0x846ca68bu;
	x ^= x >> 16;
	return x;
}

__global__ void atomic_or_kernel(uint32_t* table, uint64_t words, uint32_t iters, int pattern) {
	const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
	const uint32_t lane = threadIdx.x & 31u;
	for (uint32_t i = 0; i < iters; i++) {
		const uint32_t h = mix(tid * 0x9E3779B9u + i * 0x85EBCA6Bu);
		if (pattern == 0) {
			atomicOr(table + (h % words), 1u << (h & 31u));
		} else if (pattern == 1) {
			const uint32_t base = mix((tid >> 5) * 0x9E3779B9u + i) % (uint32_t)(words >> 5);
			atomicOr(table + (uint64_t)base * 32 + lane, 1u << (h & 31u));
		} else {
			const uint64_t w = h % (words - 8);
			for (int k = 0; k < 8; k++) atomicOr(table + w + k, 0xFFFFFFFFu >> (h & 31u));
		}
	}
}

}  // namespace

extern "C" {

// Atomics per second of `pattern` into a table of `words` 32-bit words (device memory), measured
// with CUDA events around one launch of `blocks` x 256 threads x `iters` atomics each.
double cvx_microbench_atomic_or(uint32_t* d_table, uint64_t words, int pattern, uint32_t blocks, uint32_t iters) {
	cudaEvent_t a, b;
	cudaEventCreate(&a);
	cudaEventCreate(&b);
	atomic_or_kernel<<<blocks, 256>>>(d_table, words, 1, pattern);  // warm-up
	cudaEventRecord(a);
	atomic_or_kernel<<<blocks, 256>>>(d_table, words, iters, pattern);
	cudaEventRecord(b);
	cudaEventSynchronize(b);
	float ms = 0.0f;
	cudaEventElapsedTime(&ms, a, b);
	cudaEventDestroy(a);
	cudaEventDestroy(b);
	if (cudaGetLastError() != cudaSuccess || ms <= 0.0f) return 0.0;
	const double n = (double)blocks * 256.0 * iters * (pattern == 2 ? 8.0 : 1.0);
	return n / (ms * 1e-3);
}

}  // extern "C"
