// transcode.cu -- Morton <-> linear conversion of a bit table (cubic power-of-two grids).
//
// The reference's writers read tables in linear order only (checkVoxel, src/util.h:25-38), and a
// Morton table (src/voxelize.cuh:20-34, bits MSB-first like the linear one) is written out raw
// (src/util_io.cpp:192-200).  These kernels let any caller move between the two layouts on the
// GPU.  A Morton word holds the codes 32m..32m+31: a 4 x 4 x 2 block of voxels (x and y in their two
// low bits, z in its low bit), i.e. eight 4-bit x-runs of eight linear rows.
#include <cuda_runtime.h>

#include "cvx.h"
#include "engine.h"

namespace cvx {
namespace {

// One thread per Morton word: gather the block's eight row nibbles from the linear table.
__global__ void __launch_bounds__(256) linear_to_morton(const uint32_t* __restrict__ lin, uint32_t* __restrict__ mor,
                                                        uint64_t words, uint32_t lg) {
	const uint64_t m = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (m >= words) return;
	const uint64_t code = m << 5;
	const uint64_t x0 = compact3(code), y0 = compact3(code >> 1), z0 = compact3(code >> 2);
	uint32_t out = 0;
#pragma unroll
	for (uint32_t dz = 0; dz < 2; dz++)
#pragma unroll
		for (uint32_t dy = 0; dy < 4; dy++) {
			const uint64_t bit = x0 + ((y0 + dy) << lg) + ((z0 + dz) << (2 * lg));
			const uint32_t nib = (lin[bit >> 5] >> (28u - (uint32_t)(bit & 31u))) & 0xFu;
			out |= nibble_mask(nib) >> (2u * (dy & 1u) + 4u * dz + 16u * (dy >> 1));
		}
	mor[m] = out;
}

// One thread per linear word: 32 voxels of one row, eight 4-voxel groups from eight Morton words.
__global__ void __launch_bounds__(256) morton_to_linear(const uint32_t* __restrict__ mor, uint32_t* __restrict__ lin,
                                                        uint64_t words, uint32_t lg) {
	const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (w >= words) return;
	const uint64_t bit = w << 5;
	const uint64_t g = 1ull << lg;
	const uint32_t x0 = (uint32_t)(bit & (g - 1)), y = (uint32_t)((bit >> lg) & (g - 1)), z = (uint32_t)(bit >> (2 * lg));
	const uint64_t yz = (spread3(y) << 1) | (spread3(z) << 2);
	uint32_t out = 0;
	const uint32_t groups = g < 32 ? (uint32_t)(g / 4) : 8u;  // g = 4, 8, 16: several rows per word
	for (uint32_t q = 0; q < 8; q++) {
		// voxel run q of this word: bits 4q..4q+3 (MSB first) are x = x0 + 4q' .. of row (y', z')
		const uint64_t b = bit + 4 * q;
		uint32_t xq, yq = y, zq = z;
		uint64_t yzq = yz;
		if (groups == 8) {
			xq = x0 + 4 * q;
		} else {
			xq = (uint32_t)(b & (g - 1));
			yq = (uint32_t)((b >> lg) & (g - 1));
			zq = (uint32_t)(b >> (2 * lg));
			yzq = (spread3(yq) << 1) | (spread3(zq) << 2);
		}
		const uint64_t code = spread3(xq) | yzq;
		const uint32_t word = mor[code >> 5], off = (uint32_t)(code & 31u);
		const uint32_t nib = (((word >> (31u - off)) & 1u) << 3) | (((word >> (30u - off)) & 1u) << 2) |
		                     (((word >> (23u - off)) & 1u) << 1) | ((word >> (22u - off)) & 1u);
		out |= nib << (28u - 4u * q);
	}
	lin[w] = out;
}

}  // namespace
}  // namespace cvx

using namespace cvx;

extern "C" cvx_status cvx_transcode(const uint32_t* d_src, uint32_t* d_dst, uint32_t gridsize, int to_morton,
                                    cvx_stream_t stream) {
	if (!d_src || !d_dst) {
		set_message("cvx_transcode: null argument");
		return CVX_ERR_INVALID_VALUE;
	}
	if (d_src == d_dst) {
		set_message("cvx_transcode: source and destination must not overlap");
		return CVX_ERR_INVALID_VALUE;
	}
	if (gridsize < 4 || (gridsize & (gridsize - 1)) || gridsize > (1u << 16)) {
		set_message("cvx_transcode: needs a cubic power-of-two grid between 4 and 65536");
		return CVX_ERR_UNSUPPORTED;
	}
	const uint32_t lg = 31u - (uint32_t)__builtin_clz(gridsize);
	const uint64_t words = ((uint64_t)gridsize * gridsize * gridsize) >> 5;
	const unsigned blocks = (unsigned)((words + 255) / 256);
	cudaStream_t s = (cudaStream_t)stream;
	if (to_morton) linear_to_morton<<<blocks, 256, 0, s>>>(d_src, d_dst, words, lg);
	else morton_to_linear<<<blocks, 256, 0, s>>>(d_src, d_dst, words, lg);
	const cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) {
		set_message(std::string("cvx_transcode: ") + cudaGetErrorString(e));
		return CVX_ERR_CUDA;
	}
	return CVX_OK;
}
