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

// 32 <= g <= 1024: one CTA per slab of 16 x 16 rows (y block by, z block bz), the whole x extent.
// The slab's voxels are exactly the 16^3 Morton blocks (bx, by, bz) for every bx, each 128
// consecutive Morton words, so both directions read and write contiguous memory: the linear rows
// of the slab (16 contiguous rows per z-slice) and the slab's Morton blocks.

__device__ __forceinline__ uint64_t slab_block(uint32_t bx, uint32_t by, uint32_t bz) {
	return spread3(bx) | (spread3(by) << 1) | (spread3(bz) << 2);
}

// linear -> Morton: rows into shared memory (row stride wpr | 1 words: odd, no bank conflicts
// between the rows a warp reads), then one thread per Morton word of each block.
__global__ void __launch_bounds__(256) linear_to_morton_slab(const uint32_t* __restrict__ lin, uint32_t* __restrict__ mor,
                                                             uint32_t lg) {
	extern __shared__ __align__(16) uint32_t s_rows[];
	const uint32_t g = 1u << lg, wpr = g >> 5, stride = wpr | 1u, nb = g >> 4;
	const uint32_t by = blockIdx.x & (nb - 1u), bz = blockIdx.x >> (lg - 4);
	const uint32_t chunk = 16u * wpr;  // words of the slab in one z-slice (16 contiguous rows)
	for (uint32_t i = threadIdx.x; i < 16u * (chunk / 4u); i += 256) {
		const uint32_t zi = i / (chunk / 4u), q = i % (chunk / 4u);
		const uint4 v = reinterpret_cast<const uint4*>(lin + ((uint64_t)(bz * 16 + zi) * g + by * 16) * wpr)[q];
		const uint32_t vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
		for (int k = 0; k < 4; k++) {
			const uint32_t idx = 4 * q + k;
			s_rows[slab_row(zi * 16 + idx / wpr, stride) + idx % wpr] = vv[k];
		}
	}
	__syncthreads();
	const uint32_t half = threadIdx.x >> 7, m = threadIdx.x & 127u;
	const uint32_t X = compact3(m >> 1), Y = compact3(m >> 2), Z = compact3(m);
	for (uint32_t bx = half; bx < nb; bx += 2) {
		const uint32_t wsel = bx >> 1, xoff = (bx & 1u) * 16u + 4u * X;
		uint32_t out = 0;
#pragma unroll
		for (uint32_t dz = 0; dz < 2; dz++)
#pragma unroll
			for (uint32_t dy = 0; dy < 4; dy++) {
				const uint32_t rw = s_rows[slab_row((2 * Z + dz) * 16 + 4 * Y + dy, stride) + wsel];
				out |= nibble_mask((rw >> (28u - xoff)) & 0xFu) >> (2u * (dy & 1u) + 4u * dz + 16u * (dy >> 1));
			}
		mor[(slab_block(bx, by, bz) << 7) + m] = out;
	}
}

// Morton -> linear: the slab's Morton blocks into shared memory (block stride 129 words), then one
// thread per linear word of the slab's rows, built from two blocks' four x-groups each.
__global__ void __launch_bounds__(256) morton_to_linear_slab(const uint32_t* __restrict__ mor, uint32_t* __restrict__ lin,
                                                             uint32_t lg) {
	extern __shared__ __align__(16) uint32_t s_mor[];
	const uint32_t g = 1u << lg, wpr = g >> 5, nb = g >> 4;
	const uint32_t by = blockIdx.x & (nb - 1u), bz = blockIdx.x >> (lg - 4);
	for (uint32_t i = threadIdx.x; i < nb * 32u; i += 256) {
		const uint32_t bx = i >> 5, q = i & 31u;
		const uint4 v = reinterpret_cast<const uint4*>(mor + (slab_block(bx, by, bz) << 7))[q];
		uint32_t* d = s_mor + bx * 129u + 4u * q;
		d[0] = v.x;
		d[1] = v.y;
		d[2] = v.z;
		d[3] = v.w;
	}
	__syncthreads();
	for (uint32_t i = threadIdx.x; i < 256u * wpr; i += 256) {
		const uint32_t r = i / wpr, w = i % wpr;  // row r = zi * 16 + yi of the slab, word w
		const uint32_t zi = r >> 4, yi = r & 15u;
		const uint32_t Y = yi >> 2, dy = yi & 3u, Z = zi >> 1, dz = zi & 1u;
		const uint32_t sh = 2u * (dy & 1u) + 4u * dz + 16u * (dy >> 1);
		uint32_t out = 0;
#pragma unroll
		for (uint32_t h = 0; h < 2; h++)
#pragma unroll
			for (uint32_t X = 0; X < 4; X++) {
				const uint32_t m = (uint32_t)(spread3(Z) | (spread3(X) << 1) | (spread3(Y) << 2));
				const uint32_t mw = s_mor[(2u * w + h) * 129u + m] << sh;  // (dx) bits now at 31, 30, 23, 22
				const uint32_t nib = ((mw >> 28) & 8u) | ((mw >> 28) & 4u) | ((mw >> 22) & 2u) | ((mw >> 22) & 1u);
				out |= nib << (28u - 16u * h - 4u * X);
			}
		lin[((uint64_t)(bz * 16 + zi) * g + by * 16 + yi) * wpr + w] = out;
	}
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
	const bool aligned = ((reinterpret_cast<uintptr_t>(d_src) | reinterpret_cast<uintptr_t>(d_dst)) & 15u) == 0;
	if (gridsize >= 32 && gridsize <= 1024 && aligned) {
		static bool attr_set[64] = {};
		int dev = 0;
		cudaGetDevice(&dev);
		const uint32_t wpr = gridsize >> 5, nb = gridsize >> 4;
		const size_t smem_l2m = (256u * (wpr | 1u) + kSlabSkewWords) * 4u, smem_m2l = nb * 129u * 4u;
		if (dev >= 0 && dev < 64 && !attr_set[dev]) {
			cudaFuncSetAttribute(linear_to_morton_slab, cudaFuncAttributeMaxDynamicSharedMemorySize,
			                     (256 * 33 + kSlabSkewWords) * 4);
			cudaFuncSetAttribute(morton_to_linear_slab, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 129 * 4);
			attr_set[dev] = true;
		}
		const unsigned slabs = nb * nb;
		if (to_morton) linear_to_morton_slab<<<slabs, 256, smem_l2m, s>>>(d_src, d_dst, lg);
		else morton_to_linear_slab<<<slabs, 256, smem_m2l, s>>>(d_src, d_dst, lg);
	} else if (to_morton) {
		linear_to_morton<<<blocks, 256, 0, s>>>(d_src, d_dst, words, lg);
	} else {
		morton_to_linear<<<blocks, 256, 0, s>>>(d_src, d_dst, words, lg);
	}
	const cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) {
		set_message(std::string("cvx_transcode: ") + cudaGetErrorString(e));
		return CVX_ERR_CUDA;
	}
	return CVX_OK;
}
