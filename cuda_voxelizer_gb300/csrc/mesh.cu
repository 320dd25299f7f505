// mesh.cu -- mesh ingest on the GPU: the vertex bounding box of a triangle soup and the expansion
// of an indexed mesh into the soup the voxelizer reads.
//
// Reference: src/main.cpp:61-80 (meshToGPU_managed: a host loop copying each face's three vertices
// into managed memory, 9 floats per triangle) and src/main.cpp:179 (Trimesh need_bbox: min/max over
// the vertices), followed by createMeshBBCube and the voxinfo constructor (src/main.cpp:180-186).
// Min and max are exact, so the device box equals the host one for finite coordinates.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

#include "cvx.h"
#include "engine.h"

namespace cvx {
namespace {

constexpr uint32_t kReduceThreads = 256;

// Order-preserving map of a float to an unsigned key (finite values and infinities).
__device__ __forceinline__ uint32_t order_key(float f) {
	const uint32_t b = __float_as_uint(f);
	return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// out[0..2] = min keys, out[3..5] = max keys; initialised to 0xFFFFFFFF / 0 by the host.
__global__ void __launch_bounds__(kReduceThreads) bbox_reduce(const float* __restrict__ tris, uint64_t n_vertices,
                                                              uint32_t* out) {
	float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n_vertices; v += stride) {
#pragma unroll
		for (int k = 0; k < 3; k++) {
			const float c = tris[3 * v + k];
			lo[k] = fminf(lo[k], c);
			hi[k] = fmaxf(hi[k], c);
		}
	}
#pragma unroll
	for (int k = 0; k < 3; k++) {
#pragma unroll
		for (int d = 16; d >= 1; d >>= 1) {
			lo[k] = fminf(lo[k], __shfl_xor_sync(0xFFFFFFFFu, lo[k], d));
			hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xFFFFFFFFu, hi[k], d));
		}
	}
	__shared__ float s_lo[3][kReduceThreads / 32], s_hi[3][kReduceThreads / 32];
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	if (lane == 0)
		for (int k = 0; k < 3; k++) {
			s_lo[k][warp] = lo[k];
			s_hi[k][warp] = hi[k];
		}
	__syncthreads();
	if (threadIdx.x < 3) {
		const int k = threadIdx.x;
		float a = INFINITY, b = -INFINITY;
		for (uint32_t w = 0; w < kReduceThreads / 32; w++) {
			a = fminf(a, s_lo[k][w]);
			b = fmaxf(b, s_hi[k][w]);
		}
		atomicMin(out + k, order_key(a));
		atomicMax(out + 3 + k, order_key(b));
	}
}

// One thread per face: three vertex indices -> 9 floats.  A face with an index out of range
// becomes a NaN triangle and is counted in *bad (the caller must not voxelize such a soup).
__global__ void __launch_bounds__(256) gather_faces(const float* __restrict__ verts, uint64_t n_verts,
                                                    const uint32_t* __restrict__ faces, uint64_t n_faces,
                                                    float* __restrict__ soup, unsigned long long* bad) {
	const uint64_t f = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (f >= n_faces) return;
	const uint32_t i0 = faces[3 * f], i1 = faces[3 * f + 1], i2 = faces[3 * f + 2];
	float* o = soup + 9 * f;
	if (i0 >= n_verts || i1 >= n_verts || i2 >= n_verts) {
		for (int k = 0; k < 9; k++) o[k] = __int_as_float(0x7FC00000);
		if (bad) atomicAdd(bad, 1ull);
		return;
	}
	const uint32_t idx[3] = {i0, i1, i2};
#pragma unroll
	for (int c = 0; c < 3; c++)
#pragma unroll
		for (int k = 0; k < 3; k++) o[3 * c + k] = verts[3 * (uint64_t)idx[c] + k];
}

float key_to_float(uint32_t k) {
	const uint32_t b = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
	float f;
	std::memcpy(&f, &b, 4);
	return f;
}

cvx_status cuda_status(cudaError_t e, const char* what) {
	if (e == cudaSuccess) return CVX_OK;
	set_message(std::string(what) + ": " + cudaGetErrorString(e));
	return CVX_ERR_CUDA;
}

}  // namespace
}  // namespace cvx

using namespace cvx;

extern "C" {

cvx_status cvx_mesh_bbox_device(const float* d_triangles, uint64_t n_triangles, float out_min[3], float out_max[3],
                                cvx_stream_t stream) {
	if (!d_triangles || !out_min || !out_max) {
		set_message("cvx_mesh_bbox_device: null argument");
		return CVX_ERR_INVALID_VALUE;
	}
	if (n_triangles == 0) {
		set_message("cvx_mesh_bbox_device: empty mesh has no bounding box");
		return CVX_ERR_INVALID_VALUE;
	}
	cudaStream_t s = (cudaStream_t)stream;
	uint32_t* d_out = nullptr;
	cvx_status st = cuda_status(cudaMallocAsync((void**)&d_out, 6 * sizeof(uint32_t), s), "cudaMallocAsync");
	if (st != CVX_OK) return st;
	const uint32_t init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
	uint32_t keys[6];
	int dev = 0, sms = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	const uint64_t nv = 3 * n_triangles;
	const uint64_t want = (nv + kReduceThreads * 8 - 1) / (kReduceThreads * 8);
	const uint32_t blocks = (uint32_t)(want < (uint64_t)sms * 8 ? (want ? want : 1) : (uint64_t)sms * 8);
	if ((st = cuda_status(cudaMemcpyAsync(d_out, init, sizeof(init), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync")) ==
	    CVX_OK) {
		bbox_reduce<<<blocks, kReduceThreads, 0, s>>>(d_triangles, nv, d_out);
		st = cuda_status(cudaGetLastError(), "bbox_reduce");
	}
	if (st == CVX_OK)
		st = cuda_status(cudaMemcpyAsync(keys, d_out, sizeof(keys), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
	cudaFreeAsync(d_out, s);
	if (st == CVX_OK) st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize");
	if (st != CVX_OK) return st;
	for (int k = 0; k < 3; k++) {
		out_min[k] = key_to_float(keys[k]);
		out_max[k] = key_to_float(keys[3 + k]);
	}
	return CVX_OK;
}

cvx_status cvx_voxinfo_from_device(const float* d_triangles, uint64_t n_triangles, const uint32_t gridsize[3],
                                   cvx_voxinfo* out, cvx_stream_t stream) {
	if (!gridsize || !out) {
		set_message("cvx_voxinfo_from_device: null argument");
		return CVX_ERR_INVALID_VALUE;
	}
	float lo[3], hi[3], clo[3], chi[3];
	cvx_status st = cvx_mesh_bbox_device(d_triangles, n_triangles, lo, hi, stream);
	if (st != CVX_OK) return st;
	if ((st = cvx_bbox_cube(lo, hi, clo, chi)) != CVX_OK) return st;
	return cvx_voxinfo_init(out, clo, chi, gridsize, n_triangles);
}

cvx_status cvx_gather_soup(const float* d_vertices, uint64_t n_vertices, const uint32_t* d_faces, uint64_t n_faces,
                           float* d_soup, unsigned long long* d_bad_faces, cvx_stream_t stream) {
	if ((n_faces && (!d_faces || !d_soup)) || (n_vertices && !d_vertices)) {
		set_message("cvx_gather_soup: null argument");
		return CVX_ERR_INVALID_VALUE;
	}
	if (n_faces == 0) return CVX_OK;
	cudaStream_t s = (cudaStream_t)stream;
	gather_faces<<<(unsigned)((n_faces + 255) / 256), 256, 0, s>>>(d_vertices, n_vertices, d_faces, n_faces, d_soup,
	                                                              d_bad_faces);
	return cuda_status(cudaGetLastError(), "gather_faces");
}

}  // extern "C"
