/*
 * cvx_dropin.h -- the reference's own C++ entry points, provided by libcvx.so.
 *
 * Forceflow/cuda_voxelizer's caller forward-declares (src/main.cpp:22-24)
 *     void voxelize(const voxinfo& v, float* triangle_data, unsigned int* vtable, bool morton_code);
 *     void voxelize_solid(const voxinfo& v, float* triangle_data, unsigned int* vtable, bool morton_code);
 * with voxinfo from src/util.h:50-69, and links them from src/voxelize.cu:192 and
 * src/voxelize_solid.cu:147.  libcvx.so defines both symbols with the same C++ linkage and the same
 * behaviour, so that caller relinks against this library unchanged:
 *   - launch on the default stream, then cudaDeviceSynchronize (src/voxelize.cu:216-218);
 *   - print "[Perf] Voxelization GPU time: %.1f ms" measured with CUDA events (:215-222);
 *   - on a CUDA error, print it and exit(EXIT_FAILURE), as the reference's checkCudaErrors does
 *     (src/libs/cuda/helper_cuda.h:567-579).  Unlike the reference, an unsupported request
 *     (Morton order on a grid that is not a cubic power of two, which the reference would write
 *     out of bounds for) is also reported this way instead of corrupting memory.
 * New code should prefer the C ABI in cvx.h (asynchronous, status codes, batches).
 *
 * Include this header only where the reference's util.h is not included; it declares a voxinfo
 * with the same layout.
 */
#ifndef CVX_DROPIN_H_
#define CVX_DROPIN_H_

#include <cstddef>
#include <cuda_runtime.h>

#ifndef CVX_HAVE_REFERENCE_VOXINFO
template <typename T>
struct AABox {
	T min;
	T max;
};
struct voxinfo {
	AABox<float3> bbox;
	uint3 gridsize;
	size_t n_triangles;
	float3 unit;
};
#endif

void voxelize(const voxinfo& v, float* triangle_data, unsigned int* vtable, bool morton_code);
void voxelize_solid(const voxinfo& v, float* triangle_data, unsigned int* vtable, bool morton_code);

#endif /* CVX_DROPIN_H_ */
