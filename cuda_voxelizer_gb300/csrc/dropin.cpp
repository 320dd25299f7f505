// dropin.cpp -- voxelize() / voxelize_solid() with the reference's C++ signatures
// (src/voxelize.cu:192, src/voxelize_solid.cu:147), implemented on the C ABI.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "cvx.h"
#include "cvx_dropin.h"

static_assert(sizeof(voxinfo) == sizeof(cvx_voxinfo), "voxinfo layout");
static_assert(offsetof(voxinfo, gridsize) == offsetof(cvx_voxinfo, gridsize), "voxinfo.gridsize");
static_assert(offsetof(voxinfo, n_triangles) == offsetof(cvx_voxinfo, n_triangles), "voxinfo.n_triangles");
static_assert(offsetof(voxinfo, unit) == offsetof(cvx_voxinfo, unit), "voxinfo.unit");

namespace {

[[noreturn]] void die(const char* what, const char* msg) {
	std::fprintf(stderr, "CUDA error at %s: %s\n", what, msg);
	std::exit(EXIT_FAILURE);
}

void check(cudaError_t e, const char* what) {
	if (e != cudaSuccess) die(what, cudaGetErrorString(e));
}

void run(const voxinfo& v, float* tris, unsigned int* table, bool morton, int solid) {
	cvx_voxinfo info;
	std::memcpy(&info, &v, sizeof(info));
	cudaEvent_t start, stop;
	check(cudaEventCreate(&start), "cudaEventCreate");
	check(cudaEventCreate(&stop), "cudaEventCreate");
	check(cudaEventRecord(start, 0), "cudaEventRecord");
	cvx_status st = solid ? cvx_voxelize_solid(&info, tris, table, morton ? 1 : 0, nullptr)
	                      : cvx_voxelize(&info, tris, table, morton ? 1 : 0, nullptr);
	if (st != CVX_OK) die(solid ? "voxelize_solid" : "voxelize", cvx_last_error_message());
	check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
	check(cudaEventRecord(stop, 0), "cudaEventRecord");
	check(cudaEventSynchronize(stop), "cudaEventSynchronize");
	float ms = 0.0f;
	check(cudaEventElapsedTime(&ms, start, stop), "cudaEventElapsedTime");
	std::printf("[Perf] Voxelization GPU time: %.1f ms\n", ms);
	st = cvx_device_status(nullptr);
	if (st != CVX_OK) die("device check", cvx_last_error_message());
	check(cudaEventDestroy(start), "cudaEventDestroy");
	check(cudaEventDestroy(stop), "cudaEventDestroy");
}

}  // namespace

void voxelize(const voxinfo& v, float* triangle_data, unsigned int* vtable, bool morton_code) {
	run(v, triangle_data, vtable, morton_code, 0);
}

void voxelize_solid(const voxinfo& v, float* triangle_data, unsigned int* vtable, bool morton_code) {
	run(v, triangle_data, vtable, morton_code, 1);
}
