// ref_gpu_runner.cu -- runs the reference's own CUDA kernels.  TEST INFRASTRUCTURE ONLY.
//
// oracle/build_ref.sh compiles the reference's src/voxelize.cu and src/voxelize_solid.cu, from the
// reference tree, into device code for sm_103a (oracle/_ref/ref_voxelize*.cubin).  This runner
// loads those modules with the CUDA driver API and launches the kernels the way the reference's
// host wrappers do (src/voxelize.cu:192-238, src/voxelize_solid.cu:147-193):
//   * block size from the occupancy calculator, grid = ceil(n_triangles / block)  (:208-213);
//     the solid kernel's `return` on near-vertical triangles (src/voxelize_solid.cu:92) needs
//     exactly one triangle per thread, which this grid gives;
//   * the Morton tables morton256_{x,y,z} (src/voxelize.cuh:15-17) filled with the values of
//     src/morton_LUTs.h, which are the 3-way bit spread of the byte index.
// Differences from the reference wrapper, none of which touch the kernels: the launch goes to the
// caller's stream and is not followed by a device synchronize or a printf, and an empty mesh
// launches nothing (the reference would issue an invalid <<<0, bs>>> launch and ignore the error).
//
// The kernels take `voxinfo` by value (src/util.h:50-69: 64 bytes on LP64).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

namespace {

struct RefModule {
	CUmodule mod = nullptr;
	CUfunction fn = nullptr;
	int block = 0;
};

RefModule g_surface, g_solid;
int g_ready = 0;
char g_err[512] = {0};

int fail(const char* what, CUresult r) {
	const char* s = nullptr;
	cuGetErrorString(r, &s);
	std::snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "unknown");
	return -1;
}

void spread_luts(uint32_t lx[256], uint32_t ly[256], uint32_t lz[256]) {
	for (uint32_t v = 0; v < 256; v++) {
		uint32_t s = 0;
		for (int i = 0; i < 8; i++) s |= ((v >> i) & 1u) << (3 * i);
		lx[v] = s;
		ly[v] = s << 1;
		lz[v] = s << 2;
	}
}

int load(RefModule& m, const std::string& path, const char* kernel) {
	CUresult r = cuModuleLoad(&m.mod, path.c_str());
	if (r != CUDA_SUCCESS) return fail(path.c_str(), r);
	r = cuModuleGetFunction(&m.fn, m.mod, kernel);
	if (r != CUDA_SUCCESS) return fail(kernel, r);
	int min_grid = 0;
	r = cuOccupancyMaxPotentialBlockSize(&min_grid, &m.block, m.fn, nullptr, 0, 0);
	if (r != CUDA_SUCCESS) return fail("occupancy", r);
	uint32_t lut[3][256];
	spread_luts(lut[0], lut[1], lut[2]);
	const char* names[3] = {"morton256_x", "morton256_y", "morton256_z"};
	for (int a = 0; a < 3; a++) {
		CUdeviceptr p = 0;
		size_t bytes = 0;
		r = cuModuleGetGlobal(&p, &bytes, m.mod, names[a]);
		if (r != CUDA_SUCCESS || bytes != sizeof(lut[a])) return fail(names[a], r);
		r = cuMemcpyHtoD(p, lut[a], sizeof(lut[a]));
		if (r != CUDA_SUCCESS) return fail("lut upload", r);
	}
	return 0;
}

}  // namespace

extern "C" {

const char* refgpu_last_error() { return g_err; }

// Load both reference modules from `dir` (the oracle/_ref directory) into the current device's
// primary context.  Returns 0 on success.
int refgpu_init(const char* dir) {
	if (g_ready) return 0;
	cudaError_t e = cudaFree(nullptr);  // make the runtime's primary context current
	if (e != cudaSuccess) {
		std::snprintf(g_err, sizeof(g_err), "cudaFree(0): %s", cudaGetErrorString(e));
		return -1;
	}
	std::string d(dir);
	if (load(g_surface, d + "/ref_voxelize.cubin", "_Z17voxelize_triangle7voxinfoPfPjb")) return -1;
	if (load(g_solid, d + "/ref_voxelize_solid.cubin", "_Z23voxelize_triangle_solid7voxinfoPfPjb")) return -1;
	g_ready = 1;
	return 0;
}

// Launch voxelize_triangle (solid == 0) or voxelize_triangle_solid (solid != 0) on `stream`.
int refgpu_voxelize(const void* info64, const float* d_tris, uint32_t* d_table, int morton, int solid, void* stream) {
	if (!g_ready) {
		std::snprintf(g_err, sizeof(g_err), "refgpu_init was not called");
		return -1;
	}
	unsigned char info[64];
	std::memcpy(info, info64, 64);
	uint64_t n = 0;
	std::memcpy(&n, info + 40, 8);
	if (n == 0) return 0;
	RefModule& m = solid ? g_solid : g_surface;
	uint64_t grid = (n + (uint64_t)m.block - 1) / (uint64_t)m.block;
	const float* t = d_tris;
	uint32_t* v = d_table;
	bool mo = morton != 0;
	void* args[4] = {info, &t, &v, &mo};
	CUresult r = cuLaunchKernel(m.fn, (unsigned)grid, 1, 1, (unsigned)m.block, 1, 1, 0, (CUstream)stream, args, nullptr);
	if (r != CUDA_SUCCESS) return fail("cuLaunchKernel", r);
	return 0;
}

int refgpu_block_size(int solid) { return solid ? g_solid.block : g_surface.block; }

// out[i] = rsqrtf(in[i]) evaluated on the device: the 1/|n| factor of the reference kernels'
// normalize() (helper_math.h:1436-1439), for the oracle's GPU-arithmetic mode (ovx_mode.inv_len).
__global__ void rsqrt_kernel(const float* in, float* out, uint64_t n) {
	const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) out[i] = rsqrtf(in[i]);
}

int refgpu_rsqrt(const float* d_in, float* d_out, uint64_t n, void* stream) {
	if (n == 0) return 0;
	const uint64_t blocks = (n + 255) / 256;
	rsqrt_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(d_in, d_out, n);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) {
		std::snprintf(g_err, sizeof(g_err), "rsqrt_kernel: %s", cudaGetErrorString(e));
		return -1;
	}
	return 0;
}

}  // extern "C"
