// noalloc.cu -- solid voxelization that allocates nothing.
//
// Who needs this: callers that must not allocate device memory at voxelization time.  Examples are
// real-time code that budgets all GPU memory once at start-up (a cudaMalloc in the middle of a
// frame can stall the whole device and can fail under memory pressure), and host processes whose
// memory policy forbids driver allocations outside their own allocator.  cvx_voxelize_solid
// allocates its scratch on first use and cvx_voxelize_ws needs the caller to provide some; this
// entry point needs neither: its scratch is a fixed array compiled into the library.
//
// The scratch below is a file-scope __device__ array of kNoallocScratchBytes (4 MiB + 256 B).  Every
// GPU that loads libcvx.so holds one copy of it until the process exits.  It bounds the grid:
// at most kNoallocMaxVoxels voxels (2^24, e.g. 256^3); meshes of any triangle count are processed
// in slices of kNoallocMaxTriangles triangles.
//
// Host code must not use the array's name as a device address (on the host it only names a
// stand-in): the first call on each device looks up the real address with cudaGetSymbolAddress,
// with that device current, and caches it.  That first call should therefore come before any
// stream capture.  Every call shares the one array: calls that overlap on the GPU (two streams, or
// two host threads) race on it and corrupt each other's results; issue them one after another.
// Each call clears the parts that must start at zero (counters, the flip table of its grid).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>

#include "cvx.h"
#include "engine.h"

namespace cvx {
namespace {

constexpr uint64_t kNoallocMaxVoxels = 1ull << 24;               // flip table: 2 MiB
constexpr uint64_t kNoallocMaxTriangles = 1ull << 16;            // queue: 65,536 triangles per slice
constexpr size_t kNoallocFlipBytes = kNoallocMaxVoxels / 8;
constexpr size_t kNoallocBigOff = 256;                           // counters live in the first 256 bytes
constexpr size_t kNoallocMidOff = kNoallocBigOff + kNoallocMaxTriangles * sizeof(BigRec);
constexpr size_t kNoallocFlipOff = kNoallocMidOff + kNoallocMaxTriangles * sizeof(MidRec);
constexpr size_t kNoallocScratchBytes = kNoallocFlipOff + kNoallocFlipBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};
int g_cols_grid[kMaxDevices] = {};

// Device address of the scratch array for the current device (looked up once per device).
cvx_status scratch_address(int dev, void** out, int* cols_grid) {
	std::lock_guard<std::mutex> lk(g_mu);
	if (!g_addr[dev]) {
		void* p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e != cudaSuccess || p == nullptr) {
			set_message(std::string("cudaGetSymbolAddress(noalloc scratch): ") + cudaGetErrorString(e));
			return CVX_ERR_CUDA;
		}
		int sms = 0;
		e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		if (e != cudaSuccess) {
			set_message(std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
			return CVX_ERR_CUDA;
		}
		g_cols_grid[dev] = sms * solid_cols_blocks_per_sm();
		g_addr[dev] = p;
	}
	*out = g_addr[dev];
	*cols_grid = g_cols_grid[dev];
	return CVX_OK;
}

cvx_status cuda_status(cudaError_t e, const char* what) {
	if (e == cudaSuccess) return CVX_OK;
	set_message(std::string(what) + ": " + cudaGetErrorString(e));
	return CVX_ERR_CUDA;
}

}  // namespace
}  // namespace cvx

using namespace cvx;

extern "C" cvx_status cvx_voxelize_solid_noalloc(const cvx_voxinfo* info, const float* d_triangles, uint32_t* d_table,
                                                 int morton, cvx_stream_t stream) {
	if (!info || !d_table || (info->n_triangles && !d_triangles)) {
		set_message("cvx_voxelize_solid_noalloc: null argument");
		return CVX_ERR_INVALID_VALUE;
	}
	const uint64_t g0 = info->gridsize[0], g1 = info->gridsize[1], g2 = info->gridsize[2];
	if (!g0 || !g1 || !g2) {
		set_message("cvx_voxelize_solid_noalloc: gridsize has a zero dimension");
		return CVX_ERR_INVALID_VALUE;
	}
	if (g0 * g1 * g2 > kNoallocMaxVoxels) {
		char buf[256];
		std::snprintf(buf, sizeof(buf),
		              "cvx_voxelize_solid_noalloc: grid %llux%llux%llu exceeds the fixed scratch (at most %llu voxels, "
		              "e.g. 256^3); use cvx_voxelize_solid",
		              (unsigned long long)g0, (unsigned long long)g1, (unsigned long long)g2,
		              (unsigned long long)kNoallocMaxVoxels);
		set_message(buf);
		return CVX_ERR_INVALID_VALUE;
	}
	if (morton && (g0 != g1 || g1 != g2 || (g0 & (g0 - 1)))) {
		set_message("cvx_voxelize_solid_noalloc: Morton order needs a cubic power-of-two grid");
		return CVX_ERR_UNSUPPORTED;
	}
	if (info->n_triangles == 0) return CVX_OK;
	int dev = 0;
	cvx_status st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
	if (st != CVX_OK) return st;
	if (dev < 0 || dev >= kMaxDevices) {
		set_message("cvx_voxelize_solid_noalloc: device index out of range");
		return CVX_ERR_UNSUPPORTED;
	}
	void* base = nullptr;
	int cols_grid = 0;
	if ((st = scratch_address(dev, &base, &cols_grid)) != CVX_OK) return st;
	cvx_tuning tv;
	cvx_get_tuning(dev, &tv);
	Tune tune;
	tune.small_vox = tv.small_vox;
	tune.small_cols = tv.small_cols;

	cudaStream_t s = (cudaStream_t)stream;
	char* scr = static_cast<char*>(base);
	const uint64_t words = (g0 * g1 * g2 + 31) / 32;
	uint32_t* flips = reinterpret_cast<uint32_t*>(scr + kNoallocFlipOff);
	if ((st = cuda_status(cudaMemsetAsync(flips, 0, words * 4, s), "cudaMemsetAsync(flips)")) != CVX_OK) return st;
	if ((st = cuda_status(cudaMemsetAsync(scr, 0, sizeof(Counters), s), "cudaMemsetAsync(counters)")) != CVX_OK)
		return st;

	JobDesc job{};
	job.tris = d_triangles;
	job.table = d_table;
	job.flips = flips;
	for (int i = 0; i < 3; i++) {
		job.bmin[i] = info->bbox_min[i];
		job.unit[i] = info->unit[i];
		volatile float one = 1.0f;
		job.inv_unit[i] = one / info->unit[i];
		job.grid[i] = info->gridsize[i];
	}
	job.flags = (morton ? JOB_MORTON : 0u) | JOB_SOLID;
	const SolidUnits su = solid_units(job.grid);

	LaunchDesc L{};
	L.n_jobs = 1;
	L.scr.ctr = reinterpret_cast<Counters*>(scr);
	L.scr.big = reinterpret_cast<BigRec*>(scr + kNoallocBigOff);
	L.scr.mid = reinterpret_cast<MidRec*>(scr + kNoallocMidOff);
	L.scr.cap = (uint32_t)kNoallocMaxTriangles;
	// toggles, one triangle slice at a time (the queue holds one slice)
	for (uint64_t off = 0; off < info->n_triangles; off += kNoallocMaxTriangles) {
		const uint64_t n = info->n_triangles - off < kNoallocMaxTriangles ? info->n_triangles - off : kNoallocMaxTriangles;
		L.single = job;
		L.single.tris = d_triangles + off * 9;
		L.single.n_tri = n;
		L.n_tiles = (uint32_t)((n + kTile - 1) / kTile);
		if ((st = cuda_status(cudaMemsetAsync(scr, 0, kCountersResetBytes, s), "cudaMemsetAsync(counters)")) != CVX_OK)
			return st;
		if ((st = cuda_status(launch_solid(L, tune, cols_grid, s, kSolidToggles, nullptr), "solid toggles")) != CVX_OK)
			return st;
	}
	// one resolve over the whole table
	L.single = job;
	L.single.n_tri = 0;
	L.n_tiles = 0;
	L.n_units = (uint32_t)su.units;
	if (morton) {
		if (morton_slab_grid(g0)) {
			L.n_units = 0;  // solid_morton_slab resolves these grids alone
			L.n_mslabs = (g0 / 16) * (g0 / 16);
			L.slab_smem = (256u * ((uint32_t)(g0 / 32) | 1u) + kSlabSkewWords) * 4u;
		} else if (g0 >= 32) {
			L.n_mbricks = ((g0 * g1 * g2) >> 15) / (g0 >= 128 ? 4 : g0 / 32);
		} else {
			L.n_mwords = words;
		}
	}
	return cuda_status(launch_solid(L, tune, cols_grid, s, kSolidResolve, nullptr), "solid resolve");
}
