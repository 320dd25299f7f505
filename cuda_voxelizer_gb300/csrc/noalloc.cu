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
// with that device current, and caches it together with the id of the CUDA context it belongs to.
// That first call should therefore come before any stream capture.  A later call from another
// context (after cudaDeviceReset, or after the primary context was released and made again) sees
// the id change and looks the address up afresh.  Every call shares the one array: calls that
// overlap on the GPU (two streams, or two host threads) race on it and corrupt each other's
// results; issue them one after another.  Each call clears the parts that must start at zero
// (counters, the flip table of its grid).  cvx_device_status reports the device-side checks of the
// last call on the current device (its error word lives in the array too).
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
unsigned long long g_ctx_id[kMaxDevices] = {};
int g_cols_grid[kMaxDevices] = {};

// Id of the current CUDA context (cuCtxGetCurrent + cuCtxGetId, reached through the runtime so the
// library needs no link dependency on the driver library).  Ids are unique within the process.
typedef int (*CtxGetCurrentFn)(void** ctx);
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);
cvx_status current_context_id(unsigned long long* id) {
	static CtxGetCurrentFn get_current = nullptr;
	static CtxGetIdFn get_id = nullptr;
	if (!get_current || !get_id) {
		void* f0 = nullptr;
		void* f1 = nullptr;
		cudaDriverEntryPointQueryResult q0, q1;
		if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) != cudaSuccess ||
		    cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
		    q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1) {
			cudaGetLastError();
			set_message("cvx_voxelize_solid_noalloc: cuCtxGetCurrent/cuCtxGetId not available");
			return CVX_ERR_CUDA;
		}
		get_current = reinterpret_cast<CtxGetCurrentFn>(f0);
		get_id = reinterpret_cast<CtxGetIdFn>(f1);
	}
	void* ctx = nullptr;
	if (get_current(&ctx) != 0 || !ctx || get_id(ctx, id) != 0) {
		set_message("cvx_voxelize_solid_noalloc: no current CUDA context");
		return CVX_ERR_CUDA;
	}
	return CVX_OK;
}

// Device address of the scratch array for the current device and context (looked up once per
// context).
cvx_status scratch_address(int dev, void** out, int* cols_grid) {
	cudaError_t e = cudaSetDevice(dev);  // makes the device's primary context current (no allocation)
	if (e != cudaSuccess) {
		set_message(std::string("cvx_voxelize_solid_noalloc: cannot initialise the device: ") + cudaGetErrorString(e));
		return CVX_ERR_CUDA;
	}
	unsigned long long ctx = 0;
	cvx_status st = current_context_id(&ctx);
	if (st != CVX_OK) return st;
	std::lock_guard<std::mutex> lk(g_mu);
	if (!g_addr[dev] || g_ctx_id[dev] != ctx) {
		void* p = nullptr;
		e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
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
		g_ctx_id[dev] = ctx;
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

cvx_status noalloc_error(int dev, unsigned* err) {
	*err = 0;
	if (dev < 0 || dev >= kMaxDevices) return CVX_OK;
	void* base = nullptr;
	{
		std::lock_guard<std::mutex> lk(g_mu);
		if (!g_addr[dev]) return CVX_OK;  // no call on this device yet
		unsigned long long ctx = 0;
		if (current_context_id(&ctx) != CVX_OK || ctx != g_ctx_id[dev]) return CVX_OK;  // none in this context
		base = g_addr[dev];
	}
	Counters c;
	cudaError_t e = cudaMemcpy(&c, base, sizeof(c), cudaMemcpyDeviceToHost);
	if (e != cudaSuccess) {
		set_message(std::string("cudaMemcpy(noalloc counters): ") + cudaGetErrorString(e));
		return CVX_ERR_CUDA;
	}
	*err = c.error;
	return CVX_OK;
}

}  // namespace cvx

using namespace cvx;

extern "C" cvx_status cvx_voxelize_solid_noalloc(const cvx_voxinfo* info, const float* d_triangles, uint32_t* d_table,
                                                 int morton, cvx_stream_t stream) {
	// the checks of cvx_voxelize_solid: null pointers, zero axes, axes above 2^22 (the solid
	// column arithmetic reproduces the reference only below that), Morton order on grids it cannot
	// address
	cvx_status st = validate_call(info, d_triangles, d_table, morton);
	if (st != CVX_OK) return st;
	const uint64_t g0 = info->gridsize[0], g1 = info->gridsize[1], g2 = info->gridsize[2];
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
	if (info->n_triangles == 0) return CVX_OK;
	int dev = 0;
	st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
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
	job.flags = (morton ? JOB_MORTON : 0u) | JOB_SOLID | (needs_plain_loads(d_triangles) ? JOB_PLAIN_LOADS : 0u);
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
