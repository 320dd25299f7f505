// engine.h -- internal interface between the C-ABI layer (api.cu) and the kernel files.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include "cvx.h"
#include "cvx_device.cuh"

namespace cvx {

constexpr uint32_t kTile = 128;        // triangles per classify CTA (one tile; 2.6% faster than 256 on the bench step's plan)
constexpr uint32_t kZch = 32;          // z-slices per surface work item (one per lane)
constexpr uint32_t kRowsThreads = 256; // threads per cooperative CTA
constexpr uint32_t kColsPerItem = 256; // solid columns per work item
constexpr uint32_t kSmallRows = 16;    // surface: rows of a small triangle (every voxel tested)
constexpr uint32_t kLocalRows = 64;    // surface: rows of a local triangle (row intervals), classify kernel
constexpr uint32_t kMaskRowVoxels = 16; // surface: local rows up to this long test every voxel (the pass mask holds 16)
constexpr uint32_t kSmallCols = 16;    // solid: columns of a triangle handled in the classify kernel

// Device-side check codes written to Counters::error.
enum : unsigned { kErrBulkTimeout = 1u, kErrQueueOverflow = 2u };

// Triangles per launch sequence (the queue counters assume fewer than 2^24); larger meshes and
// batches are split by the host.
constexpr uint64_t kMaxTriPerLaunch = (1ull << 24) - 1;

// Tunables (picked per device by the autotuner; defaults are safe everywhere).
// Pair area of the brick rasterizer: room for this many (brick, triangle) pairs per triangle of a
// launch (about 27 per queued triangle, 12.5 per triangle, on the 1024^3 stress soup).
constexpr uint32_t kMaxBrickPairs = 16;

struct Tune {
	uint32_t small_vox = 64;    // surface: bbox voxels at or below which a triangle stays in its thread
	uint32_t small_cols = kSmallCols;  // solid: columns at or below which a triangle stays in the classify kernel
	// pairs per triangle the brick rasterizer may use; 0 (the default: on the 1024^3 stress soup the
	// brick path measured about 25% slower than the row path) rasterizes every larger triangle by rows
	uint32_t brick_pairs = 0;
};

// Optional per-kernel timing: mark(name) records an event on the stream after the named kernel
// (and once with name == nullptr before the first kernel of a sequence).
struct Prof {
	void (*mark)(void* ctx, const char* name, cudaStream_t s);
	void* ctx;
	void operator()(const char* name, cudaStream_t s) const { mark(ctx, name, s); }
};

// Launch `kernel` on stream s.  Kernels of a launch sequence run strictly one after another: a
// programmatic dependent launch (the successor scheduled while its predecessor drains, waiting in
// griddepcontrol.wait) was measured and dropped -- it left the 2M-triangle soup's surf_rows 9 ms
// (18%) slower and gave nothing on the other workloads.
template <class... KArgs, class... Args>
inline cudaError_t launch_k(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t s,
                            Args... args) {
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(grid);
	cfg.blockDim = dim3(block);
	cfg.dynamicSmemBytes = smem;
	cfg.stream = s;
	return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Surface launch sequence: classify, then (when the launch has JOB_BRICKS jobs, L.n_bricks > 0) the
// brick kernels, then the cooperative rows.  Counters must be zero.
cudaError_t launch_surface(const LaunchDesc& L, const Tune& tune, int rows_grid, int raster_grid, cudaStream_t s,
                           const Prof* prof);
int surf_rows_blocks_per_sm();

// The brick kernels of a surface launch sequence (bricks.cu): bin, scan, scatter, raster.
cudaError_t launch_bricks(const LaunchDesc& L, int grid, int raster_grid, cudaStream_t s, const Prof* prof);
int brick_raster_blocks_per_sm();

// A surface job rasterizes its larger triangles in bricks when its table is larger than the L2 cache
// can hold beside other work (at least 2^29 voxels, 64 MiB: smaller tables stay in L2, where
// per-row atomics are cheap) and every axis is at most 2048 (bounds the bricks one triangle's bbox
// can span).
inline bool brick_grid(const uint32_t g[3]) {
	return (uint64_t)g[0] * g[1] * g[2] >= (1ull << 29) && g[0] <= 2048 && g[1] <= 2048 && g[2] <= 2048;
}
inline uint32_t bricks_of(const uint32_t g[3]) {
	return ((g[0] + kBrick - 1) >> kBrickShift) * ((g[1] + kBrick - 1) >> kBrickShift) * ((g[2] + kBrick - 1) >> kBrickShift);
}

// Solid launch sequence.  kSolidToggles: classify + cooperative columns (counters must be zero);
// kSolidResolve: prefix-XOR resolve into the tables (+ Morton transcode).  Every job's flips table
// must be zero before the toggles and is zero again after the resolve.
enum : unsigned { kSolidToggles = 1u, kSolidResolve = 2u };
cudaError_t launch_solid(const LaunchDesc& L, const Tune& tune, int cols_grid, cudaStream_t s, unsigned phases,
                         const Prof* prof);
int solid_cols_blocks_per_sm();

// Morton grids that solid_morton_slab resolves and transcodes in one pass.
inline bool morton_slab_grid(uint64_t g) { return g >= 32 && g <= 1024; }

// Resolve-unit bookkeeping of a solid job: rows per unit and units per job.
struct SolidUnits {
	uint64_t rows_per_unit;
	uint64_t units;
	bool aligned;   // gx % 32 == 0: rows start on word boundaries
};
SolidUnits solid_units(const uint32_t grid[3]);

// Zeroing many tables in one launch: ranges sorted by chunk_begin, the prefix sum of
// clear_chunks(words) over the ranges before them.
struct ClearRange {
	uint32_t* ptr;
	uint64_t words;
	uint32_t chunk_begin;
	uint32_t pad;
};
constexpr uint32_t kClearChunkWords = 16384;  // 64 KiB per CTA
uint32_t clear_chunks(uint64_t words);
cudaError_t launch_clear(const ClearRange* d_ranges, uint32_t n, uint32_t total_chunks, cudaStream_t s);

// Sets the message returned by cvx_last_error_message() on this host thread.
void set_message(const std::string& m);

// The argument checks of cvx_voxelize / cvx_voxelize_solid (null pointers, zero or oversized grid
// axes, Morton order on a grid it cannot address); sets the message on failure.
cvx_status validate_call(const cvx_voxinfo* info, const void* tris, const void* table, int morton);

// True unless `p` is known to be plain device memory (cudaMalloc, a memory pool, a VMM mapping).
// Managed, host-registered and system memory are read with ordinary loads (JOB_PLAIN_LOADS): the
// load instructions handle their page faults and migrations.
bool needs_plain_loads(const void* p);

// Error word left by the last cvx_voxelize_solid_noalloc call on device `dev` in the library's fixed
// scratch array (0 if there was none).  The caller has synchronized the stream of that call.
cvx_status noalloc_error(int dev, unsigned* err);

// A batch run on caller-owned memory (used by the server, whose memory all comes from its budget).
// batch_scratch_bytes gives the device record bytes (256-byte aligned) and the pinned host staging
// bytes that run_batch_on needs for `jobs`.  run_batch_on takes one flip table per job in `flips`
// (read for solid jobs only: table-sized, zero on entry, zero again afterwards); the staging buffer
// must stay untouched until the stream has passed this call.  overwrite_solid: the solid jobs' tables
// belong to the caller's launch alone (no other job writes them): their resolve stores every word,
// so they need not be zeroed (JOB_TABLE_OVERWRITE); the surface jobs' tables must be zero.
cvx_status batch_scratch_bytes(const cvx_job* jobs, uint32_t n_jobs, size_t* rec_bytes, size_t* staging_bytes);
cvx_status run_batch_on(const cvx_job* jobs, uint32_t n_jobs, uint32_t* const* flips, void* d_rec, size_t rec_bytes,
                        void* h_staging, size_t staging_bytes, cudaStream_t s, bool overwrite_solid = false);

}  // namespace cvx
