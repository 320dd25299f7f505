// api.cu -- C ABI of the engine (include/cvx.h): validation, scratch management, launch grouping,
// batches and graph-captured plans.
//
// Scratch.  Every launch sequence needs a small counter block, a queue of triangle records (at
// most one per triangle) and, for solid voxelization, a linear-order flip table per job.  The
// library keeps one scratch set per (device, stream), grown on demand; the flip tables are zeroed
// when allocated and every solid launch leaves them zero again, so no per-call clearing is
// needed.  cvx_voxelize_ws takes caller-owned scratch instead (and clears its flip region).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "cvx.h"
#include "engine.h"

using namespace cvx;

static_assert(sizeof(cvx_voxinfo) == 64, "cvx_voxinfo must match the reference voxinfo (64 bytes)");
static_assert(offsetof(cvx_voxinfo, gridsize) == 24, "voxinfo.gridsize offset");
static_assert(offsetof(cvx_voxinfo, n_triangles) == 40, "voxinfo.n_triangles offset");
static_assert(offsetof(cvx_voxinfo, unit) == 48, "voxinfo.unit offset");
static_assert(sizeof(cvx_host_job) == 104, "cvx_host_job layout (the Python binding mirrors it)");

namespace {

thread_local std::string g_msg;

cvx_status fail(cvx_status s, const char* fmt, ...) {
	char buf[512];
	va_list ap;
	va_start(ap, fmt);
	std::vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	g_msg = buf;
	return s;
}

cvx_status cuda_fail(cudaError_t e, const char* where) {
	return fail(CVX_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

#define CVX_CUDA(call)                                   \
	do {                                                 \
		cudaError_t e_ = (call);                         \
		if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
	} while (0)

constexpr size_t kAlign = 256;
inline size_t align_up(size_t v) { return (v + kAlign - 1) & ~(kAlign - 1); }

struct DevState {
	int sms = 0;
	int rows_grid = 0;
	int cols_grid = 0;
	int raster_grid = 0;
	Tune tune;
};

std::mutex g_mu;
std::map<int, DevState> g_dev;

cvx_status dev_state(DevState& out, int* dev_out = nullptr) {
	int dev = 0;
	CVX_CUDA(cudaGetDevice(&dev));
	std::lock_guard<std::mutex> lk(g_mu);
	auto it = g_dev.find(dev);
	if (it == g_dev.end()) {
		DevState d;
		CVX_CUDA(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev));
		d.rows_grid = d.sms * surf_rows_blocks_per_sm();
		d.cols_grid = d.sms * solid_cols_blocks_per_sm();
		d.raster_grid = d.sms * brick_raster_blocks_per_sm();
		it = g_dev.emplace(dev, d).first;
	}
	out = it->second;
	if (dev_out) *dev_out = dev;
	return CVX_OK;
}

// ---- optional per-kernel timing (cvx_profile_*) --------------------------------------------------

bool g_profile = false;
struct Mark {
	const char* name;
	cudaEvent_t ev;
};
thread_local std::vector<Mark> t_marks;

void prof_mark(void*, const char* name, cudaStream_t s) {
	cudaEvent_t ev;
	if (cudaEventCreate(&ev) != cudaSuccess) return;
	cudaEventRecord(ev, s);
	t_marks.push_back({name, ev});
}
const Prof g_prof{prof_mark, nullptr};
const Prof* prof() { return g_profile ? &g_prof : nullptr; }

// ---- scratch ------------------------------------------------------------------------------------

// Record area of a launch sequence: counters, per-brick pair counts (for up to `bricks` bricks per
// launch; none without JOB_BRICKS jobs), the queues (cap triangles), the other brick arrays, then
// `n_jobs` uploaded job descriptors.  [0, big) must be zero before the first launch sequence on the
// area (the counts are zero again after every sequence).  Pairs: about 27 per queued triangle on the
// 1024^3 stress soup; triangles whose pairs do not fit are rasterized by surf_rows instead.
struct RecLayout {
	size_t ctr, bcnt, big, mid, bq, tri, boff, bcur, ubeg, psorted, jobs, end;
	uint64_t pair_cap;
};
RecLayout rec_layout(uint64_t cap, uint64_t n_jobs, uint32_t bricks = 0) {
	RecLayout l;
	l.ctr = 0;
	l.bcnt = align_up(sizeof(Counters));
	l.big = align_up(l.bcnt + (uint64_t)bricks * 4);
	l.mid = align_up(l.big + cap * sizeof(BigRec));
	l.bq = align_up(l.mid + cap * sizeof(MidRec));
	l.pair_cap = bricks ? std::min<uint64_t>(std::max<uint64_t>(kMaxBrickPairs * cap, 1u << 16), 1ull << 31) : 0;
	const uint64_t nq = bricks ? cap : 0;
	l.tri = align_up(l.bq + nq * sizeof(MidRec));
	l.boff = align_up(l.tri + nq * sizeof(BrickTri));
	l.bcur = align_up(l.boff + (bricks ? (uint64_t)bricks + 1 : 0) * 4);
	l.ubeg = align_up(l.bcur + (uint64_t)bricks * 4);
	l.psorted = align_up(l.ubeg + (bricks ? (uint64_t)bricks + 1 : 0) * 4);
	l.jobs = align_up(l.psorted + l.pair_cap * 4);
	l.end = align_up(l.jobs + n_jobs * sizeof(JobDesc));
	return l;
}

// Point a launch descriptor's scratch at a record area laid out by rec_layout(cap, *, bricks); the
// tuning may use less of the pair area (brick_pairs per triangle; 0 sends every triangle to surf_rows).
void bind_scratch(LaunchDesc& L, char* rec, uint64_t cap, uint32_t bricks, const Tune& tune) {
	const RecLayout l = rec_layout(cap, 0, bricks);
	L.scr.ctr = reinterpret_cast<Counters*>(rec + l.ctr);
	L.scr.big = reinterpret_cast<BigRec*>(rec + l.big);
	L.scr.mid = reinterpret_cast<MidRec*>(rec + l.mid);
	L.scr.cap = (uint32_t)cap;
	const uint64_t want = (uint64_t)std::min(tune.brick_pairs, kMaxBrickPairs) * cap;
	L.scr.pair_cap = tune.brick_pairs ? (uint32_t)std::min<uint64_t>(std::max<uint64_t>(want, 1u << 16), l.pair_cap) : 0u;
	if (!bricks) return;
	L.scr.bq = reinterpret_cast<MidRec*>(rec + l.bq);
	L.scr.tri = reinterpret_cast<BrickTri*>(rec + l.tri);
	L.scr.brick_cnt = reinterpret_cast<uint32_t*>(rec + l.bcnt);
	L.scr.brick_off = reinterpret_cast<uint32_t*>(rec + l.boff);
	L.scr.brick_cur = reinterpret_cast<uint32_t*>(rec + l.bcur);
	L.scr.unit_begin = reinterpret_cast<uint32_t*>(rec + l.ubeg);
	L.scr.pair_sorted = reinterpret_cast<uint32_t*>(rec + l.psorted);
}

struct StreamScratch {
	void* rec = nullptr;
	size_t rec_bytes = 0;
	uint32_t* flips = nullptr;  // zero between launch sequences
	size_t flip_bytes = 0;
	JobDesc* staging = nullptr; // pinned host copy of uploaded job arrays
	size_t staging_n = 0;
	cudaEvent_t staging_done = nullptr;
};
std::map<std::pair<int, cudaStream_t>, StreamScratch> g_ws;

bool capturing(cudaStream_t s) {
	cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
	if (cudaStreamIsCapturing(s, &st) != cudaSuccess) return false;
	return st != cudaStreamCaptureStatusNone;
}

cvx_status ensure_scratch(int dev, cudaStream_t s, size_t rec_bytes, size_t flip_bytes, size_t staging_n,
                          StreamScratch** out) {
	std::lock_guard<std::mutex> lk(g_mu);
	StreamScratch& w = g_ws[{dev, s}];
	const bool grow_rec = rec_bytes > w.rec_bytes, grow_flip = flip_bytes > w.flip_bytes;
	const bool grow_stage = staging_n > w.staging_n;
	if ((grow_rec || grow_flip || grow_stage) && capturing(s))
		return fail(CVX_ERR_CAPTURING, "scratch must grow while the stream is being captured; make one call before capture "
		                               "or use cvx_voxelize_ws");
	if (grow_rec || grow_flip) CVX_CUDA(cudaStreamSynchronize(s));
	if (grow_rec) {
		if (w.rec) cudaFree(w.rec);
		w.rec = nullptr;
		w.rec_bytes = 0;
		size_t b = std::max(rec_bytes, (size_t)1 << 20);
		if (cudaMalloc(&w.rec, b) != cudaSuccess) {
			cudaGetLastError();
			return fail(CVX_ERR_OUT_OF_MEMORY, "cannot allocate %zu bytes of scratch", b);
		}
		w.rec_bytes = b;
	}
	if (grow_flip) {
		if (w.flips) cudaFree(w.flips);
		w.flips = nullptr;
		w.flip_bytes = 0;
		if (cudaMalloc((void**)&w.flips, flip_bytes) != cudaSuccess) {
			cudaGetLastError();
			return fail(CVX_ERR_OUT_OF_MEMORY, "cannot allocate %zu bytes of flip table", flip_bytes);
		}
		CVX_CUDA(cudaMemsetAsync(w.flips, 0, flip_bytes, s));
		w.flip_bytes = flip_bytes;
	}
	if (grow_stage) {
		if (w.staging) {
			if (w.staging_done) cudaEventSynchronize(w.staging_done);
			cudaFreeHost(w.staging);
		}
		w.staging = nullptr;
		w.staging_n = 0;
		size_t n = std::max<size_t>(staging_n, 64);
		CVX_CUDA(cudaMallocHost((void**)&w.staging, n * sizeof(JobDesc)));
		w.staging_n = n;
		if (!w.staging_done) CVX_CUDA(cudaEventCreateWithFlags(&w.staging_done, cudaEventDisableTiming));
	}
	*out = &w;
	return CVX_OK;
}

// ---- validation and job descriptors -------------------------------------------------------------

uint64_t words_of(const cvx_voxinfo& v) {
	const uint64_t bits = (uint64_t)v.gridsize[0] * v.gridsize[1] * v.gridsize[2];
	return (bits + 31) / 32;
}

// For each table range (first word, word count): does it overlap another job's range?  Jobs that
// share table words accumulate into them (OR / XOR, as repeated reference calls would), so the
// engine may neither overwrite such a table nor run those jobs on concurrent lanes.
std::vector<char> overlapping_tables(const std::vector<std::pair<uint32_t*, uint64_t>>& t) {
	std::vector<char> shared(t.size(), 0);
	std::vector<size_t> order(t.size());
	for (size_t i = 0; i < order.size(); i++) order[i] = i;
	std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return t[a].first < t[b].first; });
	size_t reach = 0;  // the job whose range ends last among those seen
	for (size_t k = 0; k < order.size(); k++) {
		const size_t i = order[k];
		if (k > 0 && t[i].first < t[reach].first + t[reach].second) shared[i] = shared[reach] = 1;
		if (k == 0 || t[i].first + t[i].second > t[reach].first + t[reach].second) reach = i;
	}
	return shared;
}

cvx_status validate(const cvx_voxinfo* info, const void* tris, const void* table, int morton) {
	if (!info) return fail(CVX_ERR_INVALID_VALUE, "info is null");
	for (int i = 0; i < 3; i++) {
		if (info->gridsize[i] == 0) return fail(CVX_ERR_INVALID_VALUE, "gridsize[%d] is 0", i);
		if (info->gridsize[i] > (1u << 22)) return fail(CVX_ERR_UNSUPPORTED, "gridsize[%d] above 2^22", i);
	}
	if (info->n_triangles > 0 && !tris) return fail(CVX_ERR_INVALID_VALUE, "triangle pointer is null");
	if (!table) return fail(CVX_ERR_INVALID_VALUE, "table pointer is null");
	if (morton) {
		const uint32_t g = info->gridsize[0];
		// Morton codes of a g^3 grid fill [0, g^3) only for a cubic power-of-two grid; anything else
		// addresses words beyond the table (the reference writes out of bounds there).
		if (info->gridsize[1] != g || info->gridsize[2] != g || (g & (g - 1)) != 0)
			return fail(CVX_ERR_UNSUPPORTED, "Morton order needs a cubic power-of-two grid (got %u x %u x %u)", g,
			            info->gridsize[1], info->gridsize[2]);
	}
	return CVX_OK;
}

// brick_pairs of the current device's tuning (the default before any call has set it).
uint32_t current_brick_pairs() {
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) {
		cudaGetLastError();
		return Tune().brick_pairs;
	}
	std::lock_guard<std::mutex> lk(g_mu);
	auto it = g_dev.find(dev);
	return it == g_dev.end() ? Tune().brick_pairs : it->second.tune.brick_pairs;
}

JobDesc make_job(const cvx_voxinfo& v, const float* tris, uint32_t* table, int morton, int solid) {
	JobDesc j;
	std::memset(&j, 0, sizeof(j));
	j.tris = tris;
	j.table = table;
	j.n_tri = v.n_triangles;
	for (int i = 0; i < 3; i++) {
		j.bmin[i] = v.bbox_min[i];
		j.unit[i] = v.unit[i];
		volatile float one = 1.0f;
		j.inv_unit[i] = one / v.unit[i];  // IEEE single division: correctly rounded
		j.grid[i] = v.gridsize[i];
	}
	j.flags = (morton ? JOB_MORTON : 0u) | (solid ? JOB_SOLID : 0u);
	const uint64_t voxels = (uint64_t)v.gridsize[0] * v.gridsize[1] * v.gridsize[2];
	if (morton ? v.gridsize[0] <= 1024 : voxels <= (1ull << 32)) j.flags |= JOB_NARROW;
	if (!solid && brick_grid(j.grid) && current_brick_pairs()) j.flags |= JOB_BRICKS;
	if (v.n_triangles && needs_plain_loads(tris)) j.flags |= JOB_PLAIN_LOADS;
	return j;
}

uint32_t tiles_of(uint64_t n) { return (uint32_t)((n + kTile - 1) / kTile); }

// A group of jobs launched together (same mode), with prefix fields filled in.
struct Group {
	std::vector<JobDesc> jobs;
	uint64_t tris = 0;
	uint32_t tiles = 0, units = 0;
	uint64_t mwords = 0, mbricks = 0, mslabs = 0;
	uint32_t slab_smem = 0;
	uint32_t bricks = 0;  // 64^3 bricks of the group's JOB_BRICKS jobs
};

void finish_group(Group& g, bool solid) {
	uint32_t tile = 0, unit = 0, brick = 0;
	uint64_t mw = 0, mb = 0, ms = 0;
	g.tris = 0;
	g.slab_smem = 0;
	for (JobDesc& j : g.jobs) {
		j.tile_begin = tile;
		tile += tiles_of(j.n_tri);
		g.tris += j.n_tri;
		j.brick_begin = brick;  // running count: jobs without bricks take the next job's value
		if (!solid && (j.flags & JOB_BRICKS)) brick += bricks_of(j.grid);
		if (solid) {
			j.unit_begin = unit;
			// Morton slab grids are resolved by solid_morton_slab alone: no resolve units
			if (!((j.flags & JOB_MORTON) && morton_slab_grid(j.grid[0]))) unit += (uint32_t)solid_units(j.grid).units;
			j.mword_begin = mw;
			j.mbrick_begin = mb;
			j.mslab_begin = ms;
			const uint64_t vox = (uint64_t)j.grid[0] * j.grid[1] * j.grid[2];
			if (j.flags & JOB_MORTON) {
				const uint64_t gx = j.grid[0];
				if (morton_slab_grid(gx)) {
					ms += (gx / 16) * (gx / 16);  // slabs of 16 x 16 rows
					const uint32_t stride = (uint32_t)(gx / 32) | 1u;
					g.slab_smem = std::max(g.slab_smem, (256u * stride + kSlabSkewWords) * 4u);
				} else if (gx >= 32) {
					const uint64_t w = gx >= 128 ? 4 : gx / 32;  // x-adjacent 32^3 bricks per CTA
					mb += (vox >> 15) / w;
				} else {
					mw += (vox + 31) / 32;
				}
			}
		}
	}
	g.tiles = tile;
	g.units = unit;
	g.bricks = brick;
	g.mwords = mw;
	g.mbricks = mb;
	g.mslabs = ms;
}

// Split jobs of one mode into launch groups of fewer than kMaxTriPerLaunch triangles.  A job above
// the limit is cut into triangle ranges (same table: the results accumulate exactly).
std::vector<Group> make_groups(const std::vector<JobDesc>& jobs, bool solid) {
	std::vector<Group> out;
	Group cur;
	for (const JobDesc& j0 : jobs) {
		JobDesc j = j0;
		uint64_t off = 0;
		do {
			JobDesc part = j;
			const uint64_t room = kMaxTriPerLaunch - cur.tris;
			const uint64_t take = std::min<uint64_t>(j.n_tri - off, room);
			part.tris = j.tris + off * 9;
			part.n_tri = take;
			cur.jobs.push_back(part);
			cur.tris += take;
			off += take;
			if (cur.tris >= kMaxTriPerLaunch) {
				out.push_back(cur);
				cur = Group();
			}
		} while (off < j.n_tri);
	}
	if (!cur.jobs.empty()) out.push_back(cur);
	for (Group& g : out) finish_group(g, solid);
	return out;
}

// Solid jobs whose resolve must follow all their toggle launches: one resolve group per distinct
// table (jobs cut into ranges share one).
Group resolve_group(const std::vector<JobDesc>& jobs) {
	Group g;
	g.jobs = jobs;
	for (JobDesc& j : g.jobs) j.n_tri = 0;  // resolve only
	finish_group(g, true);
	return g;
}

uint64_t flip_bytes_of(const JobDesc& j) {
	return align_up(((uint64_t)j.grid[0] * j.grid[1] * j.grid[2] + 31) / 32 * 4);
}

// Run every launch of a mixed job list on stream s using the scratch at (rec, flips).  `upload`
// copies job arrays to the device (stream-ordered).
struct Runner {
	cudaStream_t s;
	DevState dev;
	char* rec;
	size_t rec_bytes;
	uint32_t* flips;  // solid flip tables, laid out back to back in job order
	JobDesc* staging;
	size_t staging_cap;
	size_t staging_used = 0;
	size_t jobs_used = 0;  // JobDesc slots used in the device job area
	uint64_t cap;          // queue capacity (triangles)
	size_t jobs_off;
	uint32_t bricks = 0;   // brick capacity of the record area (largest group's bricks)
	bool timed = true;     // per-kernel events for cvx_profile_collect (callers on this thread only)
	const Prof* p() const { return timed ? prof() : nullptr; }

	cvx_status prepare(Group& g, LaunchDesc& L) {
		std::memset(&L, 0, sizeof(L));
		L.n_jobs = (uint32_t)g.jobs.size();
		L.n_tiles = g.tiles;
		L.n_units = g.units;
		L.n_mwords = g.mwords;
		L.n_mbricks = g.mbricks;
		L.n_mslabs = g.mslabs;
		L.slab_smem = g.slab_smem;
		if (g.bricks > bricks) return fail(CVX_ERR_INVALID_VALUE, "brick scratch too small");
		L.n_bricks = g.bricks;
		bind_scratch(L, rec, cap, bricks, dev.tune);
		if (g.jobs.size() == 1) {
			L.single = g.jobs[0];
			L.jobs = nullptr;
			return CVX_OK;
		}
		if (staging_used + g.jobs.size() > staging_cap) return fail(CVX_ERR_INVALID_VALUE, "job staging overflow");
		JobDesc* host = staging + staging_used;
		std::memcpy(host, g.jobs.data(), g.jobs.size() * sizeof(JobDesc));
		JobDesc* devp = reinterpret_cast<JobDesc*>(rec + jobs_off) + jobs_used;
		CVX_CUDA(cudaMemcpyAsync(devp, host, g.jobs.size() * sizeof(JobDesc), cudaMemcpyHostToDevice, s));
		staging_used += g.jobs.size();
		jobs_used += g.jobs.size();
		L.jobs = devp;
		return CVX_OK;
	}

	cvx_status run(const std::vector<JobDesc>& surf, const std::vector<JobDesc>& solid) {
		for (Group& g : make_groups(surf, false)) {
			LaunchDesc L;
			cvx_status st = prepare(g, L);
			if (st != CVX_OK) return st;
			CVX_CUDA(cudaMemsetAsync(rec, 0, kCountersResetBytes, s));
			CVX_CUDA(launch_surface(L, dev.tune, dev.rows_grid, dev.raster_grid, s, p()));
		}
		if (!solid.empty()) {
			for (Group& g : make_groups(solid, true)) {
				LaunchDesc L;
				cvx_status st = prepare(g, L);
				if (st != CVX_OK) return st;
				CVX_CUDA(cudaMemsetAsync(rec, 0, kCountersResetBytes, s));
				CVX_CUDA(launch_solid(L, dev.tune, dev.cols_grid, s, kSolidToggles, p()));
			}
			Group r = resolve_group(solid);
			LaunchDesc L;
			cvx_status st = prepare(r, L);
			if (st != CVX_OK) return st;
			CVX_CUDA(launch_solid(L, dev.tune, dev.cols_grid, s, kSolidResolve, p()));
		}
		return CVX_OK;
	}
};

// Number of JobDesc slots the uploads of run() need.
size_t job_slots(const std::vector<JobDesc>& surf, const std::vector<JobDesc>& solid) {
	size_t n = 0;
	for (const Group& g : make_groups(surf, false)) n += g.jobs.size() > 1 ? g.jobs.size() : 0;
	if (!solid.empty()) {
		for (const Group& g : make_groups(solid, true)) n += g.jobs.size() > 1 ? g.jobs.size() : 0;
		n += solid.size() > 1 ? solid.size() : 0;
	}
	return n;
}

// Largest brick count of a surface launch group.
uint32_t max_bricks(const std::vector<JobDesc>& surf) {
	uint32_t m = 0;
	for (const Group& g : make_groups(surf, false)) m = std::max(m, g.bricks);
	return m;
}

uint64_t queue_cap(const std::vector<JobDesc>& a, const std::vector<JobDesc>& b) {
	uint64_t m = 1;
	for (const Group& g : make_groups(a, false)) m = std::max(m, g.tris);
	for (const Group& g : make_groups(b, true)) m = std::max(m, g.tris);
	return m;
}

// Assign each solid job its flip table inside one buffer.
uint64_t assign_flips(std::vector<JobDesc>& solid, uint32_t* base) {
	uint64_t off = 0;
	for (JobDesc& j : solid) {
		j.flips = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(base) + off);
		off += flip_bytes_of(j);
	}
	return off;
}

cvx_status run_internal(std::vector<JobDesc> surf, std::vector<JobDesc> solid, cudaStream_t s) {
	if (surf.empty() && solid.empty()) return CVX_OK;
	DevState dev;
	int devid = 0;
	cvx_status st = dev_state(dev, &devid);
	if (st != CVX_OK) return st;
	uint64_t flip_total = 0;
	for (const JobDesc& j : solid) flip_total += flip_bytes_of(j);
	const uint64_t cap = queue_cap(surf, solid);
	const size_t slots = job_slots(surf, solid);
	const uint32_t bricks = max_bricks(surf);
	const RecLayout lay = rec_layout(cap, slots, bricks);
	StreamScratch* w = nullptr;
	st = ensure_scratch(devid, s, lay.end, (size_t)flip_total, slots, &w);
	if (st != CVX_OK) return st;
	assign_flips(solid, w->flips);
	if (slots && w->staging_done) CVX_CUDA(cudaEventSynchronize(w->staging_done));  // staging reusable
	Runner r{s, dev, reinterpret_cast<char*>(w->rec), w->rec_bytes, w->flips, w->staging, w->staging_n};
	r.cap = cap;
	r.jobs_off = lay.jobs;
	r.bricks = bricks;
	CVX_CUDA(cudaMemsetAsync(w->rec, 0, lay.big, s));  // counters and brick counts
	st = r.run(surf, solid);
	if (st != CVX_OK) return st;
	if (slots) CVX_CUDA(cudaEventRecord(w->staging_done, s));
	return CVX_OK;
}

// Job descriptors of a cvx_job array, split by mode (empty jobs dropped); flips[i], if given,
// becomes job i's flip table.
cvx_status collect_jobs(const cvx_job* jobs, uint32_t n_jobs, uint32_t* const* flips, std::vector<JobDesc>& surf,
                        std::vector<JobDesc>& solid) {
	if (n_jobs && !jobs) return fail(CVX_ERR_INVALID_VALUE, "jobs is null");
	for (uint32_t i = 0; i < n_jobs; i++) {
		cvx_status st = validate(&jobs[i].info, jobs[i].d_triangles, jobs[i].d_table, jobs[i].morton);
		if (st != CVX_OK) return fail(st, "job %u: %s", i, g_msg.c_str());
		if (jobs[i].info.n_triangles == 0) continue;
		JobDesc j = make_job(jobs[i].info, jobs[i].d_triangles, jobs[i].d_table, jobs[i].morton, jobs[i].solid);
		if (flips && jobs[i].solid) {
			if (!flips[i]) return fail(CVX_ERR_INVALID_VALUE, "job %u: no flip table", i);
			j.flips = flips[i];
		}
		(jobs[i].solid ? solid : surf).push_back(j);
	}
	return CVX_OK;
}

}  // namespace

cvx_status cvx::batch_scratch_bytes(const cvx_job* jobs, uint32_t n_jobs, size_t* rec_bytes, size_t* staging_bytes) {
	std::vector<JobDesc> surf, solid;
	cvx_status st = collect_jobs(jobs, n_jobs, nullptr, surf, solid);
	if (st != CVX_OK) return st;
	const size_t slots = job_slots(surf, solid);
	*rec_bytes = rec_layout(queue_cap(surf, solid), slots, max_bricks(surf)).end;
	*staging_bytes = std::max<size_t>(slots, 1) * sizeof(JobDesc);
	return CVX_OK;
}

cvx_status cvx::run_batch_on(const cvx_job* jobs, uint32_t n_jobs, uint32_t* const* flips, void* d_rec,
                             size_t rec_bytes, void* h_staging, size_t staging_bytes, cudaStream_t s,
                             bool overwrite_solid) {
	std::vector<JobDesc> surf, solid;
	cvx_status st = collect_jobs(jobs, n_jobs, flips, surf, solid);
	if (st != CVX_OK) return st;
	if (overwrite_solid)
		for (JobDesc& j : solid) j.flags |= JOB_TABLE_OVERWRITE;
	if (surf.empty() && solid.empty()) return CVX_OK;
	if (!solid.empty() && !flips) return fail(CVX_ERR_INVALID_VALUE, "solid jobs need flip tables");
	const uint64_t cap = queue_cap(surf, solid);
	const size_t slots = job_slots(surf, solid);
	const uint32_t bricks = max_bricks(surf);
	const RecLayout lay = rec_layout(cap, slots, bricks);
	if (!d_rec || rec_bytes < lay.end || reinterpret_cast<uintptr_t>(d_rec) % kAlign)
		return fail(CVX_ERR_INVALID_VALUE, "record area too small or not 256-byte aligned");
	if (slots && (!h_staging || staging_bytes < slots * sizeof(JobDesc)))
		return fail(CVX_ERR_INVALID_VALUE, "job staging too small");
	DevState dev;
	st = dev_state(dev);
	if (st != CVX_OK) return st;
	Runner r{s, dev, static_cast<char*>(d_rec), lay.end, nullptr, static_cast<JobDesc*>(h_staging),
	         staging_bytes / sizeof(JobDesc)};
	r.cap = cap;
	r.jobs_off = lay.jobs;
	r.bricks = bricks;
	r.timed = false;  // the server's worker thread: nobody collects events there
	CVX_CUDA(cudaMemsetAsync(d_rec, 0, lay.big, s));  // counters and brick counts
	return r.run(surf, solid);
}

void cvx::set_message(const std::string& m) { g_msg = m; }

bool cvx::needs_plain_loads(const void* p) {
	if (!p) return false;
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return true;
	}
	return a.type != cudaMemoryTypeDevice;
}

cvx_status cvx::validate_call(const cvx_voxinfo* info, const void* tris, const void* table, int morton) {
	return validate(info, tris, table, morton);
}

// ==== C ABI =======================================================================================

extern "C" {

const char* cvx_status_string(cvx_status s) {
	switch (s) {
	case CVX_OK: return "CVX_OK";
	case CVX_ERR_INVALID_VALUE: return "CVX_ERR_INVALID_VALUE";
	case CVX_ERR_UNSUPPORTED: return "CVX_ERR_UNSUPPORTED";
	case CVX_ERR_OUT_OF_MEMORY: return "CVX_ERR_OUT_OF_MEMORY";
	case CVX_ERR_CUDA: return "CVX_ERR_CUDA";
	case CVX_ERR_DEVICE_CHECK: return "CVX_ERR_DEVICE_CHECK";
	case CVX_ERR_CAPTURING: return "CVX_ERR_CAPTURING";
	}
	return "CVX_ERR_UNKNOWN";
}

const char* cvx_last_error_message(void) { return g_msg.c_str(); }

int cvx_version(void) { return CVX_VERSION_MAJOR * 1000 + CVX_VERSION_MINOR; }

cvx_status cvx_voxinfo_init(cvx_voxinfo* out, const float bbox_min[3], const float bbox_max[3],
                            const uint32_t gridsize[3], uint64_t n_triangles) {
	if (!out || !bbox_min || !bbox_max || !gridsize) return fail(CVX_ERR_INVALID_VALUE, "null argument");
	std::memset(out, 0, sizeof(*out));
	for (int i = 0; i < 3; i++) {
		out->bbox_min[i] = bbox_min[i];
		out->bbox_max[i] = bbox_max[i];
		out->gridsize[i] = gridsize[i];
		// src/util.h:58-60: (bbox.max - bbox.min) / float(gridsize)
		volatile float ext = bbox_max[i] - bbox_min[i];
		out->unit[i] = ext / (float)gridsize[i];
	}
	out->n_triangles = n_triangles;
	return CVX_OK;
}

cvx_status cvx_bbox_cube(const float in_min[3], const float in_max[3], float out_min[3], float out_max[3]) {
	if (!in_min || !in_max || !out_min || !out_max) return fail(CVX_ERR_INVALID_VALUE, "null argument");
	// src/util.h:80-110, in float: lengths, max length via std::max, half-difference padding, then
	// padding by extent / 10001 on every side.
	volatile float len[3];
	for (int i = 0; i < 3; i++) len[i] = in_max[i] - in_min[i];
	const float myz = (len[1] < len[2]) ? len[2] : len[1];
	const float mx = (len[0] < myz) ? myz : len[0];
	float lo[3], hi[3];
	for (int i = 0; i < 3; i++) {
		lo[i] = in_min[i];
		hi[i] = in_max[i];
		if (mx != len[i]) {
			volatile float delta = mx - len[i];
			volatile float half = delta / 2.0f;
			lo[i] = in_min[i] - half;
			hi[i] = in_max[i] + half;
		}
	}
	for (int i = 0; i < 3; i++) {
		volatile float ext = hi[i] - lo[i];
		volatile float eps = ext / 10001.0f;
		out_min[i] = lo[i] - eps;
		out_max[i] = hi[i] + eps;
	}
	return CVX_OK;
}

cvx_status cvx_mesh_bbox(const float* tris, uint64_t n, float out_min[3], float out_max[3]) {
	if ((!tris && n) || !out_min || !out_max) return fail(CVX_ERR_INVALID_VALUE, "null argument");
	if (n == 0) return fail(CVX_ERR_INVALID_VALUE, "empty mesh has no bounding box");
	float lo[3] = {tris[0], tris[1], tris[2]}, hi[3] = {tris[0], tris[1], tris[2]};
	for (uint64_t i = 0; i < 3 * n; i++) {
		const float* v = tris + 3 * i;
		for (int k = 0; k < 3; k++) {
			lo[k] = v[k] < lo[k] ? v[k] : lo[k];
			hi[k] = v[k] > hi[k] ? v[k] : hi[k];
		}
	}
	for (int k = 0; k < 3; k++) {
		out_min[k] = lo[k];
		out_max[k] = hi[k];
	}
	return CVX_OK;
}

uint64_t cvx_table_words(const cvx_voxinfo* info) { return info ? words_of(*info) : 0; }

cvx_status cvx_voxelize(const cvx_voxinfo* info, const float* d_tris, uint32_t* d_table, int morton,
                        cvx_stream_t stream) {
	cvx_status st = validate(info, d_tris, d_table, morton);
	if (st != CVX_OK) return st;
	if (info->n_triangles == 0) return CVX_OK;
	std::vector<JobDesc> surf{make_job(*info, d_tris, d_table, morton, 0)}, solid;
	return run_internal(surf, solid, (cudaStream_t)stream);
}

cvx_status cvx_voxelize_solid(const cvx_voxinfo* info, const float* d_tris, uint32_t* d_table, int morton,
                              cvx_stream_t stream) {
	cvx_status st = validate(info, d_tris, d_table, morton);
	if (st != CVX_OK) return st;
	if (info->n_triangles == 0) return CVX_OK;
	std::vector<JobDesc> surf, solid{make_job(*info, d_tris, d_table, morton, 1)};
	return run_internal(surf, solid, (cudaStream_t)stream);
}

// Bricks of a single surface job on this voxinfo (0 if it does not use them).
static uint32_t single_job_bricks(const cvx_voxinfo& v, int solid) {
	const uint32_t g[3] = {v.gridsize[0], v.gridsize[1], v.gridsize[2]};
	return (!solid && brick_grid(g)) ? bricks_of(g) : 0u;
}

uint64_t cvx_workspace_size(const cvx_voxinfo* info, int solid) {
	if (!info) return 0;
	const uint64_t n = std::max<uint64_t>(1, std::min<uint64_t>(info->n_triangles, kMaxTriPerLaunch));
	const RecLayout lay = rec_layout(n, 0, single_job_bricks(*info, solid));
	uint64_t b = lay.end;
	if (solid) b += align_up(words_of(*info) * 4);
	return b;
}

cvx_status cvx_voxelize_ws(const cvx_voxinfo* info, const float* d_tris, uint32_t* d_table, int morton, int solid,
                           void* d_ws, uint64_t ws_bytes, cvx_stream_t stream) {
	cvx_status st = validate(info, d_tris, d_table, morton);
	if (st != CVX_OK) return st;
	if (info->n_triangles == 0) return CVX_OK;
	if (!d_ws) return fail(CVX_ERR_INVALID_VALUE, "workspace is null");
	if (reinterpret_cast<uintptr_t>(d_ws) % kAlign) return fail(CVX_ERR_INVALID_VALUE, "workspace not 256-byte aligned");
	const uint64_t need = cvx_workspace_size(info, solid);
	if (ws_bytes < need) return fail(CVX_ERR_INVALID_VALUE, "workspace too small: %llu < %llu bytes",
	                                 (unsigned long long)ws_bytes, (unsigned long long)need);
	DevState dev;
	st = dev_state(dev);
	if (st != CVX_OK) return st;
	cudaStream_t s = (cudaStream_t)stream;
	const uint64_t cap = std::max<uint64_t>(1, std::min<uint64_t>(info->n_triangles, kMaxTriPerLaunch));
	const uint32_t bricks = single_job_bricks(*info, solid);
	const RecLayout lay = rec_layout(cap, 0, bricks);
	char* rec = static_cast<char*>(d_ws);
	std::vector<JobDesc> surf, sol;
	JobDesc j = make_job(*info, d_tris, d_table, morton, solid);
	if (solid) {
		j.flips = reinterpret_cast<uint32_t*>(rec + lay.end);
		CVX_CUDA(cudaMemsetAsync(j.flips, 0, words_of(*info) * 4, s));
		sol.push_back(j);
	} else {
		surf.push_back(j);
	}
	CVX_CUDA(cudaMemsetAsync(rec, 0, lay.big, s));  // counters and brick counts
	Runner r{s, dev, rec, (size_t)lay.end, j.flips, nullptr, 0};
	r.cap = cap;
	r.jobs_off = lay.jobs;
	r.bricks = bricks;
	return r.run(surf, sol);
}

cvx_status cvx_device_status(cvx_stream_t stream) {
	int dev = 0;
	CVX_CUDA(cudaGetDevice(&dev));
	cudaStream_t s = (cudaStream_t)stream;
	CVX_CUDA(cudaStreamSynchronize(s));
	void* rec = nullptr;
	{
		std::lock_guard<std::mutex> lk(g_mu);
		auto it = g_ws.find({dev, s});
		if (it != g_ws.end()) rec = it->second.rec;
	}
	if (rec) {
		Counters c;
		CVX_CUDA(cudaMemcpy(&c, rec, sizeof(c), cudaMemcpyDeviceToHost));
		if (c.error) return fail(CVX_ERR_DEVICE_CHECK, "device check failed (code %u)", c.error);
	}
	// the last cvx_voxelize_solid_noalloc call on this device keeps its counters in the library's
	// fixed scratch array
	unsigned err = 0;
	cvx_status st = noalloc_error(dev, &err);
	if (st != CVX_OK) return st;
	if (err) return fail(CVX_ERR_DEVICE_CHECK, "device check failed in cvx_voxelize_solid_noalloc (code %u)", err);
	return CVX_OK;
}

cvx_status cvx_stream_release(cvx_stream_t stream) {
	int dev = 0;
	CVX_CUDA(cudaGetDevice(&dev));
	cudaStream_t s = (cudaStream_t)stream;
	StreamScratch w;
	{
		std::lock_guard<std::mutex> lk(g_mu);
		auto it = g_ws.find({dev, s});
		if (it == g_ws.end()) return CVX_OK;
		w = it->second;
		g_ws.erase(it);
	}
	CVX_CUDA(cudaStreamSynchronize(s));  // no kernel of the stream still uses the scratch
	if (w.staging_done) cudaEventDestroy(w.staging_done);
	if (w.staging) cudaFreeHost(w.staging);
	if (w.rec) cudaFree(w.rec);
	if (w.flips) cudaFree(w.flips);
	return CVX_OK;
}

cvx_status cvx_voxelize_batch(const cvx_job* jobs, uint32_t n_jobs, cvx_stream_t stream) {
	if (n_jobs && !jobs) return fail(CVX_ERR_INVALID_VALUE, "jobs is null");
	std::vector<JobDesc> surf, solid;
	for (uint32_t i = 0; i < n_jobs; i++) {
		cvx_status st = validate(&jobs[i].info, jobs[i].d_triangles, jobs[i].d_table, jobs[i].morton);
		if (st != CVX_OK) return fail(st, "job %u: %s", i, g_msg.c_str());
		JobDesc j = make_job(jobs[i].info, jobs[i].d_triangles, jobs[i].d_table, jobs[i].morton, jobs[i].solid);
		if (jobs[i].info.n_triangles == 0) continue;
		(jobs[i].solid ? solid : surf).push_back(j);
	}
	return run_internal(surf, solid, (cudaStream_t)stream);
}

// ---- plans: a batch captured once into a CUDA graph ----------------------------------------------

struct cvx_plan {
	cudaGraphExec_t exec = nullptr;
	cudaGraph_t graph = nullptr;
	std::vector<void*> recs;       // counters and queues of each lane
	JobDesc* job_area = nullptr;   // the job arrays of every lane's multi-job launches
	uint32_t* flips = nullptr;
	ClearRange* clears = nullptr;  // the tables the graph zeroes (CVX_PLAN_CLEAR_TABLES)
};

// A plan runs its jobs in lanes: the surface jobs split into up to kPlanSurfaceLanes groups of
// about equal triangle count, and the solid jobs in one more.  Each lane has its own counters and
// queues and its own captured stream, so the graph lets the lanes' kernels overlap (a lane's
// latency-bound cooperative kernel runs beside another lane's classify kernel).
constexpr int kPlanSurfaceLanes = 2;

// One group's launches on a capturing stream, as Runner::run issues them but with the group's job
// array (when it has more than one job) already resident at `jobs_dev`.
static cudaError_t capture_group(const Group& g, bool solid, bool resolve, void* rec, uint64_t cap, uint32_t bricks,
                                 JobDesc* jobs_dev, const DevState& dev, cudaStream_t s) {
	if (g.bricks > bricks) return cudaErrorInvalidValue;
	LaunchDesc L;
	std::memset(&L, 0, sizeof(L));
	L.n_jobs = (uint32_t)g.jobs.size();
	L.n_tiles = g.tiles;
	L.n_units = g.units;
	L.n_mwords = g.mwords;
	L.n_mbricks = g.mbricks;
	L.n_mslabs = g.mslabs;
	L.slab_smem = g.slab_smem;
	L.n_bricks = g.bricks;
	bind_scratch(L, static_cast<char*>(rec), cap, bricks, dev.tune);
	if (g.jobs.size() == 1)
		L.single = g.jobs[0];
	else
		L.jobs = jobs_dev;
	if (resolve) return launch_solid(L, dev.tune, dev.cols_grid, s, kSolidResolve, nullptr);
	const cudaError_t e = cudaMemsetAsync(rec, 0, kCountersResetBytes, s);
	if (e != cudaSuccess) return e;
	return solid ? launch_solid(L, dev.tune, dev.cols_grid, s, kSolidToggles, nullptr)
	             : launch_surface(L, dev.tune, dev.rows_grid, dev.raster_grid, s, nullptr);
}

cvx_status cvx_plan_create(const cvx_job* jobs, uint32_t n_jobs, uint32_t flags, cvx_plan** out) {
	if (!out) return fail(CVX_ERR_INVALID_VALUE, "out is null");
	*out = nullptr;
	if (n_jobs && !jobs) return fail(CVX_ERR_INVALID_VALUE, "jobs is null");
	std::vector<JobDesc> surf, solid;
	std::vector<std::pair<uint32_t*, uint64_t>> tables;
	for (uint32_t i = 0; i < n_jobs; i++) {
		cvx_status st = validate(&jobs[i].info, jobs[i].d_triangles, jobs[i].d_table, jobs[i].morton);
		if (st != CVX_OK) return fail(st, "job %u: %s", i, g_msg.c_str());
		tables.push_back({jobs[i].d_table, words_of(jobs[i].info)});
	}
	// With CVX_PLAN_CLEAR_TABLES every table starts from zero.  A solid job with its own table
	// overwrites it (no clear needed); the others' tables are zeroed by their lane before its kernels
	// (or all at the start when jobs share tables: such a plan runs its lanes one after another).
	const std::vector<char> shared = overlapping_tables(tables);
	bool any_shared = false;
	for (char c : shared) any_shared = any_shared || c;
	const bool clear = (flags & CVX_PLAN_CLEAR_TABLES) != 0;
	const bool lane_clears = clear && !any_shared;  // surface tables zeroed in their own lane
	std::vector<std::pair<uint32_t*, uint64_t>> pre_clears;  // zeroed before the lanes fork
	for (uint32_t i = 0; i < n_jobs; i++) {
		if (jobs[i].info.n_triangles == 0) {
			if (clear) pre_clears.push_back(tables[i]);  // complete once cleared
			continue;
		}
		JobDesc j = make_job(jobs[i].info, jobs[i].d_triangles, jobs[i].d_table, jobs[i].morton, jobs[i].solid);
		if (clear && jobs[i].solid && !shared[i]) j.flags |= JOB_TABLE_OVERWRITE;
		else if (clear && !(lane_clears && !jobs[i].solid)) pre_clears.push_back(tables[i]);
		(jobs[i].solid ? solid : surf).push_back(j);
	}
	DevState dev;
	cvx_status st = dev_state(dev);
	if (st != CVX_OK) return st;
	cvx_plan* p = new cvx_plan();
	auto bail = [&](cvx_status s2) {
		cvx_plan_destroy(p);
		return s2;
	};

	struct Lane {
		bool solid = false;
		std::vector<JobDesc> jobs;
		std::vector<Group> groups;  // toggles / surface launches; the solid lane's resolve is last
		uint64_t cap = 1;
		uint32_t bricks = 0;         // largest brick count of the lane's groups
		size_t job_off = 0;          // first JobDesc slot of the lane in the job area
		size_t clear_off = 0;        // the lane's tables to zero: ranges [clear_off, clear_off + clear_n)
		uint32_t clear_n = 0, clear_chunks = 0;
		cudaStream_t stream = nullptr;
		cudaEvent_t done = nullptr;
	};
	std::vector<Lane> lanes;
	if (!surf.empty()) {
		const size_t k = std::min<size_t>(kPlanSurfaceLanes, surf.size());
		std::vector<Lane> sl(k);
		std::vector<uint64_t> load(k, 0);
		std::vector<size_t> order(surf.size());
		for (size_t i = 0; i < order.size(); i++) order[i] = i;
		std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return surf[x].n_tri > surf[y].n_tri; });
		for (size_t i : order) {
			const size_t b = (size_t)(std::min_element(load.begin(), load.end()) - load.begin());
			sl[b].jobs.push_back(surf[i]);
			load[b] += surf[i].n_tri;
		}
		for (Lane& l : sl) lanes.push_back(std::move(l));
	}
	uint64_t flip_total = 0;
	for (const JobDesc& j : solid) flip_total += flip_bytes_of(j);
	if (flip_total) {
		if (cudaMalloc((void**)&p->flips, flip_total) != cudaSuccess) {
			cudaGetLastError();
			return bail(fail(CVX_ERR_OUT_OF_MEMORY, "plan flip tables"));
		}
		if (cudaMemset(p->flips, 0, flip_total) != cudaSuccess) return bail(cuda_fail(cudaGetLastError(), "memset"));
		assign_flips(solid, p->flips);
	}
	if (!solid.empty()) {
		Lane l;
		l.solid = true;
		l.jobs = solid;
		lanes.push_back(std::move(l));
	}
	size_t slots = 0;
	for (Lane& l : lanes) {
		l.groups = make_groups(l.jobs, l.solid);
		if (l.solid) l.groups.push_back(resolve_group(l.jobs));
		l.job_off = slots;
		for (size_t gi = 0; gi < l.groups.size(); gi++) {
			const Group& g = l.groups[gi];
			if (!(l.solid && gi + 1 == l.groups.size())) l.cap = std::max<uint64_t>(l.cap, g.tris);
			if (!l.solid) l.bricks = std::max(l.bricks, g.bricks);
			if (g.jobs.size() > 1) slots += g.jobs.size();
		}
	}
	if (slots) {
		if (cudaMalloc((void**)&p->job_area, slots * sizeof(JobDesc)) != cudaSuccess) {
			cudaGetLastError();
			return bail(fail(CVX_ERR_OUT_OF_MEMORY, "plan job arrays"));
		}
		size_t used = 0;
		for (const Lane& l : lanes)
			for (const Group& g : l.groups) {
				if (g.jobs.size() <= 1) continue;
				if (cudaMemcpy(p->job_area + used, g.jobs.data(), g.jobs.size() * sizeof(JobDesc), cudaMemcpyHostToDevice) !=
				    cudaSuccess)
					return bail(cuda_fail(cudaGetLastError(), "job upload"));
				used += g.jobs.size();
			}
	}
	for (const Lane& l : lanes) {
		void* rec = nullptr;
		if (cudaMalloc(&rec, rec_layout(l.cap, 0, l.bricks).end) != cudaSuccess) {
			cudaGetLastError();
			return bail(fail(CVX_ERR_OUT_OF_MEMORY, "plan scratch"));
		}
		p->recs.push_back(rec);
	}
	// The clear list: the tables zeroed before the fork, then each surface lane's own tables (each
	// segment numbers its chunks from 0: one clear_ranges launch per segment).
	std::vector<ClearRange> clears;
	uint32_t clear_total = 0;
	if (clear) {
		for (auto& t : pre_clears) {
			clears.push_back(ClearRange{t.first, t.second, clear_total, 0u});
			clear_total += clear_chunks(t.second);
		}
		for (Lane& l : lanes) {
			if (l.solid || !lane_clears) continue;
			l.clear_off = clears.size();
			for (const JobDesc& j : l.jobs) {
				const uint64_t words = ((uint64_t)j.grid[0] * j.grid[1] * j.grid[2] + 31) / 32;
				clears.push_back(ClearRange{j.table, words, l.clear_chunks, 0u});
				l.clear_chunks += clear_chunks(words);
			}
			l.clear_n = (uint32_t)(clears.size() - l.clear_off);
		}
		if (!clears.empty()) {
			if (cudaMalloc((void**)&p->clears, clears.size() * sizeof(ClearRange)) != cudaSuccess) {
				cudaGetLastError();
				return bail(fail(CVX_ERR_OUT_OF_MEMORY, "plan clear list"));
			}
			if (cudaMemcpy(p->clears, clears.data(), clears.size() * sizeof(ClearRange), cudaMemcpyHostToDevice) !=
			    cudaSuccess)
				return bail(cuda_fail(cudaGetLastError(), "clear list upload"));
		}
	}

	cudaStream_t cs;
	cudaEvent_t fork_ev;
	if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return bail(cuda_fail(cudaGetLastError(), "stream"));
	cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming);
	const bool fork = lanes.size() > 1 && !any_shared;  // jobs sharing a table run one after another
	cvx_status cst = CVX_OK;
	for (Lane& l : lanes) {
		l.stream = cs;
		if (fork && cst == CVX_OK) {
			if (cudaStreamCreateWithFlags(&l.stream, cudaStreamNonBlocking) != cudaSuccess ||
			    cudaEventCreateWithFlags(&l.done, cudaEventDisableTiming) != cudaSuccess) {
				l.stream = cs;
				cst = cuda_fail(cudaGetLastError(), "stream");
			}
		}
	}
	auto drop_streams = [&]() {
		for (Lane& l : lanes) {
			if (l.stream && l.stream != cs) cudaStreamDestroy(l.stream);
			if (l.done) cudaEventDestroy(l.done);
		}
		cudaStreamDestroy(cs);
		cudaEventDestroy(fork_ev);
	};
	if (cst != CVX_OK) {
		drop_streams();
		return bail(cst);
	}
	if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
		drop_streams();
		return bail(cuda_fail(cudaGetLastError(), "begin capture"));
	}
	if (!pre_clears.empty() && launch_clear(p->clears, (uint32_t)pre_clears.size(), clear_total, cs) != cudaSuccess)
		cst = cuda_fail(cudaGetLastError(), "table clear");
	if (cst == CVX_OK && fork && cudaEventRecord(fork_ev, cs) != cudaSuccess) cst = cuda_fail(cudaGetLastError(), "capture fork");
	// Launch exactly like Runner::run, but with the job arrays already resident.
	for (size_t li = 0; li < lanes.size() && cst == CVX_OK; li++) {
		Lane& l = lanes[li];
		void* rec = p->recs[li];
		if ((fork && cudaStreamWaitEvent(l.stream, fork_ev, 0) != cudaSuccess) ||
		    cudaMemsetAsync(rec, 0, rec_layout(l.cap, 0, l.bricks).big, l.stream) != cudaSuccess ||
		    (l.clear_n && launch_clear(p->clears + l.clear_off, l.clear_n, l.clear_chunks, l.stream) != cudaSuccess)) {
			cst = cuda_fail(cudaGetLastError(), "capture lane");
			break;
		}
		size_t used = l.job_off;
		for (size_t gi = 0; gi < l.groups.size() && cst == CVX_OK; gi++) {
			const Group& g = l.groups[gi];
			const bool resolve = l.solid && gi + 1 == l.groups.size();
			const cudaError_t e = capture_group(g, l.solid, resolve, rec, l.cap, l.bricks, p->job_area + used, dev, l.stream);
			if (g.jobs.size() > 1) used += g.jobs.size();
			if (e != cudaSuccess) cst = cuda_fail(e, "capture launch");
		}
		if (cst == CVX_OK && fork &&
		    (cudaEventRecord(l.done, l.stream) != cudaSuccess || cudaStreamWaitEvent(cs, l.done, 0) != cudaSuccess))
			cst = cuda_fail(cudaGetLastError(), "capture join");
	}
	cudaGraph_t graph = nullptr;
	cudaError_t ee = cudaStreamEndCapture(cs, &graph);
	drop_streams();
	if (cst != CVX_OK) {
		if (graph) cudaGraphDestroy(graph);
		return bail(cst);
	}
	if (ee != cudaSuccess) return bail(cuda_fail(ee, "end capture"));
	p->graph = graph;
	if (cudaGraphInstantiate(&p->exec, graph, 0) != cudaSuccess) return bail(cuda_fail(cudaGetLastError(), "instantiate"));
	*out = p;
	return CVX_OK;
}

// ---- host-buffer plans: upload, voxelize and read back as one graph -------------------------------

namespace {

constexpr uint32_t kHostPlanDefaultChunks = 2;
constexpr uint32_t kHostPlanMaxChunks = 64;

bool page_locked(const void* p) {
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	return a.type == cudaMemoryTypeHost;
}

// One mesh's triangles on their way up: the host source, the device destination and the chunk
// bounds (in triangles; interior bounds on whole kTile-triangle tiles, so every chunk but the last
// starts 16-byte aligned when the buffer does and keeps the classify kernels' bulk tile copy).
struct Upload {
	const float* h = nullptr;
	const float* d = nullptr;
	uint64_t n = 0;
	std::vector<uint64_t> bounds;
};

// One step of a host plan's compute stream, in issue order.
struct HostStep {
	enum Kind { kWait, kLaunch, kResolve, kFinal } kind;
	uint32_t u = 0, c = 0;  // kWait: upload u's chunk c has landed
	uint32_t job = 0;       // kFinal: the caller's job whose table is now complete
	bool solid = false;
	Group g;                // kLaunch / kResolve
	size_t slot = 0;        // first JobDesc slot of g's job array (groups of more than one job)
};

}  // namespace

// A host-buffer plan is the round trip of plain calls on host memory -- copy the triangles up,
// voxelize, copy the tables down -- arranged for a link that is slower than the kernels: the copies
// bound it, so the plan keeps the link busy.  Meshes go up one after another, each in chunks, on a
// copy stream; one compute stream runs the surface jobs on each chunk as soon as it lands (exact: a
// surface table is the OR of its chunks' bits), so they complete with the last chunk; then each
// solid table in turn over the whole mesh.  Tables are completed one at a time so that a read-back
// stream can copy each down while the next is still being computed.
cvx_status cvx_plan_create_host(const cvx_host_job* jobs, uint32_t n_jobs, uint32_t n_chunks, cvx_plan** out) {
	if (!out) return fail(CVX_ERR_INVALID_VALUE, "out is null");
	*out = nullptr;
	if (n_jobs && !jobs) return fail(CVX_ERR_INVALID_VALUE, "jobs is null");
	if (n_chunks == 0) n_chunks = kHostPlanDefaultChunks;
	if (n_chunks > kHostPlanMaxChunks) return fail(CVX_ERR_INVALID_VALUE, "n_chunks above %u", kHostPlanMaxChunks);
	for (uint32_t i = 0; i < n_jobs; i++) {
		const cvx_host_job& J = jobs[i];
		cvx_status st = validate(&J.info, J.d_triangles, J.d_table, J.morton);
		if (st != CVX_OK) return fail(st, "job %u: %s", i, g_msg.c_str());
		if (!J.h_table) return fail(CVX_ERR_INVALID_VALUE, "job %u: h_table is null", i);
		if (J.info.n_triangles && !J.h_triangles) return fail(CVX_ERR_INVALID_VALUE, "job %u: h_triangles is null", i);
	}
	DevState dev;
	cvx_status st = dev_state(dev);
	if (st != CVX_OK) return st;
	std::vector<Upload> ups;
	std::vector<int> up_of(n_jobs, -1);
	for (uint32_t i = 0; i < n_jobs; i++) {
		const cvx_host_job& J = jobs[i];
		if (!page_locked(J.h_table)) return fail(CVX_ERR_INVALID_VALUE, "job %u: h_table is not page-locked host memory", i);
		if (J.info.n_triangles == 0) continue;
		if (!page_locked(J.h_triangles))
			return fail(CVX_ERR_INVALID_VALUE, "job %u: h_triangles is not page-locked host memory", i);
		int u = -1;
		for (size_t k = 0; k < ups.size(); k++) {
			if (ups[k].d != J.d_triangles) continue;
			if (ups[k].h != J.h_triangles || ups[k].n != J.info.n_triangles)
				return fail(CVX_ERR_INVALID_VALUE, "job %u: d_triangles receives a different upload in another job", i);
			u = (int)k;
		}
		if (u < 0) {
			Upload up;
			up.h = J.h_triangles;
			up.d = J.d_triangles;
			up.n = J.info.n_triangles;
			up.bounds.resize(n_chunks + 1);
			for (uint32_t c = 0; c < n_chunks; c++) up.bounds[c] = up.n * c / n_chunks / kTile * kTile;
			up.bounds[n_chunks] = up.n;
			u = (int)ups.size();
			ups.push_back(std::move(up));
		}
		up_of[i] = u;
	}

	cvx_plan* p = new cvx_plan();
	auto bail = [&](cvx_status s2) {
		cvx_plan_destroy(p);
		return s2;
	};
	// Flip tables of the solid jobs.
	std::vector<uint32_t*> flips(n_jobs, nullptr);
	{
		std::vector<JobDesc> full;
		std::vector<uint32_t> idx;
		for (uint32_t i = 0; i < n_jobs; i++)
			if (jobs[i].solid && up_of[i] >= 0) {
				full.push_back(make_job(jobs[i].info, jobs[i].d_triangles, jobs[i].d_table, jobs[i].morton, 1));
				idx.push_back(i);
			}
		uint64_t flip_total = 0;
		for (const JobDesc& j : full) flip_total += flip_bytes_of(j);
		if (flip_total) {
			if (cudaMalloc((void**)&p->flips, flip_total) != cudaSuccess) {
				cudaGetLastError();
				return bail(fail(CVX_ERR_OUT_OF_MEMORY, "plan flip tables"));
			}
			if (cudaMemset(p->flips, 0, flip_total) != cudaSuccess) return bail(cuda_fail(cudaGetLastError(), "memset"));
			assign_flips(full, p->flips);
			for (size_t k = 0; k < idx.size(); k++) flips[idx[k]] = full[k].flips;
		}
	}
	// Every launch rewrites every table: a solid job with a table of its own overwrites it (its
	// resolve stores every word); the other tables are zeroed at the start of the launch.
	std::vector<std::pair<uint32_t*, uint64_t>> ranges;
	for (uint32_t i = 0; i < n_jobs; i++) ranges.push_back({jobs[i].d_table, words_of(jobs[i].info)});
	const std::vector<char> shared = overlapping_tables(ranges);
	auto overwrites = [&](uint32_t i) { return jobs[i].solid && up_of[i] >= 0 && !shared[i]; };
	auto job_of = [&](uint32_t i, uint64_t b0, uint64_t b1) {
		cvx_voxinfo v = jobs[i].info;
		v.n_triangles = b1 - b0;
		JobDesc j = make_job(v, jobs[i].d_triangles + 9 * b0, jobs[i].d_table, jobs[i].morton, jobs[i].solid);
		j.flips = flips[i];
		if (overwrites(i)) j.flags |= JOB_TABLE_OVERWRITE;
		return j;
	};
	// The compute stream's steps.  Jobs without triangles are complete once cleared.
	std::vector<HostStep> steps;
	for (uint32_t i = 0; i < n_jobs; i++)
		if (up_of[i] < 0) {
			HostStep f;
			f.kind = HostStep::kFinal;
			f.job = i;
			steps.push_back(std::move(f));
		}
	uint64_t cap = 1;
	uint32_t bricks = 0;
	size_t slots = 0;
	auto add_groups = [&](std::vector<JobDesc>& part, bool solid) {
		if (part.empty()) return;
		for (Group& g : make_groups(part, solid)) {
			HostStep st;
			st.kind = HostStep::kLaunch;
			st.solid = solid;
			cap = std::max<uint64_t>(cap, g.tris);
			if (!solid) bricks = std::max(bricks, g.bricks);
			st.slot = slots;
			if (g.jobs.size() > 1) slots += g.jobs.size();
			st.g = std::move(g);
			steps.push_back(std::move(st));
		}
		part.clear();
	};
	for (uint32_t u = 0; u < (uint32_t)ups.size(); u++) {
		std::vector<uint32_t> mine;
		for (uint32_t i = 0; i < n_jobs; i++)
			if (up_of[i] == (int)u) mine.push_back(i);
		for (uint32_t c = 0; c < n_chunks; c++) {
			const uint64_t b0 = ups[u].bounds[c], b1 = ups[u].bounds[c + 1];
			if (b1 == b0) continue;
			HostStep w;
			w.kind = HostStep::kWait;
			w.u = u;
			w.c = c;
			steps.push_back(std::move(w));
			const bool last = b1 == ups[u].n;
			std::vector<JobDesc> part;
			if (!last) {
				for (uint32_t i : mine)
					if (!jobs[i].solid) part.push_back(job_of(i, b0, b1));
				add_groups(part, false);
				continue;
			}
			// The last chunk one surface job at a time, each table read back as soon as it is done:
			// the link starts on the first table after a fraction of the chunk's work.
			for (uint32_t i : mine)
				if (!jobs[i].solid) {
					part.push_back(job_of(i, b0, b1));
					add_groups(part, false);
					HostStep f;
					f.kind = HostStep::kFinal;
					f.job = i;
					steps.push_back(std::move(f));
				}
			// The solid tables one at a time over the whole mesh: toggles, resolve, read back.  (Per
			// chunk they would cost a persistent column launch each, which the upload cannot hide.)
			for (uint32_t i : mine)
				if (jobs[i].solid) {
					part.push_back(job_of(i, 0, ups[u].n));
					add_groups(part, true);
					HostStep r;
					r.kind = HostStep::kResolve;
					r.solid = true;
					r.g = resolve_group(std::vector<JobDesc>{job_of(i, 0, ups[u].n)});
					r.slot = slots;
					steps.push_back(std::move(r));
					HostStep f;
					f.kind = HostStep::kFinal;
					f.job = i;
					steps.push_back(std::move(f));
				}
		}
	}
	if (slots) {
		if (cudaMalloc((void**)&p->job_area, slots * sizeof(JobDesc)) != cudaSuccess) {
			cudaGetLastError();
			return bail(fail(CVX_ERR_OUT_OF_MEMORY, "plan job arrays"));
		}
		std::vector<JobDesc> all;
		for (const HostStep& st : steps)
			if (st.kind == HostStep::kLaunch && st.g.jobs.size() > 1) all.insert(all.end(), st.g.jobs.begin(), st.g.jobs.end());
		if (cudaMemcpy(p->job_area, all.data(), all.size() * sizeof(JobDesc), cudaMemcpyHostToDevice) != cudaSuccess)
			return bail(cuda_fail(cudaGetLastError(), "job upload"));
	}
	void* rec = nullptr;
	if (cudaMalloc(&rec, rec_layout(cap, 0, bricks).end) != cudaSuccess) {
		cudaGetLastError();
		return bail(fail(CVX_ERR_OUT_OF_MEMORY, "plan scratch"));
	}
	p->recs.push_back(rec);

	// The capture: compute on the origin stream, uploads on cp, read-backs on rb.
	cudaStream_t cs = nullptr, cp = nullptr, rb = nullptr;
	cudaEvent_t fork_ev = nullptr, copied = nullptr, read = nullptr;
	std::vector<std::vector<cudaEvent_t>> landed(ups.size(), std::vector<cudaEvent_t>(n_chunks, nullptr));
	std::vector<cudaEvent_t> final_ev(n_jobs, nullptr);
	cvx_status cst = CVX_OK;
	auto mk_stream = [&](cudaStream_t* st) {
		if (cst == CVX_OK && cudaStreamCreateWithFlags(st, cudaStreamNonBlocking) != cudaSuccess) {
			*st = nullptr;
			cst = cuda_fail(cudaGetLastError(), "stream");
		}
	};
	auto mk_event = [&](cudaEvent_t* e) {
		if (cst == CVX_OK && cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) {
			*e = nullptr;
			cst = cuda_fail(cudaGetLastError(), "event");
		}
	};
	mk_stream(&cs);
	mk_stream(&cp);
	mk_stream(&rb);
	mk_event(&fork_ev);
	mk_event(&copied);
	mk_event(&read);
	for (auto& v : landed)
		for (cudaEvent_t& e : v) mk_event(&e);
	for (cudaEvent_t& e : final_ev) mk_event(&e);
	auto drop = [&]() {
		for (auto& v : landed)
			for (cudaEvent_t e : v)
				if (e) cudaEventDestroy(e);
		for (cudaEvent_t e : final_ev)
			if (e) cudaEventDestroy(e);
		for (cudaStream_t st : {cs, cp, rb})
			if (st) cudaStreamDestroy(st);
		for (cudaEvent_t e : {fork_ev, copied, read})
			if (e) cudaEventDestroy(e);
	};
	if (cst != CVX_OK) {
		drop();
		return bail(cst);
	}
	if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
		drop();
		return bail(cuda_fail(cudaGetLastError(), "begin capture"));
	}
	auto ck = [&](cudaError_t e, const char* what) {
		if (cst == CVX_OK && e != cudaSuccess) cst = cuda_fail(e, what);
	};
	ck(cudaEventRecord(fork_ev, cs), "capture fork");
	ck(cudaStreamWaitEvent(cp, fork_ev, 0), "capture fork");
	ck(cudaStreamWaitEvent(rb, fork_ev, 0), "capture fork");
	for (size_t u = 0; u < ups.size() && cst == CVX_OK; u++)
		for (uint32_t c = 0; c < n_chunks && cst == CVX_OK; c++) {
			const uint64_t b0 = ups[u].bounds[c], b1 = ups[u].bounds[c + 1];
			if (b1 == b0) continue;
			ck(cudaMemcpyAsync(const_cast<float*>(ups[u].d) + 9 * b0, ups[u].h + 9 * b0, (b1 - b0) * 36,
			                   cudaMemcpyHostToDevice, cp),
			   "capture upload");
			ck(cudaEventRecord(landed[u][c], cp), "capture upload");
		}
	ck(cudaEventRecord(copied, cp), "capture upload");
	for (uint32_t i = 0; i < n_jobs; i++)
		if (!overwrites(i)) ck(cudaMemsetAsync(jobs[i].d_table, 0, words_of(jobs[i].info) * 4, cs), "capture clear");
	ck(cudaMemsetAsync(rec, 0, rec_layout(cap, 0, bricks).big, cs), "capture clear");
	for (const HostStep& st : steps) {
		if (cst != CVX_OK) break;
		switch (st.kind) {
		case HostStep::kWait:
			ck(cudaStreamWaitEvent(cs, landed[st.u][st.c], 0), "capture wait");
			break;
		case HostStep::kLaunch:
		case HostStep::kResolve:
			ck(capture_group(st.g, st.solid, st.kind == HostStep::kResolve, rec, cap, bricks, p->job_area + st.slot, dev, cs),
			   "capture launch");
			break;
		case HostStep::kFinal: {
			const cvx_host_job& J = jobs[st.job];
			ck(cudaEventRecord(final_ev[st.job], cs), "capture read-back");
			ck(cudaStreamWaitEvent(rb, final_ev[st.job], 0), "capture read-back");
			ck(cudaMemcpyAsync(J.h_table, J.d_table, words_of(J.info) * 4, cudaMemcpyDeviceToHost, rb), "capture read-back");
			break;
		}
		}
	}
	ck(cudaEventRecord(read, rb), "capture join");
	ck(cudaStreamWaitEvent(cs, read, 0), "capture join");
	ck(cudaStreamWaitEvent(cs, copied, 0), "capture join");
	cudaGraph_t graph = nullptr;
	const cudaError_t ee = cudaStreamEndCapture(cs, &graph);
	drop();
	if (cst != CVX_OK) {
		if (graph) cudaGraphDestroy(graph);
		return bail(cst);
	}
	if (ee != cudaSuccess) return bail(cuda_fail(ee, "end capture"));
	p->graph = graph;
	if (cudaGraphInstantiate(&p->exec, graph, 0) != cudaSuccess) return bail(cuda_fail(cudaGetLastError(), "instantiate"));
	*out = p;
	return CVX_OK;
}

cvx_status cvx_plan_launch(cvx_plan* p, cvx_stream_t stream) {
	if (!p || !p->exec) return fail(CVX_ERR_INVALID_VALUE, "plan is null");
	CVX_CUDA(cudaGraphLaunch(p->exec, (cudaStream_t)stream));
	return CVX_OK;
}

cvx_status cvx_plan_kernel_nodes(const cvx_plan* p, uint32_t* n_kernels) {
	if (!p || !p->graph || !n_kernels) return fail(CVX_ERR_INVALID_VALUE, "plan or output is null");
	size_t n = 0;
	CVX_CUDA(cudaGraphGetNodes(p->graph, nullptr, &n));
	std::vector<cudaGraphNode_t> nodes(n);
	if (n) CVX_CUDA(cudaGraphGetNodes(p->graph, nodes.data(), &n));
	uint32_t k = 0;
	for (size_t i = 0; i < n; i++) {
		cudaGraphNodeType t;
		CVX_CUDA(cudaGraphNodeGetType(nodes[i], &t));
		if (t == cudaGraphNodeTypeKernel) k++;
	}
	*n_kernels = k;
	return CVX_OK;
}

cvx_status cvx_plan_destroy(cvx_plan* p) {
	if (!p) return CVX_OK;
	if (p->exec) cudaGraphExecDestroy(p->exec);
	if (p->graph) cudaGraphDestroy(p->graph);
	for (void* r : p->recs) cudaFree(r);
	if (p->job_area) cudaFree(p->job_area);
	if (p->flips) cudaFree(p->flips);
	if (p->clears) cudaFree(p->clears);
	delete p;
	return CVX_OK;
}

cvx_status cvx_profile_enable(int on) {
	g_profile = on != 0;
	return CVX_OK;
}

int cvx_profile_collect(const char** names, float* ms, int max_entries) {
	int n = 0;
	cudaEvent_t prev = nullptr;
	for (const Mark& m : t_marks) {
		if (cudaEventSynchronize(m.ev) != cudaSuccess) break;
		if (m.name && prev && n < max_entries) {
			float t = 0.0f;
			cudaEventElapsedTime(&t, prev, m.ev);
			if (names) names[n] = m.name;
			if (ms) ms[n] = t;
			n++;
		}
		prev = m.ev;
	}
	for (const Mark& m : t_marks) cudaEventDestroy(m.ev);
	t_marks.clear();
	return n;
}

cvx_status cvx_get_tuning(int device, cvx_tuning* out) {
	if (!out) return fail(CVX_ERR_INVALID_VALUE, "out is null");
	std::lock_guard<std::mutex> lk(g_mu);
	Tune t;
	auto it = g_dev.find(device);
	if (it != g_dev.end()) t = it->second.tune;
	out->small_vox = t.small_vox;
	out->small_cols = t.small_cols;
	out->brick_pairs = t.brick_pairs;
	return CVX_OK;
}

cvx_status cvx_set_tuning(int device, const cvx_tuning* in) {
	if (!in) return fail(CVX_ERR_INVALID_VALUE, "in is null");
	int cur = 0;
	CVX_CUDA(cudaGetDevice(&cur));
	if (cur != device) CVX_CUDA(cudaSetDevice(device));
	DevState d;
	cvx_status st = dev_state(d);
	if (cur != device) cudaSetDevice(cur);
	if (st != CVX_OK) return st;
	std::lock_guard<std::mutex> lk(g_mu);
	g_dev[device].tune.small_vox = in->small_vox;
	g_dev[device].tune.small_cols = in->small_cols;
	g_dev[device].tune.brick_pairs = std::min(in->brick_pairs, kMaxBrickPairs);
	return CVX_OK;
}

}  // extern "C"
