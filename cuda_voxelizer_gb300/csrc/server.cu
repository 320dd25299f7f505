// server.cu -- serving: voxelization requests admitted by device memory and batched continuously.
//
// Requests (a voxinfo, host triangles, a host table, a mode) arrive at any time from any host
// thread.  One worker thread runs the loop:
//   1. retire: batches whose stream has passed their last copy (a host callback marks them) free
//      their memory and wake the waiters;
//   2. admit and launch: while a stream is free, take pending requests in arrival order for as long
//      as their memory fits in the free part of the budget (at most max_batch), then launch them as
//      one batch on that stream: copies in, clears, one engine launch sequence, copies out.
// Requests that arrive while batches are on the GPU wait only until a stream is free and then go
// into the next batch, which overlaps with those still running.
//
// Memory.  All device memory of a request -- triangles, table, solid flip table -- and its batch's
// work records come from one arena of the budget's size, allocated when the server is created and
// carved first-fit, so nothing is allocated while serving and the budget is a hard limit.
// Requests may keep their buffers on the device: triangles already resident (d_triangles, read in
// place) and the table left resident in the arena (no host table) until cvx_server_release, for
// consumers that use it on the GPU.
// Admission is strictly in arrival order: a request that does not fit waits (and so do the ones
// behind it) until batches finish.  A request larger than the whole budget is refused at submission.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "cvx.h"
#include "engine.h"

namespace {

using Clock = std::chrono::steady_clock;
constexpr size_t kAlign = 256;
inline size_t align_up(size_t v) { return (v + kAlign - 1) & ~(kAlign - 1); }

// First-fit allocator over one device arena (offsets kept in ordered maps; coalesces on release).
class Arena {
public:
	cudaError_t init(size_t bytes) {
		cudaError_t e = cudaMalloc(&base_, bytes);
		if (e != cudaSuccess) {
			base_ = nullptr;
			return e;
		}
		size_ = bytes;
		free_[0] = bytes;
		return cudaSuccess;
	}
	~Arena() {
		if (base_) cudaFree(base_);
	}
	void* alloc(size_t bytes) {
		bytes = align_up(std::max<size_t>(bytes, 1));
		for (auto it = free_.begin(); it != free_.end(); ++it) {
			if (it->second < bytes) continue;
			const size_t off = it->first, rem = it->second - bytes;
			free_.erase(it);
			if (rem) free_[off + bytes] = rem;
			live_[off] = bytes;
			used_ += bytes;
			peak_ = std::max(peak_, used_);
			return static_cast<char*>(base_) + off;
		}
		return nullptr;
	}
	void release(void* p) {
		if (!p) return;
		const size_t off = static_cast<size_t>(static_cast<char*>(p) - static_cast<char*>(base_));
		auto lv = live_.find(off);
		if (lv == live_.end()) return;
		size_t start = off, bytes = lv->second;
		live_.erase(lv);
		used_ -= bytes;
		auto next = free_.find(off + bytes);
		if (next != free_.end()) {
			bytes += next->second;
			free_.erase(next);
		}
		auto prev = free_.lower_bound(off);
		if (prev != free_.begin()) {
			--prev;
			if (prev->first + prev->second == off) {
				start = prev->first;
				bytes += prev->second;
				free_.erase(prev);
			}
		}
		free_[start] = bytes;
	}
	size_t size() const { return size_; }
	size_t used() const { return used_; }
	size_t peak() const { return peak_; }

private:
	void* base_ = nullptr;
	size_t size_ = 0, used_ = 0, peak_ = 0;
	std::map<size_t, size_t> free_, live_;
};

// The requests of one cvx_server_replay call.  They are not entered in the server's id map (a
// replay of millions of requests would grow it without bound, and each rehash of a large map, made
// under the server mutex, stopped the worker and the completion callbacks for tens of
// milliseconds); the worker writes each latency straight into the caller's array at retirement
// and counts the group down.  Guarded by the server mutex.
struct ReplayGroup {
	uint64_t remaining = 0;
	cvx_status first_err = CVX_OK;
	std::string first_msg;
};

struct Request {
	uint64_t id = 0;
	ReplayGroup* group = nullptr;  // set for cvx_server_replay's requests
	double* latency_out = nullptr; // where the worker stores the group request's latency
	cvx_server_request req{};
	bool device_tris = false;     // triangles read in place from req.d_triangles
	bool resident_table = false;  // no host table and kept: the table stays in the arena until released
	bool copy_out = true;         // the table is copied to req.h_table
	bool waited = false;
	size_t tri_bytes = 0, table_bytes = 0, flip_bytes = 0;  // arena bytes (tri_bytes 0 for device_tris)
	void* d_tris = nullptr;
	void* d_table = nullptr;
	void* d_flips = nullptr;
	Clock::time_point arrival;
	double latency_ms = 0;
	cvx_status status = CVX_OK;
	std::string message;
	bool done = false;
};
using RequestP = std::shared_ptr<Request>;

// The most recent kWindow samples of a statistic (a ring once full): a long-running server keeps
// bounded memory, and its percentiles describe recent traffic.
struct Window {
	static constexpr size_t kWindow = size_t(1) << 20;
	std::vector<double> v;
	size_t next = 0;
	Window() { v.reserve(kWindow); }  // grown once here, never under the server mutex
	void push(double x) {
		if (v.size() < kWindow) {
			v.push_back(x);
		} else {
			v[next] = x;
			next = (next + 1) % kWindow;
		}
	}
	bool empty() const { return v.empty(); }
};

struct Slot {
	cudaStream_t stream = nullptr;
	void* staging = nullptr;  // pinned job staging for the engine
	size_t staging_bytes = 0;
	bool busy = false;
	bool finished = false;  // set by the stream callback (under the server mutex)
	Clock::time_point launch_time, finish_time;
	std::vector<RequestP> reqs;
	void* d_rec = nullptr;     // engine records, then the clear list
	size_t rec_bytes = 0;
	cvx::ClearRange* d_clears = nullptr;
	cvx::ClearRange* h_clears = nullptr;  // pinned
	size_t h_clears_n = 0;
	struct cvx_server* server = nullptr;
};

}  // namespace

struct cvx_server {
	cvx_server_config cfg{};
	int device = 0;
	Arena arena;
	std::vector<std::unique_ptr<Slot>> slots;
	std::mutex mu;
	std::condition_variable cv_work, cv_done;
	std::deque<RequestP> pending;
	std::unordered_map<uint64_t, RequestP> live;
	Window latencies;
	Window queue_waits;  // submission to the launch of the request's batch (ms)
	Window services;     // launch to completion of each batch (ms)
	Window issue_us;     // worker time spent issuing each batch's work (us)
	Window replay_late;  // cvx_server_replay: submission after the scheduled arrival (ms)
	uint64_t next_id = 1, completed = 0, batches = 0, batched_requests = 0;
	Clock::time_point first_arrival, last_done;
	bool have_first = false, stop = false;
	std::thread worker;

	static void CUDART_CB on_done(void* p) {
		Slot* sl = static_cast<Slot*>(p);
		cvx_server* s = sl->server;
		{
			std::lock_guard<std::mutex> lk(s->mu);
			sl->finish_time = Clock::now();
			sl->finished = true;
		}
		s->cv_work.notify_one();
	}

	bool any_busy() const {
		for (auto& sl : slots)
			if (sl->busy) return true;
		return false;
	}

	// Allocates a request's device memory; false (nothing held) if the free budget is too small.
	bool admit(Request& r) {
		r.d_tris = r.tri_bytes ? arena.alloc(r.tri_bytes) : nullptr;
		r.d_table = arena.alloc(r.table_bytes);
		r.d_flips = r.flip_bytes ? arena.alloc(r.flip_bytes) : nullptr;
		if ((r.tri_bytes && !r.d_tris) || !r.d_table || (r.flip_bytes && !r.d_flips)) {
			unadmit(r);
			return false;
		}
		return true;
	}
	void unadmit(Request& r) {
		release_work(r);
		arena.release(r.d_table);
		r.d_table = nullptr;
	}
	// The memory a request needs only while its batch runs (its table may stay resident).
	void release_work(Request& r) {
		arena.release(r.d_tris);
		arena.release(r.d_flips);
		r.d_tris = r.d_flips = nullptr;
	}

	static cvx_job job_of(const Request& r) {
		cvx_job j{};
		j.info = r.req.info;
		j.d_triangles = r.device_tris ? r.req.d_triangles : static_cast<const float*>(r.d_tris);
		j.d_table = static_cast<uint32_t*>(r.d_table);
		j.morton = r.req.morton;
		j.solid = r.req.solid;
		return j;
	}

	// Fills slot `sl` with pending requests and their record area; false if nothing fits now.
	bool fill(Slot& sl, size_t* staging_need) {
		while (!pending.empty() && sl.reqs.size() < cfg.max_batch) {
			RequestP r = pending.front();
			if (!admit(*r)) break;
			sl.reqs.push_back(r);
			pending.pop_front();
		}
		while (!sl.reqs.empty()) {
			std::vector<cvx_job> jobs;
			for (auto& r : sl.reqs) jobs.push_back(job_of(*r));
			size_t rec = 0, stage = 0;  // the jobs were validated at submission
			const size_t clears = 2 * sl.reqs.size() * sizeof(cvx::ClearRange);
			if (cvx::batch_scratch_bytes(jobs.data(), (uint32_t)jobs.size(), &rec, &stage) == CVX_OK &&
			    (sl.d_rec = arena.alloc(align_up(rec) + clears)) != nullptr) {
				sl.rec_bytes = rec;
				sl.d_clears = reinterpret_cast<cvx::ClearRange*>(static_cast<char*>(sl.d_rec) + align_up(rec));
				*staging_need = stage;
				return true;
			}
			RequestP back = sl.reqs.back();  // records do not fit: hand the last request back
			sl.reqs.pop_back();
			unadmit(*back);
			pending.push_front(back);
		}
		return false;
	}

	void fail_batch(Slot& sl, cvx_status st, const std::string& msg) {
		for (auto& r : sl.reqs) {
			if (r->status == CVX_OK) {
				r->status = st;
				r->message = msg;
			}
		}
	}

	// Issues a filled slot's work on its stream (no lock held).
	void launch(Slot& sl, size_t staging_need) {
		cudaStream_t st = sl.stream;
		auto cuda_ok = [&](cudaError_t e, const char* what) {
			if (e == cudaSuccess) return true;
			fail_batch(sl, CVX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
			return false;
		};
		bool ok = true;
		if (staging_need > sl.staging_bytes) {
			if (sl.staging) cudaFreeHost(sl.staging);
			sl.staging = nullptr;
			sl.staging_bytes = 0;
			const size_t b = std::max<size_t>(staging_need * 2, 64 << 10);
			ok = cuda_ok(cudaMallocHost(&sl.staging, b), "cudaMallocHost(job staging)");
			if (ok) sl.staging_bytes = b;
		}
		// every table and flip table of the batch zeroed by one kernel
		const size_t n_clears = 2 * sl.reqs.size();
		if (ok && n_clears > sl.h_clears_n) {
			if (sl.h_clears) cudaFreeHost(sl.h_clears);
			sl.h_clears = nullptr;
			sl.h_clears_n = 0;
			ok = cuda_ok(cudaMallocHost((void**)&sl.h_clears, 2 * n_clears * sizeof(cvx::ClearRange)),
			             "cudaMallocHost(clear list)");
			if (ok) sl.h_clears_n = 2 * n_clears;
		}
		uint32_t n_ranges = 0, chunks = 0;
		std::vector<cvx_job> jobs;
		std::vector<uint32_t*> flips;
		for (auto& r : sl.reqs) {
			if (!ok) break;
			if (r->tri_bytes)  // host triangles (device triangles are read in place)
				ok = cuda_ok(cudaMemcpyAsync(r->d_tris, r->req.h_triangles, r->tri_bytes, cudaMemcpyHostToDevice, st),
				             "cudaMemcpyAsync(triangles)");
			const uint64_t words = r->table_bytes / 4;
			if (!r->req.solid || r->req.info.n_triangles == 0) {  // solid tables are overwritten by their resolve
				sl.h_clears[n_ranges++] = cvx::ClearRange{static_cast<uint32_t*>(r->d_table), words, chunks, 0u};
				chunks += cvx::clear_chunks(words);
			}
			if (r->flip_bytes) {
				sl.h_clears[n_ranges++] = cvx::ClearRange{static_cast<uint32_t*>(r->d_flips), words, chunks, 0u};
				chunks += cvx::clear_chunks(words);
			}
			jobs.push_back(job_of(*r));
			flips.push_back(static_cast<uint32_t*>(r->d_flips));
		}
		if (ok)
			ok = cuda_ok(cudaMemcpyAsync(sl.d_clears, sl.h_clears, n_ranges * sizeof(cvx::ClearRange),
			                             cudaMemcpyHostToDevice, st),
			             "cudaMemcpyAsync(clear list)");
		if (ok) ok = cuda_ok(cvx::launch_clear(sl.d_clears, n_ranges, chunks, st), "clear tables");
		if (ok) {
			const cvx_status rs = cvx::run_batch_on(jobs.data(), (uint32_t)jobs.size(), flips.data(), sl.d_rec,
			                                        sl.rec_bytes, sl.staging, sl.staging_bytes, st, true);
			if (rs != CVX_OK) {
				fail_batch(sl, rs, cvx_last_error_message());
				ok = false;
			}
		}
		for (auto& r : sl.reqs) {
			if (!ok) break;
			if (!r->copy_out) continue;
			ok = cuda_ok(cudaMemcpyAsync(r->req.h_table, r->d_table, r->table_bytes, cudaMemcpyDeviceToHost, st),
			             "cudaMemcpyAsync(table)");
		}
		if (cudaLaunchHostFunc(st, on_done, &sl) != cudaSuccess) {
			cudaGetLastError();
			cudaStreamSynchronize(st);  // nothing of this batch may still use its memory
			fail_batch(sl, CVX_ERR_CUDA, "cudaLaunchHostFunc failed");
			std::lock_guard<std::mutex> lk(mu);
			sl.finish_time = Clock::now();
			sl.finished = true;
		}
	}

	void retire(Slot& sl) {
		for (auto& r : sl.reqs) {
			r->latency_ms = std::chrono::duration<double, std::milli>(sl.finish_time - r->arrival).count();
			r->done = true;
			if (r->resident_table) release_work(*r);
			else unadmit(*r);
			latencies.push(r->latency_ms);
			queue_waits.push(std::chrono::duration<double, std::milli>(sl.launch_time - r->arrival).count());
			completed++;
			if (ReplayGroup* g = r->group) {
				*r->latency_out = r->latency_ms;
				if (r->status != CVX_OK && g->first_err == CVX_OK) {
					g->first_err = r->status;
					g->first_msg = r->message;
				}
				g->remaining--;
			}
		}
		last_done = sl.finish_time;
		services.push(std::chrono::duration<double, std::milli>(sl.finish_time - sl.launch_time).count());
		arena.release(sl.d_rec);
		sl.d_rec = nullptr;
		sl.d_clears = nullptr;
		sl.reqs.clear();
		sl.busy = sl.finished = false;
	}

	void run() {
		cudaSetDevice(device);
		std::unique_lock<std::mutex> lk(mu);
		while (true) {
			bool retired = false;
			for (auto& sl : slots) {
				if (sl->busy && sl->finished) {
					retire(*sl);
					retired = true;
				}
			}
			if (retired) cv_done.notify_all();
			bool launched = false;
			for (auto& slp : slots) {
				Slot& sl = *slp;
				if (sl.busy || pending.empty()) continue;
				size_t staging_need = 0;
				if (!fill(sl, &staging_need)) break;  // the head request waits for memory
				sl.busy = true;
				sl.launch_time = Clock::now();
				batches++;
				batched_requests += sl.reqs.size();
				lk.unlock();
				const Clock::time_point t_issue = Clock::now();
				launch(sl, staging_need);
				const double us = std::chrono::duration<double, std::micro>(Clock::now() - t_issue).count();
				lk.lock();
				issue_us.push(us);
				launched = true;
			}
			if (stop && pending.empty() && !any_busy()) break;
			if (!launched && !retired) cv_work.wait_for(lk, std::chrono::milliseconds(10));
		}
	}

	// group (cvx_server_replay): the request is counted in the group and its latency stored at
	// *latency_out instead of being entered in the id map; a group request without a host table is
	// freed at completion instead of staying resident (nobody will read it).
	cvx_status submit(const cvx_server_request* q, Clock::time_point arrival, uint64_t* out_id,
	                  ReplayGroup* group = nullptr, double* latency_out = nullptr) {
		const bool discard_table = group != nullptr;
		if (!q || !out_id) {
			cvx::set_message("cvx_server_submit: null argument");
			return CVX_ERR_INVALID_VALUE;
		}
		const cvx_voxinfo& v = q->info;
		for (int i = 0; i < 3; i++) {
			if (v.gridsize[i] == 0 || v.gridsize[i] > (1u << 22)) {
				cvx::set_message("cvx_server_submit: gridsize out of range");
				return CVX_ERR_INVALID_VALUE;
			}
		}
		if (v.n_triangles && !q->h_triangles && !q->d_triangles) {
			cvx::set_message("cvx_server_submit: no triangles (host or device)");
			return CVX_ERR_INVALID_VALUE;
		}
		if (q->morton) {
			const uint32_t g = v.gridsize[0];
			if (v.gridsize[1] != g || v.gridsize[2] != g || (g & (g - 1))) {
				cvx::set_message("cvx_server_submit: Morton order needs a cubic power-of-two grid");
				return CVX_ERR_UNSUPPORTED;
			}
		}
		auto r = std::make_shared<Request>();
		r->req = *q;
		r->device_tris = q->d_triangles != nullptr;
		r->copy_out = q->h_table != nullptr;
		r->resident_table = !r->copy_out && !discard_table;
		r->tri_bytes = r->device_tris ? 0 : (size_t)v.n_triangles * 9 * sizeof(float);
		r->table_bytes = (size_t)cvx_table_words(&v) * 4;
		r->flip_bytes = q->solid ? r->table_bytes : 0;
		// Fits an empty budget? (its own memory plus the records of a batch holding it alone)
		cvx_job j{};
		j.info = v;
		j.d_triangles = reinterpret_cast<const float*>(kAlign);  // placeholders for validation only
		j.d_table = reinterpret_cast<uint32_t*>(kAlign);
		j.morton = q->morton;
		j.solid = q->solid;
		size_t rec = 0, stage = 0;
		cvx_status st = cvx::batch_scratch_bytes(&j, 1, &rec, &stage);
		if (st != CVX_OK) return st;
		const size_t need = align_up(r->tri_bytes) + align_up(r->table_bytes) + align_up(r->flip_bytes) + align_up(rec);
		if (need > arena.size()) {
			cvx::set_message("cvx_server_submit: request needs " + std::to_string(need) +
			                 " bytes, more than the whole memory budget");
			return CVX_ERR_OUT_OF_MEMORY;
		}
		{
			std::lock_guard<std::mutex> lk(mu);
			r->id = next_id++;
			r->arrival = arrival;
			if (!have_first || arrival < first_arrival) first_arrival = arrival;
			have_first = true;
			pending.push_back(r);
			if (group) {
				r->group = group;
				r->latency_out = latency_out;
				group->remaining++;
			} else {
				live[r->id] = r;
			}
			*out_id = r->id;
		}
		cv_work.notify_one();
		return CVX_OK;
	}

	// A completed request's resident table: its device address, or its release.
	cvx_status table(uint64_t id, uint32_t** d_table) {
		std::lock_guard<std::mutex> lk(mu);
		auto it = live.find(id);
		if (it == live.end() || !it->second->resident_table || !it->second->done) {
			cvx::set_message("cvx_server_table: no completed request with a resident table under this id");
			return CVX_ERR_INVALID_VALUE;
		}
		*d_table = static_cast<uint32_t*>(it->second->d_table);
		return CVX_OK;
	}
	cvx_status release(uint64_t id) {
		std::lock_guard<std::mutex> lk(mu);
		auto it = live.find(id);
		if (it == live.end() || !it->second->resident_table || !it->second->done) {
			cvx::set_message("cvx_server_release: no completed request with a resident table under this id");
			return CVX_ERR_INVALID_VALUE;
		}
		arena.release(it->second->d_table);
		it->second->d_table = nullptr;
		live.erase(it);
		cv_work.notify_one();  // memory came free: pending requests may fit now
		return CVX_OK;
	}

	cvx_status wait(uint64_t id, double timeout_ms, double* latency_ms) {
		std::unique_lock<std::mutex> lk(mu);
		auto it = live.find(id);
		if (it == live.end()) {
			cvx::set_message("cvx_server_wait: unknown request id");
			return CVX_ERR_INVALID_VALUE;
		}
		RequestP r = it->second;
		auto is_done = [&] { return r->done; };
		if (timeout_ms < 0) {
			cv_done.wait(lk, is_done);
		} else if (!cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), is_done)) {
			cvx::set_message("cvx_server_wait: timed out");
			return CVX_ERR_INVALID_VALUE;
		}
		r->waited = true;
		if (!r->resident_table || r->status != CVX_OK) {
			if (r->resident_table) {
				arena.release(r->d_table);
				r->d_table = nullptr;
			}
			live.erase(id);
		}
		if (latency_ms) *latency_ms = r->latency_ms;
		if (r->status != CVX_OK) cvx::set_message(r->message);
		return r->status;
	}
};

static_assert(sizeof(cvx_server_stats) == 136, "cvx_server_stats layout (the Python binding mirrors it)");
static_assert(sizeof(cvx_server_request) == 96, "cvx_server_request layout (the Python binding mirrors it)");

extern "C" {

cvx_status cvx_server_create(const cvx_server_config* cfg, cvx_server** out) {
	if (!cfg || !out || cfg->memory_budget_bytes < (1u << 20) || cfg->max_batch == 0 || cfg->max_batch > 65536 ||
	    cfg->max_inflight == 0 || cfg->max_inflight > 64) {
		cvx::set_message("cvx_server_create: need a budget of at least 1 MiB, 0 < max_batch <= 65536, "
		                 "0 < max_inflight <= 64");
		return CVX_ERR_INVALID_VALUE;
	}
	auto s = std::make_unique<cvx_server>();
	s->cfg = *cfg;
	if (cudaGetDevice(&s->device) != cudaSuccess) {
		cvx::set_message("cvx_server_create: no CUDA device");
		return CVX_ERR_CUDA;
	}
	if (s->arena.init(cfg->memory_budget_bytes) != cudaSuccess) {
		cudaGetLastError();
		cvx::set_message("cvx_server_create: cannot allocate the memory budget");
		return CVX_ERR_OUT_OF_MEMORY;
	}
	// Each slot's pinned host buffers are allocated here, not while serving: a pinned allocation is
	// a slow driver call that holds up the other streams' launches.  The clear list is exact
	// (a table and a flip table per request); the job staging covers every batch of max_batch
	// jobs that no launch has to split (over 2^24 triangles), and only grows for one that does.
	const size_t staging_bytes = std::max<size_t>((4 * (size_t)cfg->max_batch + 64) * sizeof(cvx::JobDesc), (size_t)64 << 10);
	for (uint32_t i = 0; i < cfg->max_inflight; i++) {
		auto sl = std::make_unique<Slot>();
		sl->server = s.get();
		bool ok = cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking) == cudaSuccess;
		if (ok) ok = cudaMallocHost(&sl->staging, staging_bytes) == cudaSuccess;
		if (ok) sl->staging_bytes = staging_bytes;
		if (ok) ok = cudaMallocHost((void**)&sl->h_clears, 2 * (size_t)cfg->max_batch * sizeof(cvx::ClearRange)) == cudaSuccess;
		if (ok) sl->h_clears_n = 2 * (size_t)cfg->max_batch;
		s->slots.push_back(std::move(sl));
		if (!ok) {
			cudaGetLastError();
			for (auto& o : s->slots) {
				if (o->stream) cudaStreamDestroy(o->stream);
				if (o->staging) cudaFreeHost(o->staging);
				if (o->h_clears) cudaFreeHost(o->h_clears);
			}
			cvx::set_message("cvx_server_create: cannot create streams or pinned staging");
			return CVX_ERR_CUDA;
		}
	}
	// Room for a burst of requests up front: growing these under the server mutex (a rehash of the
	// request map) would hold up the worker while it is copied.
	s->live.reserve(1 << 16);
	cvx_server* p = s.release();
	p->worker = std::thread([p] { p->run(); });
	*out = p;
	return CVX_OK;
}

cvx_status cvx_server_submit(cvx_server* s, const cvx_server_request* req, uint64_t* out_id) {
	if (!s) {
		cvx::set_message("cvx_server_submit: server is null");
		return CVX_ERR_INVALID_VALUE;
	}
	return s->submit(req, Clock::now(), out_id);
}

cvx_status cvx_server_wait(cvx_server* s, uint64_t id, double timeout_ms, double* latency_ms) {
	if (!s) {
		cvx::set_message("cvx_server_wait: server is null");
		return CVX_ERR_INVALID_VALUE;
	}
	return s->wait(id, timeout_ms, latency_ms);
}

cvx_status cvx_server_table(cvx_server* s, uint64_t id, uint32_t** d_table) {
	if (!s || !d_table) {
		cvx::set_message("cvx_server_table: null argument");
		return CVX_ERR_INVALID_VALUE;
	}
	return s->table(id, d_table);
}

cvx_status cvx_server_release(cvx_server* s, uint64_t id) {
	if (!s) {
		cvx::set_message("cvx_server_release: server is null");
		return CVX_ERR_INVALID_VALUE;
	}
	return s->release(id);
}

cvx_status cvx_server_stats_get(cvx_server* s, cvx_server_stats* out) {
	if (!s || !out) {
		cvx::set_message("cvx_server_stats_get: null argument");
		return CVX_ERR_INVALID_VALUE;
	}
	std::memset(out, 0, sizeof(*out));
	// Copy under the lock, sort outside it: the worker and the completion callbacks need the mutex.
	std::vector<double> lat, queue, svc, issue, late;
	double span = 0.0;
	{
		std::lock_guard<std::mutex> lk(s->mu);
		out->completed = s->completed;
		out->pending = s->pending.size();
		out->batches = s->batches;
		out->mean_batch = s->batches ? (double)s->batched_requests / (double)s->batches : 0.0;
		out->memory_used = s->arena.used();
		out->memory_budget = s->arena.size();
		out->memory_peak = s->arena.peak();
		lat = s->latencies.v;
		queue = s->queue_waits.v;
		svc = s->services.v;
		issue = s->issue_us.v;
		late = s->replay_late.v;
		if (!lat.empty()) span = std::chrono::duration<double>(s->last_done - s->first_arrival).count();
	}
	auto pct = [](std::vector<double>& v, double q) {
		return v[std::min(v.size() - 1, (size_t)(q * (double)(v.size() - 1) + 0.5))];
	};
	for (std::vector<double>* v : {&lat, &queue, &svc, &issue, &late}) std::sort(v->begin(), v->end());
	if (!queue.empty()) out->queue_p99_ms = pct(queue, 0.99);
	if (!svc.empty()) {
		out->service_p50_ms = pct(svc, 0.50);
		out->service_p99_ms = pct(svc, 0.99);
	}
	if (!issue.empty()) out->issue_p50_us = pct(issue, 0.50);
	if (!late.empty()) {
		out->replay_late_p99_ms = pct(late, 0.99);
		out->replay_late_max_ms = late.back();
	}
	if (!lat.empty()) {
		out->p50_ms = pct(lat, 0.50);
		out->p99_ms = pct(lat, 0.99);
		out->max_ms = lat.back();
		out->meshes_per_s = span > 0 ? (double)out->completed / span : 0.0;
	}
	return CVX_OK;
}

cvx_status cvx_server_replay(cvx_server* s, const cvx_server_request* reqs, uint32_t n, const double* arrival_s,
                             double* latency_ms) {
	if (!s || (n && (!reqs || !arrival_s || !latency_ms))) {
		cvx::set_message("cvx_server_replay: null argument");
		return CVX_ERR_INVALID_VALUE;
	}
	for (uint32_t i = 1; i < n; i++) {
		if (arrival_s[i] < arrival_s[i - 1]) {
			cvx::set_message("cvx_server_replay: arrival times must ascend");
			return CVX_ERR_INVALID_VALUE;
		}
	}
	std::vector<double> late(n);
	ReplayGroup group;
	const Clock::time_point t0 = Clock::now();
	cvx_status st = CVX_OK;
	uint32_t submitted = 0;
	for (uint32_t i = 0; i < n && st == CVX_OK; i++) {
		const auto due = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[i]));
		// sleep to 50 us before the arrival, then spin: a generator that spins longer keeps a whole
		// core busy at high rates and competes with the server's own threads
		if (due - Clock::now() > std::chrono::microseconds(100)) std::this_thread::sleep_until(due - std::chrono::microseconds(50));
		Clock::time_point now;
		while ((now = Clock::now()) < due) {
		}
		late[i] = std::chrono::duration<double, std::milli>(now - due).count();
		uint64_t id = 0;
		st = s->submit(&reqs[i], due, &id, &group, &latency_ms[i]);
		if (st == CVX_OK) submitted++;
	}
	const std::string submit_msg = st == CVX_OK ? std::string() : cvx_last_error_message();
	// Generator lateness into the statistics, a slice at a time so the worker is not held up.
	for (uint32_t i = 0; i < submitted; i += 4096) {
		std::lock_guard<std::mutex> lk(s->mu);
		for (uint32_t k = i; k < std::min(submitted, i + 4096); k++) s->replay_late.push(late[k]);
	}
	std::unique_lock<std::mutex> lk(s->mu);
	s->cv_done.wait(lk, [&] { return group.remaining == 0; });  // every submitted request retired
	if (st != CVX_OK) {
		cvx::set_message(submit_msg);
		return st;
	}
	if (group.first_err != CVX_OK) cvx::set_message(group.first_msg);
	return group.first_err;
}

cvx_status cvx_server_destroy(cvx_server* s) {
	if (!s) return CVX_OK;
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->stop = true;
	}
	s->cv_work.notify_all();
	if (s->worker.joinable()) s->worker.join();
	for (auto& sl : s->slots) {
		cudaStreamSynchronize(sl->stream);
		cudaStreamDestroy(sl->stream);
		if (sl->staging) cudaFreeHost(sl->staging);
		if (sl->h_clears) cudaFreeHost(sl->h_clears);
	}
	delete s;
	return CVX_OK;
}

}  // extern "C"
