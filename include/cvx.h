/*
 * cvx.h -- C ABI of the GB300 voxelization engine (cuda_voxelizer_gb300).
 *
 * Drop-in for the voxelization path of Forceflow/cuda_voxelizer v0.6: surface voxelization
 * (`voxelize`, src/voxelize.cu:192-238) and solid voxelization (`voxelize_solid`,
 * src/voxelize_solid.cu:147-193) of an fp32 triangle soup into a bit-packed uint32 table, in linear
 * or Morton order.  Plain pointers and sizes only; device pointers may be cudaMalloc'ed or managed
 * memory (the reference's callers pass cudaMallocManaged buffers, src/main.cpp:66,214).
 *
 * Semantics kept from the reference:
 *   - the table holds ceil(gx*gy*gz/32) words; voxel (x,y,z) is linear index x + y*gx + z*gx*gy
 *     (src/voxelize.cu:175-178) or its Morton code (src/voxelize.cuh:20-34); word = idx/32 and the
 *     bit is 31 - idx%32, most significant bit first (src/voxelize.cu:50-55, src/util.h:25-38);
 *   - surface ORs into the table and solid XORs into it, so the caller zeroes it first
 *     (the reference relies on fresh managed pages, src/main.cpp:214);
 *   - every bit is identical to the reference kernels' result on the same input.
 * Differences, all at the interface: calls are asynchronous on the given stream, return a status
 * instead of calling exit(), never print, and allocate their scratch once per (device, stream)
 * (see cvx_voxelize_ws for caller-owned scratch).  The C++ symbols with the reference's exact
 * signatures are declared in cvx_dropin.h.
 */
#ifndef CVX_H_
#define CVX_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CVX_VERSION_MAJOR 1
#define CVX_VERSION_MINOR 1

/* Same bytes as the reference's voxinfo (src/util.h:50-69) on LP64 targets:
 * AABox<float3> bbox @0, uint3 gridsize @24, size_t n_triangles @40, float3 unit @48, 64 bytes. */
typedef struct cvx_voxinfo {
	float bbox_min[3];
	float bbox_max[3];
	uint32_t gridsize[3];
	uint32_t _pad0;
	uint64_t n_triangles;
	float unit[3];
	uint32_t _pad1;
} cvx_voxinfo;

typedef enum cvx_status {
	CVX_OK = 0,
	CVX_ERR_INVALID_VALUE = 1,   /* null pointer, zero grid, bad size */
	CVX_ERR_UNSUPPORTED = 2,     /* e.g. Morton order on a grid that is not a cubic power of two */
	CVX_ERR_OUT_OF_MEMORY = 3,   /* scratch allocation failed */
	CVX_ERR_CUDA = 4,            /* a CUDA runtime call failed (see cvx_last_error_message) */
	CVX_ERR_DEVICE_CHECK = 5,    /* a device-side check reported a problem (cvx_device_status) */
	CVX_ERR_CAPTURING = 6        /* the call would allocate while the stream is being captured */
} cvx_status;

/* cudaStream_t without including the CUDA headers (the same type). */
typedef struct CUstream_st* cvx_stream_t;

const char* cvx_status_string(cvx_status s);
/* Message of the last failed call on this host thread. */
const char* cvx_last_error_message(void);
int cvx_version(void); /* MAJOR*1000 + MINOR */

/* ---- host-side setup (replaces src/util.h:56-61, :80-110 and src/main.cpp:179,190) ---------- */

/* voxinfo constructor: unit = (bbox_max - bbox_min) / float(gridsize), per axis. */
cvx_status cvx_voxinfo_init(cvx_voxinfo* out, const float bbox_min[3], const float bbox_max[3],
                            const uint32_t gridsize[3], uint64_t n_triangles);
/* createMeshBBCube: pad the box to a cube, then by extent/10001 on every side. */
cvx_status cvx_bbox_cube(const float in_min[3], const float in_max[3], float out_min[3], float out_max[3]);
/* Vertex min/max of a host triangle soup (9 floats per triangle); what Trimesh need_bbox computes. */
cvx_status cvx_mesh_bbox(const float* triangles, uint64_t n_triangles, float out_min[3], float out_max[3]);
/* Words of the bit table: ceil(gx*gy*gz / 32), computed exactly (src/main.cpp:190 goes through a
 * float ceil, which is exact for power-of-two grids). */
uint64_t cvx_table_words(const cvx_voxinfo* info);

/* ---- single mesh ------------------------------------------------------------------------------ */

/* Surface voxelization; replaces voxelize() (src/voxelize.cu:192) and its kernel voxelize_triangle
 * (src/voxelize.cu:58).  ORs into d_table.  morton != 0 needs a cubic power-of-two grid. */
cvx_status cvx_voxelize(const cvx_voxinfo* info, const float* d_triangles, uint32_t* d_table, int morton,
                        cvx_stream_t stream);

/* Solid voxelization; replaces voxelize_solid() (src/voxelize_solid.cu:147) and its kernel
 * voxelize_triangle_solid (src/voxelize_solid.cu:73).  XORs into d_table. */
cvx_status cvx_voxelize_solid(const cvx_voxinfo* info, const float* d_triangles, uint32_t* d_table, int morton,
                              cvx_stream_t stream);

/* Bytes of caller-owned scratch needed by cvx_voxelize_ws for this mesh and mode. */
uint64_t cvx_workspace_size(const cvx_voxinfo* info, int solid);

/* cvx_voxelize / cvx_voxelize_solid with caller-owned scratch (no allocation inside; usable while
 * the stream is being captured into a CUDA graph).  d_workspace: device memory of at least
 * cvx_workspace_size() bytes, 256-byte aligned; its contents need not be preserved between calls. */
cvx_status cvx_voxelize_ws(const cvx_voxinfo* info, const float* d_triangles, uint32_t* d_table, int morton,
                           int solid, void* d_workspace, uint64_t workspace_bytes, cvx_stream_t stream);

/* Solid voxelization that allocates nothing (no counterpart in the reference).  For callers that must
 * not allocate device memory while voxelizing -- e.g. per-frame code that budgets all GPU memory at
 * start-up (an allocation mid-frame can stall the device or fail under memory pressure), or hosts
 * whose memory policy forbids driver allocations.  Same result as cvx_voxelize_solid.  Its scratch
 * is a fixed 4 MiB array inside the library (held by every GPU that loads it until exit), so the
 * grid may hold at most 2^24 voxels (e.g. 256^3); larger grids return CVX_ERR_INVALID_VALUE, and
 * the other argument checks are those of cvx_voxelize_solid (axes up to 2^22).  The first call on a
 * device (and in each new CUDA context of it, e.g. after cudaDeviceReset) looks up that array's
 * device address and should come before any stream capture.  All calls share the array: calls that
 * overlap on the GPU race, so issue them one at a time.  Device-side checks of the last call are
 * reported by cvx_device_status (pass the stream the call ran on). */
cvx_status cvx_voxelize_solid_noalloc(const cvx_voxinfo* info, const float* d_triangles, uint32_t* d_table,
                                      int morton, cvx_stream_t stream);

/* Synchronizes `stream` and reports device-side checks of the last calls made on it through the
 * library-owned scratch, and of the last cvx_voxelize_solid_noalloc call on the current device:
 * CVX_OK, or CVX_ERR_DEVICE_CHECK (a queue overflow or a timed-out copy; the call's table is then
 * incomplete). */
cvx_status cvx_device_status(cvx_stream_t stream);

/* Synchronizes `stream` and frees the scratch the library allocated for it (on the current device).
 * Call it before destroying a stream used with the library: a later stream can get the same handle,
 * and would otherwise share scratch with work still running on the old one.  Calls on the stream
 * afterwards allocate afresh; a stream the library never used returns CVX_OK at once. */
cvx_status cvx_stream_release(cvx_stream_t stream);

/* ---- batches: many meshes of different sizes, grids and modes in one launch sequence ---------- */

typedef struct cvx_job {
	cvx_voxinfo info;
	const float* d_triangles;
	uint32_t* d_table;
	int32_t morton;
	int32_t solid;
} cvx_job;

/* All jobs in one launch sequence (a fixed handful of kernels whatever the job count); the
 * tables of different jobs must not overlap.  Results are bit-identical to one call per job. */
cvx_status cvx_voxelize_batch(const cvx_job* jobs, uint32_t n_jobs, cvx_stream_t stream);

/* A batch prepared once and replayed as one CUDA graph launch. */
typedef struct cvx_plan cvx_plan;
/* CVX_PLAN_CLEAR_TABLES: every launch gives each table exactly what voxelizing into a zeroed table
 * gives, whatever the table held (surface tables are zeroed inside the graph, solid tables are
 * written word by word).  Jobs whose tables share words accumulate into them (OR, then XOR).
 * Without the flag, jobs OR / XOR into their tables like the per-call functions. */
#define CVX_PLAN_CLEAR_TABLES 1u
cvx_status cvx_plan_create(const cvx_job* jobs, uint32_t n_jobs, uint32_t flags, cvx_plan** out);
cvx_status cvx_plan_launch(cvx_plan* plan, cvx_stream_t stream);
/* Number of kernel launches one cvx_plan_launch makes (the graph's kernel nodes; copies and memsets
 * not counted).  Works for host-buffer plans too. */
cvx_status cvx_plan_kernel_nodes(const cvx_plan* plan, uint32_t* n_kernels);
cvx_status cvx_plan_destroy(cvx_plan* plan);

/* Host-buffer plans: the reference's round trip (src/main.cpp:209-222 hands voxelize host-visible
 * triangles and table) as one graph.  Each launch copies every job's triangles from h_triangles into
 * d_triangles, zeroes d_table, voxelizes, and copies d_table into h_table; the tables are
 * bit-identical to plain calls.  Meshes go up in job order, each in n_chunks pieces (0 = 2, at most
 * 64); the surface jobs voxelize each piece as soon as it lands, the solid jobs follow the mesh's
 * last piece, and each table is copied down as soon as it is complete, so the kernels run under
 * the copies and the link stays busy.  Jobs that share
 * d_triangles must share h_triangles and n_triangles (one upload serves them); different uploads
 * and different tables must not overlap.  Host buffers must be page-locked (cudaHostAlloc or
 * cudaHostRegister).  Launch with cvx_plan_launch; the host tables are complete when the launch's
 * stream reaches the point after it.  Destroy with cvx_plan_destroy.  Plans share no device state:
 * host plans over their own device buffers and host tables may be in flight at once on different
 * streams (one plan's launches run one after another), which overlaps one round trip's upload with
 * another's read-back. */
typedef struct cvx_host_job {
	cvx_voxinfo info;
	const float* h_triangles; /* host source, n_triangles * 9 floats */
	float* d_triangles;       /* device copy of them, written by the plan */
	uint32_t* d_table;        /* device table (zeroed by the plan) */
	uint32_t* h_table;        /* host destination of the table */
	int32_t morton;
	int32_t solid;
} cvx_host_job;
cvx_status cvx_plan_create_host(const cvx_host_job* jobs, uint32_t n_jobs, uint32_t n_chunks, cvx_plan** out);

/* ---- serving: requests admitted by device memory and batched continuously --------------------
 * No counterpart in the reference (src/main.cpp voxelizes one mesh per process).  A server owns
 * one device arena of memory_budget_bytes (allocated at creation, nothing else is allocated while
 * serving) holding every admitted request's triangles, table, solid flip table and its batch's
 * work records, and max_inflight streams.  A worker thread launches pending requests as one
 * batch (at most max_batch requests, in arrival order, as many as the free budget holds) whenever
 * a stream is free, so requests that arrive while others run go into the next batch and overlap
 * with them.  A request's host triangles are copied in and its table copied out within its batch
 * (host buffers should be pinned for the copies to overlap); device-resident triangles are read in
 * place and a request without a host table keeps its table resident on the device.  Results are
 * identical to cvx_voxelize / cvx_voxelize_solid on the same request. */
typedef struct cvx_server cvx_server;
typedef struct cvx_server_config {
	uint64_t memory_budget_bytes;
	uint32_t max_batch;     /* requests per launch sequence, 1 .. 65536 */
	uint32_t max_inflight;  /* batches on the GPU at once (one stream each) */
} cvx_server_config;
typedef struct cvx_server_request {
	cvx_voxinfo info;
	const float* h_triangles;  /* host, 9 floats per triangle, copied in; read until completion */
	const float* d_triangles;  /* or device-resident triangles, read in place (then h_ is ignored) */
	uint32_t* h_table;         /* host table, cvx_table_words(&info) words, written by completion;
	                            * NULL: the table stays resident in the server's budget after
	                            * completion (cvx_server_table) until cvx_server_release */
	int32_t morton;
	int32_t solid;
} cvx_server_request;
typedef struct cvx_server_stats {
	uint64_t completed, pending, batches;
	double mean_batch;                    /* requests per batch */
	uint64_t memory_used, memory_budget;  /* arena bytes now in use / in total */
	uint64_t memory_peak;                 /* most arena bytes ever in use at once */
	double p50_ms, p99_ms, max_ms;        /* latency, submission to table written; these and the
	                                       * other percentiles cover the last 2^20 samples */
	double meshes_per_s;                  /* completed / (last completion - first submission) */
	double queue_p99_ms;                  /* submission to the launch of the request's batch, p99 */
	double replay_late_p99_ms;            /* cvx_server_replay: how late its submissions were against */
	double replay_late_max_ms;            /*   the schedule (p99, maximum); latency counts from the schedule */
	double service_p50_ms, service_p99_ms; /* a batch's launch to completion (copies in, kernels, copies out) */
	double issue_p50_us;                  /* host time the worker spends issuing one batch's work */
} cvx_server_stats;
/* CVX_ERR_OUT_OF_MEMORY if the budget cannot be allocated. */
cvx_status cvx_server_create(const cvx_server_config* cfg, cvx_server** out);
/* Queues one request.  CVX_ERR_OUT_OF_MEMORY if it would not fit even in an empty budget. */
cvx_status cvx_server_submit(cvx_server* s, const cvx_server_request* req, uint64_t* out_id);
/* Waits for request `id` (timeout_ms < 0: no limit) and forgets it; returns its status.  A timeout
 * returns CVX_ERR_INVALID_VALUE and keeps the request. */
cvx_status cvx_server_wait(cvx_server* s, uint64_t id, double timeout_ms, double* latency_ms);
/* Device address of a completed request's resident table (valid until cvx_server_release). */
cvx_status cvx_server_table(cvx_server* s, uint64_t id, uint32_t** d_table);
/* Frees a completed request's resident table and forgets the request. */
cvx_status cvx_server_release(cvx_server* s, uint64_t id);
cvx_status cvx_server_stats_get(cvx_server* s, cvx_server_stats* out);
/* Open-loop load: submits reqs[i] at arrival_s[i] seconds after the call starts (arrival_s
 * ascending), waits for all and writes each latency, counted from its scheduled arrival.
 * Tables of requests without a host table are freed as the requests complete (nothing reads
 * them), so a replay measures voxelization with device-resident output. */
cvx_status cvx_server_replay(cvx_server* s, const cvx_server_request* reqs, uint32_t n, const double* arrival_s,
                             double* latency_ms);
/* Finishes the queued requests, then frees everything. */
cvx_status cvx_server_destroy(cvx_server* s);

/* ---- mesh ingest on the GPU (replaces src/main.cpp:61-80 and :179-186) ------------------------ */

/* Vertex bounding box of a device triangle soup (min/max over the 3n vertices, as Trimesh's
 * need_bbox); synchronizes `stream` and writes the host arrays.  Equal to cvx_mesh_bbox for finite
 * coordinates. */
cvx_status cvx_mesh_bbox_device(const float* d_triangles, uint64_t n_triangles, float out_min[3], float out_max[3],
                                cvx_stream_t stream);
/* main()'s setup from a device soup: bounding box, createMeshBBCube, voxinfo (synchronizes). */
cvx_status cvx_voxinfo_from_device(const float* d_triangles, uint64_t n_triangles, const uint32_t gridsize[3],
                                   cvx_voxinfo* out, cvx_stream_t stream);
/* Indexed mesh -> soup: face f's vertices d_vertices[3*d_faces[3f+k] ..] become floats 9f..9f+8
 * of d_soup (the loop of meshToGPU_managed, src/main.cpp:68-77).  A face with an index >=
 * n_vertices is written as NaNs and counted into *d_bad_faces (device counter, may be NULL);
 * such a soup must not be voxelized.  Asynchronous. */
cvx_status cvx_gather_soup(const float* d_vertices, uint64_t n_vertices, const uint32_t* d_faces, uint64_t n_faces,
                           float* d_soup, unsigned long long* d_bad_faces, cvx_stream_t stream);

/* ---- table layouts and output encoders ------------------------------------------------------ */

/* Morton <-> linear conversion of a g^3 table (g a power of two, 4 <= g <= 65536); source and
 * destination must not overlap.  to_morton != 0: linear -> Morton.  Asynchronous. */
cvx_status cvx_transcode(const uint32_t* d_src, uint32_t* d_dst, uint32_t gridsize, int to_morton,
                         cvx_stream_t stream);
/* binvox payload of a linear-order table: the (value, count) byte pairs write_binvox emits after
 * its ASCII header (src/util_io.cpp:219-245: x outermost, then z, then y; runs end on a change or
 * after 255 voxels).  *out_bytes receives the payload size; with d_out == NULL only the size is
 * computed, and a capacity below it returns CVX_ERR_INVALID_VALUE.  Synchronizes `stream`; uses
 * temporary device memory. */
cvx_status cvx_encode_binvox(const cvx_voxinfo* info, const uint32_t* d_table, uint8_t* d_out, uint64_t out_capacity,
                             uint64_t* out_bytes, cvx_stream_t stream);
/* The voxels write_vox hands to VoxWriter::AddVoxel (src/util_io.cpp:264-280), in its order, as
 * int32 triples (x, gz - z, y) into d_xyz (3 * capacity int32).  Needs gridsize y == z.
 * *out_count receives the number of set voxels; d_xyz == NULL computes only that.  Synchronizes. */
cvx_status cvx_encode_voxel_list(const cvx_voxinfo* info, const uint32_t* d_table, int32_t* d_xyz, uint64_t capacity,
                                 uint64_t* out_count, cvx_stream_t stream);

/* ---- tuning ---------------------------------------------------------------------------------- */

typedef struct cvx_tuning {
	uint32_t small_vox;   /* surface: triangles with at most this many bbox voxels stay in one thread */
	uint32_t small_cols;  /* solid: triangles with at most this many columns stay in one thread */
	uint32_t brick_pairs; /* surface, grids of 2^29+ voxels: (brick, triangle) pairs per triangle the
	                       * shared-memory brick rasterizer may use, at most 16; 0 (the default)
	                       * rasterizes every larger triangle row by row with global atomics instead */
} cvx_tuning;
/* Per-device tuning used by subsequent calls (results never depend on it). */
cvx_status cvx_get_tuning(int device, cvx_tuning* out);
cvx_status cvx_set_tuning(int device, const cvx_tuning* in);

/* ---- per-kernel timing ---------------------------------------------------------------------- */

/* When enabled, calls made by this host thread record a CUDA event after each engine kernel on
 * their stream.  cvx_profile_collect waits for those events, writes up to max_entries (kernel
 * name, milliseconds) pairs in launch order and forgets them.  Names are static strings. */
cvx_status cvx_profile_enable(int on);
int cvx_profile_collect(const char** names, float* ms, int max_entries);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* CVX_H_ */
