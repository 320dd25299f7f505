/*
 * cvx_diag.h -- diagnostics beside the voxelization library: not part of its ABI, no counterpart
 * in the reference.  Provided by cuda_voxelizer_gb300/_lib/libcvx_diag.so (a separate library, so
 * that libcvx.so exports only the voxelization interface of cvx.h and cvx_dropin.h).
 *
 * cvx_microbench_atomic_or measures the rate of 32-bit global atomicOr into a table, the peak the
 * engine's roofline divides its atomic term by (the HBM and tensor peaks come from elsewhere):
 * atomics per second into d_table (`words` long), pattern 0 scattered lanes, 1 one 128-byte line
 * per warp, 2 eight consecutive words per lane; `blocks` CTAs of 256 threads, `iters` atomics per
 * thread.  Synchronous.
 */
#ifndef CVX_DIAG_H_
#define CVX_DIAG_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

double cvx_microbench_atomic_or(uint32_t* d_table, uint64_t words, int pattern, uint32_t blocks, uint32_t iters);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* CVX_DIAG_H_ */
