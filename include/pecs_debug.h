/*
 * pecs_debug.h -- diagnostics of the pecs C ABI that involve no GPU.
 *
 * pecs_lu_host_apply applies, on the host, the multifrontal factors that
 * pecs_lu_factor computed (before they are uploaded to the device by the
 * first pecs_lu_solve*).  It exists so that the ordering and factorisation
 * logic can be checked on machines without a GPU; no product path calls it.
 * pecs_debug_time_levels times the levels of a solve sweep for profiling.
 */
#ifndef PECS_DEBUG_H
#define PECS_DEBUG_H
#include "pecs.h"
#ifdef __cplusplus
extern "C" {
#endif
int pecs_lu_host_apply(pecs_lu* lu, const double* b, double* x);
/* Device time of every level launch of one carrier (which = 0) or Poisson (1)
 * solve sweep of a context with FP32 panel sweeps (forward levels, then
 * backward), CUDA events between the launches, mean of `reps` sweeps after a
 * warm-up.  Returns the number of levels written to ms (at most cap), or a
 * negative error code.  The sweep's outputs are overwritten. */
int pecs_debug_time_levels(pecs_ctx* ctx, int which, int reps, double* ms, int cap);
/* The stored factor values of a pecs_lu handle (before its first solve
 * uploads them): every node's Gf then Hb, nodes in elimination order, into
 * out (capacity n doubles); returns the count via *count (out may be NULL to
 * query it). */
int pecs_debug_lu_values(pecs_lu* lu, double* out, long long n, long long* count);
#ifdef __cplusplus
}
#endif
#endif
