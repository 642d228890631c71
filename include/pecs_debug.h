/*
 * pecs_debug.h -- diagnostics of the pecs C ABI; no product path calls them.
 *
 * pecs_lu_host_apply applies, on the host, the multifrontal factors that
 * pecs_lu_factor computed (before they are uploaded to the device by the
 * first pecs_lu_solve*), so that the ordering and factorisation logic can be
 * checked on machines without a GPU; pecs_debug_lu_values exports them.
 * pecs_debug_time_levels times the levels of a solve sweep for profiling, and
 * pecs_debug_flow_stall exercises the bounded waits of the flow sweeps.
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
/* Contexts whose carrier (which = 0) or Poisson (1) bank uses the flow sweep:
 * sets the first factor's root counter of the next forward flow sweep far
 * below its target, runs one solve sweep of that bank (the root's waits run
 * out after their poll limit), and returns in *flag the bank's flow error
 * flag (1: a wait ran out and that sweep wrote NaN), clearing it.  The
 * sweep's outputs are overwritten; the context stays usable. */
int pecs_debug_flow_stall(pecs_ctx* ctx, int which, int* flag);
#ifdef __cplusplus
}
#endif
#endif
