/*
 * pecs_debug.h -- diagnostics of the pecs C ABI that involve no GPU.
 *
 * pecs_lu_host_apply applies, on the host, the multifrontal factors that
 * pecs_lu_factor computed (before they are uploaded to the device by the
 * first pecs_lu_solve*).  It exists so that the ordering and factorisation
 * logic can be checked on machines without a GPU; no product path calls it.
 */
#ifndef PECS_DEBUG_H
#define PECS_DEBUG_H
#include "pecs.h"
#ifdef __cplusplus
extern "C" {
#endif
int pecs_lu_host_apply(pecs_lu* lu, const double* b, double* x);
#ifdef __cplusplus
}
#endif
#endif
