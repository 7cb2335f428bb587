/*
 * ggem_noalloc.h -- the local mobility matvec without any allocation.
 *
 * This entry point has no counterpart in the reference.  It exists for
 * callers that cannot call cudaMalloc: code whose device memory is entirely
 * held by another allocator (a framework's caching pool or a solver's own
 * memory arena), code running where a device allocation would block or is
 * not permitted (inside a solver callback or a real-time loop), and builds
 * that budget device memory statically.  Those callers cannot create a
 * ggem_ctx, which allocates its cell lists and workspaces.
 *
 * ggem_local_matvec_noalloc computes the same u = M_loc f as
 * ggem_local_matvec_dev on a GGEM_FP64 / GGEM_NB_CUTOFF context (the FP64
 * cut-off cell-list pair sweep plus the chosen self term), but keeps every
 * intermediate array in one fixed device array of GGEM_NOALLOC_SCRATCH_BYTES
 * (2.5 MiB) compiled into the library.  Every GPU that loads the library
 * holds that array until the process exits.
 *
 * Limits: at most GGEM_NOALLOC_MAX_PARTICLES particles and
 * GGEM_NOALLOC_MAX_CELLS cells of side >= rc (floor(edge / rc) per axis);
 * larger inputs return GGEM_ERR_BAD_ARG without launching anything.
 *
 * Sharing: all calls use the same array, which keeps the last call's
 * contents; each call clears the counters it needs.  Calls that overlap on
 * the GPU (on different streams, or from different host threads) race on
 * the array: serialise them.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.
 */
#ifndef GGEM_NOALLOC_H
#define GGEM_NOALLOC_H

#include <stdint.h>

#include "ggem_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GGEM_NOALLOC_MAX_PARTICLES 32768
#define GGEM_NOALLOC_MAX_CELLS 32768
#define GGEM_NOALLOC_SCRATCH_BYTES 2621696

/* bits of *d_status */
#define GGEM_NOALLOC_STATUS_OUT_OF_BOX 1 /* a particle outside the box on a non-periodic axis */
#define GGEM_NOALLOC_STATUS_NON_FINITE 2 /* a coordinate is NaN or infinite */

/* p: constants, box and rc (nb_mode must be GGEM_NB_CUTOFF; precision and
 * device are ignored: FP64 on the current device).  d_xyz[3n], d_f[3n] and
 * d_u[3n] are device arrays in the reference's particle order; d_status is a
 * device int the call sets to 0, or to the OR of the status bits above (the
 * context path's GGEM_ERR_OUT_OF_DOMAIN and GGEM_ERR_BAD_ARG); u is then
 * not meaningful.  Work is enqueued on `stream` (a cudaStream_t, NULL for
 * the legacy default stream); the call returns without synchronising. */
int ggem_local_matvec_noalloc(const ggem_params *p, int64_t n, const double *d_xyz,
                              const double *d_f, double *d_u, int self_mode, int *d_status,
                              void *stream);

#ifdef __cplusplus
}
#endif
#endif
