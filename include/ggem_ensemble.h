/*
 * ggem_ensemble.h -- many independent suspensions of uneven size through
 * one set of launches.
 *
 * The reference runs one suspension per COPSS job (Copss::fixman_integrate,
 * copss.C:1560-1686, with its own GGEMStokes, PointMesh and BrownianSystem).
 * An ensemble holds K periodic suspensions with their own boxes and bead
 * counts: each is built as an ordinary context (cell list, pair list,
 * stored pair tensors), and their lists are concatenated into one
 * block-diagonal operator, so that a matvec or a Chebyshev term of all K
 * suspensions and up to 8 right-hand sides each is a single kernel launch.
 * The unchecked stretch of Chebyshev terms is captured once as a CUDA graph
 * and replayed.  Every series keeps its own eigen interval, coefficients,
 * error estimators and stopping decision (brownian_system.C:967-1178).
 *
 * Vector layout: [bead][rhs][3] float64, beads in ensemble order (the K
 * suspensions' particles concatenated, each in its caller order).
 */
#ifndef GGEM_ENSEMBLE_H
#define GGEM_ENSEMBLE_H

#include <stdint.h>

#include "ggem_gb300.h"
#include "ggem_surrogate.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GGEM_ENSEMBLE_MAX_RHS 8

typedef struct ggem_ensemble ggem_ensemble;

/* K suspensions sharing base's physics (mu, alpha, br0, point type, rc,
 * cell_div, device); suspension b is the periodic cube [0, box_length[b])^3
 * (FP32 pair sums, cut-off lists, FP64 recurrence) */
int ggem_ensemble_create(const ggem_params *base, int k, const double *box_length,
                         ggem_ensemble **out);
void ggem_ensemble_destroy(ggem_ensemble *e);
const char *ggem_ensemble_last_error(const ggem_ensemble *e);

/* positions of all suspensions (device, [sum n][3], ensemble order) with
 * n[b] beads in suspension b: cell lists, pair lists and pair tensors of
 * every suspension, then the concatenated operator */
int ggem_ensemble_set_particles_dev(ggem_ensemble *e, const int64_t *n, const double *d_xyz);
/* total beads and ordered in-cutoff pairs of the current configuration */
int ggem_ensemble_sizes(const ggem_ensemble *e, int64_t *beads, int64_t *pairs);

/* u = M f for every suspension, nrhs <= 8, device vectors [bead][nrhs][3] */
int ggem_ensemble_matvec_dev(ggem_ensemble *e, int nrhs, const double *d_f, double *d_u,
                             int self_mode);

/* Brownian displacements dw = M M^{-1/2} xi of every suspension and
 * right-hand side: Chebyshev of at most N terms on [eig_min[b], eig_max[b]]
 * with the adaptive schedule of ggem_brownian_displacement (check_every 0),
 * err1 <= tol; rep[b * nrhs + r] per series.  Returns
 * GGEM_ERR_CHEB_NOT_CONVERGED when some series failed (its dw is still
 * written); the caller recomputes those intervals (Lanczos) and repeats. */
int ggem_ensemble_brownian_dev(ggem_ensemble *e, int nrhs, int N, const double *eig_min,
                               const double *eig_max, double tol, const double *d_xi,
                               double *d_dw, ggem_cheb_report *rep);

/* eigen intervals of all suspensions: features of each (pair-distance
 * histograms on the GPU) and one batched forward pass of the network */
int ggem_ensemble_intervals(ggem_ensemble *e, ggem_surrogate *s, const double *chain_fraction,
                            double margin_lo, double margin_hi, double *eig_min,
                            double *eig_max);
/* Lanczos bounds of suspension b (the fallback) */
int ggem_ensemble_lanczos(ggem_ensemble *e, int b, int k, uint64_t seed, double *eig_min,
                          double *eig_max);

/* autotune the ensemble kernels' block size on the current configuration
 * (candidates 128, 256, 512 threads; CUDA-event timing of the fused term);
 * the choice is kept and reported */
int ggem_ensemble_autotune(ggem_ensemble *e, int nrhs, int *block_threads, double *ms_per_term);
/* How ggem_ensemble_brownian_dev runs the series.  persistent = 1 (the
 * default): one cooperative launch walks the whole step (start, terms,
 * error checks and every series' stopping decision, brownian_system.C:
 * 1036-1155) with tiles of slots_per_tile slots of one suspension; a tile
 * waits only for its own suspension's previous pass, and every wait is
 * bounded by wait_polls polls (0 = the default, ~8 s) after which the call
 * returns GGEM_ERR_TIMEOUT.  persistent = 0: one launch per term with the
 * checks read back on the host.  slots_per_tile 0 keeps the current value;
 * never_ready = 1 is a test hook that makes every wait run out. */
int ggem_ensemble_set_series_mode(ggem_ensemble *e, int persistent, int slots_per_tile,
                                  uint32_t wait_polls, int never_ready);
/* Autotune the step's form: times one Brownian step of every series (N - 1
 * terms, no early stop; xi, dw as for ggem_ensemble_brownian_dev) as one
 * persistent launch for each launch shape (threads per block and the
 * register cap for 4, 6 or 12 resident blocks per SM: shapes 0, 1, 2) and
 * tile size (64, 128, 256 slots), and as one launch per term (shape 3),
 * keeps the fastest (the series mode follows it) and returns it (shape
 * index, slots per tile, ms per step).  With
 * cache_path (may be NULL) a line "key shape slots ms" per tuned ensemble is
 * appended to that text file; a later call with the same device, suspension
 * count, bead and pair counts, row width and right-hand sides reads it back
 * instead of timing. */
int ggem_ensemble_autotune_series(ggem_ensemble *e, int nrhs, int N, const double *eig_min,
                                  const double *eig_max, double tol, const double *d_xi,
                                  double *d_dw, const char *cache_path, int *shape,
                                  int *slots_per_tile, double *ms_per_step);

#ifdef __cplusplus
}
#endif
#endif
