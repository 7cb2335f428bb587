/*
 * ggem_diag.h -- measurement hooks of the GGEM library.
 *
 * Not part of the reference's interface (the reference has no GPU): these
 * report what the library launched and the FP32 issue rate of the device, so
 * that benchmarks can state kernel counts and roofline fractions.
 */
#ifndef GGEM_DIAG_H
#define GGEM_DIAG_H

#include <stdint.h>

#include "ggem_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* launch trace: with enable = 1 every kernel launch of the context is
 * followed by an event on its stream (the first marks the start); reading
 * returns, for up to max launches, the event times in ms from the start and
 * the launch names (static strings), and the number recorded in *count.
 * The differences of consecutive times are a kernel's duration plus the
 * idle gap before it.  Setting it (on or off) clears the trace. */
int ggem_set_launch_trace(ggem_ctx *ctx, int enable);
int ggem_get_launch_trace(ggem_ctx *ctx, int64_t max, double *t_ms, const char **names,
                          int64_t *count);
/* the library's integer-only double -> float conversion (used where FP64
 * conversion throughput matters) and the hardware __double2float_rn, both
 * applied to d_in[n] on the device, for a bit-for-bit check */
int ggem_diag_convert_f32(ggem_ctx *ctx, int64_t n, const double *d_in, float *d_out,
                          float *d_ref);
/* number of CUDA kernels this context has launched so far */
int ggem_get_launch_count(const ggem_ctx *ctx, int64_t *count);
/* ordered in-cutoff pairs of the current FP32 pair list (the work unit of
 * the pair kernel) */
int ggem_get_pair_count(const ggem_ctx *ctx, int64_t *count);
/* storage of the current FP32 pair list: row width (entries per row) and
 * whether per-pair tensors are stored (1: the pair kernels stream 20 B per
 * pair, 0: they evaluate the tensor per pair and matvec) */
int ggem_get_pair_storage(const ggem_ctx *ctx, int *row_width, int *tensors_stored);
/* allow (1, the default when B(s) >= 0 on [0, rc^2]) or forbid (0) stored
 * pair tensors; takes effect at the next ggem_build_cells */
int ggem_set_pair_tensors(ggem_ctx *ctx, int enable);
/* GGEM_FP64 cutoff contexts: 1 = build the exact pair list with the cells
 * and walk it in the FP64 pair kernel (only in-cutoff pairs, the
 * reference's FP64 arithmetic per pair); 0 (default) = sweep the 27 cells
 * around every bead.  Takes effect at the next ggem_build_cells. */
int ggem_set_fp64_pair_list(ggem_ctx *ctx, int enable);
/* GGEM_FP32 cutoff contexts: 1 = single-RHS matvecs with tensors evaluated
 * per pair use the symmetry G_ij = G_ji: the list build also writes the
 * half list, each unordered pair is evaluated once and its source side added
 * to the source with a vector atomic (results within the FP32 tolerance,
 * not bit-reproducible from run to run); 0 (default) = full rows.  Takes
 * effect at the next ggem_build_cells. */
int ggem_set_symmetric_pairs(ggem_ctx *ctx, int enable);
/* autotune the pair storage on the current configuration (cells and list
 * built, FP32): times `reps` single-RHS matvecs with tensors evaluated per
 * pair and with stored tensors (plus the one tensor pass per build,
 * amortised over matvecs_per_build matvecs) by CUDA events on the context's
 * stream; each form is timed for each of its kernel shapes (per-matvec
 * tensors: registers capped for 6 or for 5 blocks of 256 per SM; stored
 * tensors: lanes per target, entries in flight, pipelined stream).  The
 * fastest stays selected for this context; both costs are reported in ms
 * per matvec (the stored one with its amortised pass) and variants[0],
 * variants[1] receive the chosen computed and stored shapes */
int ggem_autotune_pair_storage(ggem_ctx *ctx, int reps, double matvecs_per_build,
                               int *use_stored, double *ms_computed, double *ms_stored,
                               int *variants);
/* select the kernel shapes directly: computed 0 .. 1, stored 0 .. 3 */
int ggem_set_pair_variant(ggem_ctx *ctx, int computed, int stored);
/* dense FP32 FMA throughput of this device in TFLOP/s (FMA = 2 flops),
 * measured with CUDA events over a register-resident FMA chain kernel on the
 * context's stream */
int ggem_probe_fp32_peak(ggem_ctx *ctx, double *tflops);
/* kernel timing: when enabled, CUDA events on the context's stream bracket
 * every launch of the kernels below; totals are read back (with a stream
 * synchronisation) by ggem_get_kernel_timing.  Enabling resets the totals. */
#define GGEM_KERNEL_PAIR_FP32 0  /* FP32 pair-list sum                        */
#define GGEM_KERNEL_PAIR_FP64 1  /* FP64 pair sum (cell sweep or pair list)   */
#define GGEM_KERNEL_CHEB_TERM 2  /* fused Chebyshev term                       */
#define GGEM_KERNEL_LIST_BUILD 3 /* pair-list count + fill                     */
#define GGEM_KERNEL_PAIR_CHEB 4  /* FP32 pair sum with the Chebyshev term fused */
int ggem_set_kernel_timing(ggem_ctx *ctx, int enable);
/* the same for a subset of the kinds above (bit k of mask = kind k), so
 * that a measurement brackets only the kernel it reports.  Consecutive
 * fused Chebyshev terms (GGEM_KERNEL_PAIR_CHEB) share one event pair, and
 * their launches count one each; the span includes the gaps between them */
int ggem_set_kernel_timing_kinds(ggem_ctx *ctx, int enable, unsigned mask);
/* CUDA graph of the fused single-RHS Brownian series (FP32 cut-off context,
 * tensors per pair, adaptive single check): the first step, the terms up to
 * the first error check and that check's matvec, sums and readback are
 * captured as one graph when a call repeats the previous call's
 * configuration (sizes, buffers, eigen interval, predicted degree), and
 * replayed while it holds.  Results are those of the launches it replaces.
 * On by default; a failed capture turns it off for the context. */
int ggem_set_series_graphs(ggem_ctx *ctx, int enable);
/* graphs captured and replays launched so far */
int ggem_get_series_graph_stats(const ggem_ctx *ctx, int64_t *captures, int64_t *replays);
int ggem_get_kernel_timing(ggem_ctx *ctx, int kernel, double *total_ms, int64_t *launches);

#ifdef __cplusplus
}
#endif
#endif
