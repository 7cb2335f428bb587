/*
 * ggem_forces.h -- the per-step particle forces that reuse the cell lists:
 * excluded volume between neighbours and spring forces along polymer bonds.
 *
 * They replace the host loops of the reference's force fixes:
 *   FixPointGaussianDNA::compute (fix/fix_point_gaussian_dna.C:69-84) with
 *     FixBase::gaussian_force (fix/fix_base.C:150-162);
 *   FixPointWLS::compute (fix/fix_point_wls.C:66-92) with
 *     FixBase::spring_force_wls / _fene / _ud / _lhs (fix/fix_base.C:55-148).
 * All arithmetic is FP64.  Forces are [n][3] in the caller's particle order
 * and are added to (accumulate = 1) or replace (0) the output.
 */
#ifndef GGEM_FORCES_H
#define GGEM_FORCES_H

#include <stdint.h>

#include "ggem_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* spring laws of FixBase (fix_base.C:55-148), f(R) along R = x_j - x_i */
#define GGEM_SPRING_WLS 0  /* c1 (1/(1-R/Ls)^2 - 1 + 4R/Ls) R/|R|      */
#define GGEM_SPRING_FENE 1 /* c1 (R/Ls) / (1 - (R/Ls)^2) R/|R|          */
#define GGEM_SPRING_UD 2   /* Underhill-Doyle polynomial in (R/Ls)^2    */
#define GGEM_SPRING_LHS 3  /* k0 (|R| - l0) R/|R| with c1 = l0, Ls = k0 */

/* excluded-volume Gaussian force over the cut-off neighbours of every
 * particle: f_i (+)= sum_j -c1 c2 exp(-c2 |r_ij|^2) r_ij with
 * r_ij = x_j - x_i (minimum image), |r_ij| < rc (the context's cut-off);
 * the cells must be built */
int ggem_ev_gaussian_forces(ggem_ctx *ctx, double c1, double c2, double *f, int accumulate);
int ggem_ev_gaussian_forces_dev(ggem_ctx *ctx, double c1, double c2, double *d_f,
                                int accumulate);

/* the bond list (caller particle ids, m x 2: bonds[k][0] -- bonds[k][1]),
 * kept on the device until replaced; every bead sums its bonds in bond order */
int ggem_set_bonds(ggem_ctx *ctx, int64_t m, const int64_t *bonds);
/* spring forces of all bonds: bead i of bond (i, j) receives f(x_j - x_i)
 * and bead j receives -f, as FixPointWLS::compute; `kind` one of
 * GGEM_SPRING_* with its two parameters (c1, Ls) */
int ggem_spring_forces(ggem_ctx *ctx, int kind, double c1, double Ls, double *f, int accumulate);
int ggem_spring_forces_dev(ggem_ctx *ctx, int kind, double c1, double Ls, double *d_f,
                           int accumulate);

#ifdef __cplusplus
}
#endif
#endif
