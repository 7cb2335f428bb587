/*
 * ggem_fem.h -- the global (FEM) velocity at the particles.
 *
 * PMSystemStokes::compute_point_velocity (pm_system_stokes.C:437-441) adds
 * to the local GGEM velocity the FEM solution of the smoothed problem,
 * evaluated at every particle with System::point_value on the element that
 * contains it: u, v and w are SECOND-order LAGRANGE variables
 * (copss.C:1147-1149) on the HEX20 box mesh of MeshTools::Generation::
 * build_cube (copss.C:993-1004).  This entry point evaluates the same
 * interpolant on the device for all particles of a context at once:
 *
 *   U_global(x) = sum_{k<20} N_k(xi(x)) U[dof(e, var, k)],  var = u, v, w,
 *
 * where e is the element containing x on the uniform n_elem[0] x n_elem[1]
 * x n_elem[2] mesh of [lo, hi] (elements numbered x fastest, the order of
 * build_cube), xi in [-1, 1]^3 the reference coordinates and N_k the
 * 20-node serendipity shape functions in libMesh's Hex20 node order:
 * corners 0-7 (z = -1: (-1,-1), (1,-1), (1,1), (-1,1); then z = +1), edge
 * nodes 8-11 on the z = -1 edges 0-1, 1-2, 2-3, 3-0, 12-15 on the vertical
 * edges 0-4, 1-5, 2-6, 3-7, 16-19 on the z = +1 edges 4-5, 5-6, 6-7, 7-4.
 *
 * The driver passes, per element, the dof indices of u, v and w at its 20
 * nodes (libMesh's DofMap::dof_indices) once, and the solution vector of
 * each solve.  All arithmetic is FP64.
 */
#ifndef GGEM_FEM_H
#define GGEM_FEM_H

#include <stdint.h>

#include "ggem_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ggem_fem ggem_fem;

/* the mesh: elem_dofs is [n_elem total][3 variables][20 nodes], each index
 * in [0, n_dofs); copied to the device.  The context provides the particle
 * positions (ggem_set_particles) and its box's periodic axes: a particle on
 * a periodic axis is wrapped into [lo, hi) first; outside [lo, hi] on a
 * non-periodic axis is GGEM_ERR_OUT_OF_DOMAIN (pm_system_stokes.C:417-424) */
int ggem_fem_create(ggem_ctx *ctx, const int n_elem[3], const double lo[3], const double hi[3],
                    int64_t n_dofs, const int64_t *elem_dofs, ggem_fem **out);
void ggem_fem_destroy(ggem_fem *fem);

/* U_global at every particle of the context, [n][3] in the caller's
 * particle order; accumulate = 1 adds it to u (U = U_global + U_local,
 * pm_system_stokes.C:446-455), 0 overwrites */
int ggem_fem_point_values(ggem_fem *fem, const double *solution, double *u, int accumulate);
int ggem_fem_point_values_dev(ggem_fem *fem, const double *d_solution, double *d_u,
                              int accumulate);

/* the 20 shape functions at reference point xi (host; for checks) */
void ggem_fem_hex20_shape(const double xi[3], double n[20]);

#ifdef __cplusplus
}
#endif
#endif
