/*
 * ggem_gb300.h -- C ABI of the GB300 (sm_103a) GGEM particle-side library.
 *
 * The library computes the local part of the GGEM Stokes mobility
 * (regularized Stokeslets over cell lists), the Gaussian force spreading onto
 * FEM quadrature points that feeds the global FEM solve, and the Chebyshev
 * M^{-1/2} xi Brownian step with its spectral bounds.  The global FEM Stokes
 * solve stays with the caller (libMesh/PETSc).
 *
 * Conventions
 *   - Vectors use the reference's PETSc layout [p0x, p0y, p0z, p1x, ...]
 *     (brownian_system.C:72-75); several right-hand sides are stored one
 *     after another: f[r * 3n + 3i + d].
 *   - Functions without a suffix take HOST pointers and copy through the
 *     library's pinned staging; `_dev` functions take DEVICE pointers and
 *     enqueue on the context's stream (ggem_set_stream), returning without a
 *     host synchronisation unless stated.
 *   - Every call returns GGEM_OK (0) or a negative ggem error code; the
 *     message of the last failure is available from ggem_last_error(ctx).
 *     No function aborts, traps or throws.
 *   - One context per host thread; a context is not thread safe.
 *
 * Each entry point names the reference interface it replaces
 * (COPSS-Hydrodynamics src/, file:line).
 */
#ifndef GGEM_GB300_H
#define GGEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ------------------------------------------------------- */
#define GGEM_OK 0
#define GGEM_ERR_BAD_ARG -1          /* invalid argument or call order     */
#define GGEM_ERR_CUDA -2             /* CUDA runtime error                  */
#define GGEM_ERR_CELL_OVERFLOW -3    /* neighbour list capacity exceeded    */
#define GGEM_ERR_TIMEOUT -4          /* a bounded device wait gave up       */
#define GGEM_ERR_NOT_SPD -5          /* eigenvalue <= 0 (brownian_system.C:835-840) */
#define GGEM_ERR_CHEB_NOT_CONVERGED -6 /* brownian_system.C:1162-1163       */
#define GGEM_ERR_SURROGATE_REJECTED -7
#define GGEM_ERR_OUT_OF_DOMAIN -8    /* point outside every cell (point_mesh.C:602-613) */
#define GGEM_ERR_NO_DEVICE -9
#define GGEM_ERR_OOM -10
#define GGEM_ERR_INVALID_RANGE -11   /* eig_min < 0, eig_max < 0 or min > max (copss.C:1609-1615) */

/* ---- enumerations ------------------------------------------------------ */
/* PointType, point_particle.h:36-41 */
#define GGEM_POLYMER_BEAD 0
#define GGEM_LAGRANGIAN_POINT 1
#define GGEM_POINT_PARTICLE 2

/* self term of the local mobility */
#define GGEM_SELF_NONE 0       /* local_solution_bead as is (ggem_stokes.C:427-503)         */
#define GGEM_SELF_BEAD 1       /* u - coeff_1 f + f  (pm_system_stokes.C:450-453)          */
#define GGEM_SELF_LAGRANGIAN 2 /* u + G(0) f         (ggem_stokes.C:485-499)               */

/* neighbour definition */
#define GGEM_NB_REFERENCE 0 /* element-as-cell lists, point_mesh.C:293-848 (no per-pair cutoff) */
#define GGEM_NB_CUTOFF 1    /* all pairs with |r| < rc                                        */

/* arithmetic of the pair sum */
#define GGEM_FP64 0 /* FP64 Green's tensors with erf/exp, plain cell-stencil sweep     */
#define GGEM_FP32 1 /* FP32 cell-relative coordinates, tabulated tensor, compensated sums,
                       cached pair list                                                  */

/* Chebyshev quadrature, chebyshev.C:68-70 */
#define GGEM_CHEB_GAUSS 0
#define GGEM_CHEB_GAUSS_RADAU 1
#define GGEM_CHEB_GAUSS_LOBATTO 2

typedef struct ggem_ctx ggem_ctx;

typedef struct ggem_params {
  /* GGEMStokes::set_mu / set_alpha / set_br0 / set_point_type / set_ibm_beta
   * / set_hmin (ggem_stokes.C:39-114, ggem_system.h:73-100) */
  double mu;
  double alpha;
  double br0;
  int point_type;
  double ibm_beta;
  double hmin;
  /* PMPeriodicBoundary box and periodicity (pm_periodic_boundary.C:350-374) */
  double box_lo[3];
  double box_hi[3];
  int periodic[3];
  /* neighbour definition */
  int nb_mode;
  double rc;              /* GGEM_NB_CUTOFF: pair cutoff radius                    */
  int n_mesh[3];          /* GGEM_NB_REFERENCE: elements per axis (copss.C:986-992) */
  double search_radius_e; /* GGEM_NB_REFERENCE: <= 0 means 0.5*hmax + 4/alpha (copss.C:1075) */
  int precision;          /* GGEM_FP64 or GGEM_FP32                                */
  int cell_div;           /* GGEM_FP32 cutoff cells per rc (1 or 2); 0 = default   */
  int device;             /* CUDA device ordinal                                    */
} ggem_params;

/* derived constants, ggem_stokes.h:315-334 and ggem_system.h:107-131 */
typedef struct ggem_constants {
  double mu, alpha, ksi, br0;
  double one_eight_pi_mu, alpha2, alpha3, alpha3_pi_23, two_alpha_sqrt_pi, coeff_1;
  double ksi2, ksi3, ksi3_pi_23, two_ksi_sqrt_pi, coeff_2;
  double r_eps;
} ggem_constants;

/* BrownianSystem::chebyshev_polynomial_approximation outcome
 * (brownian_system.C:967-1178) */
typedef struct ggem_cheb_report {
  int converged;   /* err1 <= tol_cheb reached                               */
  int n_terms;     /* highest polynomial degree used                         */
  int n_matvecs;   /* mobility applications, error checks included            */
  double err1;     /* sqrt(|y.M^2.y - xi.M.xi| / xi.M.xi) of the last check   */
  double err2;     /* |c_k| ||x_k|| / ||y||                                   */
} ggem_cheb_report;

/* ---- context ----------------------------------------------------------- */
void ggem_default_params(ggem_params *p);
/* replaces AssembleStokes::init_ggem_stokes (assemble_stokes.C:1061-1082) */
int ggem_create(const ggem_params *p, ggem_ctx **out);
void ggem_destroy(ggem_ctx *ctx);
const char *ggem_strerror(int code);
const char *ggem_last_error(const ggem_ctx *ctx);
int ggem_get_constants(const ggem_ctx *ctx, ggem_constants *out);
/* stream for all _dev calls (cudaStream_t); NULL restores the library's own */
int ggem_set_stream(ggem_ctx *ctx, void *stream);
int ggem_synchronize(ggem_ctx *ctx);

/* ---- particles and neighbour structure -------------------------------- */
/* replaces PointParticle positions + PointMesh::reinit (point_mesh.C:245-289):
 * cell assignment, sorted cell list and (FP32) the cached pair list.
 * xyz (AoS, 3n doubles) is copied on the context's stream: from pageable
 * memory the call returns once the copy has read it; from page-locked
 * memory the copy may still be reading it after the call returns, so keep
 * xyz unchanged until the next call that synchronises (ggem_build_cells
 * without deferred checks, ggem_brownian_displacement, ggem_synchronize). */
int ggem_set_particles(ggem_ctx *ctx, int64_t n, const double *xyz);
int ggem_set_particles_dev(ggem_ctx *ctx, int64_t n, const double *d_xyz);
/* (a NaN or infinite coordinate is reported by the cell build, or with
 * deferred checks by the call that reads its flags, as GGEM_ERR_BAD_ARG) */
int ggem_build_cells(ggem_ctx *ctx);
/* deferred checks: with enable = 1, a build after the first one keeps the
 * pair-list row width and returns without waiting for the device; its row
 * statistics and error word (a particle outside a non-periodic axis, a row
 * longer than the width) are read at the next synchronising call.  The
 * Chebyshev calls read them with their first error check and, when the rows
 * overflowed, rebuild the list wider and run the series again; every other
 * call that uses the cells or the list reads them on entry.  Errors of a
 * build are therefore reported by the call that reads them.  Off (0) by
 * default; switching it off reads any pending statistics. */
int ggem_set_deferred_checks(ggem_ctx *ctx, int enable);
/* number of ordered neighbour pairs (self excluded) of the current build */
int ggem_neighbor_pair_count(ggem_ctx *ctx, int64_t *count);
/* per-particle neighbour lists in original particle ids, ascending,
 * replacing PointParticle::neighbor_list (point_particle.h:189-203);
 * offsets has n+1 entries, ids has capacity `cap` */
int ggem_get_neighbors(ggem_ctx *ctx, int64_t *offsets, int32_t *ids, int64_t cap);
/* cell (element) of each particle, replacing elem_id() after
 * build_elem_point_containing_list (point_mesh.C:573-648) */
int ggem_get_cell_of_particles(ggem_ctx *ctx, int32_t *cell);

/* ---- local mobility ---------------------------------------------------- */
/* u = M_loc f for all particles: GGEMStokes::local_solution_bead
 * (ggem_stokes.C:427-503) for every bead plus the self term of
 * PMSystemStokes::compute_point_velocity (pm_system_stokes.C:446-455);
 * the local part of _MatMult_Stokes (brownian_system.C:44-140) */
int ggem_local_matvec(ggem_ctx *ctx, int nrhs, const double *f, double *u, int self_mode);
int ggem_local_matvec_dev(ggem_ctx *ctx, int nrhs, const double *d_f, double *d_u,
                          int self_mode);
/* GGEMStokes::green_tensor_local_regularized (ggem_stokes.C:304-357) at m
 * displacement vectors, G row-major 9 per vector (FP64) */
int ggem_green_tensor_local(ggem_ctx *ctx, int64_t m, const double *x, double *G);
/* GGEMStokes::local_solution_field (ggem_stokes.C:360-424) at nt field
 * points: sources are the particles within rc of the point (cutoff mode,
 * rc <= 0 uses the context rc) or the element neighbour list of the
 * point's element (reference mode) */
int ggem_local_field(ggem_ctx *ctx, int64_t nt, const double *targets, const double *f,
                     double *u);

/* ---- Gaussian force spreading ------------------------------------------ */
/* rho(q) = sum_j g_alpha(q - x_j) f_j (GGEMStokes::smoothed_force_exp,
 * ggem_stokes.C:117-128, summed as in AssembleStokes::compute_element_rhs,
 * assemble_stokes.C:645-662).  qp_elem gives the element of each point
 * (reference mode); in cutoff mode sources within spread_rc (<= 0 means
 * 0.5*hmax + 4/alpha) are used and qp_elem may be NULL. */
int ggem_spread_qp(ggem_ctx *ctx, int64_t nq, const double *qxyz, const int32_t *qp_elem,
                   const double *f, double spread_rc, double *rho);
/* the same with device arrays (f in the caller's particle order) */
int ggem_spread_qp_dev(ggem_ctx *ctx, int64_t nq, const double *d_qxyz, const int32_t *d_qp_elem,
                       const double *d_f, double spread_rc, double *d_rho);
/* fused element right-hand side, assemble_stokes.C:645-671 with the cached
 * JxW*phi of assemble_int_force (:733-757): for each element e,
 * Fe[e][j*n_u + l] = sum_q int_force[e][l*nq + q] * rho_j(q_e,q) */
int ggem_element_rhs(ggem_ctx *ctx, int64_t n_elem, int nq_per_elem, int n_u,
                     const double *qxyz, const double *int_force, const double *f,
                     double spread_rc, double *Fe);

/* ---- Gaussian spreading onto every element's quadrature points --------- */
/* The quadrature points of the mesh, element-major: qxyz[(e * nq + q) * 3 + d]
 * for the n_mesh[0] * n_mesh[1] * n_mesh[2] elements in the reference's
 * build_cube order (x fastest), nq_per_elem in [1, 32] each (8 for the
 * QGauss SECOND rule of the HEX20 velocity element, assemble_stokes.C:397).
 * Reference mode only.  The points are kept on the device (the mesh is fixed
 * for a run; the reference takes them from fe->get_xyz() per element,
 * assemble_stokes.C:404). */
int ggem_set_quadrature(ggem_ctx *ctx, int nq_per_elem, const double *qxyz);
int ggem_set_quadrature_dev(ggem_ctx *ctx, int nq_per_elem, const double *d_qxyz);
/* rho at every quadrature point of every element: the loop of
 * AssembleStokes::compute_element_rhs over the element neighbour list
 * (assemble_stokes.C:645-662) with GGEMStokes::smoothed_force_exp
 * (ggem_stokes.C:117-128) for all elements at once.  f[3n] in the caller's
 * particle order; rho[(e * nq + q) * 3 + d].  precision GGEM_FP64 (the
 * reference's arithmetic) or GGEM_FP32 (element-relative coordinates, error
 * stated against FP64).  pairs (may be NULL) receives the number of
 * (quadrature point, listed particle) pairs summed. */
int ggem_spread_elements(ggem_ctx *ctx, int precision, const double *f, double *rho);
int ggem_spread_elements_dev(ggem_ctx *ctx, int precision, const double *d_f, double *d_rho,
                             int64_t *pairs);

/* ---- Chebyshev and spectral bounds ------------------------------------ */
/* Chebyshev::chebyshev_coefficients (chebyshev.C:57-107), N+1 values */
int ggem_cheb_coeffs(int N, double da, double db, int method, double *coef);
/* BrownianSystem::chebyshev_polynomial_approximation (brownian_system.C:967-1178)
 * on the local mobility: xi_inout (nrhs x 3n) becomes y ~ M^{-1/2} xi.
 * check_every = 1 reproduces the reference exactly (an error-check matvec
 * every term); k > 1 checks err1 every k terms.  rep has nrhs entries.
 * A context without particles returns at once with every report converged
 * at degree 0 and no matvec (the pointers may then be NULL). */
int ggem_cheb_inv_sqrt(ggem_ctx *ctx, int nrhs, int N, double eig_min, double eig_max,
                       double tol_cheb, int check_every, double *xi_inout,
                       ggem_cheb_report *rep);
int ggem_cheb_inv_sqrt_dev(ggem_ctx *ctx, int nrhs, int N, double eig_min, double eig_max,
                           double tol_cheb, int check_every, double *d_xi_inout,
                           ggem_cheb_report *rep);
/* Brownian displacement of the Fixman step (copss.C:1585-1686): the
 * Chebyshev y of xi followed by dw = M y (hi_ewald).  Returns
 * GGEM_ERR_CHEB_NOT_CONVERGED (with dw untouched) when the series fails. */
int ggem_brownian_displacement(ggem_ctx *ctx, int nrhs, int N, double eig_min,
                               double eig_max, double tol_cheb, int check_every,
                               const double *xi, double *dw, ggem_cheb_report *rep);
int ggem_brownian_displacement_dev(ggem_ctx *ctx, int nrhs, int N, double eig_min,
                                   double eig_max, double tol_cheb, int check_every,
                                   const double *d_xi, double *d_dw, ggem_cheb_report *rep);
/* spectral interval of the local mobility by k-step Lanczos with full
 * reorthogonalisation, replacing BrownianSystem::compute_eigenvalues
 * (brownian_system.C:803-843, SLEPc Krylov-Schur).  Returns GGEM_ERR_NOT_SPD
 * when an eigenvalue estimate is <= 0. */
int ggem_lanczos_bounds(ggem_ctx *ctx, int k, uint64_t seed, double *eig_min,
                        double *eig_max);
/* BrownianSystem::power_iteration (brownian_system.C:846-920); returns the
 * iteration that met tol or GGEM_ERR_CHEB_NOT_CONVERGED */
int ggem_power_iteration(ggem_ctx *ctx, double tol, int maxits, double *eig);

/* ---- noise --------------------------------------------------------------- */
/* BrownianSystem::std_random_vector / RandomGenerator::random_vector_normal
 * (brownian_system.C:434-472, random_generator.C:43-67): the reference's
 * std::default_random_engine stream, host side; `skip_vectors` vectors of
 * length n are drawn first (restart fast-forward, copss.C:1544-1555) */
int ggem_std_random_vector(uint64_t seed, int64_t skip_vectors, int64_t n, double mean,
                           double stddev, double *out);
/* counter-based N(0,1) noise on the device (Philox4x32-10 + Box-Muller in
 * FP32, FP64 output) for batched right-hand sides: elements 4p .. 4p+3 from
 * counter (p, stream) */
int ggem_philox_normals_dev(ggem_ctx *ctx, uint64_t seed, uint64_t stream, int64_t n,
                            double *d_out);

#ifdef __cplusplus
}
#endif
#endif
