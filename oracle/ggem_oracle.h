/*
 * ggem_oracle.h -- FP64 CPU oracle for the GGEM particle-side hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms (COPSS-Hydrodynamics src/ggem_stokes.C, src/chebyshev.C,
 * src/brownian_system.C, src/point_mesh.C, src/pm_periodic_boundary.C,
 * src/assemble_stokes.C).  It is used by the tests, by smoke() and by the
 * cpu_baseline / reference arm of bench.py as the checker and as the timed
 * CPU baseline.  The shipped library never links, loads or calls it.
 *
 * Parity pins (see tests/): the reference's PointParticle_Stokes_GGEM golden
 * velocity profiles (local and exact columns), the reference's own
 * chebyshev.C compiled from its source (oracle/_ref), and closed-form
 * known-answer tests.
 */
#ifndef GGEM_ORACLE_H
#define GGEM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* point types, point_particle.h:36-41 */
/* PointType, point_particle.h:36-41 */
enum { ORC_POLYMER_BEAD = 0, ORC_LAGRANGIAN_POINT = 1, ORC_POINT_PARTICLE = 2 };

/* self-term handling of the local mobility */
enum {
  ORC_SELF_NONE = 0,       /* local_solution_bead for a bead: self not in list */
  ORC_SELF_BEAD = 1,       /* pm_system_stokes.C:452  u - coeff_1 f + f       */
  ORC_SELF_LAGRANGIAN = 2  /* ggem_stokes.C:485-499   u + G(0) f               */
};

/* neighbour modes */
enum { ORC_NB_REFERENCE = 0, ORC_NB_CUTOFF = 1 };

typedef struct orc_consts {
  double mu, alpha, ksi, br0;
  double one_eight_pi_mu, alpha2, alpha3, alpha3_pi_23, two_alpha_sqrt_pi, coeff_1;
  double ksi2, ksi3, ksi3_pi_23, two_ksi_sqrt_pi, coeff_2;
  double r_eps;
} orc_consts;

typedef struct orc_box {
  double lo[3], hi[3];
  int periodic[3];
} orc_box;

/* neighbour structure (CSR) */
typedef struct orc_nblist {
  int64_t n;
  int64_t *offsets; /* n+1 */
  int32_t *ids;     /* offsets[n] */
} orc_nblist;

/* element grid used by the reference-faithful neighbour mode */
typedef struct orc_mesh {
  int nx, ny, nz;
  double search_radius_e;
} orc_mesh;

int  orc_set_constants(double mu, double alpha, double br0, int point_type,
                       double ibm_beta, double hmin, orc_consts *c);
void orc_green_local(const orc_consts *c, const double x[3], double G[9]);
void orc_green_unbounded_smoothed(const orc_consts *c, const double x[3],
                                  double a_or_k, double G[9]);
double orc_smoothed_force_exp(const orc_consts *c, const double r[3]);
void orc_point_vector(const orc_box *b, const double p0[3], const double p1[3],
                      double out[3]);

/* neighbour builds; caller frees with orc_free_nblist */
int orc_build_neighbors_cutoff(const orc_box *b, int64_t n, const double *xyz,
                               double rc, orc_nblist *out);
int orc_elem_of_point(const orc_box *b, const orc_mesh *m, const double p[3]);
int orc_build_elem_lists(const orc_box *b, const orc_mesh *m, int64_t n,
                         const double *xyz, orc_nblist *elem_point_nb,
                         int32_t *elem_of_particle);
int orc_build_neighbors_reference(const orc_box *b, const orc_mesh *m,
                                  int64_t n, const double *xyz, orc_nblist *out);
void orc_free_nblist(orc_nblist *l);

/* u[r][3n] = M_loc f[r][3n] over the given neighbour lists */
void orc_local_matvec(const orc_consts *c, const orc_box *b, int64_t n,
                      const double *xyz, const orc_nblist *nb, int nrhs,
                      const double *f, double *u, int self_mode, int nthreads);
/* field-point local velocity, targets use element lists (mode R) */
void orc_local_field_reference(const orc_consts *c, const orc_box *b,
                               const orc_mesh *m, const orc_nblist *elem_nb,
                               int64_t n, const double *xyz, const double *f,
                               int64_t nt, const double *targets, double *u);
/* field-point local velocity over all particles within rc (rc<=0: all) */
void orc_local_field_cutoff(const orc_consts *c, const orc_box *b, int64_t n,
                            const double *xyz, const double *f, double rc,
                            int64_t nt, const double *targets, double *u);
/* exact unbounded solution with ksi, analytical_solution_stokes.C:66-102 */
void orc_exact_unbounded(const orc_consts *c, int64_t n, const double *xyz,
                         const double *f, int64_t nt, const double *targets,
                         double *u);
/* smoothed force density at points: rho[q] = sum_j g(q - x_j) f_j over the
 * element neighbour list of qp_elem[q] (rc<=0) or all j within rc (rc>0) */
void orc_spread_qp(const orc_consts *c, const orc_box *b,
                   const orc_nblist *elem_nb, int64_t n, const double *xyz,
                   const double *f, int64_t nq, const double *qxyz,
                   const int32_t *qp_elem, double rc, double *rho);
/* element rhs, assemble_stokes.C:645-671: Fe[e][j*n_u + l] */
void orc_element_rhs(const orc_consts *c, const orc_box *b,
                     const orc_nblist *elem_nb, int64_t n, const double *xyz,
                     const double *f, int64_t n_elem, int nq_per_elem,
                     int n_u, const double *qxyz, const double *int_force,
                     double rc, double *Fe);

/* chebyshev.C:57-107, methods 0 Gauss, 1 Gauss_Radau, 2 Gauss_Lobatto */
void orc_cheb_coeffs(int N, double da, double db, int method, double *coef);

/* operator callback u = M f (vectors of length dim) */
typedef void (*orc_op_fn)(void *ctx, const double *f, double *u);

typedef struct orc_cheb_report {
  int converged;   /* brownian_system.C:1138-1147 */
  int n_terms;     /* polynomial degree reached */
  int n_matvecs;
  double err1, err2;
} orc_cheb_report;

/* brownian_system.C:967-1178, dw is overwritten with y ~ M^{-1/2} dw */
void orc_cheb_inv_sqrt(orc_op_fn op, void *ctx, int64_t dim, int N,
                       double eig_min, double eig_max, double tol_cheb,
                       double *dw, orc_cheb_report *rep);
/* Lanczos with full reorthogonalisation; start vector given */
int orc_lanczos(orc_op_fn op, void *ctx, int64_t dim, int k, const double *v0,
                double *lmin, double *lmax, double *alpha_out, double *beta_out);
/* smallest/largest eigenvalue of the k x k symmetric tridiagonal matrix */
void orc_tridiag_extremes(int k, const double *a, const double *b, double *lmin,
                          double *lmax);
/* brownian_system.C:846-920 */
int orc_power_iteration(orc_op_fn op, void *ctx, int64_t dim, double tol,
                        int maxits, double *eig);

/* a matvec operator context for orc_op_fn */
typedef struct orc_matvec_ctx {
  const orc_consts *c;
  const orc_box *b;
  int64_t n;
  const double *xyz;
  const orc_nblist *nb;
  int self_mode;
  int nthreads;
} orc_matvec_ctx;
void orc_matvec_op(void *ctx, const double *f, double *u);
/* u_i = (i+1) f_i, brownian_system.C:1181-1211 */
void orc_diag_test_op(void *ctx, const double *f, double *u);

/* random_generator.C:43-67 stream: std::default_random_engine seeded with
 * seed, std::normal_distribution(mean, std); `skip_vectors` earlier vectors
 * of length n are drawn first (copss.C:1544-1555 fast-forward) */
void orc_std_normal_vector(uint64_t seed, int64_t skip_vectors, int64_t n,
                           double mean, double stddev, double *out);

/* Philox4x32-10 (Salmon et al., SC'11) counter-based normals, restated for
 * checking the device noise generator: the counter words bit-for-bit, the
 * FP32 Box-Muller transform to a few FP32 ulps */
void orc_philox_normals(uint64_t seed, uint64_t stream, int64_t n, double *out);

/* excluded-volume Gaussian force, FixPointGaussianDNA::compute
 * (fix/fix_point_gaussian_dna.C:69-84) with FixBase::gaussian_force
 * (fix/fix_base.C:150-162): f_i += sum over nb(i) of -c1 c2 exp(-c2 r^2) r_ij,
 * r_ij = point_vector(x_i, x_j) (minimum image) */
void orc_ev_gaussian(const orc_box *b, int64_t n, const double *xyz, const orc_nblist *nb,
                     double c1, double c2, double *f);
/* the FixBase spring laws (fix/fix_base.C:55-148): the force on bead i from
 * R_ij = x_j - x_i; kind 0 WLS, 1 FENE, 2 Underhill-Doyle, 3 LHS (c1 = l0,
 * Ls = k0) */
void orc_spring_force(int kind, const double R_ij[3], double c1, double Ls, double F[3]);
/* FixPointWLS::compute (fix/fix_point_wls.C:66-92) for any law: bonds m x 2,
 * F_ij to bead bonds[k][0] and -F_ij to bonds[k][1], in bond order */
void orc_spring_forces(const orc_box *b, int64_t n, const double *xyz, int64_t m,
                       const int64_t *bonds, int kind, double c1, double Ls, double *f);

/* the global (FEM) velocity at points: libMesh System::point_value of the
 * SECOND-order u, v, w on the HEX20 build_cube mesh
 * (pm_system_stokes.C:437-441), restated from the 20-node serendipity
 * element (libMesh Hex20 node order); elem_dofs [ne][3][20].  Returns the
 * number of points outside a non-periodic axis (clamped to the mesh). */
void orc_hex20_shape(double x, double y, double z, double n[20]);
int64_t orc_fem_point_values(int64_t n, const double *xyz, const int ne[3], const double lo[3],
                             const double hi[3], const int periodic[3],
                             const int64_t *elem_dofs, const double *sol, double *u);

#ifdef __cplusplus
}
#endif
#endif
