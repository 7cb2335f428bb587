// ggem_copss.hpp -- C++ host adapter over the GB300 GGEM C ABI.
//
// Mirrors the call surface the COPSS driver uses on the particle side, so a
// libMesh/PETSc build can swap its CPU loops for the GPU library:
//   GGEMStokes      ggem_stokes.h:58-343   (constants, Green's tensor, local
//                                          velocities, self exclusion)
//   Chebyshev       chebyshev.h:43-105     (expansion coefficients)
//   BrownianSystem  brownian_system.h:72-260 (Chebyshev approximation,
//                                          eigen bounds, power iteration,
//                                          noise, hi_ewald)
//   PMSystemStokes  pm_system_stokes.h      (compute_point_velocity: FEM
//                                          point values + local velocity)
// Vectors keep the reference's PETSc layout [f1x, f1y, f1z, f2x, ...].
// Errors follow the reference: a failing call that the reference ends with
// libmesh_error() throws ggem_copss::Error; calls that return a
// PetscErrorCode or bool keep that convention.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "ggem_fem.h"
#include "ggem_gb300.h"

namespace ggem_copss {

using Point = std::array<double, 3>;
using Tensor = std::array<double, 9>;  // row major 3x3

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc, const ggem_ctx *ctx) {
  if (rc < 0)
    throw Error(rc, std::string(ggem_strerror(rc)) + ": " + (ctx ? ggem_last_error(ctx) : ""));
}

// The particle system the library works on: box, neighbour rule, positions.
class ParticleSystem {
 public:
  explicit ParticleSystem(const ggem_params &p) {
    check(ggem_create(&p, &ctx_), nullptr);
  }
  ~ParticleSystem() { ggem_destroy(ctx_); }
  ParticleSystem(const ParticleSystem &) = delete;
  ParticleSystem &operator=(const ParticleSystem &) = delete;

  // PointMesh::reinit (point_mesh.C:245-289) for positions xyz[3n]
  void reinit(const std::vector<double> &xyz) {
    n_ = (int64_t)(xyz.size() / 3);
    check(ggem_set_particles(ctx_, n_, xyz.data()), ctx_);
    check(ggem_build_cells(ctx_), ctx_);
  }
  int64_t num_particles() const { return n_; }
  ggem_ctx *ctx() const { return ctx_; }

 private:
  ggem_ctx *ctx_ = nullptr;
  int64_t n_ = 0;
};

class GGEMStokes {
 public:
  explicit GGEMStokes(ParticleSystem &ps) : ps_(ps) {
    check(ggem_get_constants(ps.ctx(), &c_), ps.ctx());
  }
  double get_alpha() const { return c_.alpha; }
  double get_ksi() const { return c_.ksi; }
  double get_mu() const { return c_.mu; }
  double get_br0() const { return c_.br0; }

  // green_tensor_local_regularized (ggem_stokes.C:304-357)
  Tensor green_tensor_local_regularized(const Point &x) const {
    Tensor G{};
    check(ggem_green_tensor_local(ps_.ctx(), 1, x.data(), G.data()), ps_.ctx());
    return G;
  }

  // smoothed_force_exp (ggem_stokes.C:117-128), evaluated on the host: a
  // scalar of three constants, not worth a device round trip
  double smoothed_force_exp(const Point &r) const;

  // local_solution_bead for every bead at once (ggem_stokes.C:427-503);
  // self_mode chooses the compute_point_velocity self term
  std::vector<double> local_solution_beads(const std::vector<double> &f,
                                           int self_mode = GGEM_SELF_NONE) const {
    std::vector<double> u(f.size());
    check(ggem_local_matvec(ps_.ctx(), (int)(f.size() / (3 * ps_.num_particles())), f.data(),
                            u.data(), self_mode),
          ps_.ctx());
    return u;
  }

  // local_solution_field at many field points (ggem_stokes.C:360-424)
  std::vector<double> local_solution_field(const std::vector<double> &pts,
                                           const std::vector<double> &f) const {
    std::vector<double> u(pts.size());
    check(ggem_local_field(ps_.ctx(), (int64_t)(pts.size() / 3), pts.data(), f.data(), u.data()),
          ps_.ctx());
    return u;
  }

  // global_self_exclusion (ggem_stokes.C:506-523): coeff_1 * f
  Point global_self_exclusion(const Point &f) const {
    return Point{c_.coeff_1 * f[0], c_.coeff_1 * f[1], c_.coeff_1 * f[2]};
  }

  // AssembleStokes::compute_element_rhs force part (assemble_stokes.C:645-671)
  std::vector<double> element_rhs(int64_t n_elem, int nq, int n_u, const std::vector<double> &qxyz,
                                  const std::vector<double> &int_force,
                                  const std::vector<double> &f, double spread_rc = 0.0) const {
    std::vector<double> Fe((size_t)n_elem * 3 * n_u);
    check(ggem_element_rhs(ps_.ctx(), n_elem, nq, n_u, qxyz.data(), int_force.data(), f.data(),
                           spread_rc, Fe.data()),
          ps_.ctx());
    return Fe;
  }

  const ggem_constants &constants() const { return c_; }

 private:
  ParticleSystem &ps_;
  ggem_constants c_{};
};

inline double GGEMStokes::smoothed_force_exp(const Point &r) const {
  const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  const double a2r2 = c_.alpha2 * r2;
  return c_.alpha3_pi_23 * std::exp(-a2r2) * (2.5 - a2r2);
}

class Chebyshev {
 public:
  // chebyshev_coefficients (chebyshev.C:57-107); method "Gauss",
  // "Gauss_Radau" or "Gauss_Lobatto" (anything else means "Gauss", :68-70)
  std::vector<double> chebyshev_coefficients(std::size_t N, double da, double db,
                                             const std::string &method) const {
    int m = GGEM_CHEB_GAUSS;
    if (method == "Gauss_Lobatto") m = GGEM_CHEB_GAUSS_LOBATTO;
    else if (method == "Gauss_Radau") m = GGEM_CHEB_GAUSS_RADAU;
    std::vector<double> c(N + 1);
    check(ggem_cheb_coeffs((int)N, da, db, m, c.data()), nullptr);
    return c;
  }
};

class BrownianSystem {
 public:
  explicit BrownianSystem(ParticleSystem &ps) : ps_(ps) {}

  // RandomGenerator::set_seed (random_generator.C:96-99)
  void set_std_random_seed(std::size_t seed) { engine_.seed(seed); }

  // std_random_vector(a, b, "gaussian") (brownian_system.C:434-472 with
  // random_generator.C:43-67): a fresh normal distribution per vector drawn
  // from the one seeded engine
  std::vector<double> std_random_vector(double a, double b) {
    std::vector<double> v(3 * (size_t)ps_.num_particles());
    std::normal_distribution<double> dist(a, b);
    dist.reset();
    for (double &x : v) x = dist(engine_);
    return v;
  }

  // chebyshev_polynomial_approximation (brownian_system.C:967-1178):
  // dw becomes y ~ M^{-1/2} dw; returns the convergence flag
  bool chebyshev_polynomial_approximation(std::size_t N, double eigen_min, double eigen_max,
                                          double tol_cheb, std::vector<double> &dw,
                                          ggem_cheb_report *report = nullptr) {
    ggem_cheb_report rep{};
    const int rc = ggem_cheb_inv_sqrt(ps_.ctx(), 1, (int)N, eigen_min, eigen_max, tol_cheb, 1,
                                      dw.data(), &rep);
    check(rc, ps_.ctx());
    if (report) *report = rep;
    return rep.converged != 0;
  }

  // compute_eigenvalues (brownian_system.C:803-843); returns 0 like the
  // PetscErrorCode, throws on a non-positive eigenvalue as libmesh_error()
  int compute_eigenvalues(double &eig_min, double &eig_max, double /*tol*/, int k = 24,
                          uint64_t seed = 7) {
    check(ggem_lanczos_bounds(ps_.ctx(), k, seed, &eig_min, &eig_max), ps_.ctx());
    return 0;
  }

  // power_iteration (brownian_system.C:846-920)
  double power_iteration(double tol = 1e-3, int maxits = 50) {
    double eig = 0.0;
    check(ggem_power_iteration(ps_.ctx(), tol, maxits, &eig), ps_.ctx());
    return eig;
  }

  // hi_ewald (brownian_system.h:249-252) restricted to the local mobility:
  // u = M f with the bead self term of compute_point_velocity
  int hi_ewald(const std::vector<double> &f, std::vector<double> &u) {
    u.resize(f.size());
    check(ggem_local_matvec(ps_.ctx(), 1, f.data(), u.data(), GGEM_SELF_BEAD), ps_.ctx());
    return 0;
  }

 private:
  ParticleSystem &ps_;
  std::default_random_engine engine_;
};

// PMSystemStokes::compute_point_velocity (pm_system_stokes.C:383-500): the
// FEM solution at every particle (point_value of u, v, w on the HEX20 mesh)
// plus, for option "disturbed", the local velocity with the bead self term
// (U = U_global + U_local - coeff_1 f + f).  The mesh's dof map
// ([n_elem][u, v, w][20 nodes], DofMap::dof_indices per element in libMesh's
// Hex20 node order) is uploaded once.
class PMSystemStokes {
 public:
  PMSystemStokes(ParticleSystem &ps, const std::array<int, 3> &n_elem, const Point &lo,
                 const Point &hi, int64_t n_dofs, const std::vector<int64_t> &elem_dofs)
      : ps_(ps) {
    check(ggem_fem_create(ps.ctx(), n_elem.data(), lo.data(), hi.data(), n_dofs,
                          elem_dofs.data(), &fem_),
          ps.ctx());
  }
  ~PMSystemStokes() { ggem_fem_destroy(fem_); }
  PMSystemStokes(const PMSystemStokes &) = delete;
  PMSystemStokes &operator=(const PMSystemStokes &) = delete;

  void compute_point_velocity(const std::vector<double> &solution, const std::vector<double> &f,
                              const std::string &option, std::vector<double> &pv) const {
    pv.assign(3 * ps_.num_particles(), 0.0);
    if (option == "disturbed") {
      check(ggem_local_matvec(ps_.ctx(), 1, f.data(), pv.data(), GGEM_SELF_BEAD), ps_.ctx());
      check(ggem_fem_point_values(fem_, solution.data(), pv.data(), 1), ps_.ctx());
    } else if (option == "undisturbed") {
      check(ggem_fem_point_values(fem_, solution.data(), pv.data(), 0), ps_.ctx());
    } else {
      throw Error(GGEM_ERR_BAD_ARG, "compute_point_velocity: option must be disturbed or undisturbed");
    }
  }

 private:
  ParticleSystem &ps_;
  ggem_fem *fem_ = nullptr;
};

}  // namespace ggem_copss
