// ref_ggem_entry.cpp -- TEST INFRASTRUCTURE ONLY.
//
// C entry points around the reference's own GGEMStokes (ggem_stokes.h:43-340,
// ggem_stokes.C), compiled from the reference source tree into
// oracle/_ref/libref_ggem.so by oracle/Makefile, with the stand-in
// PointMesh of oracle/ref_shim_ggem/point_mesh.h.  The tests pin the
// oracle's restatement of the Green tensor and of the bead and field local
// sums against it.
//
// Constants are set as the reference's PMSystemStokes does before a solve:
// set_mu, set_alpha, set_point_type, set_br0, set_hmin, set_ibm_beta,
// set_ksi (ggem_stokes.C:41-110).
#include <cstdint>
#include <string>
#include <vector>

#include "ggem_stokes.h"

using libMesh::GGEMStokes;
using libMesh::Point;
using libMesh::PointMesh;
using libMesh::PointParticle;
using libMesh::PointType;

namespace {

bool make_ggem(GGEMStokes &g, double mu, double alpha, double br0, int point_type,
               double hmin, double ibm_beta) {
  if (point_type < 0 || point_type > 2) return false;
  g.set_mu(mu);
  g.set_alpha(alpha);
  g.set_point_type(static_cast<PointType>(point_type));
  g.set_br0(br0);
  g.set_hmin(hmin);
  g.set_ibm_beta(ibm_beta);
  g.set_ksi();
  return true;
}

struct MeshHolder {
  PointMesh<3> pm;
  std::vector<PointParticle> store;
  MeshHolder(const double *lo, const double *hi, const int *periodic, int64_t n,
             const double *xyz, const double *f, int point_type) {
    for (int d = 0; d < 3; ++d) {
      pm.pbc.lo(d) = lo[d];
      pm.pbc.L(d) = hi[d] - lo[d];
      pm.pbc.periodic[d] = periodic[d] != 0;
    }
    store.resize(static_cast<std::size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
      PointParticle &p = store[static_cast<std::size_t>(i)];
      p.pt = Point(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
      p.force = Point(f[3 * i], f[3 * i + 1], f[3 * i + 2]);
      p.type = static_cast<PointType>(point_type);
    }
    for (auto &p : store) pm.parts.push_back(&p);
  }
};

}  // namespace

// green_tensor_local_regularized (ggem_stokes.C:304-352) of one vector x
extern "C" int ref_ggem_green_local(double mu, double alpha, double br0, int point_type,
                                    double hmin, double ibm_beta, const double *x,
                                    double *G) {
  GGEMStokes g;
  if (!make_ggem(g, mu, alpha, br0, point_type, hmin, ibm_beta)) return -1;
  const libMesh::DenseMatrix<libMesh::Number> T =
      g.green_tensor_local_regularized(Point(x[0], x[1], x[2]));
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) G[3 * i + j] = T(i, j);
  return 0;
}

// Per bead: local_solution_bead (ggem_stokes.C:426-503) over the CSR
// neighbour lists (offsets[n + 1], ids) with the neighbour vectors of
// PointMesh::reinit_neighbor_vector, and global_self_exclusion
// (ggem_stokes.C:506-521).  u_local and u_self are [n, 3].
extern "C" int ref_ggem_local_bead(double mu, double alpha, double br0, int point_type,
                                   double hmin, double ibm_beta, const double *lo,
                                   const double *hi, const int *periodic, int64_t n,
                                   const double *xyz, const double *f,
                                   const int64_t *offsets, const int32_t *ids,
                                   double *u_local, double *u_self) {
  GGEMStokes g;
  if (!make_ggem(g, mu, alpha, br0, point_type, hmin, ibm_beta)) return -1;
  MeshHolder h(lo, hi, periodic, n, xyz, f, point_type);
  for (int64_t i = 0; i < n; ++i) {
    PointParticle &p = h.store[static_cast<std::size_t>(i)];
    for (int64_t k = offsets[i]; k < offsets[i + 1]; ++k)
      p.nb.push_back(static_cast<libMesh::dof_id_type>(ids[k]));
  }
  h.pm.reinit_neighbor_vector();
  const std::string ftype = "regularized";
  for (int64_t i = 0; i < n; ++i) {
    const std::size_t id = static_cast<std::size_t>(i);
    const Point ul = g.local_solution_bead(&h.pm, id, ftype);
    const Point us = g.global_self_exclusion(&h.pm, id);
    for (int d = 0; d < 3; ++d) {
      u_local[3 * i + d] = ul(d);
      u_self[3 * i + d] = us(d);
    }
  }
  return 0;
}

// local_solution_field (ggem_stokes.C:358-423) at n_t target points, each
// with the element that holds it; elem_offsets[n_elem + 1] / elem_ids are
// the element point-neighbour lists.
extern "C" int ref_ggem_local_field(double mu, double alpha, double br0, int point_type,
                                    double hmin, double ibm_beta, const double *lo,
                                    const double *hi, const int *periodic, int64_t n,
                                    const double *xyz, const double *f, int64_t n_elem,
                                    const int64_t *elem_offsets, const int32_t *elem_ids,
                                    int64_t n_t, const double *targets,
                                    const int32_t *target_elem, double *u) {
  GGEMStokes g;
  if (!make_ggem(g, mu, alpha, br0, point_type, hmin, ibm_beta)) return -1;
  MeshHolder h(lo, hi, periodic, n, xyz, f, point_type);
  h.pm.mesh.ne = static_cast<std::size_t>(n_elem);
  h.pm.elem_lists.resize(static_cast<std::size_t>(n_elem));
  for (int64_t e = 0; e < n_elem; ++e)
    for (int64_t k = elem_offsets[e]; k < elem_offsets[e + 1]; ++k)
      h.pm.elem_lists[static_cast<std::size_t>(e)].push_back(
          static_cast<libMesh::dof_id_type>(elem_ids[k]));
  const std::string ftype = "regularized";
  for (int64_t t = 0; t < n_t; ++t) {
    if (target_elem[t] < 0 || target_elem[t] >= n_elem) return -2;
    const Point x(targets[3 * t], targets[3 * t + 1], targets[3 * t + 2]);
    const Point ut = g.local_solution_field(
        &h.pm, x, ftype, static_cast<libMesh::dof_id_type>(target_elem[t]));
    for (int d = 0; d < 3; ++d) u[3 * t + d] = ut(d);
  }
  return 0;
}
