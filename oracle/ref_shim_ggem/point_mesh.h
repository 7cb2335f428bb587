// point_mesh.h -- TEST INFRASTRUCTURE ONLY.
//
// A stand-in for the reference's PointMesh, PointParticle and
// PMPeriodicBoundary, just large enough to compile the reference's own
// src/ggem_stokes.C (GGEMStokes) into oracle/_ref: it holds the particles,
// their positions, forces, neighbour lists and neighbour vectors, and the
// element lists that local_solution_field reads.  The periodic minimum image
// restates PMPeriodicBoundary::point_vector (pm_periodic_boundary.C:350-374);
// the neighbour vectors are formed as PointMesh::reinit_neighbor_vector does
// (point_mesh.C:220-241).  oracle/Makefile puts this directory ahead of the
// reference sources (-I-), so ggem_stokes.h and ggem_system.h include this
// file instead of the reference's point_mesh.h, which needs libMesh.
#pragma once
#include <cstddef>
#include <vector>

#include "libmesh/libmesh_common.h"
#include "libmesh/point.h"

namespace libMesh {

enum PointType {
  POLYMER_BEAD = 0,
  LAGRANGIAN_POINT = 1,
  POINT_PARTICLE = 2,
  NOT_DEFINED_POINTTYPE = -1
};

template <typename T>
class ReferenceCountedObject {};

class PMPeriodicBoundary {
 public:
  Point lo, L;
  bool periodic[3] = {false, false, false};
  Point point_vector(const Point &pt0, const Point &pt1) const {
    Point d = pt1 - pt0;
    for (int i = 0; i < 3; ++i) {
      if (periodic[i]) {
        const Real xs = L(i);
        if (d(i) <= -xs / 2.0) d(i) += xs;
        if (d(i) > xs / 2.0) d(i) -= xs;
      }
    }
    return d;
  }
};

class PointParticle {
 public:
  Point pt, force;
  PointType type = POLYMER_BEAD;
  std::vector<dof_id_type> nb;
  std::vector<Point> nbv;
  const Point &point() const { return pt; }
  const Point &particle_force() const { return force; }
  const std::vector<dof_id_type> &neighbor_list() const { return nb; }
  const std::vector<Point> &neighbor_vector() const { return nbv; }
  const PointType &point_type() const { return type; }
};

struct StubMesh {
  std::size_t ne = 0;
  std::size_t n_elem() const { return ne; }
};

template <unsigned int KDDim>
class PointMesh {
 public:
  std::vector<PointParticle *> parts;
  std::vector<std::vector<dof_id_type>> elem_lists;
  PMPeriodicBoundary pbc;
  StubMesh mesh;
  std::vector<PointParticle *> &particles() { return parts; }
  const std::vector<dof_id_type> &get_elem_point_neighbor_list(dof_id_type e) const {
    return elem_lists[e];
  }
  const PMPeriodicBoundary *pm_periodic_boundary() const { return &pbc; }
  const StubMesh &get_mesh() const { return mesh; }
  // PointMesh::reinit_neighbor_vector (point_mesh.C:220-241)
  void reinit_neighbor_vector() {
    for (PointParticle *p : parts) {
      p->nbv.resize(p->nb.size());
      for (std::size_t j = 0; j < p->nb.size(); ++j)
        p->nbv[j] = pbc.point_vector(p->pt, parts[p->nb[j]]->pt);
    }
  }
};

}  // namespace libMesh
