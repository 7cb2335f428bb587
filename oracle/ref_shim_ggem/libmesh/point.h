// A 3-vector with the operations the reference's ggem_stokes.C uses,
// standing in for libMesh::Point (TEST INFRASTRUCTURE ONLY).
#pragma once
#include <cmath>

#include "libmesh/libmesh_common.h"

namespace libMesh {
class Point {
 public:
  explicit Point(Real x = 0, Real y = 0, Real z = 0) : v_{x, y, z} {}
  Real &operator()(std::size_t i) { return v_[i]; }
  const Real &operator()(std::size_t i) const { return v_[i]; }
  Point operator-(const Point &o) const { return Point(v_[0] - o.v_[0], v_[1] - o.v_[1], v_[2] - o.v_[2]); }
  Point operator+(const Point &o) const { return Point(v_[0] + o.v_[0], v_[1] + o.v_[1], v_[2] + o.v_[2]); }
  Point operator*(Real a) const { return Point(v_[0] * a, v_[1] * a, v_[2] * a); }
  Point &operator+=(const Point &o) {
    for (int i = 0; i < 3; ++i) v_[i] += o.v_[i];
    return *this;
  }
  Real norm_sq() const { return v_[0] * v_[0] + v_[1] * v_[1] + v_[2] * v_[2]; }
  Real norm() const { return std::sqrt(norm_sq()); }
 private:
  Real v_[3];
};
}  // namespace libMesh
