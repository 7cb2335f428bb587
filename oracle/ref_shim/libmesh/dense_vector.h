// Row container with operator(), standing in for libMesh::DenseVector.
#pragma once
#include "libmesh/libmesh_common.h"
namespace libMesh {
template <typename T>
class DenseVector {
 public:
  explicit DenseVector(std::size_t n = 0) : v_(n, T(0)) {}
  T &operator()(std::size_t i) { return v_[i]; }
  const T &operator()(std::size_t i) const { return v_[i]; }
  std::size_t size() const { return v_.size(); }
 private:
  std::vector<T> v_;
};
}  // namespace libMesh
