// Row-major container with operator()(i, j) and scaling by a scalar,
// standing in for libMesh::DenseMatrix.
#pragma once
#include "libmesh/dense_vector.h"
namespace libMesh {
template <typename T>
class DenseMatrix {
 public:
  DenseMatrix(std::size_t m = 0, std::size_t n = 0) : m_(m), n_(n), v_(m * n, T(0)) {}
  T &operator()(std::size_t i, std::size_t j) { return v_[i * n_ + j]; }
  const T &operator()(std::size_t i, std::size_t j) const { return v_[i * n_ + j]; }
  DenseMatrix &operator*=(const T &a) {
    for (T &x : v_) x *= a;
    return *this;
  }
  std::size_t m() const { return m_; }
  std::size_t n() const { return n_; }
 private:
  std::size_t m_, n_;
  std::vector<T> v_;
};
}  // namespace libMesh
