// ref_chebyshev_entry.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A C entry point around the reference's own Chebyshev class
// (chebyshev.h:43-105, chebyshev.C:57-107), compiled from the reference
// source tree into oracle/_ref/libref_chebyshev.so by oracle/Makefile.  The
// tests compare the oracle restatement and the CUDA library's coefficients
// against it.
#include <string>

#include "chebyshev.h"

extern "C" int ref_chebyshev_coefficients(int N, double da, double db,
                                          int method, double *out) {
  const char *names[3] = {"Gauss", "Gauss_Radau", "Gauss_Lobatto"};
  if (method < 0 || method > 2 || N < 1) return -1;
  libMesh::Chebyshev cheb;
  libMesh::DenseVector<libMesh::Number> c =
      cheb.chebyshev_coefficients(static_cast<std::size_t>(N), da, db, names[method]);
  for (int k = 0; k <= N; ++k) out[k] = c(k);
  return 0;
}
