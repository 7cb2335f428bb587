// Minimal stand-in for the libMesh declarations that the reference's
// chebyshev.C uses (Real, Number, libMesh::pi, START_LOG/STOP_LOG).  Only
// for compiling that single reference file into the test oracle; no libMesh
// code is reproduced here.
#pragma once
#include <cmath>
#include <cstddef>
#include <string>
#include <vector>
namespace libMesh {
typedef double Real;
typedef double Number;
const Real pi = 3.1415926535897932384626433832795029L;
}  // namespace libMesh
#define START_LOG(a, b) ((void)0)
#define STOP_LOG(a, b) ((void)0)
