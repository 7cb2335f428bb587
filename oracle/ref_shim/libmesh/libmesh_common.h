// Minimal stand-in for the libMesh declarations that the reference's
// chebyshev.C and ggem_stokes.C use (Real, Number, dof_id_type, libMesh::pi,
// START_LOG/STOP_LOG, libmesh_error).  Only for compiling those reference
// files into the test oracle; no libMesh code is reproduced here.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>
namespace libMesh {
typedef double Real;
typedef double Number;
typedef uint32_t dof_id_type;
const Real pi = 3.1415926535897932384626433832795029L;
}  // namespace libMesh
#define START_LOG(a, b) ((void)0)
#define STOP_LOG(a, b) ((void)0)
#define libmesh_error() throw std::runtime_error("libmesh_error")
