// ggem_fem.cu -- the global (FEM) velocity at the particles: System::point_value
// of the SECOND-order u, v, w on the HEX20 box mesh, as called by
// PMSystemStokes::compute_point_velocity (pm_system_stokes.C:437-441).
//
// One thread per particle: element from the uniform mesh (the floor rule of
// the cell build), reference coordinates, the 20 serendipity shape
// functions, and a gather of the 60 nodal values through the driver's dof
// map.  Per particle: 60 dof indices + 60 solution values read, 24 bytes
// written; FP64 throughout.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "ggem_fem.h"
#include "ggem_internal.cuh"

namespace ggem {
namespace {

// libMesh Hex20 node positions on [-1, 1]^3 (corners, then edge midpoints)
struct Hex20Nodes {
  signed char x[20], y[20], z[20];
};
__host__ __device__ constexpr Hex20Nodes hex20_nodes() {
  return Hex20Nodes{{-1, 1, 1, -1, -1, 1, 1, -1, 0, 1, 0, -1, -1, 1, 1, -1, 0, 1, 0, -1},
                    {-1, -1, 1, 1, -1, -1, 1, 1, -1, 0, 1, 0, -1, -1, 1, 1, -1, 0, 1, 0},
                    {-1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0, 1, 1, 1, 1}};
}

// serendipity shape functions: corner (a, b, c) = +-1:
//   N = (1 + a x)(1 + b y)(1 + c z)(a x + b y + c z - 2) / 8;
// edge node with one zero coordinate, e.g. (0, b, c):
//   N = (1 - x^2)(1 + b y)(1 + c z) / 4
__host__ __device__ inline void hex20_shape(double x, double y, double z, double n[20]) {
  constexpr Hex20Nodes P = hex20_nodes();
#pragma unroll
  for (int k = 0; k < 20; ++k) {
    const double a = P.x[k], b = P.y[k], c = P.z[k];
    if (k < 8) {
      n[k] = 0.125 * (1.0 + a * x) * (1.0 + b * y) * (1.0 + c * z) * (a * x + b * y + c * z - 2.0);
    } else if (a == 0.0) {
      n[k] = 0.25 * (1.0 - x * x) * (1.0 + b * y) * (1.0 + c * z);
    } else if (b == 0.0) {
      n[k] = 0.25 * (1.0 + a * x) * (1.0 - y * y) * (1.0 + c * z);
    } else {
      n[k] = 0.25 * (1.0 + a * x) * (1.0 + b * y) * (1.0 - z * z);
    }
  }
}

struct FemGrid {
  double lo[3], L[3], h[3], inv_h[3];
  int ne[3];
  int periodic[3];
};

// element index and reference coordinate along one axis (the wrap and floor
// rule of k_assign); false when x lies outside a non-periodic axis
__device__ inline bool locate(const FemGrid &g, int d, double x, int &e, double &xi) {
  double t = x - g.lo[d];
  bool ok = true;
  if (g.periodic[d]) {
    if (!(t >= 0.0 && t < g.L[d])) {
      t = fmod(t, g.L[d]);
      if (t < 0) t += g.L[d];
      if (t >= g.L[d]) t = 0.0;
    }
  } else if (!(t >= 0.0 && t <= g.L[d])) {
    ok = false;
  }
  const double q = t * g.inv_h[d];
  double fq = floor(q);
  if (q - fq < 1e-9 || (fq + 1.0) - q < 1e-9 || !(fabs(q) < 1e6)) fq = floor(t / g.h[d]);
  int k = (int)fq;
  k = k < 0 ? 0 : (k >= g.ne[d] ? g.ne[d] - 1 : k);
  e = k;
  // xi = 2 (t - k h) / h - 1, in [-1, 1] inside the element
  xi = (t - k * g.h[d]) * (2.0 * g.inv_h[d]) - 1.0;
  return ok;
}

template <typename I>
__global__ void k_fem_values(int64_t n, const double *__restrict__ xyz, FemGrid g,
                             const I *__restrict__ dofs, const double *__restrict__ sol,
                             double *__restrict__ u, int accumulate, int *__restrict__ err) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int e[3];
  double xi[3];
  bool ok = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) ok &= locate(g, d, xyz[3 * i + d], e[d], xi[d]);
  if (!ok) atomicOr(err, kErrOutOfDomain);
  double nf[20];
  hex20_shape(xi[0], xi[1], xi[2], nf);
  const int64_t elem = e[0] + (int64_t)g.ne[0] * (e[1] + (int64_t)g.ne[1] * e[2]);
  const I *ed = dofs + elem * 60;
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 20; ++k) s = fma(nf[k], sol[ed[20 * v + k]], s);
    u[3 * i + v] = accumulate ? u[3 * i + v] + s : s;
  }
}

struct FemGuard {
  int prev = -1;
  explicit FemGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~FemGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

}  // namespace
}  // namespace ggem

using namespace ggem;

struct ggem_fem {
  ggem_ctx *ctx = nullptr;
  FemGrid grid{};
  int64_t n_elem = 0, n_dofs = 0;
  bool wide = false;  // dof indices kept as int64 (n_dofs >= 2^31)
  DevBuf<int32_t> dofs32;
  DevBuf<int64_t> dofs64;
  DevBuf<double> sol, u;
  DevBuf<int> err;
};

extern "C" void ggem_fem_hex20_shape(const double xi[3], double n[20]) {
  hex20_shape(xi[0], xi[1], xi[2], n);
}

extern "C" int ggem_fem_create(ggem_ctx *ctx, const int n_elem[3], const double lo[3],
                               const double hi[3], int64_t n_dofs, const int64_t *elem_dofs,
                               ggem_fem **out) {
  if (!ctx || !n_elem || !lo || !hi || !elem_dofs || !out || n_dofs < 1) return GGEM_ERR_BAD_ARG;
  *out = nullptr;
  int64_t ne = 1;
  for (int d = 0; d < 3; ++d) {
    if (n_elem[d] < 1 || !(hi[d] > lo[d]))
      return fail(ctx, GGEM_ERR_BAD_ARG, "fem mesh: n_elem >= 1 and hi > lo on every axis");
    ne *= n_elem[d];
  }
  for (int64_t k = 0; k < ne * 60; ++k)
    if (elem_dofs[k] < 0 || elem_dofs[k] >= n_dofs)
      return fail(ctx, GGEM_ERR_BAD_ARG, "fem mesh: dof index out of [0, n_dofs)");
  FemGuard g(ctx->device);
  ggem_fem *f = new ggem_fem();
  f->ctx = ctx;
  f->n_elem = ne;
  f->n_dofs = n_dofs;
  f->wide = n_dofs > 0x7fffffffLL;
  for (int d = 0; d < 3; ++d) {
    f->grid.lo[d] = lo[d];
    f->grid.L[d] = hi[d] - lo[d];
    f->grid.ne[d] = n_elem[d];
    f->grid.h[d] = f->grid.L[d] / n_elem[d];
    f->grid.inv_h[d] = 1.0 / f->grid.h[d];
    f->grid.periodic[d] = ctx->prm.periodic[d];
  }
  cudaError_t e = f->err.ensure(1);
  if (e == cudaSuccess) {
    if (f->wide) {
      e = f->dofs64.ensure((size_t)ne * 60);
      if (e == cudaSuccess)
        e = cudaMemcpy(f->dofs64.p, elem_dofs, sizeof(int64_t) * ne * 60, cudaMemcpyHostToDevice);
    } else {
      std::vector<int32_t> d32((size_t)ne * 60);
      for (size_t k = 0; k < d32.size(); ++k) d32[k] = (int32_t)elem_dofs[k];
      e = f->dofs32.ensure(d32.size());
      if (e == cudaSuccess)
        e = cudaMemcpy(f->dofs32.p, d32.data(), sizeof(int32_t) * d32.size(),
                       cudaMemcpyHostToDevice);
    }
  }
  if (e != cudaSuccess) {
    const int rc = cuda_fail(ctx, e, "fem mesh upload");
    delete f;
    return rc;
  }
  *out = f;
  return GGEM_OK;
}

extern "C" void ggem_fem_destroy(ggem_fem *f) {
  if (!f) return;
  FemGuard g(f->ctx->device);
  cudaStreamSynchronize(f->ctx->stream);
  delete f;
}

extern "C" int ggem_fem_point_values_dev(ggem_fem *f, const double *d_solution, double *d_u,
                                         int accumulate) {
  if (!f || !d_solution || (!d_u && f->ctx->n)) return GGEM_ERR_BAD_ARG;
  ggem_ctx *c = f->ctx;
  if (c->n == 0) return GGEM_OK;
  FemGuard g(c->device);
  cudaStream_t st = c->stream;
  cudaError_t e = cudaMemsetAsync(f->err.p, 0, sizeof(int), st);
  if (e) return cuda_fail(c, e, "fem memset");
  const unsigned bn = (unsigned)((c->n + 127) / 128);
  if (f->wide)
    k_fem_values<<<bn, 128, 0, st>>>(c->n, c->xyz_in.p, f->grid, f->dofs64.p, d_solution, d_u,
                                     accumulate, f->err.p);
  else
    k_fem_values<<<bn, 128, 0, st>>>(c->n, c->xyz_in.p, f->grid, f->dofs32.p, d_solution, d_u,
                                     accumulate, f->err.p);
  if (int rc = check_launch(c, "fem point values")) return rc;
  int flags = 0;
  e = cudaMemcpyAsync(&flags, f->err.p, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e) return cuda_fail(c, e, "fem flags");
  if (flags & kErrOutOfDomain)
    return fail(c, GGEM_ERR_OUT_OF_DOMAIN,
                "a particle lies outside the FEM mesh on a non-periodic axis "
                "(pm_system_stokes.C:417-424)");
  return GGEM_OK;
}

extern "C" int ggem_fem_point_values(ggem_fem *f, const double *solution, double *u,
                                     int accumulate) {
  if (!f || !solution || (!u && f->ctx->n)) return GGEM_ERR_BAD_ARG;
  ggem_ctx *c = f->ctx;
  if (c->n == 0) return GGEM_OK;
  FemGuard g(c->device);
  cudaStream_t st = c->stream;
  const size_t len = (size_t)c->n * 3;
  cudaError_t e;
  if ((e = f->sol.ensure((size_t)f->n_dofs)) || (e = f->u.ensure(len)))
    return cuda_fail(c, e, "fem buffers");
  if ((e = cudaMemcpyAsync(f->sol.p, solution, sizeof(double) * f->n_dofs,
                           cudaMemcpyHostToDevice, st)))
    return cuda_fail(c, e, "fem solution copy");
  if (accumulate && (e = cudaMemcpyAsync(f->u.p, u, sizeof(double) * len,
                                         cudaMemcpyHostToDevice, st)))
    return cuda_fail(c, e, "fem velocity copy");
  if (int rc = ggem_fem_point_values_dev(f, f->sol.p, f->u.p, accumulate)) return rc;
  if ((e = cudaMemcpyAsync(u, f->u.p, sizeof(double) * len, cudaMemcpyDeviceToHost, st)) ||
      (e = cudaStreamSynchronize(st)))
    return cuda_fail(c, e, "fem velocity copy back");
  return GGEM_OK;
}
