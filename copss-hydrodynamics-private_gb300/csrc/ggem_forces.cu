// ggem_forces.cu -- excluded-volume and spring forces on the GPU
// (include/ggem_forces.h), FP64.
//
// Excluded volume: one thread per target slot sweeps the same neighbour
// cells as the FP64 mobility sweep (cut-off mode: stencil + |r| < rc with the
// oracle's predicate; reference mode: own element then the element stencil,
// no cut-off), summing FixBase::gaussian_force (fix/fix_base.C:150-162) as
// FixPointGaussianDNA::compute does (fix/fix_point_gaussian_dna.C:69-84).
// Springs: one thread per bead sums the spring law over its bonds (the
// adjacency keeps bond order); bead i of bond (i, j) gets f(x_j - x_i), bead
// j gets f(x_i - x_j) = -f(x_j - x_i), as FixPointWLS::compute
// (fix/fix_point_wls.C:66-92) adds F_ij and F_ji.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "ggem_forces.h"
#include "ggem_internal.cuh"

namespace ggem {
namespace {

__device__ __forceinline__ void min_image_f(const Grid &g, double d[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (g.periodic[k]) {
      const double xs = g.L[k];
      if (d[k] <= -xs / 2.0) d[k] += xs;
      if (d[k] > xs / 2.0) d[k] -= xs;
    }
  }
}

__device__ __forceinline__ int wrap_f(int k, int n) {
  k %= n;
  return k < 0 ? k + n : k;
}

__global__ void __launch_bounds__(128) k_ev_gaussian(int64_t n, Grid g,
                                                     const int4 *__restrict__ stencil, int nst,
                                                     int own_first, int use_cutoff, double rc2,
                                                     const int32_t *__restrict__ start,
                                                     const int32_t *__restrict__ order,
                                                     const double4_32a *__restrict__ pos64,
                                                     const float4 *__restrict__ pos32, double c1,
                                                     double c2, double *__restrict__ f,
                                                     int accumulate) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const double4_32a pi = pos64[s];
  const int32_t cid = __float_as_int(pos32[s].w);
  const int cx = cid % g.nc[0], cy = (cid / g.nc[0]) % g.nc[1], cz = cid / (g.nc[0] * g.nc[1]);
  double acc[3] = {0.0, 0.0, 0.0};
  const double c12 = c1 * c2;
  for (int k = own_first ? -1 : 0; k < nst; ++k) {
    const int4 o = (k < 0) ? make_int4(0, 0, 0, 0) : stencil[k];
    int c[3] = {cx + o.x, cy + o.y, cz + o.z};
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (c[d] < 0 || c[d] >= g.nc[d]) {
        if (!g.periodic[d]) ok = false;
        else c[d] = wrap_f(c[d], g.nc[d]);
      }
    }
    if (!ok) continue;
    const int32_t nc = c[0] + g.nc[0] * (c[1] + g.nc[1] * c[2]);
    for (int32_t t = start[nc]; t < start[nc + 1]; ++t) {
      if (t == s) continue;
      const double4_32a pj = pos64[t];
      double x[3] = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z};
      min_image_f(g, x);
      if (use_cutoff) {
        const double r2c = __dadd_rn(__dadd_rn(__dmul_rn(x[0], x[0]), __dmul_rn(x[1], x[1])),
                                     __dmul_rn(x[2], x[2]));
        if (!(r2c < rc2)) continue;
      }
      const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
      const double w = -c12 * exp(-c2 * r * r);
      acc[0] += w * x[0];
      acc[1] += w * x[1];
      acc[2] += w * x[2];
    }
  }
  double *fi = f + 3 * (int64_t)order[s];
#pragma unroll
  for (int d = 0; d < 3; ++d) fi[d] = accumulate ? fi[d] + acc[d] : acc[d];
}

// FixBase spring laws (fix_base.C:55-148) on R = x_j - x_i
__device__ __forceinline__ double spring_scale(int kind, double R, double c1, double Ls) {
  const double tol = 1e-3;  // fix_base.h:50
  if (kind == GGEM_SPRING_WLS) {
    const double ratio = R / Ls;
    double v0 = 1.0 - ratio;
    if (fabs(v0) < tol) v0 = v0 / fabs(v0) * tol;
    return c1 * (1.0 / (v0 * v0) - 1.0 + 4.0 * ratio) / R;
  }
  if (kind == GGEM_SPRING_FENE) {
    const double ratio = R / Ls;
    double v0 = 1.0 - ratio * ratio;
    if (fabs(v0) < tol) v0 = v0 / fabs(v0) * tol * tol;
    return c1 * ratio / v0 / R;
  }
  if (kind == GGEM_SPRING_UD) {
    const double ratio = R / Ls, r2 = ratio * ratio, cc = c1 * c1;
    const double a1 = 1.0, a2 = -7.0 * c1, a3 = 3.0 / 32.0 - 0.75 * c1 - 6.0 * cc;
    const double a4 = (13.0 / 32.0 + 0.8172 * c1 - 14.79 * cc) / (1.0 - 4.225 * c1 + 4.87 * cc);
    const double T4 = 1.0 - r2, T2 = 1.0 / T4, T1 = T2 / T4;
    return (a1 * T1 + a2 * T2 + a3 + a4 * T4) / R;
  }
  // GGEM_SPRING_LHS: k0 (|R| - l0) with l0 = c1, k0 = Ls
  return Ls * (R - c1) / R;
}

__global__ void k_springs(int64_t n, Grid g, const double4_32a *__restrict__ xyz,
                          const int64_t *__restrict__ off, const int32_t *__restrict__ nbr,
                          int kind, double c1, double Ls, double *__restrict__ f,
                          int accumulate) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4_32a pi = xyz[i];
  double acc[3] = {0.0, 0.0, 0.0};
  for (int64_t k = off[i]; k < off[i + 1]; ++k) {
    const double4_32a pj = xyz[nbr[k]];
    double x[3] = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z};
    min_image_f(g, x);
    const double R = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    const double w = spring_scale(kind, R, c1, Ls);
    acc[0] += w * x[0];
    acc[1] += w * x[1];
    acc[2] += w * x[2];
  }
  double *fi = f + 3 * i;
#pragma unroll
  for (int d = 0; d < 3; ++d) fi[d] = accumulate ? fi[d] + acc[d] : acc[d];
}

struct FGuard {
  int prev = -1;
  explicit FGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~FGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// host-pointer wrappers: copy f in (accumulate) and out through w_a
template <typename Fn>
int with_host_forces(ggem_ctx *c, double *f, int accumulate, Fn fn) {
  const size_t len = (size_t)3 * std::max<int64_t>(c->n, 1);
  cudaError_t e = c->w_a.ensure(len);
  if (e) return cuda_fail(c, e, "force buffer");
  if (c->n && accumulate &&
      (e = cudaMemcpyAsync(c->w_a.p, f, sizeof(double) * 3 * c->n, cudaMemcpyHostToDevice,
                           c->stream)))
    return cuda_fail(c, e, "forces in");
  if (int rc = fn(c->w_a.p)) return rc;
  if (c->n && (e = cudaMemcpyAsync(f, c->w_a.p, sizeof(double) * 3 * c->n,
                                   cudaMemcpyDeviceToHost, c->stream)))
    return cuda_fail(c, e, "forces out");
  if ((e = cudaStreamSynchronize(c->stream))) return cuda_fail(c, e, "forces");
  return GGEM_OK;
}

}  // namespace
}  // namespace ggem

using namespace ggem;

extern "C" int ggem_ev_gaussian_forces_dev(ggem_ctx *ctx, double c1, double c2, double *d_f,
                                           int accumulate) {
  if (!ctx || (!d_f && ctx->n)) return GGEM_ERR_BAD_ARG;
  if (int rc = settle_list(ctx)) return rc;
  if (!ctx->cells_built) return fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_build_cells first");
  FGuard g(ctx->device);
  if (ctx->n == 0) return GGEM_OK;
  const bool ref = ctx->prm.nb_mode == GGEM_NB_REFERENCE;
  k_ev_gaussian<<<(unsigned)((ctx->n + 127) / 128), 128, 0, ctx->stream>>>(
      ctx->n, ctx->grid, ctx->d_stencil.p, (int)ctx->stencil.size(), ref ? 1 : 0, ref ? 0 : 1,
      ctx->rc2, ctx->cell_start.p, ctx->order.p, ctx->pos64.p, ctx->pos32.p, c1, c2, d_f,
      accumulate);
  return check_launch(ctx, "excluded volume");
}

extern "C" int ggem_ev_gaussian_forces(ggem_ctx *ctx, double c1, double c2, double *f,
                                       int accumulate) {
  if (!ctx || (!f && ctx->n)) return GGEM_ERR_BAD_ARG;
  if (int rc = settle_list(ctx)) return rc;
  if (!ctx->cells_built) return fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_build_cells first");
  FGuard g(ctx->device);
  return with_host_forces(ctx, f, accumulate, [&](double *d) {
    return ggem_ev_gaussian_forces_dev(ctx, c1, c2, d, accumulate);
  });
}

extern "C" int ggem_set_bonds(ggem_ctx *ctx, int64_t m, const int64_t *bonds) {
  if (!ctx || m < 0 || (m && !bonds)) return GGEM_ERR_BAD_ARG;
  if (ctx->n <= 0) return fail(ctx, GGEM_ERR_BAD_ARG, "set the particles before the bonds");
  FGuard g(ctx->device);
  const int64_t n = ctx->n;
  std::vector<int64_t> off(n + 1, 0);
  for (int64_t k = 0; k < m; ++k) {
    const int64_t a = bonds[2 * k], b = bonds[2 * k + 1];
    if (a < 0 || a >= n || b < 0 || b >= n || a == b)
      return fail(ctx, GGEM_ERR_BAD_ARG, "bond " + std::to_string(k) + " names a bad bead");
    off[a + 1] += 1;
    off[b + 1] += 1;
  }
  for (int64_t i = 0; i < n; ++i) off[i + 1] += off[i];
  std::vector<int32_t> nbr(std::max<int64_t>(2 * m, 1));
  std::vector<int64_t> fill(off.begin(), off.end() - 1);
  for (int64_t k = 0; k < m; ++k) {  // bond order per bead
    const int64_t a = bonds[2 * k], b = bonds[2 * k + 1];
    nbr[fill[a]++] = (int32_t)b;
    nbr[fill[b]++] = (int32_t)a;
  }
  cudaError_t e;
  if ((e = ctx->bond_off.ensure(n + 1)) || (e = ctx->bond_nbr.ensure(nbr.size())) ||
      (e = cudaMemcpyAsync(ctx->bond_off.p, off.data(), sizeof(int64_t) * (n + 1),
                           cudaMemcpyHostToDevice, ctx->stream)) ||
      (e = cudaMemcpyAsync(ctx->bond_nbr.p, nbr.data(), sizeof(int32_t) * nbr.size(),
                           cudaMemcpyHostToDevice, ctx->stream)) ||
      (e = cudaStreamSynchronize(ctx->stream)))
    return cuda_fail(ctx, e, "bonds");
  ctx->bond_n = n;
  return GGEM_OK;
}

extern "C" int ggem_spring_forces_dev(ggem_ctx *ctx, int kind, double c1, double Ls, double *d_f,
                                      int accumulate) {
  if (!ctx || (!d_f && ctx->n) || kind < GGEM_SPRING_WLS || kind > GGEM_SPRING_LHS)
    return GGEM_ERR_BAD_ARG;
  if (int rc = settle_list(ctx)) return rc;
  if (!ctx->cells_built) return fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_build_cells first");
  if (ctx->bond_n != ctx->n) return fail(ctx, GGEM_ERR_BAD_ARG, "set the bonds for these particles");
  FGuard g(ctx->device);
  if (ctx->n == 0) return GGEM_OK;
  k_springs<<<(unsigned)((ctx->n + 255) / 256), 256, 0, ctx->stream>>>(
      ctx->n, ctx->grid, ctx->wrapped.p, ctx->bond_off.p, ctx->bond_nbr.p, kind, c1, Ls, d_f,
      accumulate);
  return check_launch(ctx, "springs");
}

extern "C" int ggem_spring_forces(ggem_ctx *ctx, int kind, double c1, double Ls, double *f,
                                  int accumulate) {
  if (!ctx || (!f && ctx->n)) return GGEM_ERR_BAD_ARG;
  if (int rc = settle_list(ctx)) return rc;
  if (!ctx->cells_built) return fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_build_cells first");
  FGuard g(ctx->device);
  return with_host_forces(ctx, f, accumulate, [&](double *d) {
    return ggem_spring_forces_dev(ctx, kind, c1, Ls, d, accumulate);
  });
}
