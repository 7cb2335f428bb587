// ggem_spread.cu -- Kernel D and the field-point sums: the Gaussian force
// spreading onto FEM quadrature points (GGEMStokes::smoothed_force_exp,
// ggem_stokes.C:117-128, summed as in AssembleStokes::compute_element_rhs,
// assemble_stokes.C:645-671), the fused element right-hand side, and the
// local velocity at arbitrary field points (GGEMStokes::local_solution_field,
// ggem_stokes.C:360-424).
//
// One thread per target point sweeps the cells within the source radius of
// the target's cell (cut-off mode) or the element stencil of the target's
// element (reference mode).  FP64 throughout.  Algorithmic work per
// (target, source in range): 20 flops + 1 exp (spread), 28 + 19 (field).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "ggem_internal.cuh"

namespace ggem {
namespace {

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

__device__ __forceinline__ int wrap_i(int k, int n) {
  k %= n;
  return k < 0 ? k + n : k;
}

__device__ __forceinline__ void min_image(const Grid &g, double d[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (g.periodic[k]) {
      const double xs = g.L[k];
      if (d[k] <= -xs / 2.0) d[k] += xs;
      if (d[k] > xs / 2.0) d[k] -= xs;
    }
  }
}

struct SweepAxis {
  int first, count, wrap;  // absolute start cell, number of cells, wrap flag
};

__device__ __forceinline__ SweepAxis axis_range(const Grid &g, int d, int c, int range) {
  SweepAxis a;
  if (g.periodic[d]) {
    if (2 * range + 1 >= g.nc[d]) {
      a.first = 0;
      a.count = g.nc[d];
      a.wrap = 0;
    } else {
      a.first = c - range;
      a.count = 2 * range + 1;
      a.wrap = 1;
    }
  } else {
    const int lo = max(0, c - range), hi = min(g.nc[d] - 1, c + range);
    a.first = lo;
    a.count = hi - lo + 1;
    a.wrap = 0;
  }
  return a;
}

// KIND 0: local regularized Stokeslet (3-vector result); KIND 1: Gaussian
// smoothed force density (3-vector rho)
template <int KIND>
__global__ void __launch_bounds__(128) k_field(
    int64_t nt, const double *__restrict__ targets, const int32_t *__restrict__ telem,
    int ref_mode, Grid g, DevConsts K, const int4 *__restrict__ stencil, int nst, int range0,
    int range1, int range2, double R2, const int32_t *__restrict__ start,
    const double4_32a *__restrict__ pos64, const double *__restrict__ f, double *__restrict__ out,
    int *__restrict__ err) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const double p[3] = {targets[3 * t], targets[3 * t + 1], targets[3 * t + 2]};
  int c[3];
  bool outside = false;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double s = p[d] - g.lo[d];
    if (g.periodic[d]) {
      s = fmod(s, g.L[d]);
      if (s < 0) s += g.L[d];
    } else if (!(s >= 0.0 && s <= g.L[d])) {
      outside = true;
    }
    int k = (int)floor(s / g.h[d]);
    c[d] = k < 0 ? 0 : (k >= g.nc[d] ? g.nc[d] - 1 : k);
  }
  double acc[3] = {0.0, 0.0, 0.0};
  if (ref_mode) {
    int e;
    if (telem) {
      e = telem[t];
      if (e < 0 || e >= g.ncell) {
        atomicOr(err, kErrBadIndex);
        e = -1;
      }
    } else {
      if (outside) atomicOr(err, kErrOutOfDomain);
      e = outside ? -1 : c[0] + g.nc[0] * (c[1] + g.nc[1] * c[2]);
    }
    if (e >= 0) {
      const int ex = e % g.nc[0], ey = (e / g.nc[0]) % g.nc[1], ez = e / (g.nc[0] * g.nc[1]);
      for (int k = -1; k < nst; ++k) {
        const int4 o = k < 0 ? make_int4(0, 0, 0, 0) : stencil[k];
        int cc[3] = {ex + o.x, ey + o.y, ez + o.z};
        bool ok = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          if (cc[d] < 0 || cc[d] >= g.nc[d]) {
            if (!g.periodic[d]) ok = false;
            else cc[d] = wrap_i(cc[d], g.nc[d]);
          }
        }
        if (!ok) continue;
        const int32_t cell = cc[0] + g.nc[0] * (cc[1] + g.nc[1] * cc[2]);
        for (int32_t s = start[cell]; s < start[cell + 1]; ++s) {
          const double4_32a q = pos64[s];
          double x[3] = {q.x - p[0], q.y - p[1], q.z - p[2]};
          min_image(g, x);
          const double *fj = f + 3 * (int64_t)s;
          if (KIND == 0) {
            const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
            if (r < K.r_eps) {
              acc[0] += K.coeff_2 * fj[0];
              acc[1] += K.coeff_2 * fj[1];
              acc[2] += K.coeff_2 * fj[2];
            } else {
              const double r2 = r * r;
              const double kr = K.ksi * r, ar = K.alpha * r;
              const double c1 = (erf(kr) - erf(ar)) / r;
              const double c2 =
                  K.two_ksi_sqrt_pi * exp(-kr * kr) - K.two_alpha_sqrt_pi * exp(-ar * ar);
              const double xf = (x[0] * fj[0] + x[1] * fj[1] + x[2] * fj[2]) / r2;
              const double pp = (c1 + c2) * K.one_eight_pi_mu, mm = (c1 - c2) * xf * K.one_eight_pi_mu;
              acc[0] += pp * fj[0] + mm * x[0];
              acc[1] += pp * fj[1] + mm * x[1];
              acc[2] += pp * fj[2] + mm * x[2];
            }
          } else {
            const double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
            const double a2r2 = K.alpha2 * r2;
            const double gv = K.alpha3_pi_23 * exp(-a2r2) * (2.5 - a2r2);
            acc[0] += gv * fj[0];
            acc[1] += gv * fj[1];
            acc[2] += gv * fj[2];
          }
        }
      }
    }
  } else {
    // cut-off mode: a target beyond a non-periodic face has no complete cell
    // neighbourhood, so it is rejected like a point outside every element
    if (outside) atomicOr(err, kErrOutOfDomain);
    const int rng[3] = {range0, range1, range2};
    SweepAxis ax[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) ax[d] = axis_range(g, d, c[d], rng[d]);
    for (int iz = 0; iz < ax[2].count; ++iz) {
      const int cz = ax[2].wrap ? wrap_i(ax[2].first + iz, g.nc[2]) : ax[2].first + iz;
      for (int iy = 0; iy < ax[1].count; ++iy) {
        const int cy = ax[1].wrap ? wrap_i(ax[1].first + iy, g.nc[1]) : ax[1].first + iy;
        for (int ix = 0; ix < ax[0].count; ++ix) {
          const int cx = ax[0].wrap ? wrap_i(ax[0].first + ix, g.nc[0]) : ax[0].first + ix;
          const int32_t cell = cx + g.nc[0] * (cy + g.nc[1] * cz);
          for (int32_t s = start[cell]; s < start[cell + 1]; ++s) {
            const double4_32a q = pos64[s];
            double x[3] = {q.x - p[0], q.y - p[1], q.z - p[2]};
            min_image(g, x);
            const double r2c = __dadd_rn(__dadd_rn(__dmul_rn(x[0], x[0]), __dmul_rn(x[1], x[1])),
                                         __dmul_rn(x[2], x[2]));
            if (!(r2c < R2)) continue;
            const double *fj = f + 3 * (int64_t)s;
            if (KIND == 0) {
              const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
              if (r < K.r_eps) {
                acc[0] += K.coeff_2 * fj[0];
                acc[1] += K.coeff_2 * fj[1];
                acc[2] += K.coeff_2 * fj[2];
              } else {
                const double r2 = r * r;
                const double kr = K.ksi * r, ar = K.alpha * r;
                const double c1 = (erf(kr) - erf(ar)) / r;
                const double c2 =
                    K.two_ksi_sqrt_pi * exp(-kr * kr) - K.two_alpha_sqrt_pi * exp(-ar * ar);
                const double xf = (x[0] * fj[0] + x[1] * fj[1] + x[2] * fj[2]) / r2;
                const double pp = (c1 + c2) * K.one_eight_pi_mu,
                             mm = (c1 - c2) * xf * K.one_eight_pi_mu;
                acc[0] += pp * fj[0] + mm * x[0];
                acc[1] += pp * fj[1] + mm * x[1];
                acc[2] += pp * fj[2] + mm * x[2];
              }
            } else {
              const double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
              const double a2r2 = K.alpha2 * r2;
              const double gv = K.alpha3_pi_23 * exp(-a2r2) * (2.5 - a2r2);
              acc[0] += gv * fj[0];
              acc[1] += gv * fj[1];
              acc[2] += gv * fj[2];
            }
          }
        }
      }
    }
  }
  out[3 * t] = acc[0];
  out[3 * t + 1] = acc[1];
  out[3 * t + 2] = acc[2];
}

// Fe[e][j*n_u + l] = sum_q int_force[e][l*nq + q] * rho[e*nq + q][j]
__global__ void k_element_rhs(int64_t n_elem, int nq, int n_u, const double *__restrict__ IF,
                              const double *__restrict__ rho, double *__restrict__ Fe) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n_elem * n_u) return;
  const int64_t e = k / n_u;
  const int l = (int)(k - e * n_u);
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  const double *w = IF + e * (int64_t)n_u * nq + (int64_t)l * nq;
  const double *r = rho + e * (int64_t)nq * 3;
  for (int q = 0; q < nq; ++q) {
    const double wq = w[q];
    a0 += wq * r[3 * q];
    a1 += wq * r[3 * q + 1];
    a2 += wq * r[3 * q + 2];
  }
  double *F = Fe + e * 3 * (int64_t)n_u;
  F[l] = a0;
  F[n_u + l] = a1;
  F[2 * n_u + l] = a2;
}

__global__ void k_green_full(int64_t m, DevConsts K, const double *__restrict__ x,
                             double *__restrict__ G) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= m) return;
  const double v[3] = {x[3 * t], x[3 * t + 1], x[3 * t + 2]};
  double *o = G + 9 * t;
  const double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (r < K.r_eps) {
    for (int i = 0; i < 9; ++i) o[i] = (i % 4 == 0) ? K.coeff_2 : 0.0;
    return;
  }
  const double r2 = r * r;
  const double kr = K.ksi * r, kr2 = kr * kr;
  const double ar = K.alpha * r, ar2 = ar * ar;
  const double c1 = (erf(kr) - erf(ar)) / r;
  const double c2 = K.two_ksi_sqrt_pi * exp(-kr2) - K.two_alpha_sqrt_pi * exp(-ar2);
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j) {
      const double d = (i == j) ? 1.0 : 0.0;
      const double xx = v[i] * v[j] / r2;
      const double gij = ((d + xx) * c1 + (d - xx) * c2) * K.one_eight_pi_mu;
      o[3 * i + j] = gij;
      o[3 * j + i] = gij;
    }
}

int field_sums(ggem_ctx *c, int kind, int64_t nt, const double *d_targets, const int32_t *d_elem,
               double radius, const double *d_f_slot, double *d_out) {
  const Grid &g = c->grid;
  const bool ref = c->prm.nb_mode == GGEM_NB_REFERENCE;
  int rng[3] = {0, 0, 0};
  if (!ref) {
    for (int d = 0; d < 3; ++d) rng[d] = (int)std::ceil(radius / g.h[d]);
  }
  cudaError_t e = cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream);
  if (e) return cuda_fail(c, e, "memset");
  const unsigned bn = (unsigned)((nt + 127) / 128);
  if (nt > 0) {
    if (kind == 0)
      k_field<0><<<bn, 128, 0, c->stream>>>(nt, d_targets, d_elem, ref ? 1 : 0, g, c->dc,
                                             c->d_stencil.p, (int)c->stencil.size(), rng[0],
                                             rng[1], rng[2], radius * radius, c->cell_start.p,
                                             c->pos64.p, d_f_slot, d_out, c->err.p);
    else
      k_field<1><<<bn, 128, 0, c->stream>>>(nt, d_targets, d_elem, ref ? 1 : 0, g, c->dc,
                                             c->d_stencil.p, (int)c->stencil.size(), rng[0],
                                             rng[1], rng[2], radius * radius, c->cell_start.p,
                                             c->pos64.p, d_f_slot, d_out, c->err.p);
    if (int rc = check_launch(c, "field sums")) return rc;
  }
  int flags = 0;
  if (int rc = read_error_flags(c, &flags)) return rc;
  if (flags & kErrOutOfDomain)
    return fail(c, GGEM_ERR_OUT_OF_DOMAIN, "a target point lies outside every element");
  if (flags & kErrBadIndex) return fail(c, GGEM_ERR_BAD_ARG, "element index out of range");
  return GGEM_OK;
}

// host arrays -> device, forces permuted to slots
int stage_common(ggem_ctx *c, int64_t nt, const double *targets, const double *f) {
  const size_t n3 = (size_t)c->n * 3;
  cudaError_t e;
  if ((e = c->w_a.ensure(std::max<size_t>(n3, 1))) || (e = c->w_in.ensure(std::max<size_t>(n3, 1))) ||
      (e = c->w_c.ensure(std::max<size_t>(3 * nt, 1))) || (e = c->w_d.ensure(std::max<size_t>(3 * nt, 1))))
    return cuda_fail(c, e, "field buffers");
  if (n3 && (e = cudaMemcpyAsync(c->w_a.p, f, 8 * n3, cudaMemcpyHostToDevice, c->stream)))
    return cuda_fail(c, e, "forces h2d");
  if (nt && (e = cudaMemcpyAsync(c->w_c.p, targets, 8 * 3 * nt, cudaMemcpyHostToDevice, c->stream)))
    return cuda_fail(c, e, "targets h2d");
  return permute_to_slots(c, 1, c->w_a.p, c->w_in.p);
}

}  // namespace
}  // namespace ggem

using namespace ggem;

extern "C" int ggem_green_tensor_local(ggem_ctx *ctx, int64_t m, const double *x, double *G) {
  if (!ctx || m < 0 || (m > 0 && (!x || !G))) return GGEM_ERR_BAD_ARG;
  if (m == 0) return GGEM_OK;
  DeviceGuard dg(ctx->device);
  cudaError_t e;
  if ((e = ctx->w_c.ensure(3 * m)) || (e = ctx->w_d.ensure(9 * m))) return cuda_fail(ctx, e, "green buffers");
  if ((e = cudaMemcpyAsync(ctx->w_c.p, x, 8 * 3 * m, cudaMemcpyHostToDevice, ctx->stream)))
    return cuda_fail(ctx, e, "green h2d");
  k_green_full<<<(unsigned)((m + 127) / 128), 128, 0, ctx->stream>>>(m, ctx->dc, ctx->w_c.p, ctx->w_d.p);
  if (int rc = check_launch(ctx, "green")) return rc;
  if ((e = cudaMemcpyAsync(G, ctx->w_d.p, 8 * 9 * m, cudaMemcpyDeviceToHost, ctx->stream)) ||
      (e = cudaStreamSynchronize(ctx->stream)))
    return cuda_fail(ctx, e, "green d2h");
  return GGEM_OK;
}

extern "C" int ggem_local_field(ggem_ctx *ctx, int64_t nt, const double *targets, const double *f,
                                double *u) {
  if (!ctx || nt < 0 || (nt > 0 && (!targets || !u)) || (ctx->n > 0 && !f)) return GGEM_ERR_BAD_ARG;
  if (int rc = ggem::settle_list(ctx)) return rc;
  if (!ctx->cells_built) return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_build_cells first");
  DeviceGuard dg(ctx->device);
  if (int rc = stage_common(ctx, nt, targets, f)) return rc;
  const double R = ctx->prm.rc;
  if (int rc = field_sums(ctx, 0, nt, ctx->w_c.p, nullptr, R, ctx->w_in.p, ctx->w_d.p)) return rc;
  cudaError_t e;
  if (nt && ((e = cudaMemcpyAsync(u, ctx->w_d.p, 8 * 3 * nt, cudaMemcpyDeviceToHost, ctx->stream)) ||
             (e = cudaStreamSynchronize(ctx->stream))))
    return cuda_fail(ctx, e, "field d2h");
  return GGEM_OK;
}

static double spread_radius(const ggem_ctx *ctx, double spread_rc) {
  // search_radius_p = 4 / alpha (copss.C:1074) unless given
  return spread_rc > 0 ? spread_rc : 4.0 / ctx->prm.alpha;
}

extern "C" int ggem_spread_qp(ggem_ctx *ctx, int64_t nq, const double *qxyz, const int32_t *qp_elem,
                              const double *f, double spread_rc, double *rho) {
  if (!ctx || nq < 0 || (nq > 0 && (!qxyz || !rho)) || (ctx->n > 0 && !f)) return GGEM_ERR_BAD_ARG;
  if (int rc = ggem::settle_list(ctx)) return rc;
  if (!ctx->cells_built) return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_build_cells first");
  const bool ref = ctx->prm.nb_mode == GGEM_NB_REFERENCE;
  if (ref && !qp_elem && nq > 0)
    return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "reference mode needs the element of each point");
  DeviceGuard dg(ctx->device);
  if (int rc = stage_common(ctx, nq, qxyz, f)) return rc;
  ggem::DevBuf<int32_t> elem;
  cudaError_t e;
  if (ref && nq > 0) {
    if ((e = elem.ensure(nq)) ||
        (e = cudaMemcpyAsync(elem.p, qp_elem, 4 * nq, cudaMemcpyHostToDevice, ctx->stream)))
      return cuda_fail(ctx, e, "qp elements");
  }
  if (int rc = field_sums(ctx, 1, nq, ctx->w_c.p, ref ? elem.p : nullptr,
                          spread_radius(ctx, spread_rc), ctx->w_in.p, ctx->w_d.p))
    return rc;
  if (nq && ((e = cudaMemcpyAsync(rho, ctx->w_d.p, 8 * 3 * nq, cudaMemcpyDeviceToHost, ctx->stream)) ||
             (e = cudaStreamSynchronize(ctx->stream))))
    return cuda_fail(ctx, e, "rho d2h");
  return GGEM_OK;
}

extern "C" int ggem_spread_qp_dev(ggem_ctx *ctx, int64_t nq, const double *d_qxyz,
                                  const int32_t *d_qp_elem, const double *d_f, double spread_rc,
                                  double *d_rho) {
  if (!ctx || nq < 0 || (nq > 0 && (!d_qxyz || !d_rho)) || (ctx->n > 0 && !d_f))
    return GGEM_ERR_BAD_ARG;
  if (int rc = ggem::settle_list(ctx)) return rc;
  if (!ctx->cells_built) return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_build_cells first");
  const bool ref = ctx->prm.nb_mode == GGEM_NB_REFERENCE;
  if (ref && !d_qp_elem && nq > 0)
    return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "reference mode needs the element of each point");
  DeviceGuard dg(ctx->device);
  const size_t n3 = (size_t)ctx->n * 3;
  cudaError_t e = ctx->w_in.ensure(std::max<size_t>(n3, 1));
  if (e) return cuda_fail(ctx, e, "spread buffers");
  if (n3) {
    if (int rc = permute_to_slots(ctx, 1, d_f, ctx->w_in.p)) return rc;
  }
  return field_sums(ctx, 1, nq, d_qxyz, ref ? d_qp_elem : nullptr, spread_radius(ctx, spread_rc),
                    ctx->w_in.p, d_rho);
}

extern "C" int ggem_element_rhs(ggem_ctx *ctx, int64_t n_elem, int nq_per_elem, int n_u,
                                const double *qxyz, const double *int_force, const double *f,
                                double spread_rc, double *Fe) {
  if (!ctx || n_elem < 0 || nq_per_elem < 1 || n_u < 1 ||
      (n_elem > 0 && (!qxyz || !int_force || !Fe)) || (ctx->n > 0 && !f))
    return GGEM_ERR_BAD_ARG;
  if (int rc = ggem::settle_list(ctx)) return rc;
  if (!ctx->cells_built) return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_build_cells first");
  const bool ref = ctx->prm.nb_mode == GGEM_NB_REFERENCE;
  if (ref && n_elem != ctx->grid.ncell)
    return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "reference mode: one entry per mesh element");
  DeviceGuard dg(ctx->device);
  const int64_t nq = n_elem * nq_per_elem;
  if (int rc = stage_common(ctx, nq, qxyz, f)) return rc;
  ggem::DevBuf<int32_t> elem;
  ggem::DevBuf<double> IF, FE;
  cudaError_t e;
  if ((e = IF.ensure(std::max<int64_t>(1, n_elem * n_u * nq_per_elem))) ||
      (e = FE.ensure(std::max<int64_t>(1, n_elem * 3 * n_u))))
    return cuda_fail(ctx, e, "element buffers");
  if (n_elem && (e = cudaMemcpyAsync(IF.p, int_force, 8 * n_elem * n_u * nq_per_elem,
                                     cudaMemcpyHostToDevice, ctx->stream)))
    return cuda_fail(ctx, e, "int_force h2d");
  if (ref && nq > 0) {
    std::vector<int32_t> qe(nq);
    for (int64_t q = 0; q < nq; ++q) qe[q] = (int32_t)(q / nq_per_elem);
    if ((e = elem.ensure(nq)) ||
        (e = cudaMemcpyAsync(elem.p, qe.data(), 4 * nq, cudaMemcpyHostToDevice, ctx->stream)) ||
        (e = cudaStreamSynchronize(ctx->stream)))
      return cuda_fail(ctx, e, "qp elements");
  }
  if (int rc = field_sums(ctx, 1, nq, ctx->w_c.p, ref ? elem.p : nullptr,
                          spread_radius(ctx, spread_rc), ctx->w_in.p, ctx->w_d.p))
    return rc;
  if (n_elem > 0) {
    k_element_rhs<<<(unsigned)((n_elem * n_u + 127) / 128), 128, 0, ctx->stream>>>(
        n_elem, nq_per_elem, n_u, IF.p, ctx->w_d.p, FE.p);
    if (int rc = check_launch(ctx, "element rhs")) return rc;
    if ((e = cudaMemcpyAsync(Fe, FE.p, 8 * n_elem * 3 * n_u, cudaMemcpyDeviceToHost, ctx->stream)) ||
        (e = cudaStreamSynchronize(ctx->stream)))
      return cuda_fail(ctx, e, "Fe d2h");
  }
  return GGEM_OK;
}
