// ggem_api.cu -- context management and the particle / mobility entry points
// of the C ABI (include/ggem_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ggem_internal.cuh"

ggem_ctx::~ggem_ctx() {
  for (auto &t : ktimer)
    for (cudaEvent_t e : t.ev) cudaEventDestroy(e);
  for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
  for (auto &t : trace_ev) cudaEventDestroy(t.second);
  if (ev_readback) cudaEventDestroy(ev_readback);
  for (cudaGraphExec_t g : sg_exec)
    if (g) cudaGraphExecDestroy(g);
  if (ev_copy) cudaEventDestroy(ev_copy);
  if (copy_stream) cudaStreamDestroy(copy_stream);
  for (auto *b : scan_scratch) delete b;
  if (h_red) cudaFreeHost(h_red);
  if (h_stage) cudaFreeHost(h_stage);
  if (own_stream) cudaStreamDestroy(own_stream);
}

namespace ggem {

int fail(ggem_ctx *c, int code, const std::string &msg) {
  if (c) c->last_error = msg;
  return code;
}

int cuda_fail(ggem_ctx *c, cudaError_t e, const char *what) {
  std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  cudaGetLastError();  // clear a non-sticky error
  return fail(c, e == cudaErrorMemoryAllocation ? GGEM_ERR_OOM : GGEM_ERR_CUDA, m);
}

int check_launch(ggem_ctx *c, const char *what) {
  ++c->launches;
  if (c->trace) trace_mark(c, what);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(c, e, what);
  return GGEM_OK;
}

int read_error_flags(ggem_ctx *c, int *flags) {
  int v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, c->err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "error flags");
  *flags = v;
  return GGEM_OK;
}

int ensure_host_stage(ggem_ctx *c, size_t bytes) {
  if (bytes <= c->h_stage_bytes && c->h_stage) return GGEM_OK;
  if (c->h_stage) cudaFreeHost(c->h_stage);
  c->h_stage = nullptr;
  c->h_stage_bytes = 0;
  cudaError_t e = cudaMallocHost((void **)&c->h_stage, bytes ? bytes : 8);
  if (e != cudaSuccess) return cuda_fail(c, e, "pinned staging");
  c->h_stage_bytes = bytes ? bytes : 8;
  return GGEM_OK;
}

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


// reference-mode element stencil: every element offset whose centroid lies
// within search_radius_e (minimum image) of the element's own centroid,
// build_elem_elem_neighbor_list (point_mesh.C:293-443); each periodic axis
// uses one representative per residue class so no element appears twice
int build_reference_stencil(ggem_ctx *c) {
  const Grid &g = c->grid;
  const double R = c->search_radius_e;
  int lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    const int r = (int)std::ceil(R / g.h[d]) + 1;
    if (g.periodic[d] && 2 * r + 1 >= g.nc[d]) {
      lo[d] = -((g.nc[d] - 1) / 2);
      hi[d] = g.nc[d] / 2;
    } else {
      lo[d] = -std::min(r, g.nc[d] - 1);
      hi[d] = std::min(r, g.nc[d] - 1);
    }
  }
  c->stencil.clear();
  // centroid arithmetic as the oracle / reference: lo + (k + 0.5) h, the
  // neighbour measured from a reference element near the box centre
  int base[3];
  for (int d = 0; d < 3; ++d) base[d] = g.nc[d] / 2;
  for (int dz = lo[2]; dz <= hi[2]; ++dz)
    for (int dy = lo[1]; dy <= hi[1]; ++dy)
      for (int dx = lo[0]; dx <= hi[0]; ++dx) {
        if (dx == 0 && dy == 0 && dz == 0) continue;
        const int off[3] = {dx, dy, dz};
        double dist2 = 0.0;
        for (int d = 0; d < 3; ++d) {
          const double c0 = g.lo[d] + (base[d] + 0.5) * g.h[d];
          const double c1 = g.lo[d] + (base[d] + off[d] + 0.5) * g.h[d];
          double v = c1 - c0;
          if (g.periodic[d]) {
            if (v <= -g.L[d] / 2.0) v += g.L[d];
            if (v > g.L[d] / 2.0) v -= g.L[d];
          }
          dist2 += v * v;
        }
        const double dist = std::sqrt(dist2);
        if (std::fabs(dist - R) <= 1e-12 * R)
          return fail(c, GGEM_ERR_BAD_ARG,
                      "search_radius_e coincides with an element centroid distance; perturb it");
        if (dist < R) c->stencil.push_back(make_int4(dx, dy, dz, 0));
      }
  return GGEM_OK;
}

int upload_stencil(ggem_ctx *c) {
  cudaError_t e = c->d_stencil.ensure(std::max<size_t>(1, c->stencil.size()));
  if (e) return cuda_fail(c, e, "stencil");
  if (!c->stencil.empty()) {
    e = cudaMemcpy(c->d_stencil.p, c->stencil.data(), sizeof(int4) * c->stencil.size(),
                   cudaMemcpyHostToDevice);
    if (e) return cuda_fail(c, e, "stencil upload");
  }
  // FP32 cell shift per entry code (cut-off mode only: codes < kMaxCode)
  std::vector<float4> sh(kMaxCode, make_float4(0.f, 0.f, 0.f, 0.f));
  if (c->prm.nb_mode == GGEM_NB_CUTOFF) {
    for (size_t k = 0; k < c->stencil.size(); ++k) {
      const int4 o = c->stencil[k];
      sh[o.w] = make_float4((float)(o.x * c->grid.h[0]), (float)(o.y * c->grid.h[1]),
                            (float)(o.z * c->grid.h[2]), 0.f);
    }
  }
  e = c->d_shift.ensure(sh.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(c->d_shift.p, sh.data(), sizeof(float4) * sh.size(), cudaMemcpyHostToDevice);
  if (e) return cuda_fail(c, e, "shift upload");
  return GGEM_OK;
}

int validate_and_setup(ggem_ctx *c) {
  ggem_params &p = c->prm;
  if (!(p.mu > 0) || !(p.alpha > 0) || !(p.br0 > 0) || p.point_type < 0 || p.point_type > 2)
    return fail(c, GGEM_ERR_BAD_ARG, "mu, alpha and br0 must be > 0 and point_type valid");
  if (p.point_type == GGEM_LAGRANGIAN_POINT && !(p.ibm_beta > 0 && p.hmin > 0))
    return fail(c, GGEM_ERR_BAD_ARG, "Lagrangian points need ibm_beta > 0 and hmin > 0");
  compute_constants(p, &c->cst);
  if (!(c->cst.ksi > p.alpha))
    return fail(c, GGEM_ERR_BAD_ARG,
                "ksi must exceed alpha for a positive-definite local mobility");
  const ggem_constants &k = c->cst;
  c->dc = DevConsts{k.one_eight_pi_mu, k.alpha, k.alpha2, k.alpha3_pi_23, k.two_alpha_sqrt_pi,
                    k.coeff_1, k.ksi, k.two_ksi_sqrt_pi, k.coeff_2, k.r_eps};
  Grid &g = c->grid;
  for (int d = 0; d < 3; ++d) {
    if (!std::isfinite(p.box_lo[d]) || !std::isfinite(p.box_hi[d]) || !(p.box_hi[d] > p.box_lo[d]))
      return fail(c, GGEM_ERR_BAD_ARG, "box_hi must exceed box_lo on every axis");
    g.lo[d] = p.box_lo[d];
    g.L[d] = p.box_hi[d] - p.box_lo[d];
    g.periodic[d] = p.periodic[d] ? 1 : 0;
  }
  if (p.precision != GGEM_FP64 && p.precision != GGEM_FP32)
    return fail(c, GGEM_ERR_BAD_ARG, "precision must be GGEM_FP64 or GGEM_FP32");
  if (p.nb_mode == GGEM_NB_REFERENCE) {
    if (p.precision != GGEM_FP64)
      return fail(c, GGEM_ERR_BAD_ARG, "the reference neighbour mode runs in FP64 only");
    double hmax = 0.0;
    for (int d = 0; d < 3; ++d) {
      if (p.n_mesh[d] < 1 || p.n_mesh[d] > 4096)
        return fail(c, GGEM_ERR_BAD_ARG, "n_mesh must be in [1, 4096] per axis");
      g.nc[d] = p.n_mesh[d];
      g.h[d] = g.L[d] / g.nc[d];
      hmax = std::max(hmax, g.h[d]);
    }
    // copss.C:986-992 (hmaxf = largest element size), :1075
    c->search_radius_e = (p.search_radius_e > 0) ? p.search_radius_e : 0.5 * hmax + 4. / p.alpha;
    g.ncell = (int64_t)g.nc[0] * g.nc[1] * g.nc[2];
    if (g.ncell > (int64_t)1 << 30) return fail(c, GGEM_ERR_BAD_ARG, "too many elements");
    if (int rc = build_reference_stencil(c)) return rc;
    c->rc2 = 0.0;
  } else if (p.nb_mode == GGEM_NB_CUTOFF) {
    if (!(p.rc > 0) || !std::isfinite(p.rc)) return fail(c, GGEM_ERR_BAD_ARG, "rc must be > 0");
    int div = p.cell_div;
    if (div <= 0) div = 1;
    if (div > 2) return fail(c, GGEM_ERR_BAD_ARG, "cell_div must be 1 or 2");
    if (p.precision == GGEM_FP64) div = 1;
    p.cell_div = div;
    for (int d = 0; d < 3; ++d) {
      int nc = (int)std::floor(g.L[d] * div / p.rc);
      nc = std::max(1, std::min(nc, 2048));
      if (g.periodic[d] && nc < 2 * div + 1)
        return fail(c, GGEM_ERR_BAD_ARG,
                    "periodic box edge must be at least 3 * rc (each image within rc unique)");
      g.nc[d] = nc;
      g.h[d] = g.L[d] / nc;
    }
    g.ncell = (int64_t)g.nc[0] * g.nc[1] * g.nc[2];
    c->stencil.clear();
    for (int dz = -div; dz <= div; ++dz)
      for (int dy = -div; dy <= div; ++dy)
        for (int dx = -div; dx <= div; ++dx) {
          // drop cells whose nearest point is beyond rc
          const double gx = std::max(0, std::abs(dx) - 1) * g.h[0];
          const double gy = std::max(0, std::abs(dy) - 1) * g.h[1];
          const double gz = std::max(0, std::abs(dz) - 1) * g.h[2];
          if (gx * gx + gy * gy + gz * gz >= p.rc * p.rc) continue;
          // w: the offset's index in the full (2 div + 1)^3 cube, the code a
          // pair entry carries (decoded arithmetically by the pair kernel)
          const int side = 2 * div + 1;
          const int code = ((dz + div) * side + (dy + div)) * side + (dx + div);
          c->stencil.push_back(make_int4(dx, dy, dz, code));
        }
    c->rc2 = p.rc * p.rc;
    c->rc2_lo = (float)(c->rc2 * (1.0 - 1e-4));
    c->rc2_hi = (float)(c->rc2 * (1.0 + 1e-4));
    if (p.precision == GGEM_FP32) {
      std::vector<float4> tab;
      const double s_max = c->rc2 * (1.0 + 2e-4);
      if (fit_tensor_table(c->cst, s_max, kTableN, tab, &c->tab_max_err))
        return fail(c, GGEM_ERR_BAD_ARG, "tensor table fit failed for these constants");
      c->tab_inv_ds = (float)(kTableN / s_max);
      cudaError_t e = c->tab.ensure(tab.size());
      if (e == cudaSuccess)
        e = cudaMemcpy(c->tab.p, tab.data(), sizeof(float4) * tab.size(), cudaMemcpyHostToDevice);
      if (e) return cuda_fail(c, e, "table upload");
      // the analytic exp x polynomial form replaces the table lookup when its
      // FP32 evaluation error stays within 1e-6 of the tensor scale
      c->use_poly = fit_tensor_poly(c->cst, s_max, c->poly_a, c->poly_b, &c->poly_x0,
                                    &c->poly_x1, c->poly_e, &c->poly_max_err) == 0;
      c->use_pretensor = tensor_b_nonnegative(c->cst, s_max);
    }
  } else {
    return fail(c, GGEM_ERR_BAD_ARG, "nb_mode must be GGEM_NB_REFERENCE or GGEM_NB_CUTOFF");
  }
  // the FP32 pair entry carries the stencil index in kCodeBits bits; the
  // (larger) reference-mode element stencil is only swept in FP64
  if (p.precision == GGEM_FP32 && (int)c->stencil.size() > kMaxCode)
    return fail(c, GGEM_ERR_BAD_ARG, "stencil larger than the pair-entry code space");
  for (int d = 0; d < 3; ++d) {
    g.h32[d] = (float)g.h[d];
    g.inv_h[d] = 1.0 / g.h[d];
    // FP32 cell index (k_assign): xf - lo32 is within 2^-24 (|x| + |lo| +
    // |t|) <= 2^-23 (|lo| + |hi|) of x - lo; the margins are four times the
    // worst case, and the cell band adds the rounding of t / h up to nc
    const double eps = std::ldexp(1.0, -24);
    const double mag = std::fabs(g.lo[d]) + std::fabs(g.lo[d] + g.L[d]);
    g.lo32[d] = (float)g.lo[d];
    g.L32[d] = (float)g.L[d];
    g.inv_h32[d] = (float)g.inv_h[d];
    g.margin32[d] = (float)(8.0 * eps * mag + 1e-30);
    g.band32[d] = (float)(8.0 * eps * mag / g.h[d] + 8.0 * eps * (g.nc[d] + 2));
  }
  return upload_stencil(c);
}

}  // namespace
}  // namespace ggem

using namespace ggem;

extern "C" void ggem_default_params(ggem_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->mu = 1.0 / (6.0 * 3.14159265358979323846);  // copss.C:173
  p->alpha = 0.5;
  p->br0 = 1.0;  // copss_point_particle_system.C:208-209
  p->point_type = GGEM_POLYMER_BEAD;
  p->ibm_beta = 0.75;
  p->hmin = 1.0;
  for (int d = 0; d < 3; ++d) {
    p->box_lo[d] = 0.0;
    p->box_hi[d] = 1.0;
    p->periodic[d] = 1;
    p->n_mesh[d] = 1;
  }
  p->nb_mode = GGEM_NB_CUTOFF;
  p->rc = 7.0;
  p->search_radius_e = 0.0;
  p->precision = GGEM_FP32;
  p->cell_div = 0;
  p->device = 0;
}

extern "C" const char *ggem_strerror(int code) {
  switch (code) {
    case GGEM_OK: return "ok";
    case GGEM_ERR_BAD_ARG: return "invalid argument or call order";
    case GGEM_ERR_CUDA: return "CUDA runtime error";
    case GGEM_ERR_CELL_OVERFLOW: return "neighbour list capacity exceeded";
    case GGEM_ERR_TIMEOUT: return "bounded device wait gave up";
    case GGEM_ERR_NOT_SPD: return "eigenvalue <= 0: mobility not positive definite";
    case GGEM_ERR_CHEB_NOT_CONVERGED: return "Chebyshev polynomial failed to converge";
    case GGEM_ERR_SURROGATE_REJECTED: return "surrogate eigen interval rejected";
    case GGEM_ERR_OUT_OF_DOMAIN: return "particle outside the domain";
    case GGEM_ERR_NO_DEVICE: return "no CUDA device";
    case GGEM_ERR_OOM: return "device memory exhausted";
    case GGEM_ERR_INVALID_RANGE: return "invalid eigenvalue range";
    default: return "unknown error";
  }
}

extern "C" const char *ggem_last_error(const ggem_ctx *ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

extern "C" int ggem_create(const ggem_params *p, ggem_ctx **out) {
  if (!p || !out) return GGEM_ERR_BAD_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return GGEM_ERR_NO_DEVICE;
  }
  if (p->device < 0 || p->device >= ndev) return GGEM_ERR_BAD_ARG;
  ggem_ctx *c = new ggem_ctx();
  c->prm = *p;
  c->device = p->device;
  DeviceGuard dg(c->device);
  cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return GGEM_ERR_CUDA;
  }
  c->stream = c->own_stream;
  int rc = validate_and_setup(c);
  if (rc == GGEM_OK) {
    if ((e = c->err.ensure(1)) || (e = cudaMemset(c->err.p, 0, sizeof(int))) ||
        (e = cudaMallocHost((void **)&c->h_red, 4096 * sizeof(double))))
      rc = cuda_fail(c, e, "context buffers");
  }
  if (rc != GGEM_OK) {
    // keep the message on stderr: the context is gone
    std::fprintf(stderr, "ggem_create: %s\n", c->last_error.c_str());
    delete c;
    return rc;
  }
  *out = c;
  return GGEM_OK;
}

extern "C" void ggem_destroy(ggem_ctx *ctx) {
  if (!ctx) return;
  DeviceGuard dg(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  delete ctx;
}

extern "C" int ggem_get_constants(const ggem_ctx *ctx, ggem_constants *out) {
  if (!ctx || !out) return GGEM_ERR_BAD_ARG;
  *out = ctx->cst;
  return GGEM_OK;
}

extern "C" int ggem_set_stream(ggem_ctx *ctx, void *stream) {
  if (!ctx) return GGEM_ERR_BAD_ARG;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return GGEM_OK;
}

extern "C" int ggem_synchronize(ggem_ctx *ctx) {
  if (!ctx) return GGEM_ERR_BAD_ARG;
  DeviceGuard dg(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e) return cuda_fail(ctx, e, "synchronize");
  return GGEM_OK;
}

static int set_particles_common(ggem_ctx *ctx, int64_t n, const double *xyz, bool dev) {
  if (!ctx || n < 0 || (n > 0 && !xyz)) return GGEM_ERR_BAD_ARG;
  if (n >= ((int64_t)1 << (32 - kCodeBits)))
    return fail(ctx, GGEM_ERR_BAD_ARG, "at most 2^25 particles per context");
  DeviceGuard dg(ctx->device);
  // non-finite coordinates are found by the cell build on the device (a host
  // scan of the positions cost more than the copy itself)
  cudaError_t e = ctx->xyz_in.ensure((size_t)std::max<int64_t>(3 * n, 1));
  if (e) return cuda_fail(ctx, e, "positions");
  if (n > 0) {
    e = cudaMemcpyAsync(ctx->xyz_in.p, xyz, sizeof(double) * 3 * n,
                        dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream);
    if (e) return cuda_fail(ctx, e, "positions copy");
  }
  ctx->n = n;
  ctx->cells_built = false;
  ctx->list_built = false;
  ctx->list_unchecked = false;  // the pending statistics describe the old positions
  return GGEM_OK;
}

extern "C" int ggem_set_particles(ggem_ctx *ctx, int64_t n, const double *xyz) {
  return set_particles_common(ctx, n, xyz, false);
}

extern "C" int ggem_set_particles_dev(ggem_ctx *ctx, int64_t n, const double *d_xyz) {
  return set_particles_common(ctx, n, d_xyz, true);
}

extern "C" int ggem_set_deferred_checks(ggem_ctx *ctx, int enable) {
  if (!ctx) return GGEM_ERR_BAD_ARG;
  DeviceGuard dg(ctx->device);
  if (!enable)
    if (int rc = settle_list(ctx)) return rc;
  ctx->defer_checks = enable != 0;
  return GGEM_OK;
}

extern "C" int ggem_build_cells(ggem_ctx *ctx) {
  if (!ctx) return GGEM_ERR_BAD_ARG;
  DeviceGuard dg(ctx->device);
  // statistics of an earlier deferred build that nothing has read yet
  if (int rc = settle_list(ctx)) return rc;
  // the FP32 path builds its pair list right after the cells; both error
  // checks then share the list's single host readback
  const bool cutoff = ctx->prm.nb_mode == GGEM_NB_CUTOFF;
  const bool fp32 = ctx->prm.precision == GGEM_FP32;
  const bool with_list = cutoff && (fp32 || ctx->f64_list);
  if (int rc = build_cells(ctx, with_list)) return rc;
  if (with_list) {
    if (int rc = build_pair_list(ctx)) return rc;
    return fp32 ? build_pair_tensors(ctx) : GGEM_OK;
  }
  return GGEM_OK;
}

static int require_built(ggem_ctx *ctx) {
  if (int rc = settle_list(ctx)) return rc;
  if (!ctx->cells_built)
    return fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_build_cells after setting particles");
  if ((ctx->prm.precision == GGEM_FP32 || ctx->f64_list) && !ctx->list_built)
    return fail(ctx, GGEM_ERR_BAD_ARG, "pair list not built");
  return GGEM_OK;
}

extern "C" int ggem_neighbor_pair_count(ggem_ctx *ctx, int64_t *count) {
  if (!ctx || !count) return GGEM_ERR_BAD_ARG;
  if (int rc = require_built(ctx)) return rc;
  if (ctx->prm.precision == GGEM_FP32) {
    *count = ctx->n_pairs;
    return GGEM_OK;
  }
  int64_t n = 0;
  std::vector<int64_t> off(ctx->n + 1);
  int rc = ggem_get_neighbors(ctx, off.data(), nullptr, 0);
  if (rc < 0 && rc != GGEM_ERR_CELL_OVERFLOW) return rc;
  n = off[ctx->n];
  *count = n;
  return GGEM_OK;
}

extern "C" int ggem_get_cell_of_particles(ggem_ctx *ctx, int32_t *cell) {
  if (!ctx || (!cell && ctx->n)) return GGEM_ERR_BAD_ARG;
  if (int rc = settle_list(ctx)) return rc;
  if (!ctx->cells_built) return fail(ctx, GGEM_ERR_BAD_ARG, "cells not built");
  DeviceGuard dg(ctx->device);
  if (ctx->n == 0) return GGEM_OK;
  cudaError_t e = cudaMemcpyAsync(cell, ctx->cell_of.p, sizeof(int32_t) * ctx->n,
                                  cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e) return cuda_fail(ctx, e, "cell ids");
  return GGEM_OK;
}

// Neighbour sets for parity checks.  FP32: the cached list; FP64: the same
// predicate as the sweep, evaluated on the host from the device's sorted
// cells (this path is for verification, not speed).
extern "C" int ggem_get_neighbors(ggem_ctx *ctx, int64_t *offsets, int32_t *ids, int64_t cap) {
  if (!ctx || !offsets) return GGEM_ERR_BAD_ARG;
  if (int rc = require_built(ctx)) return rc;
  DeviceGuard dg(ctx->device);
  const int64_t n = ctx->n;
  const Grid &g = ctx->grid;
  std::vector<int32_t> order(n), start(g.ncell + 1), cell_of(n);
  std::vector<double4_32a> pos(n);
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaSuccess;
  if (n > 0) {
    if ((e = cudaMemcpyAsync(order.data(), ctx->order.p, 4 * n, cudaMemcpyDeviceToHost, st)) ||
        (e = cudaMemcpyAsync(cell_of.data(), ctx->cell_of.p, 4 * n, cudaMemcpyDeviceToHost, st)) ||
        (e = cudaMemcpyAsync(pos.data(), ctx->pos64.p, sizeof(double4_32a) * n,
                             cudaMemcpyDeviceToHost, st)))
      return cuda_fail(ctx, e, "neighbour readback");
  }
  if ((e = cudaMemcpyAsync(start.data(), ctx->cell_start.p, 4 * (g.ncell + 1),
                           cudaMemcpyDeviceToHost, st)) ||
      (e = cudaStreamSynchronize(st)))
    return cuda_fail(ctx, e, "neighbour readback");
  std::vector<std::vector<int32_t>> lists(n);
  if (ctx->prm.precision == GGEM_FP32) {
    const int64_t W = ctx->nb_w;
    std::vector<int32_t> cnt(std::max<int64_t>(n, 1));
    std::vector<uint32_t> lst(std::max<int64_t>(n * W, 1));
    if (n > 0) {
      if ((e = cudaMemcpyAsync(cnt.data(), ctx->nb_cnt.p, 4 * n, cudaMemcpyDeviceToHost, st)) ||
          (e = cudaMemcpyAsync(lst.data(), ctx->nb_list.p, 4 * n * W, cudaMemcpyDeviceToHost, st)) ||
          (e = cudaStreamSynchronize(st)))
        return cuda_fail(ctx, e, "list readback");
    }
    for (int64_t s = 0; s < n; ++s) {
      auto &L = lists[order[s]];
      for (int64_t m = s * W; m < s * W + cnt[s]; ++m) L.push_back(order[lst[m] >> kCodeBits]);
    }
  } else {
    const bool ref = ctx->prm.nb_mode == GGEM_NB_REFERENCE;
    for (int64_t s = 0; s < n; ++s) {
      const int32_t cid = cell_of[order[s]];
      const int cx = cid % g.nc[0], cy = (cid / g.nc[0]) % g.nc[1], cz = cid / (g.nc[0] * g.nc[1]);
      auto &L = lists[order[s]];
      for (int k = ref ? -1 : 0; k < (int)ctx->stencil.size(); ++k) {
        const int4 o = k < 0 ? make_int4(0, 0, 0, 0) : ctx->stencil[k];
        int cc[3] = {cx + o.x, cy + o.y, cz + o.z};
        bool ok = true;
        for (int d = 0; d < 3; ++d) {
          if (cc[d] < 0 || cc[d] >= g.nc[d]) {
            if (!g.periodic[d]) ok = false;
            else cc[d] = ((cc[d] % g.nc[d]) + g.nc[d]) % g.nc[d];
          }
        }
        if (!ok) continue;
        const int32_t nc = cc[0] + g.nc[0] * (cc[1] + g.nc[1] * cc[2]);
        for (int32_t t = start[nc]; t < start[nc + 1]; ++t) {
          if (t == s) continue;
          if (!ref) {
            double d[3] = {pos[t].x - pos[s].x, pos[t].y - pos[s].y, pos[t].z - pos[s].z};
            for (int q = 0; q < 3; ++q)
              if (g.periodic[q]) {
                if (d[q] <= -g.L[q] / 2.0) d[q] += g.L[q];
                if (d[q] > g.L[q] / 2.0) d[q] -= g.L[q];
              }
            volatile double a = d[0] * d[0];
            volatile double b = d[1] * d[1];
            volatile double cz2 = d[2] * d[2];
            volatile double ab = a + b;
            const double r2 = ab + cz2;
            if (!(r2 < ctx->rc2)) continue;
          }
          L.push_back(order[t]);
        }
      }
    }
  }
  offsets[0] = 0;
  int64_t used = 0;
  bool overflow = false;
  for (int64_t i = 0; i < n; ++i) {
    auto &L = lists[i];
    std::sort(L.begin(), L.end());
    for (int32_t v : L) {
      if (ids && used < cap) ids[used] = v;
      ++used;
    }
    offsets[i + 1] = used;
  }
  if (ids && used > cap) overflow = true;
  if (overflow) return fail(ctx, GGEM_ERR_CELL_OVERFLOW, "ids capacity too small");
  return GGEM_OK;
}

extern "C" int ggem_local_matvec_dev(ggem_ctx *ctx, int nrhs, const double *d_f, double *d_u,
                                     int self_mode) {
  if (!ctx || nrhs < 1 || self_mode < 0 || self_mode > 2) return GGEM_ERR_BAD_ARG;
  if (ctx->n > 0 && (!d_f || !d_u)) return GGEM_ERR_BAD_ARG;
  if (int rc = require_built(ctx)) return rc;
  if (ctx->n == 0) return GGEM_OK;  // no particles: nothing to write
  DeviceGuard dg(ctx->device);
  const size_t len = (size_t)ctx->n * 3 * nrhs;
  cudaError_t e = ctx->w_in.ensure(len);
  if (e == cudaSuccess) e = ctx->w_out.ensure(len);
  if (e) return cuda_fail(ctx, e, "matvec workspace");
  if (nrhs == 1 && ctx->prm.precision == GGEM_FP32 && ctx->prm.nb_mode == GGEM_NB_CUTOFF &&
      !ctx->pretensor_ok && !ctx->sym_pairs && d_f != d_u)
    return matvec_orig_fused(ctx, d_f, d_u, ctx->w_in.p, self_mode);
  if (int rc = permute_to_slots(ctx, nrhs, d_f, ctx->w_in.p)) return rc;
  if (int rc = matvec_slots(ctx, nrhs, ctx->w_in.p, ctx->w_out.p, self_mode)) return rc;
  return permute_from_slots(ctx, nrhs, ctx->w_out.p, d_u);
}

extern "C" int ggem_local_matvec(ggem_ctx *ctx, int nrhs, const double *f, double *u,
                                 int self_mode) {
  if (!ctx || nrhs < 1) return GGEM_ERR_BAD_ARG;
  if (ctx->n > 0 && (!f || !u)) return GGEM_ERR_BAD_ARG;
  if (int rc = require_built(ctx)) return rc;
  DeviceGuard dg(ctx->device);
  const size_t len = (size_t)ctx->n * 3 * nrhs;
  cudaError_t e = ctx->w_a.ensure(len);
  if (e == cudaSuccess) e = ctx->w_b.ensure(len);
  if (e) return cuda_fail(ctx, e, "matvec io");
  if (len) {
    e = cudaMemcpyAsync(ctx->w_a.p, f, sizeof(double) * len, cudaMemcpyHostToDevice, ctx->stream);
    if (e) return cuda_fail(ctx, e, "matvec h2d");
  }
  if (int rc = ggem_local_matvec_dev(ctx, nrhs, ctx->w_a.p, ctx->w_b.p, self_mode)) return rc;
  if (len) {
    e = cudaMemcpyAsync(u, ctx->w_b.p, sizeof(double) * len, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e) return cuda_fail(ctx, e, "matvec d2h");
  }
  return GGEM_OK;
}
