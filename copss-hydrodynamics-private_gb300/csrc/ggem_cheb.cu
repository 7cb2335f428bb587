// ggem_cheb.cu -- Kernel C: the FP64 Chebyshev M^{-1/2} xi recurrence, the
// Lanczos spectral bounds, power iteration and the device noise generator.
//
// Vectors live on the device in slot order ([r][3n] doubles); the pair sums
// come from ggem_pair.cu.  The recurrence is fused into one pass per term
// (x_{k+1}, y += c_k x_{k+1} and both norms), bound by HBM/L2:
// 40 B x 3n per right-hand side per term of algorithmic traffic.
#include <cuda_runtime.h>

#include <cstring>

#include <algorithm>
#include <cmath>
#include <vector>

#include "ggem_ff.cuh"
#include "ggem_internal.cuh"

namespace ggem {
namespace {

constexpr int kMaxRhs = 64;
constexpr int kVecThreads = 256;

struct RhsCoef {
  double c[kMaxRhs];
};

int vec_blocks(int64_t D) {
  int64_t g = (D + 4 * kVecThreads - 1) / (4 * kVecThreads);
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, 592));
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;  // valid in thread 0
}

// partial[r][blockIdx.x] = sum_k a[r][k] * b[r][k]
__global__ void __launch_bounds__(kVecThreads) k_dot_partials(int64_t D, const double *__restrict__ a,
                                                              const double *__restrict__ b,
                                                              double *__restrict__ partial) {
  __shared__ double sh[32];
  const int r = blockIdx.y;
  const double *pa = a + (int64_t)r * D, *pb = b + (int64_t)r * D;
  double acc = 0.0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < D;
       k += (int64_t)gridDim.x * blockDim.x)
    acc += pa[k] * pb[k];
  const double t = block_sum(acc, sh);
  if (threadIdx.x == 0) partial[(int64_t)r * gridDim.x + blockIdx.x] = t;
}

// k_dot_partials with float-float products and sums (no FP64 arithmetic):
// the estimator sums of the FP32 multi-RHS series, whose matvecs carry
// ~1e-7 relative error, so that their ~1e-14 serves as well as FP64
__global__ void __launch_bounds__(kVecThreads) k_dot_ff(int64_t D, const double *__restrict__ a,
                                                        const double *__restrict__ b,
                                                        double *__restrict__ partial) {
  __shared__ float2 sh[32];
  const int r = blockIdx.y;
  const double *pa = a + (int64_t)r * D, *pb = b + (int64_t)r * D;
  float h = 0.f, l = 0.f;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < D;
       k += (int64_t)gridDim.x * blockDim.x) {
    float ph, pl;
    dot_ff(pa[k], pb[k], ph, pl);
    ff_add(h, l, ph, pl);
  }
  const double t = block_ff_sum(h, l, sh);
  if (threadIdx.x == 0) partial[(int64_t)r * gridDim.x + blockIdx.x] = t;
}

// out[q] = sum_b partial[q][b], fixed order (deterministic).  With stat and
// err given, out[nq .. nq+2] also receive the pair-list statistics (total
// and longest row, as bit patterns) and the error word of a deferred build,
// so that one readback carries both.
__global__ void __launch_bounds__(kVecThreads) k_finalize(int G, const double *__restrict__ partial,
                                                          double *__restrict__ out, int nq,
                                                          const unsigned long long *__restrict__ stat,
                                                          const int *__restrict__ err) {
  __shared__ double sh[32];
  const int q = blockIdx.x;
  // four running sums per thread keep four loads in flight (fixed order)
  const double *p = partial + (int64_t)q * G;
  const int T = blockDim.x;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  int b = threadIdx.x;
  for (; b + 3 * T < G; b += 4 * T) {
    a0 += p[b];
    a1 += p[b + T];
    a2 += p[b + 2 * T];
    a3 += p[b + 3 * T];
  }
  for (; b < G; b += T) a0 += p[b];
  const double t = block_sum((a0 + a1) + (a2 + a3), sh);
  if (threadIdx.x == 0) out[q] = t;
  if (stat && q == 0 && threadIdx.x == 0) {
    out[nq] = __longlong_as_double((long long)stat[0]);
    out[nq + 1] = __longlong_as_double((long long)stat[1]);
    out[nq + 2] = (double)*err;
  }
}

// the series' first step in one pass (brownian_system.C:1041, 1050-1056):
// x1 = db x0 + da x1 (VecAXPBY; x1 holds M x0), dw = c0 x0 + c1 x1, with
// the norms |c0 x0| -> q0 and |x1| -> q1 only where a check precedes the
// first term (the reference-faithful mode)
template <bool NORMS>
__global__ void __launch_bounds__(kVecThreads) k_cheb_start(int64_t D, double da, double db,
                                                            double c0, double c1,
                                                            const double *__restrict__ x0,
                                                            double *__restrict__ x1,
                                                            double *__restrict__ dw,
                                                            double *__restrict__ partial) {
  __shared__ double sh[32];
  const int r = blockIdx.y, nrhs = gridDim.y;
  const int64_t off = (int64_t)r * D;
  double a4 = 0.0, a3 = 0.0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < D;
       k += (int64_t)gridDim.x * blockDim.x) {
    const double x = x0[off + k];
    const double v = db * x + da * x1[off + k];
    x1[off + k] = v;
    const double t = c0 * x;
    dw[off + k] = t + c1 * v;
    if (NORMS) {
      a4 += t * t;
      a3 += v * v;
    }
  }
  if (NORMS) {
    const double s4 = block_sum(a4, sh);
    const double s3 = block_sum(a3, sh);
    if (threadIdx.x == 0) {
      partial[(int64_t)(0 * nrhs + r) * gridDim.x + blockIdx.x] = s4;
      partial[(int64_t)(1 * nrhs + r) * gridDim.x + blockIdx.x] = s3;
    }
  }
}

// one term (brownian_system.C:1091-1108):
//   ||dw|| -> q0 ; xm = (2db x1 + 2da xm) - x0 ; dw += c[r] xm ; ||xm|| -> q1
// The norms feed only the error estimators: a term that no check follows
// skips them (NORMS = false), a third of the term's FP64 work.
// With FF the norms are float-float sums (no FP64 arithmetic; the FP32
// series) instead of FP64 ones.  With REC (one right-hand side) the term
// also writes the 32-byte pair-kernel records of the new x and of the new
// dw (cell-relative position from pos32, then the FP32 values, rounded as
// the records the pair kernels stage themselves), so that the next matvec
// and the check's matvec need no staging pass.
template <bool NORMS, bool FF = false, bool REC = false>
__global__ void __launch_bounds__(kVecThreads) k_cheb_term(int64_t D, double two_da,
                                                           double two_db, RhsCoef cf,
                                                           const double *__restrict__ x0,
                                                           const double *__restrict__ x1,
                                                           double *__restrict__ xm,
                                                           double *__restrict__ dw,
                                                           double *__restrict__ partial,
                                                           const float4 *__restrict__ pos32 = nullptr,
                                                           float4 *__restrict__ rec_x = nullptr,
                                                           float4 *__restrict__ rec_dw = nullptr) {
  __shared__ double sh[32];
  __shared__ float2 shf[32];
  const int r = blockIdx.y, nrhs = gridDim.y;
  const int64_t off = (int64_t)r * D;
  const double c = cf.c[r];
  double a4 = 0.0, a3 = 0.0;
  float h4 = 0.f, l4 = 0.f, h3 = 0.f, l3 = 0.f;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < D;
       k += (int64_t)gridDim.x * blockDim.x) {
    const double y = dw[off + k];
    double v = two_db * x1[off + k] + two_da * xm[off + k];
    v -= x0[off + k];
    xm[off + k] = v;
    const double yn = y + c * v;
    dw[off + k] = yn;
    if (REC) {
      const int64_t s = k / 3;
      const int comp = (int)(k - 3 * s);
      float *rx = reinterpret_cast<float *>(rec_x + 2 * s);
      float *rd = reinterpret_cast<float *>(rec_dw + 2 * s);
      rx[4 + comp] = d2f_bits(v);
      rd[4 + comp] = d2f_bits(yn);
      if (comp == 0) {
        const float4 p = pos32[s];
        rec_x[2 * s] = p;
        rec_dw[2 * s] = p;
        rx[7] = 0.f;
        rd[7] = 0.f;
      }
    }
    if (NORMS && FF) {
      float ph, pl;
      sq_ff(y, ph, pl);
      ff_add(h4, l4, ph, pl);
      sq_ff(v, ph, pl);
      ff_add(h3, l3, ph, pl);
    } else if (NORMS) {
      a4 += y * y;
      a3 += v * v;
    }
  }
  if (NORMS) {
    const double s4 = FF ? block_ff_sum(h4, l4, shf) : block_sum(a4, sh);
    const double s3 = FF ? block_ff_sum(h3, l3, shf) : block_sum(a3, sh);
    if (threadIdx.x == 0) {
      partial[(int64_t)(0 * nrhs + r) * gridDim.x + blockIdx.x] = s4;
      partial[(int64_t)(1 * nrhs + r) * gridDim.x + blockIdx.x] = s3;
    }
  }
}

__global__ void k_copy(int64_t tot, const double *__restrict__ a, double *__restrict__ b) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < tot;
       k += (int64_t)gridDim.x * blockDim.x)
    b[k] = a[k];
}

__global__ void k_scale(int64_t tot, double s, const double *__restrict__ a, double *__restrict__ b) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < tot;
       k += (int64_t)gridDim.x * blockDim.x)
    b[k] = a[k] * s;
}

__global__ void k_fill(int64_t tot, double v, double *__restrict__ b) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < tot;
       k += (int64_t)gridDim.x * blockDim.x)
    b[k] = v;
}

// b = a + s * b
__global__ void k_axpy_into(int64_t tot, double s, const double *__restrict__ a,
                            double *__restrict__ b) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < tot;
       k += (int64_t)gridDim.x * blockDim.x)
    b[k] = b[k] + s * a[k];
}

// Lanczos: partial[i][b] = Q_i . w for i < m
__global__ void __launch_bounds__(kVecThreads) k_multi_dot(int64_t D, const double *__restrict__ Q,
                                                           const double *__restrict__ w,
                                                           double *__restrict__ partial) {
  __shared__ double sh[32];
  const int i = blockIdx.y;
  const double *q = Q + (int64_t)i * D;
  double acc = 0.0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < D;
       k += (int64_t)gridDim.x * blockDim.x)
    acc += q[k] * w[k];
  const double t = block_sum(acc, sh);
  if (threadIdx.x == 0) partial[(int64_t)i * gridDim.x + blockIdx.x] = t;
}

// w -= sum_i h_i Q_i
__global__ void k_sub_proj(int64_t D, int m, const double *__restrict__ Q,
                           const double *__restrict__ h, double *__restrict__ w) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < D;
       k += (int64_t)gridDim.x * blockDim.x) {
    double v = w[k];
    for (int i = 0; i < m; ++i) v -= h[i] * Q[(int64_t)i * D + k];
    w[k] = v;
  }
}

// Philox4x32-10 (Salmon et al., SC'11) + Box-Muller
__device__ __forceinline__ void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
    const uint32_t n0 = hi1 ^ c[1] ^ k0;
    const uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// Counter (p, stream) gives elements 4p .. 4p+3: words (c0, c1) and (c2, c3)
// each make one Box-Muller pair from u1 = (c0 + 1/2) 2^-32 (rounded to
// FP32) and u2 = (floor(c1 / 2^9) + 1/2) 2^-23 (exact), transformed in FP32
// (the FP64 transcendentals would run at 1/64 of the FP32 rate); the tail
// reaches 6.8 sigma.
__global__ void k_philox_normals(int64_t n, uint64_t seed, uint64_t stream,
                                 double *__restrict__ out) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (4 * p >= n) return;
  uint32_t c[4] = {(uint32_t)p, (uint32_t)((uint64_t)p >> 32), (uint32_t)stream,
                   (uint32_t)(stream >> 32)};
  philox10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const float u1 = fmaf(__uint2float_rn(c[2 * h]), 0x1p-32f, 0x1p-33f);
    const float u2 = fmaf((float)(c[2 * h + 1] >> 9), 0x1p-23f, 0x1p-24f);
    const float r = sqrtf(-2.f * logf(u1));
    float sn, cs;
    sincospif(2.f * u2, &sn, &cs);
    const int64_t k = 4 * p + 2 * h;
    if (k < n) out[k] = (double)(r * cs);
    if (k + 1 < n) out[k + 1] = (double)(r * sn);
  }
}

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

int grid1(int64_t tot) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((tot + 255) / 256, 4096));
}

// results[q] of the partial arrays, copied to the pinned host mirror; with
// list_stats, host[nq .. nq+2] receive a deferred build's statistics too.
// before_wait (optional) queues more work behind the readback before the
// host waits for it.
// the finalized sums copied to the pinned host mirror (no wait)
int finalize_issue(ggem_ctx *c, int nq, int G, double *host, bool list_stats) {
  double *out = c->w_red.p + (size_t)nq * G;
  k_finalize<<<nq, kVecThreads, 0, c->stream>>>(G, c->w_red.p, out, nq,
                                                list_stats ? c->nb_stat.p : nullptr,
                                                list_stats ? c->err.p : nullptr);
  if (int rc = check_launch(c, "finalize")) return rc;
  const int nv = nq + (list_stats ? 3 : 0);
  cudaError_t e = cudaMemcpyAsync(host, out, sizeof(double) * nv, cudaMemcpyDeviceToHost, c->stream);
  if (e) return cuda_fail(c, e, "reduction readback");
  return GGEM_OK;
}

// the event the host waits on for a readback, recorded after the work so far
int record_readback(ggem_ctx *c) {
  cudaError_t e;
  if (!c->ev_readback &&
      (e = cudaEventCreateWithFlags(&c->ev_readback, cudaEventDisableTiming)))
    return cuda_fail(c, e, "readback event");
  if ((e = cudaEventRecord(c->ev_readback, c->stream))) return cuda_fail(c, e, "readback event");
  return GGEM_OK;
}

int wait_readback(ggem_ctx *c) {
  cudaError_t e = cudaEventSynchronize(c->ev_readback);
  if (e) return cuda_fail(c, e, "reduction readback");
  return GGEM_OK;
}

template <typename F>
int finalize_to_host_then(ggem_ctx *c, int nq, int G, double *host, bool list_stats,
                          F &&before_wait) {
  if (int rc = finalize_issue(c, nq, G, host, list_stats)) return rc;
  // the host waits for the readback only: work queued by before_wait runs on
  if (int rc = record_readback(c)) return rc;
  if (int rc = before_wait()) return rc;
  return wait_readback(c);
}

// ---- the series prefix as CUDA graphs ---------------------------------
// 0: run live (a new key; it is kept), 1: capture now (the key came back),
// 2: replay the graphs of this key
int series_graph_state(ggem_ctx *c, const std::vector<uint64_t> &key) {
  if (key == c->sg_key) return c->sg_exec[0] ? 2 : 1;
  for (cudaGraphExec_t &g : c->sg_exec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  c->sg_key = key;
  return 0;
}

// capture issue(seg) for seg = 0, 1, 2 into the prefix's three graphs and
// instantiate them.  The kernel timer records no events inside a capture.
// On a failed capture the graphs stay off for this context and *fallback
// is set, with the host state the capture touched put back, so that the
// caller runs the prefix live.
template <typename F>
int series_graph_capture(ggem_ctx *c, F &&issue, bool *fallback) {
  *fallback = false;
  const int64_t l0 = c->launches;
  const int rec0 = c->rec_cur;
  const bool timing = c->timing;
  cudaGraphExec_t exec[3] = {nullptr, nullptr, nullptr};
  bool ok = true;
  c->timing = false;
  for (int seg = 0; seg < 3 && ok; ++seg) {
    if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal)) {
      ok = false;
      break;
    }
    const int rc = issue(seg);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (!rc && !e) e = cudaGraphInstantiate(&exec[seg], g, 0);
    if (g) cudaGraphDestroy(g);
    ok = !rc && !e && exec[seg];
  }
  c->timing = timing;
  if (!ok) {
    cudaGetLastError();
    for (cudaGraphExec_t g : exec)
      if (g) cudaGraphExecDestroy(g);
    c->launches = l0;
    c->rec_cur = rec0;
    c->series_graphs = false;
    c->sg_key.clear();
    *fallback = true;
    return GGEM_OK;
  }
  for (int seg = 0; seg < 3; ++seg) c->sg_exec[seg] = exec[seg];
  c->sg_launches = c->launches - l0;
  ++c->sg_captures;
  return GGEM_OK;
}

// one replay: the first step, the fused terms inside the kernel timer's
// span (i_terms launches), the check
int series_graph_launch(ggem_ctx *c, int i_terms) {
  cudaError_t e;
  if ((e = cudaGraphLaunch(c->sg_exec[0], c->stream))) return cuda_fail(c, e, "series graph");
  kt_span_begin(c, kKPairCheb);
  if ((e = cudaGraphLaunch(c->sg_exec[1], c->stream))) return cuda_fail(c, e, "series graph");
  if (c->span_kind == kKPairCheb) c->span_n = i_terms;
  kt_span_end(c);
  if ((e = cudaGraphLaunch(c->sg_exec[2], c->stream))) return cuda_fail(c, e, "series graph");
  ++c->sg_replays;
  return GGEM_OK;
}

int finalize_to_host(ggem_ctx *c, int nq, int G, double *host, bool list_stats = false) {
  return finalize_to_host_then(c, nq, G, host, list_stats, [] { return GGEM_OK; });
}

int sumsq_to_host(ggem_ctx *c, int nrhs, int64_t D, const double *v, double *host) {
  const int G = vec_blocks(D);
  k_dot_partials<<<dim3(G, nrhs), kVecThreads, 0, c->stream>>>(D, v, v, c->w_red.p);
  if (int rc = check_launch(c, "sumsq")) return rc;
  return finalize_to_host(c, nrhs, G, host);
}

int dot_to_host(ggem_ctx *c, int nrhs, int64_t D, const double *a, const double *b, double *host) {
  const int G = vec_blocks(D);
  k_dot_partials<<<dim3(G, nrhs), kVecThreads, 0, c->stream>>>(D, a, b, c->w_red.p);
  if (int rc = check_launch(c, "dot")) return rc;
  return finalize_to_host(c, nrhs, G, host);
}

int brownian_self_mode(const ggem_ctx *c) {
  // the mobility of _MatMult_Stokes: compute_point_velocity adds -coeff_1 f + f
  // for beads (pm_system_stokes.C:450-453); Lagrangian points carry G(0) f in
  // local_solution_bead (ggem_stokes.C:485-499)
  return c->prm.point_type == GGEM_LAGRANGIAN_POINT ? GGEM_SELF_LAGRANGIAN : GGEM_SELF_BEAD;
}

int ensure_cheb_buffers(ggem_ctx *c, size_t len) {
  cudaError_t e;
  if ((e = c->w_in.ensure(len)) || (e = c->w_out.ensure(len)) || (e = c->w_c.ensure(len)) ||
      (e = c->w_d.ensure(len)) || (e = c->w_e.ensure(len)) || (e = c->w_y.ensure(len)) ||
      (e = c->w_red.ensure(4 * kMaxRhs * 600)))
    return cuda_fail(c, e, "chebyshev workspace");
  return GGEM_OK;
}

// cheb_slots' answer when a deferred list build turned out to have
// overflowing rows: the list has been rebuilt and the series must restart
constexpr int kRestartCheb = 1;

// Chebyshev on xi (caller order, device; left unchanged); leaves y in c->w_y
// (slot order).
//
// check_every = 1: the reference's loop (brownian_system.C:1089-1155): the
//   error-check matvec dw_mid = M dw and both estimators every term.
// check_every = k > 1: err1/err2 are evaluated at every k-th term (and the
//   last); the norms of a term come from the fused term kernel.
// check_every = 0: the first check is at the degree the previous call
//   converged at (8 on the first call), then every term; the prediction is
//   lowered by one when the first check passed with room for one degree
//   less (see the end of cheb_slots).
// Only check points synchronise with the host.  On return *dm_is_my tells
// whether c->w_out holds M y for every right-hand side (the last check ran
// on the final y), which the Brownian displacement reuses.
// spec_dw (optional, caller order): every error check also queues M dw into
// it before the host waits for the check's readback; when the series ends at
// a check, *spec_done says that spec_dw already holds M y.
int cheb_slots_impl(ggem_ctx *c, int nrhs, int N, double eig_min, double eig_max, double tol,
                    int check_every, const double *xi, ggem_cheb_report *rep, bool *dm_is_my,
                    double *spec_dw, bool *spec_done) {
  if (spec_done) *spec_done = false;
  const int64_t D = 3 * c->n;
  const int sm = brownian_self_mode(c);
  const bool faithful = check_every == 1;
  // the FP32 series' estimator sums run as float-float sums (the FP64
  // precision and the reference-faithful mode keep FP64 dots)
  const bool ff_sums = c->prm.precision == GGEM_FP32 && !faithful;
  // Terms that no error check follows need neither norm: on the FP32
  // single-RHS path they run as one fused pair-sum + recurrence kernel that
  // also writes the FP32 records of the next x1 (records_fresh).  With
  // per-matvec pair tensors outside the reference-faithful mode the whole
  // series is fused: the first step is one pair kernel (m = M x0, x1, dw)
  // and a checked term is a fused term followed by its two norms.
  const bool can_fuse = nrhs == 1 && c->prm.precision == GGEM_FP32 &&
                        c->prm.nb_mode == GGEM_NB_CUTOFF;
  const bool fused = can_fuse && !faithful && !c->pretensor_ok && c->n > 0;
  // 16 .. 64 right-hand sides: an unchecked term is one batched kernel
  const bool batch_fused = !faithful && c->n > 0 && batch_term_fusable(c, nrhs);
  // one right-hand side on the unfused path with per-pair tensors (the
  // reference-faithful checks): each term also writes the pair records of
  // its new x (w_rec[0]) and dw (w_src), so the next matvec and the check's
  // matvec skip their staging passes
  const bool rec_terms = can_fuse && !fused && !c->pretensor_ok && c->n > 0;
  bool xrec_fresh = false, dwrec_fresh = false;
  if (rec_terms) {
    cudaError_t e;
    if ((e = c->w_rec[0].ensure(2 * (size_t)c->n)) || (e = c->w_src.ensure(2 * (size_t)c->n)))
      return cuda_fail(c, e, "chebyshev records");
  }
  bool staged_fresh = false;
  // partial sums per reduction: vector-kernel blocks, or in a fused series
  // the pair kernels' blocks (the first step, the checked terms and the
  // check matvec leave their estimator sums themselves)
  const int G = fused ? (int)pair_partials(c) : vec_blocks(D);
  cudaStream_t st = c->stream;
  if (fused) {
    cudaError_t e = c->w_red.ensure((size_t)4 * G + 64);
    if (e) return cuda_fail(c, e, "reduction partials");
  }
  double *x0 = c->w_c.p, *x1 = c->w_d.p, *xm = c->w_e.p, *dw = c->w_y.p, *dm = c->w_out.p;
  // reduction regions: term norms [2 nrhs][G], |dm|^2 [nrhs][G], xi.M.xi
  // [nrhs][G], then the 4 nrhs finalized values
  double *p_term = c->w_red.p;
  double *p_dm = p_term + (size_t)2 * nrhs * G;
  double *p_aux2 = p_dm + (size_t)nrhs * G;
  // brownian_system.C:1001-1003 and the coefficients of :1021-1024
  const double d_eig = eig_max - eig_min;
  const double da = 2.0 / d_eig;
  const double db = -(eig_max + eig_min) / d_eig;
  std::vector<double> X(N + 1);
  cheb_coeffs_host(N, da, db, GGEM_CHEB_GAUSS, X.data());
  std::vector<int> active(nrhs, 1);
  for (int r = 0; r < nrhs; ++r) rep[r] = ggem_cheb_report{0, 1, 0, 0.0, 0.0};
  double *h = c->h_red;
  const int k_first = (check_every == 0) ? std::max(2, c->cheb_pred_terms > 0 ? c->cheb_pred_terms : 8)
                                         : 0;
  *dm_is_my = false;
  // x0 = xi; x1 = M x0; aux2 = x1.x0; x1 = db x0 + da x1   (:1036-1041)
  // dw = c0 x0, dw += c1 x1 (with both norms unless fused)  (:1050-1056)
  bool records_fresh = false;
  const double two_da = 2. * da, two_db = 2. * db;
  int first_check = -1;
  // The fused adaptive series' prefix: the first step, the unchecked terms,
  // the first checked term (i_chk) and the device half of its check.  It is
  // issued by issue_prefix, live or as one CUDA graph (series_graph).
  const int i_chk = std::min(k_first - 1, N - 1);
  const bool prefix = fused && check_every == 0 && N >= 2;
  if (!prefix) {
    if (fused) {
      // dm holds m = M x0 until the first check
      if (int rc = cheb_start_fused(c, xi, x0, dm, x1, dw, da, db, X[0], X[1], sm, p_aux2))
        return rc;
      records_fresh = true;
    } else {
      int prc = GGEM_OK;
      if (batch_fused && to_slots_staged(c, nrhs, xi, x0, &prc)) {
        if (prc) return prc;
        if (int rc = matvec_slots_prestaged(c, nrhs, x0, x1, sm)) return rc;
      } else {
        if (int rc = permute_to_slots(c, nrhs, xi, x0)) return rc;
        if (int rc = matvec_slots(c, nrhs, x0, x1, sm)) return rc;
      }
      if (ff_sums) k_dot_ff<<<dim3(G, nrhs), kVecThreads, 0, st>>>(D, x1, x0, p_aux2);
      else k_dot_partials<<<dim3(G, nrhs), kVecThreads, 0, st>>>(D, x1, x0, p_aux2);
      if (int rc = check_launch(c, "aux2")) return rc;
      // the start's norms feed only a check before the first term
      if (batch_fused) {  // (not faithful) x1's staging for the first fused term
        if (int rc = cheb_start_staged(c, nrhs, da, db, X[0], X[1], x0, x1, dw)) return rc;
        staged_fresh = true;
      } else if (faithful)
        k_cheb_start<true><<<dim3(G, nrhs), kVecThreads, 0, st>>>(D, da, db, X[0], X[1], x0, x1,
                                                                  dw, p_term);
      else
        k_cheb_start<false><<<dim3(G, nrhs), kVecThreads, 0, st>>>(D, da, db, X[0], X[1], x0,
                                                                   x1, dw, p_term);
      if (!batch_fused)
        if (int rc = check_launch(c, "cheb start")) return rc;
    }
  }
  for (int r = 0; r < nrhs; ++r) rep[r].n_matvecs = 1;

  // the device half of an error check: M dw with |M dw|^2, the finalized
  // estimator sums (and a deferred list build's statistics) copied to the
  // host mirror, then the caller's speculative M y.  The host half
  // (check_eval) waits for the copy; with event_first the wait does not
  // cover the speculative permute.
  bool pending = false;
  auto check_issue = [&](bool event_first) -> int {
    if (fused) {  // dw's records come from the checked term
      if (int rc = matvec_dw_records(c, dw, dm, sm, p_dm)) return rc;
    } else {
      if (int rc = rec_terms && dwrec_fresh ? matvec_dw_records(c, dw, dm, sm, nullptr)
                                            : matvec_slots(c, nrhs, dw, dm, sm))
        return rc;
      if (ff_sums) k_dot_ff<<<dim3(G, nrhs), kVecThreads, 0, st>>>(D, dm, dm, p_dm);
      else k_dot_partials<<<dim3(G, nrhs), kVecThreads, 0, st>>>(D, dm, dm, p_dm);
      if (int rc = check_launch(c, "dm norm")) return rc;
    }
    // a deferred list build is checked in the same readback; the caller's
    // M y is queued behind it in case this check ends the series
    pending = c->list_unchecked;
    if (int rc = finalize_issue(c, 4 * nrhs, G, h, pending)) return rc;
    if (event_first)
      if (int rc = record_readback(c)) return rc;
    // (with a check after every term the caller permutes the last check's
    // M y once, after the series, instead of every check speculatively)
    return spec_dw && !faithful ? permute_from_slots(c, nrhs, dm, spec_dw) : GGEM_OK;
  };
  // evaluate err1 / err2 of the current dw for the active right-hand sides
  auto check_eval = [&](double coef_abs, bool apply_rules) -> int {
    if (int rc = wait_readback(c)) return rc;
    if (pending) {
      const double *v = h + 4 * nrhs;
      bool rebuilt = false;
      unsigned long long total = 0, longest = 0;
      std::memcpy(&total, &v[0], sizeof total);
      std::memcpy(&longest, &v[1], sizeof longest);
      if (int rc = finish_list_check(c, total, longest, (int)v[2], &rebuilt))
        return rc;
      if (rebuilt) return kRestartCheb;
    }
    for (int r = 0; r < nrhs; ++r) {
      if (!active[r]) continue;
      const double aux4 = std::sqrt(h[r]);
      const double aux3 = std::sqrt(h[nrhs + r]) * coef_abs;
      const double aux1 = h[2 * nrhs + r], aux2 = h[3 * nrhs + r];
      rep[r].n_matvecs += 1;
      if (aux2 != 0.0) rep[r].err1 = std::sqrt(std::fabs(aux1 - aux2) / aux2);
      if (aux4 != 0.0) rep[r].err2 = aux3 / aux4;
      if (!apply_rules) continue;
      if (rep[r].err1 <= tol) {  // :1138-1147
        rep[r].converged = 1;
        active[r] = 0;
        continue;
      }
      if (rep[r].err2 <= 1E-9) active[r] = 0;  // :1150
    }
    return GGEM_OK;
  };
  auto check_now = [&](double coef_abs, bool apply_rules) -> int {
    if (int rc = check_issue(true)) return rc;
    return check_eval(coef_abs, apply_rules);
  };

  int i_begin = 1;
  if (prefix) {
    // the prefix's kernels, in the order of the loop below; span_begin /
    // span_end bracket the fused terms for the kernel timer
    auto issue_prefix = [&](int seg) -> int {  // seg -1: all of it, live
      if (seg <= 0)
        if (int rc = cheb_start_fused(c, xi, x0, dm, x1, dw, da, db, X[0], X[1], sm, p_aux2))
          return rc;
      if (seg == -1 || seg == 1) {
        double *a = x0, *b = x1, *m = xm;
        if (seg == -1) kt_span_begin(c, kKPairCheb);
        for (int i = 1; i <= i_chk; ++i) {
          const bool chk = i == i_chk;
          if (int rc = pair_cheb_term(c, true, a, b, m, dw, two_da, two_db, X[i + 1], sm,
                                      chk ? p_term : nullptr))
            return rc;
          double *t = a;
          a = b;
          b = m;
          m = t;
        }
        if (seg == -1) kt_span_end(c);
      }
      if (seg == -1 || seg == 2) return check_issue(seg == -1);
      return GGEM_OK;
    };
    // the records' ping-pong starts from buffer 0 (both are scratch here),
    // so that the graph's baked pointers hold from one call to the next
    c->rec_cur = 0;
    const int rc_cur0 = 0;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(c->stream, &cap) != cudaSuccess) {
      cudaGetLastError();
      cap = cudaStreamCaptureStatusActive;
    }
    // the kernel timer can bracket the graphs' fused terms only: timing of
    // any other kind runs the prefix live
    const bool timed_other = c->timing && (c->timing_mask & ~(1u << kKPairCheb));
    std::vector<uint64_t> key;
    if (c->series_graphs && !c->trace && !timed_other && cap == cudaStreamCaptureStatusNone) {
      auto u = [&](uint64_t v) { key.push_back(v); };
      auto pbits = [&](const void *q) { u((uint64_t)(uintptr_t)q); };
      auto dbits = [&](double v) {
        uint64_t b;
        std::memcpy(&b, &v, 8);
        u(b);
      };
      u((uint64_t)c->n);
      u((uint64_t)c->nb_w);
      u((uint64_t)G);
      u((uint64_t)i_chk);
      u((uint64_t)sm);
      u((uint64_t)c->use_poly);
      u((uint64_t)c->computed_variant);
      u((uint64_t)c->list_unchecked);
      u((uint64_t)rc_cur0);
      dbits(eig_min);
      dbits(eig_max);
      for (const void *q : {(const void *)xi, (const void *)spec_dw, (const void *)c->stream,
                            (const void *)x0, (const void *)x1, (const void *)xm,
                            (const void *)dw, (const void *)dm, (const void *)c->w_red.p,
                            (const void *)c->w_rec[0].p, (const void *)c->w_rec[1].p,
                            (const void *)c->w_src.p, (const void *)h, (const void *)c->order.p,
                            (const void *)c->rank.p, (const void *)c->pos32.p,
                            (const void *)c->nb_cnt.p, (const void *)c->nb_list.p,
                            (const void *)c->d_shift.p, (const void *)c->tab.p,
                            (const void *)c->nb_stat.p, (const void *)c->err.p})
        pbits(q);
    }
    pending = c->list_unchecked;
    int gs = key.empty() ? 0 : series_graph_state(c, key);
    if (gs == 1) {  // the key came back: capture the prefix once
      bool fallback = false;
      if (int rc = series_graph_capture(c, [&](int seg) { return issue_prefix(seg); },
                                        &fallback))
        return rc;
      if (fallback) gs = 0;
    } else if (gs == 2) {
      c->launches += c->sg_launches;
      c->rec_cur = rc_cur0 ^ ((1 + i_chk) & 1);
    }
    if (gs == 0) {  // live (a new key, graphs off, or a failed capture)
      if (int rc = issue_prefix(-1)) return rc;
    } else {
      if (int rc = series_graph_launch(c, i_chk)) return rc;
      if (int rc = record_readback(c)) return rc;
    }
    records_fresh = true;
    for (int i = 1; i <= i_chk; ++i) {  // the loop's bookkeeping for the prefix's terms
      for (int r = 0; r < nrhs; ++r) {
        rep[r].n_matvecs += 1;
        rep[r].n_terms = i + 1;
      }
      double *t = x0;
      x0 = x1;
      x1 = xm;
      xm = t;
    }
    if (int rc = check_eval(std::fabs(X[i_chk + 1]), true)) return rc;  // incl. kRestartCheb
    *dm_is_my = true;
    if (spec_done) *spec_done = spec_dw != nullptr && !faithful;
    first_check = i_chk + 1;
    i_begin = i_chk + 1;
  }

  if (faithful) {  // the estimators before the loop (:1064-1072)
    if (int rc = check_now(std::fabs(X[1]), false)) return rc;
    *dm_is_my = true;
    if (spec_done) *spec_done = spec_dw != nullptr && !faithful;
  }
  for (int i = i_begin; i < N; ++i) {
    int n_active = 0;
    for (int r = 0; r < nrhs; ++r) n_active += active[r];
    if (n_active == 0) break;
    bool check;
    if (faithful) check = true;
    else if (check_every > 1) check = (i % check_every == 0) || (i == N - 1);
    else check = (i + 1 >= k_first) || (i == N - 1);
    if (can_fuse && (!check || fused)) {
      // consecutive fused terms share one timing span (closed before the
      // check's matvec, the next launch of another kernel)
      if (fused && c->span_kind < 0) kt_span_begin(c, kKPairCheb);
      // a checked fused term leaves its two norms and the records of dw
      if (int rc = pair_cheb_term(c, records_fresh, x0, x1, xm, dw, two_da, two_db, X[i + 1], sm,
                                  check ? p_term : nullptr))
        return rc;
      records_fresh = true;
    } else if (batch_fused && !check) {
      double cf[kMaxRhs];
      for (int r = 0; r < nrhs; ++r) cf[r] = active[r] ? X[i + 1] : 0.0;
      if (int rc = batch_cheb_term(c, nrhs, staged_fresh, x0, x1, xm, dw, two_da, two_db, cf, sm))
        return rc;
      staged_fresh = true;
    } else {
      // (a fused batched term before this one left x1's staging; a recorded
      // term before this one left x1's pair records)
      int mrc;
      if (batch_fused && staged_fresh) mrc = matvec_slots_prestaged(c, nrhs, x1, xm, sm);
      else if (rec_terms && xrec_fresh) mrc = matvec_records(c, c->w_rec[0].p, x1, xm, sm, nullptr);
      else mrc = matvec_slots(c, nrhs, x1, xm, sm);
      if (mrc) return mrc;
      RhsCoef cf;
      for (int r = 0; r < nrhs; ++r) cf.c[r] = active[r] ? X[i + 1] : 0.0;
      kt_start(c, kKChebTerm);
      if (check && ff_sums)
        k_cheb_term<true, true><<<dim3(G, nrhs), kVecThreads, 0, st>>>(D, two_da, two_db, cf,
                                                                        x0, x1, xm, dw, p_term);
      else if (check && rec_terms)
        k_cheb_term<true, false, true><<<dim3(G, nrhs), kVecThreads, 0, st>>>(
            D, two_da, two_db, cf, x0, x1, xm, dw, p_term, c->pos32.p, c->w_rec[0].p,
            c->w_src.p);
      else if (check)
        k_cheb_term<true><<<dim3(G, nrhs), kVecThreads, 0, st>>>(D, two_da, two_db, cf, x0, x1,
                                                                  xm, dw, p_term);
      else
        k_cheb_term<false><<<dim3(G, nrhs), kVecThreads, 0, st>>>(D, two_da, two_db, cf, x0, x1,
                                                                   xm, dw, p_term);
      kt_stop(c, kKChebTerm);
      if (int rc = check_launch(c, "cheb term")) return rc;
      records_fresh = false;
      staged_fresh = false;
      xrec_fresh = dwrec_fresh = check && rec_terms;
    }
    for (int r = 0; r < nrhs; ++r)
      if (active[r]) {
        rep[r].n_matvecs += 1;
        rep[r].n_terms = i + 1;
      }
    *dm_is_my = false;
    if (spec_done) *spec_done = false;
    if (check) {
      kt_span_end(c);
      if (int rc = check_now(std::fabs(X[i + 1]), true)) return rc;  // incl. kRestartCheb
      *dm_is_my = true;
      if (spec_done) *spec_done = spec_dw != nullptr && !faithful;
      if (first_check < 0) first_check = i + 1;
    }
    // x0 <- x1, x1 <- xm (:1152-1153) by rotating the buffers
    double *t = x0;
    x0 = x1;
    x1 = xm;
    xm = t;
  }
  if (check_every == 0) {
    int worst = 0;
    bool all = true;
    for (int r = 0; r < nrhs; ++r) {
      all = all && rep[r].converged;
      worst = std::max(worst, rep[r].n_terms);
    }
    // The series error shrinks by about rho = (sqrt(k) - 1) / (sqrt(k) + 1)
    // per degree (k = eig_max / eig_min, the Chebyshev rate for x^(-1/2));
    // the next call tries one degree less only when the first check passed
    // with that much room, so a workload converging at a steady degree does
    // not pay a failing check (an extra matvec and host round trip) every
    // other call.
    double e1 = 0.0;
    for (int r = 0; r < nrhs; ++r) e1 = std::max(e1, rep[r].err1);
    const double kap = eig_min > 0 ? eig_max / eig_min : 1e30;
    const double rho = (std::sqrt(kap) - 1.0) / (std::sqrt(kap) + 1.0);
    const bool lower = worst == first_check && e1 <= 0.8 * rho * tol;
    if (all) c->cheb_pred_terms = lower ? std::max(2, worst - 1) : worst;
  }
  return GGEM_OK;
}

int cheb_slots(ggem_ctx *c, int nrhs, int N, double eig_min, double eig_max, double tol,
               int check_every, const double *xi, ggem_cheb_report *rep, bool *dm_is_my,
               double *spec_dw = nullptr, bool *spec_done = nullptr) {
  const int rc = cheb_slots_impl(c, nrhs, N, eig_min, eig_max, tol, check_every, xi, rep,
                                 dm_is_my, spec_dw, spec_done);
  kt_span_end(c);  // a span left open by an early return or a series ending unchecked
  return rc;
}

}  // namespace
}  // namespace ggem

using namespace ggem;

static int cheb_common(ggem_ctx *ctx, int nrhs, int N, double eig_min, double eig_max,
                       double tol, int check_every, ggem_cheb_report *rep) {
  if (!ctx || nrhs < 1 || nrhs > kMaxRhs || N < 1 || !rep || !(tol >= 0))
    return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "chebyshev: bad arguments (nrhs in [1, 64], N >= 1)");
  if (!(eig_min >= 0) || !(eig_max >= 0) || !(eig_min < eig_max))
    return ggem::fail(ctx, GGEM_ERR_INVALID_RANGE, "invalid eigenvalue range (copss.C:1609-1615)");
  if (!ctx->cells_built || (ctx->prm.precision == GGEM_FP32 && !ctx->list_built))
    return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_build_cells first");
  return GGEM_OK;
}

// a context without particles: the series of an empty vector is exact at
// degree 0 (no operator application), reported converged
static bool empty_series(const ggem_ctx *ctx, int nrhs, ggem_cheb_report *rep) {
  if (ctx->n != 0) return false;
  for (int r = 0; r < nrhs; ++r) rep[r] = ggem_cheb_report{1, 0, 0, 0.0, 0.0};
  return true;
}

extern "C" int ggem_cheb_inv_sqrt_dev(ggem_ctx *ctx, int nrhs, int N, double eig_min,
                                      double eig_max, double tol_cheb, int check_every,
                                      double *d_xi, ggem_cheb_report *rep) {
  if (int rc = cheb_common(ctx, nrhs, N, eig_min, eig_max, tol_cheb, check_every, rep)) return rc;
  if (empty_series(ctx, nrhs, rep)) return GGEM_OK;
  DeviceGuard dg(ctx->device);
  const size_t len = (size_t)ctx->n * 3 * nrhs;
  if (int rc = ensure_cheb_buffers(ctx, len)) return rc;
  bool dm_is_my = false;
  int rc = cheb_slots(ctx, nrhs, N, eig_min, eig_max, tol_cheb, check_every, d_xi, rep, &dm_is_my);
  if (rc == kRestartCheb)  // the deferred list was rebuilt wider: run the series again
    rc = cheb_slots(ctx, nrhs, N, eig_min, eig_max, tol_cheb, check_every, d_xi, rep, &dm_is_my);
  if (rc) return rc;
  return permute_from_slots(ctx, nrhs, ctx->w_y.p, d_xi);
}

extern "C" int ggem_cheb_inv_sqrt(ggem_ctx *ctx, int nrhs, int N, double eig_min, double eig_max,
                                  double tol_cheb, int check_every, double *xi,
                                  ggem_cheb_report *rep) {
  if (int rc = cheb_common(ctx, nrhs, N, eig_min, eig_max, tol_cheb, check_every, rep)) return rc;
  if (!xi && ctx->n) return GGEM_ERR_BAD_ARG;
  DeviceGuard dg(ctx->device);
  const size_t len = (size_t)ctx->n * 3 * nrhs;
  cudaError_t e = ctx->w_a.ensure(len);
  if (e) return cuda_fail(ctx, e, "cheb io");
  if (len && (e = cudaMemcpyAsync(ctx->w_a.p, xi, 8 * len, cudaMemcpyHostToDevice, ctx->stream)))
    return cuda_fail(ctx, e, "cheb h2d");
  if (int rc = ggem_cheb_inv_sqrt_dev(ctx, nrhs, N, eig_min, eig_max, tol_cheb, check_every,
                                      ctx->w_a.p, rep))
    return rc;
  if (len && (e = cudaMemcpyAsync(xi, ctx->w_a.p, 8 * len, cudaMemcpyDeviceToHost, ctx->stream)))
    return cuda_fail(ctx, e, "cheb d2h");
  if ((e = cudaStreamSynchronize(ctx->stream))) return cuda_fail(ctx, e, "cheb sync");
  return GGEM_OK;
}

extern "C" int ggem_brownian_displacement(ggem_ctx *ctx, int nrhs, int N, double eig_min,
                                          double eig_max, double tol_cheb, int check_every,
                                          const double *xi, double *dw, ggem_cheb_report *rep) {
  if (int rc = cheb_common(ctx, nrhs, N, eig_min, eig_max, tol_cheb, check_every, rep)) return rc;
  if (ctx->n && (!xi || !dw)) return GGEM_ERR_BAD_ARG;
  DeviceGuard dg(ctx->device);
  const size_t len = (size_t)ctx->n * 3 * nrhs;
  cudaError_t e;
  if ((e = ctx->w_hin.ensure(len)) || (e = ctx->w_b.ensure(len)))
    return cuda_fail(ctx, e, "bd io");
  if (len) {
    // xi travels on a copy stream into a buffer only this call uses, so the
    // copy overlaps the work already queued (a deferred cell and list
    // build); the series waits for it
    if (!ctx->copy_stream &&
        (e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking)))
      return cuda_fail(ctx, e, "copy stream");
    if (!ctx->ev_copy && (e = cudaEventCreateWithFlags(&ctx->ev_copy, cudaEventDisableTiming)))
      return cuda_fail(ctx, e, "copy event");
    if ((e = cudaMemcpyAsync(ctx->w_hin.p, xi, 8 * len, cudaMemcpyHostToDevice,
                             ctx->copy_stream)) ||
        (e = cudaEventRecord(ctx->ev_copy, ctx->copy_stream)) ||
        (e = cudaStreamWaitEvent(ctx->stream, ctx->ev_copy, 0)))
      return cuda_fail(ctx, e, "bd h2d");
  }
  int rc = ggem_brownian_displacement_dev(ctx, nrhs, N, eig_min, eig_max, tol_cheb, check_every,
                                          ctx->w_hin.p, ctx->w_b.p, rep);
  if (rc) {
    // the next call's copy stream is ordered only before its own series:
    // let the kernels this call queued before failing finish reading w_hin
    // (a successful call synchronises below)
    cudaStreamSynchronize(ctx->stream);
    cudaGetLastError();
    return rc;
  }
  if (len && (e = cudaMemcpyAsync(dw, ctx->w_b.p, 8 * len, cudaMemcpyDeviceToHost, ctx->stream)))
    return cuda_fail(ctx, e, "bd d2h");
  if ((e = cudaStreamSynchronize(ctx->stream))) return cuda_fail(ctx, e, "bd sync");
  return GGEM_OK;
}

extern "C" int ggem_brownian_displacement_dev(ggem_ctx *ctx, int nrhs, int N, double eig_min,
                                              double eig_max, double tol_cheb, int check_every,
                                              const double *d_xi, double *d_dw,
                                              ggem_cheb_report *rep) {
  if (int rc = cheb_common(ctx, nrhs, N, eig_min, eig_max, tol_cheb, check_every, rep)) return rc;
  if (ctx->n && (!d_xi || !d_dw)) return GGEM_ERR_BAD_ARG;
  if (empty_series(ctx, nrhs, rep)) return GGEM_OK;
  DeviceGuard dg(ctx->device);
  const size_t len = (size_t)ctx->n * 3 * nrhs;
  if (int rc = ensure_cheb_buffers(ctx, len)) return rc;
  bool dm_is_my = false, spec_done = false;
  // d_dw is the caller's output alone (unless it is xi itself), so every
  // check may already queue M dw into it (overwritten if the series goes on)
  double *spec = d_dw != d_xi ? d_dw : nullptr;
  int rc = cheb_slots(ctx, nrhs, N, eig_min, eig_max, tol_cheb, check_every, d_xi, rep, &dm_is_my,
                      spec, &spec_done);
  if (rc == kRestartCheb)  // the deferred list was rebuilt wider: run the series again
    rc = cheb_slots(ctx, nrhs, N, eig_min, eig_max, tol_cheb, check_every, d_xi, rep, &dm_is_my,
                    spec, &spec_done);
  if (rc) return rc;
  bool all = true;
  for (int r = 0; r < nrhs; ++r) all = all && rep[r].converged;
  if (!all)
    return ggem::fail(ctx, GGEM_ERR_CHEB_NOT_CONVERGED,
                      "Chebyshev polynomial fails to converge (brownian_system.C:1162-1163)");
  // hi_ewald: dw = M y (copss.C:1686); the last error check already
  // computed M y when it ran on the final y (and queued it into d_dw)
  if (spec_done) return GGEM_OK;
  if (!dm_is_my) {
    if (int rc = matvec_slots(ctx, nrhs, ctx->w_y.p, ctx->w_out.p, brownian_self_mode(ctx)))
      return rc;
  }
  return permute_from_slots(ctx, nrhs, ctx->w_out.p, d_dw);
}

extern "C" int ggem_lanczos_bounds(ggem_ctx *ctx, int k, uint64_t seed, double *eig_min,
                                   double *eig_max) {
  if (!ctx || !eig_min || !eig_max) return GGEM_ERR_BAD_ARG;
  if (k < 2 || k > 512) return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "Lanczos steps must be in [2, 512]");
  if (int rc = settle_list(ctx)) return rc;
  if (!ctx->cells_built || (ctx->prm.precision == GGEM_FP32 && !ctx->list_built))
    return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_build_cells first");
  DeviceGuard dg(ctx->device);
  const int64_t D = 3 * ctx->n;
  if (D == 0) return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "no particles");
  k = (int)std::min<int64_t>(k, D);
  cudaError_t e;
  if ((e = ctx->lz_Q.ensure((size_t)D * (k + 1))) || (e = ctx->w_out.ensure(D)) ||
      (e = ctx->w_red.ensure(std::max(4 * kMaxRhs * 600, (k + 2) * 600 + 1024))))
    return cuda_fail(ctx, e, "lanczos workspace");
  cudaStream_t st = ctx->stream;
  const int sm = brownian_self_mode(ctx);
  const int G = vec_blocks(D);
  double *Q = ctx->lz_Q.p, *w = ctx->w_out.p, *h = ctx->h_red;
  // start vector: N(0,1) from the counter-based generator
  k_philox_normals<<<(unsigned)(((D + 3) / 4 + 255) / 256), 256, 0, st>>>(D, seed, 0x4C414E43ull, Q);
  if (int rc = check_launch(ctx, "lanczos start")) return rc;
  if (int rc = sumsq_to_host(ctx, 1, D, Q, h)) return rc;
  k_scale<<<grid1(D), 256, 0, st>>>(D, 1.0 / std::sqrt(h[0]), Q, Q);
  std::vector<double> a(k), b(k);
  int m = k;
  double *hdev = ctx->w_red.p + (size_t)(k + 2) * 600;
  for (int j = 0; j < k; ++j) {
    double *q = Q + (size_t)j * D;
    if (int rc = matvec_slots(ctx, 1, q, w, sm)) return rc;
    if (int rc = dot_to_host(ctx, 1, D, q, w, h)) return rc;
    a[j] = h[0];
    for (int pass = 0; pass < 2; ++pass) {
      k_multi_dot<<<dim3(G, j + 1), kVecThreads, 0, st>>>(D, Q, w, ctx->w_red.p);
      if (int rc = check_launch(ctx, "lanczos dots")) return rc;
      k_finalize<<<j + 1, kVecThreads, 0, st>>>(G, ctx->w_red.p, hdev, j + 1, nullptr, nullptr);
      if (int rc = check_launch(ctx, "lanczos finalize")) return rc;
      k_sub_proj<<<grid1(D), 256, 0, st>>>(D, j + 1, Q, hdev, w);
      if (int rc = check_launch(ctx, "lanczos project")) return rc;
    }
    if (int rc = sumsq_to_host(ctx, 1, D, w, h)) return rc;
    const double beta = std::sqrt(h[0]);
    b[j] = beta;
    if (j == k - 1) break;
    if (beta < 1e-14 * std::fabs(a[j]) + 1e-300) {
      m = j + 1;
      break;
    }
    k_scale<<<grid1(D), 256, 0, st>>>(D, 1.0 / beta, w, Q + (size_t)(j + 1) * D);
    if (int rc = check_launch(ctx, "lanczos next")) return rc;
  }
  tridiag_extremes(m, a.data(), b.data(), eig_min, eig_max);
  if (!(*eig_min > 0.0) || !(*eig_max > 0.0))
    return ggem::fail(ctx, GGEM_ERR_NOT_SPD,
                      "eigenvalue <= 0 (brownian_system.C:835-840): mobility not positive definite");
  return GGEM_OK;
}

extern "C" int ggem_power_iteration(ggem_ctx *ctx, double tol, int maxits, double *eig) {
  if (!ctx || !(tol > 0) || maxits < 1 || !eig) return GGEM_ERR_BAD_ARG;
  if (int rc = settle_list(ctx)) return rc;
  if (!ctx->cells_built || (ctx->prm.precision == GGEM_FP32 && !ctx->list_built))
    return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_build_cells first");
  DeviceGuard dg(ctx->device);
  const int64_t D = 3 * ctx->n;
  if (D == 0) return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "no particles");
  if (int rc = ensure_cheb_buffers(ctx, D)) return rc;
  cudaStream_t st = ctx->stream;
  const int sm = brownian_self_mode(ctx);
  double *v0 = ctx->w_c.p, *v1 = ctx->w_d.p, *w0 = ctx->w_e.p, *h = ctx->h_red;
  *eig = NAN;
  // brownian_system.C:868-871
  k_fill<<<grid1(D), 256, 0, st>>>(D, 1.0, v0);
  if (int rc = sumsq_to_host(ctx, 1, D, v0, h)) return rc;
  k_scale<<<grid1(D), 256, 0, st>>>(D, 1.0 / std::sqrt(h[0]), v0, v0);
  for (int it = 0; it < maxits; ++it) {
    if (int rc = matvec_slots(ctx, 1, v0, w0, sm)) return rc;
    if (int rc = sumsq_to_host(ctx, 1, D, w0, h)) return rc;
    k_scale<<<grid1(D), 256, 0, st>>>(D, 1.0 / std::sqrt(h[0]), w0, w0);
    k_copy<<<grid1(D), 256, 0, st>>>(D, w0, v1);
    k_axpy_into<<<grid1(D), 256, 0, st>>>(D, -1.0, v0, w0);
    if (int rc = check_launch(ctx, "power step")) return rc;
    if (int rc = sumsq_to_host(ctx, 1, D, w0, h)) return rc;
    const double norm = std::sqrt(h[0]);
    k_copy<<<grid1(D), 256, 0, st>>>(D, v1, v0);
    if (norm < tol) {
      if (int rc = matvec_slots(ctx, 1, v0, w0, sm)) return rc;
      if (int rc = dot_to_host(ctx, 1, D, v0, w0, h)) return rc;
      *eig = h[0];
      return it;
    }
  }
  return ggem::fail(ctx, GGEM_ERR_CHEB_NOT_CONVERGED, "power iteration did not reach tol");
}

extern "C" int ggem_philox_normals_dev(ggem_ctx *ctx, uint64_t seed, uint64_t stream, int64_t n,
                                       double *d_out) {
  if (!ctx || n < 0 || (n > 0 && !d_out)) return GGEM_ERR_BAD_ARG;
  if (n == 0) return GGEM_OK;
  DeviceGuard dg(ctx->device);
  const int64_t quads = (n + 3) / 4;
  k_philox_normals<<<(unsigned)((quads + 255) / 256), 256, 0, ctx->stream>>>(n, seed, stream, d_out);
  return check_launch(ctx, "philox");
}
