// ggem_ensemble.cu -- K independent suspensions as one block-diagonal
// operator (include/ggem_ensemble.h).
//
// Each suspension is an ordinary FP32 context (its own box, cell list, pair
// list and stored pair tensors t = (A, sqrt(B) x)).  The ensemble
// concatenates the rows of all K lists into one fixed-width list over a
// global slot space (source slots offset by the suspension's first slot),
// so that the pair kernel needs neither positions nor a cell grid: one launch
// applies M to every suspension.  Vectors inside the ensemble are
// [slot][8][3] float64 (right-hand sides padded to 8); the pair kernel maps
// 8 lanes to one target slot, one lane per right-hand side, so that the
// 8 forces of a source (FP32, [slot][8] float4) are one 128-byte load.
//
// The Chebyshev series of every (suspension, right-hand side) keeps its own
// interval, coefficients (chebyshev.C:44-151), estimators and stopping
// decision (brownian_system.C:967-1178); a term of all series is one fused
// launch, the norms of the estimators are segmented reductions (one block
// per suspension), and the stretch of terms before the first error check is
// captured once as a CUDA graph and replayed on later calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cmath>
#include <map>
#include <string>
#include <vector>

#include "ggem_ensemble.h"
#include "ggem_internal.cuh"

namespace ggem {
namespace ens {

constexpr int kR = GGEM_ENSEMBLE_MAX_RHS;  // right-hand-side lanes per slot
constexpr int kE = 3 * kR;                 // doubles per slot in a vector

struct SubView {
  const int32_t *cnt;
  const uint32_t *list;
  const float4 *ten;
  const int32_t *order;
  const int32_t *rank;
  int64_t n, off;
  int W;
};

// the K lists into the global list: rows re-strided to Wg, source slots
// offset, suspension id, slot <-> ensemble-index maps
__global__ void k_ens_gather(const SubView *__restrict__ views, int Wg,
                             int32_t *__restrict__ cnt_g, uint32_t *__restrict__ list_g,
                             float4 *__restrict__ ten_g, int32_t *__restrict__ susp,
                             int32_t *__restrict__ order_g, int32_t *__restrict__ rank_g) {
  const SubView v = views[blockIdx.y];
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < v.n;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t gs = v.off + s;
    const int c = v.cnt[s];
    cnt_g[gs] = c;
    susp[gs] = (int32_t)blockIdx.y;
    order_g[gs] = (int32_t)(v.off + v.order[s]);
    rank_g[v.off + s] = (int32_t)(v.off + v.rank[s]);  // s as the caller index here
    for (int m = 0; m < c; ++m) {
      const uint32_t en = v.list[s * v.W + m];
      list_g[gs * Wg + m] = (uint32_t)(((int64_t)(en >> kCodeBits) + v.off) << kCodeBits);
      ten_g[gs * Wg + m] = v.ten[s * v.W + m];
    }
  }
}

// [bead][nrhs][3] (ensemble order) <-> [slot][8][3] (zero padded)
__global__ void k_ens_to_slots(int64_t ntot, int nrhs, const int32_t *__restrict__ order_g,
                               const double *__restrict__ src, double *__restrict__ dst) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= ntot * kE) return;
  const int64_t s = k / kE;
  const int q = (int)(k - s * kE), r = q / 3, c = q - 3 * r;
  dst[k] = r < nrhs ? src[((int64_t)order_g[s] * nrhs + r) * 3 + c] : 0.0;
}

__global__ void k_ens_from_slots(int64_t ntot, int nrhs, const int32_t *__restrict__ order_g,
                                 const double *__restrict__ src, double *__restrict__ dst) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= ntot * kE) return;
  const int64_t s = k / kE;
  const int q = (int)(k - s * kE), r = q / 3, c = q - 3 * r;
  if (r < nrhs) dst[((int64_t)order_g[s] * nrhs + r) * 3 + c] = src[k];
}

// FP32 forces [slot][8] float4 of an FP64 vector [slot][8][3]
__global__ void k_ens_stage(int64_t ntot, const double *__restrict__ v, float4 *__restrict__ f4) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= ntot * kR) return;
  const double *p = v + 3 * k;
  f4[k] = make_float4((float)p[0], (float)p[1], (float)p[2], 0.f);
}

__device__ __forceinline__ void kahan(float &sum, float &comp, float v) {
  const float y = v - comp;
  const float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

__device__ __forceinline__ double f2d(float x) {
  const uint32_t b = __float_as_uint(x);
  const uint32_t sign = b & 0x80000000u, ex = (b >> 23) & 0xffu, m = b & 0x7fffffu;
  if (ex == 0u) return __hiloint2double((int)sign, 0);
  const uint32_t e64 = ex == 0xffu ? 0x7ffu : ex + (1023u - 127u);
  return __hiloint2double((int)(sign | (e64 << 20) | (m >> 3)), (int)(m << 29));
}

// Pair sums of all suspensions over the stored tensors: 8 lanes per target
// slot, lane r its r-th right-hand side.  TERM = false: u = M f (+ self term
// from the FP64 f).  TERM = true: one Chebyshev term of every series,
// xm = (2db x1 + 2da M x1) - x0, dw += c xm (c of the series' suspension,
// zero once the series has stopped), and the FP32 forces of xm.  With
// c1 = 2db + 2da self_c (per suspension) the term is
// xm = 2da (pair sum) + (c1 x1 - x0): four FP64 operations per element
// (GB300 runs FP64 at 1/64 of the FP32 rate).
template <bool TERM>
__global__ void k_ens_pair(int64_t ntot, const int32_t *__restrict__ cnt, int W,
                           const uint32_t *__restrict__ list, const float4 *__restrict__ ten,
                           const float4 *__restrict__ f4, double self_c,
                           const double *__restrict__ f, double *__restrict__ u,
                           const int32_t *__restrict__ susp, const double *__restrict__ two_da,
                           const double *__restrict__ c1x, const double *__restrict__ coef,
                           int ldc, int term, const uint8_t *__restrict__ active,
                           const double *__restrict__ x0, double *__restrict__ dw,
                           float4 *__restrict__ next) {
  const int64_t gid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t s = gid / kR;
  const int r = (int)(gid % kR);
  if (s >= ntot) return;  // 8 consecutive lanes share s: whole groups leave
  const int64_t b0 = s * (int64_t)W, e = b0 + cnt[s];
  float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  float bx = 0.f, by = 0.f, bz = 0.f;
  int blk = 0;
  for (int64_t m = b0; m < e; ++m) {
    const uint32_t en = __ldg(list + m);
    const float4 t = __ldg(ten + m);
    const float4 fj = __ldg(f4 + (int64_t)(en >> kCodeBits) * kR + r);
    const float d = fmaf(t.w, fj.z, fmaf(t.z, fj.y, t.y * fj.x));
    bx += fmaf(t.x, fj.x, d * t.y);
    by += fmaf(t.x, fj.y, d * t.z);
    bz += fmaf(t.x, fj.z, d * t.w);
    if (++blk == 8) {
      kahan(sx, cx, bx);
      kahan(sy, cy, by);
      kahan(sz, cz, bz);
      bx = by = bz = 0.f;
      blk = 0;
    }
  }
  kahan(sx, cx, bx);
  kahan(sy, cy, by);
  kahan(sz, cz, bz);
  const float hs[3] = {sx, sy, sz}, ls[3] = {-cx, -cy, -cz};
  const int64_t k0 = (s * kR + r) * 3;
  if (!TERM) {
#pragma unroll
    for (int c = 0; c < 3; ++c) u[k0 + c] = fma(self_c, f[k0 + c], f2d(hs[c]) + f2d(ls[c]));
  } else {
    const int b = susp[s];
    const double cf = active[b * kR + r] ? coef[(int64_t)b * ldc + term] : 0.0;
    const double tda = two_da[b], c1 = c1x[b];
    float out[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double xk = f[k0 + c];  // f is x1 here
      const double v = fma(tda, f2d(hs[c]) + f2d(ls[c]), fma(c1, xk, -x0[k0 + c]));
      u[k0 + c] = v;  // u is xm here
      dw[k0 + c] = fma(cf, v, dw[k0 + c]);
      out[c] = d2f_bits(v);
    }
    next[s * kR + r] = make_float4(out[0], out[1], out[2], 0.f);
  }
}

// x1 = db x0 + da x1 and dw = c0 x0 + c1 x1 of every series
__global__ void k_ens_start(int64_t ntot, const int32_t *__restrict__ susp,
                            const double *__restrict__ da, const double *__restrict__ db,
                            const double *__restrict__ coef, int ldc,
                            const double *__restrict__ x0, double *__restrict__ x1,
                            double *__restrict__ dw) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= ntot * kE) return;
  const int b = susp[k / kE];
  const double v = db[b] * x0[k] + da[b] * x1[k];
  x1[k] = v;
  dw[k] = coef[(int64_t)b * ldc] * x0[k] + coef[(int64_t)b * ldc + 1] * v;
}

// out[b][r] = sum over the slots of suspension b of a . b (per right-hand
// side), fixed order.  Element k of a vector belongs to right-hand side
// (k % 24) / 3; a block's stride (a multiple of 24) keeps every thread on one
// right-hand side.
constexpr int kDotThreads = 192;

// The sums are split into chunks of at most kDotSlots slots (one block per
// whole suspension made the largest suspension's block the critical path):
// one block per chunk, four running sums per thread, then the chunks of each
// suspension added in order (k_ens_dot_fin).  part[c][r] per chunk c and
// right-hand side r.
constexpr int kDotSlots = 256;

__global__ void __launch_bounds__(kDotThreads) k_ens_dot_part(const int64_t *__restrict__ cs,
                                                              const double *__restrict__ a,
                                                              const double *__restrict__ bv,
                                                              double *__restrict__ part) {
  __shared__ double sh[kDotThreads];
  const int64_t c = blockIdx.x;
  const int64_t k0 = cs[c] * kE, k1 = cs[c + 1] * kE;
  double v0 = 0.0, v1 = 0.0, v2 = 0.0, v3 = 0.0;
  int64_t k = k0 + threadIdx.x;
  for (; k + 3 * kDotThreads < k1; k += 4 * kDotThreads) {
    v0 = fma(a[k], bv[k], v0);
    v1 = fma(a[k + kDotThreads], bv[k + kDotThreads], v1);
    v2 = fma(a[k + 2 * kDotThreads], bv[k + 2 * kDotThreads], v2);
    v3 = fma(a[k + 3 * kDotThreads], bv[k + 3 * kDotThreads], v3);
  }
  for (; k < k1; k += kDotThreads) v0 = fma(a[k], bv[k], v0);
  sh[threadIdx.x] = (v0 + v1) + (v2 + v3);
  __syncthreads();
  if (threadIdx.x < kR) {
    double t = 0.0;
    for (int i = 0; i < kDotThreads; ++i)
      if ((i % kE) / 3 == (int)threadIdx.x) t += sh[i];
    part[c * kR + threadIdx.x] = t;
  }
}

__global__ void k_ens_dot_fin(const int32_t *__restrict__ coff, const double *__restrict__ part,
                              double *__restrict__ out) {
  const int b = blockIdx.x, r = threadIdx.x;
  if (r >= kR) return;
  double t = 0.0;
  for (int c = coff[b]; c < coff[b + 1]; ++c) t += part[(int64_t)c * kR + r];
  out[b * kR + r] = t;
}

// ---- the whole Brownian series of every suspension in one launch ----------
// A persistent cooperative kernel walks a fixed list of passes:
//   START       m = M x0, x0 . m per series, x1 = db x0 + da m,
//               dw = c0 x0 + c1 x1, FP32 forces of x1
//   TERM        x_{k+1} = 2da M x_k + (c1 x_k - x_{k-1}), dw += c_{k+1} x_{k+1}
//               (brownian_system.C:1091-1108)
//   TERM_CHECK  the same, plus |dw|^2 before the term, |x_{k+1}|^2 and the
//               FP32 forces of the new dw
//   CHECK       M dw, |M dw|^2; the stopping decision of every series of the
//               suspension (brownian_system.C:1117-1155): err1 <= tol
//               converged, err2 <= 1e-9 stopped
// Each pass is cut into tiles of S slots of one suspension.  A tile of
// pass p waits until its suspension has completed pass p - 1 (a per-
// suspension counter that the suspension's last tile of a pass advances,
// after the decision when the pass is a CHECK); nothing waits on other
// suspensions, so suspensions of different sizes and states overlap.  A
// free block takes the next tile in index order from one counter: a tile
// only waits on tiles of smaller index, all of which have been taken by
// running blocks (the launch is cooperative, every block resident), so the
// smallest unfinished tile can always proceed.  Every wait is bounded: a block that gives up sets the
// error word and all blocks leave.  A tile's reads of data other blocks
// wrote in earlier passes follow the wait's acquire fence and a block
// barrier; the per-series state and the partial sums are read through L2
// (volatile / ld.global.cg).  The estimator sums are per tile and then per
// suspension in tile order (deterministic).
enum : int { kPassStart = 0, kPassTerm = 1, kPassTermCheck = 2, kPassCheck = 3 };
constexpr int kPartKinds = 4;  // aux2 (x0 . M x0), |dw|^2, |x_{k+1}|^2, |M dw|^2

struct SeriesArgs {
  int64_t ntot;
  int W, K, S, T, npass, ldc;
  double tol, self_c;
  const int32_t *cnt;
  const uint32_t *list;
  const float4 *ten;
  const int32_t *susp;
  const int32_t *tile_b;      // [T] suspension of every tile of a pass
  const int64_t *tile_s0;     // [T] first slot of every tile
  const int32_t *susp_tile0;  // [K] first tile of every suspension
  const int32_t *susp_ntile;  // [K] its number of tiles
  const int64_t *off;         // [K + 1] first slot of every suspension
  const int32_t *pass_type;   // [npass]
  const int32_t *pass_term;   // [npass] term index t (x_{t+1} is formed)
  double *X0, *X1, *X2, *dw, *dm;
  float4 *F0, *F1, *Fdw;
  const double *da, *db, *two_da, *c1x, *coef;
  uint8_t *active;            // [K * 8]
  ggem_cheb_report *rep;      // [K * 8]
  double *part;               // [T][kPartKinds][8]
  double *aux2;               // [K * 8]
  unsigned int *arrive, *done;  // [K] tiles finished / passes completed
  int *n_active, *all_done, *err;
  unsigned long long *claim;  // next tile to take (tiles are taken in order)
  uint32_t polls;
  int never_ready;            // test hook: every wait runs out
};

__device__ __forceinline__ double series_x(const SeriesArgs &a, int q, int64_t k) {
  const double *X = q == 0 ? a.X0 : (q == 1 ? a.X1 : a.X2);
  return __ldcg(X + k);
}
__device__ __forceinline__ double *series_xp(const SeriesArgs &a, int q) {
  return q == 0 ? a.X0 : (q == 1 ? a.X1 : a.X2);
}

// sum over r-lanes of a per-thread value: lane % 8 is the right-hand side;
// sums of the 8 right-hand sides land in sh[w][r], then in out[r] (warps in
// order; fixed tree, deterministic)
template <int NT>
__device__ __forceinline__ void tile_rsum(double v, double (*sh)[kR], double *out) {
  v += __shfl_xor_sync(0xffffffffu, v, 8);
  v += __shfl_xor_sync(0xffffffffu, v, 16);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane < kR) sh[w][lane] = v;
  __syncthreads();
  if (threadIdx.x < kR) {
    double t = 0.0;
    for (int q = 0; q < NT / 32; ++q) t += sh[q][threadIdx.x];
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

// launch shapes of the persistent kernel (threads, blocks per SM that the
// register cap must allow); the autotuner picks one with the tile size
constexpr int kSeriesShapes = 3;
constexpr int kSeriesShapeThreads[kSeriesShapes] = {256, 256, 128};
constexpr int kSeriesShapeMinBlocks[kSeriesShapes] = {4, 6, 12};

template <int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_ens_series(SeriesArgs a) {
  __shared__ double sh[NT / 32][kR];
  __shared__ double dsum[kPartKinds][kR];
  __shared__ int s_go, s_last;
  __shared__ long long s_g;
  const int tid = threadIdx.x;
  const int64_t total = (int64_t)a.T * a.npass;
  for (;;) {
    // the next tile in pass-major order: a block that is free takes it, so
    // cheap and expensive tiles balance over the blocks
    if (tid == 0) s_g = (long long)atomicAdd(a.claim, 1ull);
    __syncthreads();
    const int64_t g = s_g;
    if (g >= total) return;
    const int p = (int)(g / a.T);
    const int tl = (int)(g - (int64_t)p * a.T);
    const int b = a.tile_b[tl];
    const int type = a.pass_type[p], t = a.pass_term[p];
    // ---- wait until this suspension has completed pass p - 1 ----
    if (tid == 0) {
      int go = 1;
      const unsigned need = (unsigned)p + (a.never_ready ? 0x40000000u : 0u);
      uint32_t n = 0;
      while (true) {
        if (*(volatile int *)a.err || *(volatile int *)a.all_done) {
          go = 0;
          break;
        }
        if (*(volatile unsigned *)(a.done + b) >= need) break;
        if (++n > a.polls) {
          atomicOr(a.err, kErrTimeout);
          go = 0;
          break;
        }
        __nanosleep(128);
      }
      __threadfence();
      // a suspension whose series have all stopped skips the work of its
      // later passes (its tiles still arrive, so that its passes complete);
      // the flags are read after the wait, when every earlier decision of
      // this suspension is visible
      if (go && type != kPassStart) {
        int any = 0;
        for (int r = 0; r < kR; ++r) any |= *(volatile const uint8_t *)(a.active + b * kR + r);
        if (!any) go = 2;
      }
      s_go = go;
    }
    __syncthreads();
    if (!s_go) return;  // an error, or every series has stopped
    const bool work = s_go == 1;
    const int64_t s_begin = a.tile_s0[tl];
    const int64_t s_end = min(s_begin + a.S, a.off[b + 1]);
    const double tda = a.two_da[b], c1 = a.c1x[b];
    const int q0 = (t + 2) % 3, q1 = t % 3, qm = (t + 1) % 3;  // x_{t-1}, x_t, x_{t+1}
    const float4 *Fsrc = type == kPassStart ? a.F1
                                            : (type == kPassCheck ? a.Fdw
                                                                  : ((t - 1) % 2 ? a.F1 : a.F0));
    float4 *Fout = type == kPassStart ? a.F0 : (t % 2 ? a.F1 : a.F0);
    double v0 = 0.0, v1 = 0.0;  // this thread's estimator terms
    for (int64_t i = tid; work && i < (int64_t)a.S * kR; i += NT) {
      const int64_t s = s_begin + i / kR;
      const int r = (int)(i % kR);
      if (s >= s_end) continue;
      const uint8_t act = *(volatile const uint8_t *)(a.active + b * kR + r);
      // pair sum over the stored tensors (entries and tensors are read-only)
      const int64_t e0 = s * (int64_t)a.W, e1 = e0 + __ldg(a.cnt + s);
      float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
      float bx = 0.f, by = 0.f, bz = 0.f;
      int blk = 0;
      for (int64_t m = e0; m < e1; ++m) {
        const uint32_t en = __ldg(a.list + m);
        const float4 tt = __ldg(a.ten + m);
        // a plain (L1-cacheable) load: the wait above ended with an acquire
        // fence at gpu scope and a block barrier, which orders these reads
        // after every write another block released for the previous pass
        // (PTX memory model, message passing); L1 keeps the sources that
        // neighbouring targets share
        const float4 fj = Fsrc[(int64_t)(en >> kCodeBits) * kR + r];
        const float d = fmaf(tt.w, fj.z, fmaf(tt.z, fj.y, tt.y * fj.x));
        bx += fmaf(tt.x, fj.x, d * tt.y);
        by += fmaf(tt.x, fj.y, d * tt.z);
        bz += fmaf(tt.x, fj.z, d * tt.w);
        if (++blk == 8) {
          kahan(sx, cx, bx);
          kahan(sy, cy, by);
          kahan(sz, cz, bz);
          bx = by = bz = 0.f;
          blk = 0;
        }
      }
      kahan(sx, cx, bx);
      kahan(sy, cy, by);
      kahan(sz, cz, bz);
      const float hs[3] = {sx, sy, sz}, ls[3] = {-cx, -cy, -cz};
      const int64_t k0 = (s * kR + r) * 3;
      float out[3];
      if (type == kPassStart) {
        const double cc0 = __ldg(a.coef + (int64_t)b * a.ldc),
                     cc1 = __ldg(a.coef + (int64_t)b * a.ldc + 1);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const double x0 = __ldcg(a.X0 + k0 + c);
          const double m = fma(a.self_c, x0, f2d(hs[c]) + f2d(ls[c]));
          v0 = fma(x0, m, v0);
          const double x1 = a.db[b] * x0 + a.da[b] * m;
          a.X1[k0 + c] = x1;
          a.dw[k0 + c] = cc0 * x0 + cc1 * x1;
          out[c] = d2f_bits(x1);
        }
        Fout[s * kR + r] = make_float4(out[0], out[1], out[2], 0.f);
      } else if (type == kPassCheck) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const double m = fma(a.self_c, __ldcg(a.dw + k0 + c), f2d(hs[c]) + f2d(ls[c]));
          v0 = fma(m, m, v0);
          if (act) a.dm[k0 + c] = m;  // a stopped series keeps its final M y
        }
      } else {
        const double cf = act ? __ldg(a.coef + (int64_t)b * a.ldc + t + 1) : 0.0;
        double *XM = series_xp(a, qm);
        float o2[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const double xk = series_x(a, q1, k0 + c);
          const double v = fma(tda, f2d(hs[c]) + f2d(ls[c]), fma(c1, xk, -series_x(a, q0, k0 + c)));
          XM[k0 + c] = v;
          const double y = __ldcg(a.dw + k0 + c);
          const double yn = fma(cf, v, y);
          a.dw[k0 + c] = yn;
          out[c] = d2f_bits(v);
          o2[c] = d2f_bits(yn);
          if (type == kPassTermCheck) {
            v0 = fma(y, y, v0);
            v1 = fma(v, v, v1);
          }
        }
        Fout[s * kR + r] = make_float4(out[0], out[1], out[2], 0.f);
        if (type == kPassTermCheck) a.Fdw[s * kR + r] = make_float4(o2[0], o2[1], o2[2], 0.f);
      }
    }
    // ---- this tile's estimator sums ----
    double *pt = a.part + (int64_t)tl * kPartKinds * kR;
    if (type == kPassStart) tile_rsum<NT>(v0, sh, pt + 0 * kR);
    if (type == kPassTermCheck) {
      tile_rsum<NT>(v0, sh, pt + 1 * kR);
      tile_rsum<NT>(v1, sh, pt + 2 * kR);
    }
    if (type == kPassCheck) tile_rsum<NT>(v0, sh, pt + 3 * kR);
    // ---- finish the tile; the suspension's last tile of the pass completes it ----
    __syncthreads();
    const int nt = a.susp_ntile[b];
    if (tid == 0) {
      __threadfence();
      const unsigned old = atomicAdd(a.arrive + b, 1u);
      s_last = old == (unsigned)(p + 1) * (unsigned)nt - 1u;
      if (s_last) __threadfence();
    }
    __syncthreads();
    if (!s_last) continue;
    if (type == kPassStart || type == kPassCheck) {
      // the suspension's sums in tile order (fixed assignment and tree)
      const int kind = type == kPassStart ? 0 : 3;
      const int nk = type == kPassStart ? 1 : 3;
      for (int q = 0; q < nk; ++q) {
        const int kd = type == kPassStart ? 0 : q + 1;
        double acc = 0.0;
        const int r = tid % kR;
        for (int j = tid / kR; j < nt; j += NT / kR)
          acc += __ldcg(a.part + ((int64_t)(a.susp_tile0[b] + j) * kPartKinds + kd) * kR + r);
        tile_rsum<NT>(acc, sh, dsum[kd]);
      }
      (void)kind;
      if (tid < kR) {
        // (state written by other blocks is read through L2: volatile / .cg)
        const int r = tid, sr = b * kR + r;
        if (type == kPassStart) {
          a.aux2[sr] = dsum[0][r];
        } else if (*(volatile const uint8_t *)(a.active + sr)) {
          volatile ggem_cheb_report *R = a.rep + sr;
          R->n_terms = t + 1;
          const double a2 = __ldcg(a.aux2 + sr);
          const double aux4 = sqrt(dsum[1][r]);
          const double aux3 = sqrt(dsum[2][r]) * fabs(__ldg(a.coef + (int64_t)b * a.ldc + t + 1));
          double e1 = R->err1, e2 = R->err2;
          if (a2 != 0.0) e1 = sqrt(fabs(dsum[3][r] - a2) / a2);
          if (aux4 != 0.0) e2 = aux3 / aux4;
          R->err1 = e1;
          R->err2 = e2;
          bool stop = false;
          if (e1 <= a.tol) {  // brownian_system.C:1138-1147
            R->converged = 1;
            stop = true;
          } else if (e2 <= 1e-9) {  // :1150
            stop = true;
          }
          if (stop) {
            a.active[sr] = 0;
            if (atomicSub(a.n_active, 1) == 1) atomicExch(a.all_done, 1);
          }
        }
      }
    } else if (tid < kR && *(volatile const uint8_t *)(a.active + b * kR + tid)) {
      ((volatile ggem_cheb_report *)a.rep)[b * kR + tid].n_terms = t + 1;
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      atomicExch(a.done + b, (unsigned)(p + 1));
    }
  }
}

}  // namespace ens
}  // namespace ggem

using namespace ggem;
using namespace ggem::ens;

struct ggem_ensemble {
  ggem_params base{};
  int K = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<double> box;
  std::vector<ggem_ctx *> sub;
  std::vector<int64_t> n, off;  // beads and first slot of every suspension (off has K+1)
  int64_t ntot = 0, pairs = 0;
  int W = 0;
  double self_c = 0.0;
  bool built = false;
  int block = 256;  // threads per block of the pair kernels (autotuned)
  DevBuf<int32_t> cnt, susp, order_g, rank_g;
  DevBuf<uint32_t> list;
  DevBuf<float4> ten;
  DevBuf<int64_t> d_off;
  // dot chunks: slot starts [nchunk + 1], first chunk of every suspension
  // [K + 1], partial sums [nchunk][8]
  DevBuf<int64_t> chunk_s;
  DevBuf<int32_t> chunk_off;
  DevBuf<double> chunk_part;
  int nchunk = 0;
  DevBuf<SubView> views;
  // Chebyshev state: vectors [slot][8][3] and FP32 forces [slot][8]
  DevBuf<double> v[6];
  DevBuf<float4> f4[3];
  DevBuf<double> coef, da, db, two_da, c1x, red;  // c1x: 2db + 2da self_c
  DevBuf<uint8_t> active;
  double *h_red = nullptr;
  int pred_terms = 0;
  int64_t vec_cap = 0;
  // the persistent series launch (k_ens_series): tiles of S slots of one
  // suspension, their per-pass estimator partials, counters and reports
  bool persistent = true;
  int S = 128;                 // slots per tile (autotuned)
  int series_shape = 1;        // launch shape of k_ens_series (autotuned)
  int T = 0;                   // tiles per pass
  int tiles_for_S = 0;         // S the tile tables were built for
  int64_t tiles_for_ntot = -1;
  DevBuf<int32_t> tile_b, susp_tile0, susp_ntile, pass_type, pass_term;
  DevBuf<int64_t> tile_s0;
  DevBuf<double> part, aux2;
  DevBuf<unsigned int> sync;   // arrive[K], done[K], n_active, all_done, err
  DevBuf<unsigned long long> claim;
  DevBuf<ggem_cheb_report> d_rep;
  uint32_t series_polls = 1u << 26;  // bounded waits of the persistent launch
  int never_ready = 0;               // test hook: every wait runs out
  // captured stretches of unchecked terms: (last term, coefficient stride) -> graph
  std::map<std::pair<int, int>, cudaGraphExec_t> graphs;
  // what the captured launches hold by value: the bead count, the row width,
  // the launch shape and the operator's and tables' device pointers.  A
  // reconfiguration can change any of them (a row overflow widens W, a new
  // bead count moves ntot, ensure() reallocates a grown buffer), so the
  // graphs are dropped whenever the signature differs from the captured one.
  struct GraphSig {
    int64_t ntot = -1;
    int W = -1, block = -1;
    const void *p[14] = {nullptr};
    bool operator==(const GraphSig &o) const {
      if (ntot != o.ntot || W != o.W || block != o.block) return false;
      for (int k = 0; k < 14; ++k)
        if (p[k] != o.p[k]) return false;
      return true;
    }
  } graph_sig;
  GraphSig signature() const {
    GraphSig g;
    g.ntot = ntot;
    g.W = W;
    g.block = block;
    const void *q[14] = {cnt.p,    list.p, ten.p,  susp.p, coef.p, two_da.p, c1x.p,
                         active.p, v[0].p, v[1].p, v[2].p, v[3].p, f4[0].p, f4[1].p};
    for (int k = 0; k < 14; ++k) g.p[k] = q[k];
    return g;
  }
  void drop_graphs() {
    for (auto &g : graphs) cudaGraphExecDestroy(g.second);
    graphs.clear();
  }
  // drops the captured graphs if anything they hold by value has changed
  void check_graphs() {
    const GraphSig now = signature();
    if (!(now == graph_sig)) {
      drop_graphs();
      graph_sig = now;
    }
  }
};

namespace {

struct EnsGuard {
  int prev = -1;
  explicit EnsGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~EnsGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

int efail(ggem_ensemble *e, int code, const std::string &msg) {
  e->err = msg;
  return code;
}
int ecuda(ggem_ensemble *e, cudaError_t c, const char *what) {
  cudaGetLastError();
  e->err = std::string(what) + ": " + cudaGetErrorString(c);
  return c == cudaErrorMemoryAllocation ? GGEM_ERR_OOM : GGEM_ERR_CUDA;
}
int elaunch(ggem_ensemble *e, const char *what) {
  cudaError_t c = cudaGetLastError();
  return c == cudaSuccess ? GGEM_OK : ecuda(e, c, what);
}
unsigned eblocks(int64_t work, int t) { return (unsigned)((work + t - 1) / t); }

int ensure_vectors(ggem_ensemble *e) {
  if (e->ntot <= e->vec_cap) return GGEM_OK;
  e->drop_graphs();  // captured pointers change
  cudaError_t c;
  for (auto &b : e->v)
    if ((c = b.ensure((size_t)e->ntot * kE))) return ecuda(e, c, "ensemble vectors");
  for (auto &b : e->f4)
    if ((c = b.ensure((size_t)e->ntot * kR))) return ecuda(e, c, "ensemble forces");
  e->vec_cap = e->ntot;
  return GGEM_OK;
}

// u = M f on slot-ordered [slot][8][3] vectors
int ens_matvec_slots(ggem_ensemble *e, const double *f, double *u, float4 *f4, double self_c) {
  k_ens_stage<<<eblocks(e->ntot * kR, 256), 256, 0, e->stream>>>(e->ntot, f, f4);
  if (int rc = elaunch(e, "ensemble stage")) return rc;
  k_ens_pair<false><<<eblocks(e->ntot * kR, e->block), e->block, 0, e->stream>>>(
      e->ntot, e->cnt.p, e->W, e->list.p, e->ten.p, f4, self_c, f, u, nullptr, nullptr, nullptr,
      nullptr, 0, 0, nullptr, nullptr, nullptr, nullptr);
  return elaunch(e, "ensemble pair sum");
}

}  // namespace

extern "C" int ggem_ensemble_create(const ggem_params *base, int k, const double *box_length,
                                    ggem_ensemble **out) {
  if (!base || k < 1 || !box_length || !out) return GGEM_ERR_BAD_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || base->device < 0 || base->device >= count) {
    cudaGetLastError();
    return GGEM_ERR_NO_DEVICE;
  }
  EnsGuard g(base->device);
  ggem_ensemble *e = new ggem_ensemble();
  e->base = *base;
  e->K = k;
  e->device = base->device;
  e->box.assign(box_length, box_length + k);
  e->sub.assign(k, nullptr);
  cudaError_t c;
  if ((c = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking)) ||
      (c = cudaMallocHost((void **)&e->h_red, sizeof(double) * 4 * kR * (size_t)k)) ||
      (c = e->d_off.ensure(k + 1)) || (c = e->views.ensure(k)) || (c = e->red.ensure(4 * kR * (size_t)k)) ||
      (c = e->active.ensure(kR * (size_t)k)) || (c = e->da.ensure(k)) || (c = e->db.ensure(k)) ||
      (c = e->two_da.ensure(k)) || (c = e->c1x.ensure(k))) {
    cudaGetLastError();
    ggem_ensemble_destroy(e);
    return c == cudaErrorMemoryAllocation ? GGEM_ERR_OOM : GGEM_ERR_CUDA;
  }
  for (int b = 0; b < k; ++b) {
    ggem_params p = *base;
    for (int d = 0; d < 3; ++d) {
      p.box_lo[d] = 0.0;
      p.box_hi[d] = box_length[b];
      p.periodic[d] = 1;
    }
    p.nb_mode = GGEM_NB_CUTOFF;
    p.precision = GGEM_FP32;
    if (int rc = ggem_create(&p, &e->sub[b])) {
      ggem_ensemble_destroy(e);
      return rc;
    }
    if (!e->sub[b]->use_pretensor) {
      ggem_ensemble_destroy(e);
      return GGEM_ERR_BAD_ARG;  // the ensemble operator needs stored pair tensors (B >= 0)
    }
  }
  e->self_c = self_coefficient(e->sub[0], e->base.point_type == GGEM_LAGRANGIAN_POINT
                                              ? GGEM_SELF_LAGRANGIAN
                                              : GGEM_SELF_BEAD);
  *out = e;
  return GGEM_OK;
}

extern "C" void ggem_ensemble_destroy(ggem_ensemble *e) {
  if (!e) return;
  {
    EnsGuard g(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    e->drop_graphs();
    for (auto *c : e->sub)
      if (c) ggem_destroy(c);
    if (e->h_red) cudaFreeHost(e->h_red);
    if (e->stream) cudaStreamDestroy(e->stream);
  }
  delete e;
}

extern "C" const char *ggem_ensemble_last_error(const ggem_ensemble *e) {
  return e ? e->err.c_str() : "null ensemble";
}

extern "C" int ggem_ensemble_set_particles_dev(ggem_ensemble *e, const int64_t *n,
                                               const double *d_xyz) {
  if (!e || !n || !d_xyz) return GGEM_ERR_BAD_ARG;
  EnsGuard g(e->device);
  e->built = false;
  e->n.assign(n, n + e->K);
  e->off.assign(e->K + 1, 0);
  for (int b = 0; b < e->K; ++b) {
    if (n[b] < 1) return efail(e, GGEM_ERR_BAD_ARG, "every suspension needs beads");
    e->off[b + 1] = e->off[b] + n[b];
  }
  e->ntot = e->off[e->K];
  if (e->ntot >= ((int64_t)1 << (32 - kCodeBits)))
    return efail(e, GGEM_ERR_BAD_ARG, "ensemble larger than the pair-entry slot space");
  // every suspension: cells, list, stored tensors (on its own stream)
  e->W = 0;
  e->pairs = 0;
  std::vector<SubView> views(e->K);
  for (int b = 0; b < e->K; ++b) {
    ggem_ctx *c = e->sub[b];
    if (int rc = ggem_set_particles_dev(c, n[b], d_xyz + 3 * e->off[b]))
      return efail(e, rc, "suspension " + std::to_string(b) + ": " + c->last_error);
    if (int rc = ggem_build_cells(c))
      return efail(e, rc, "suspension " + std::to_string(b) + ": " + c->last_error);
    if (!c->pretensor_ok)
      return efail(e, GGEM_ERR_OOM, "suspension " + std::to_string(b) + ": no pair tensors");
    e->W = std::max(e->W, c->nb_w);
    e->pairs += c->n_pairs;
    views[b] = SubView{c->nb_cnt.p, c->nb_list.p, c->pair_ten.p, c->order.p, c->rank.p,
                       n[b], e->off[b], c->nb_w};
  }
  for (ggem_ctx *c : e->sub) cudaStreamSynchronize(c->stream);
  cudaError_t c;
  if ((c = e->cnt.ensure(e->ntot)) || (c = e->susp.ensure(e->ntot)) ||
      (c = e->order_g.ensure(e->ntot)) || (c = e->rank_g.ensure(e->ntot)) ||
      (c = e->list.ensure((size_t)e->ntot * e->W)) || (c = e->ten.ensure((size_t)e->ntot * e->W)))
    return ecuda(e, c, "ensemble operator");
  if ((c = cudaMemcpyAsync(e->views.p, views.data(), sizeof(SubView) * e->K,
                           cudaMemcpyHostToDevice, e->stream)) ||
      (c = cudaMemcpyAsync(e->d_off.p, e->off.data(), sizeof(int64_t) * (e->K + 1),
                           cudaMemcpyHostToDevice, e->stream)))
    return ecuda(e, c, "ensemble tables");
  // the dot chunks (each within one suspension)
  std::vector<int64_t> cs;
  std::vector<int32_t> coff(e->K + 1, 0);
  for (int b = 0; b < e->K; ++b) {
    coff[b] = (int32_t)cs.size();
    for (int64_t s0 = e->off[b]; s0 < e->off[b + 1]; s0 += kDotSlots) cs.push_back(s0);
  }
  coff[e->K] = (int32_t)cs.size();
  e->nchunk = (int)cs.size();
  cs.push_back(e->ntot);  // a chunk ends where the next one (or the next suspension) begins
  if ((c = e->chunk_s.ensure(cs.size())) || (c = e->chunk_off.ensure(coff.size())) ||
      (c = e->chunk_part.ensure((size_t)e->nchunk * kR)) ||
      (c = cudaMemcpyAsync(e->chunk_s.p, cs.data(), sizeof(int64_t) * cs.size(),
                           cudaMemcpyHostToDevice, e->stream)) ||
      (c = cudaMemcpyAsync(e->chunk_off.p, coff.data(), sizeof(int32_t) * coff.size(),
                           cudaMemcpyHostToDevice, e->stream)))
    return ecuda(e, c, "ensemble dot chunks");
  int64_t nmax = 0;
  for (int b = 0; b < e->K; ++b) nmax = std::max(nmax, n[b]);
  dim3 grid(eblocks(nmax, 256), e->K);
  k_ens_gather<<<grid, 256, 0, e->stream>>>(e->views.p, e->W, e->cnt.p, e->list.p, e->ten.p,
                                            e->susp.p, e->order_g.p, e->rank_g.p);
  if (int rc = elaunch(e, "ensemble gather")) return rc;
  if ((c = cudaStreamSynchronize(e->stream))) return ecuda(e, c, "ensemble gather");
  if (int rc = ensure_vectors(e)) return rc;
  e->built = true;
  return GGEM_OK;
}

extern "C" int ggem_ensemble_sizes(const ggem_ensemble *e, int64_t *beads, int64_t *pairs) {
  if (!e || !beads || !pairs || !e->built) return GGEM_ERR_BAD_ARG;
  *beads = e->ntot;
  *pairs = e->pairs;
  return GGEM_OK;
}

extern "C" int ggem_ensemble_matvec_dev(ggem_ensemble *e, int nrhs, const double *d_f,
                                        double *d_u, int self_mode) {
  if (!e || nrhs < 1 || nrhs > kR || !d_f || !d_u) return GGEM_ERR_BAD_ARG;
  if (!e->built) return efail(e, GGEM_ERR_BAD_ARG, "set the ensemble's particles first");
  EnsGuard g(e->device);
  const double self_c = self_coefficient(e->sub[0], self_mode);
  const unsigned gv = eblocks(e->ntot * kE, 256);
  k_ens_to_slots<<<gv, 256, 0, e->stream>>>(e->ntot, nrhs, e->order_g.p, d_f, e->v[0].p);
  if (int rc = elaunch(e, "ensemble permute")) return rc;
  if (int rc = ens_matvec_slots(e, e->v[0].p, e->v[1].p, e->f4[0].p, self_c)) return rc;
  k_ens_from_slots<<<gv, 256, 0, e->stream>>>(e->ntot, nrhs, e->order_g.p, e->v[1].p, d_u);
  if (int rc = elaunch(e, "ensemble permute")) return rc;
  cudaError_t c = cudaStreamSynchronize(e->stream);
  return c ? ecuda(e, c, "ensemble matvec") : GGEM_OK;
}

namespace {

// one Chebyshev term of every series (k_ens_pair<true>); x1's forces in fcur,
// xm's written to fnext
int ens_term(ggem_ensemble *e, int term, int ldc, const double *x0, const double *x1, double *xm,
             double *dw, const float4 *fcur, float4 *fnext) {
  k_ens_pair<true><<<eblocks(e->ntot * kR, e->block), e->block, 0, e->stream>>>(
      e->ntot, e->cnt.p, e->W, e->list.p, e->ten.p, fcur, e->self_c, x1, xm, e->susp.p,
      e->two_da.p, e->c1x.p, e->coef.p, ldc, term, e->active.p, x0, dw, fnext);
  return elaunch(e, "ensemble chebyshev term");
}

int ens_dot(ggem_ensemble *e, const double *a, const double *b, double *out) {
  k_ens_dot_part<<<e->nchunk, kDotThreads, 0, e->stream>>>(e->chunk_s.p, a, b, e->chunk_part.p);
  if (int rc = elaunch(e, "ensemble dot")) return rc;
  k_ens_dot_fin<<<e->K, 32, 0, e->stream>>>(e->chunk_off.p, e->chunk_part.p, out);
  return elaunch(e, "ensemble dot sum");
}

}  // namespace

namespace {

// tile tables of the persistent launch for the current bead counts and S.
// Within a pass the suspensions' tiles follow in order of decreasing size:
// the many tiles of the large suspensions are taken first, so their pass is
// complete by the time the next pass reaches them, and the tiles taken last
// (whose next-pass tiles wait longest) are the small suspensions' few
static_assert(sizeof(int32_t) == 4, "tile tables");
int ensure_tiles(ggem_ensemble *e) {
  if (e->tiles_for_S == e->S && e->tiles_for_ntot == e->ntot && e->T > 0) return GGEM_OK;
  std::vector<int> by_size(e->K);
  for (int b = 0; b < e->K; ++b) by_size[b] = b;
  std::stable_sort(by_size.begin(), by_size.end(),
                   [&](int x, int y) { return e->n[x] > e->n[y]; });
  std::vector<int32_t> tb, st0(e->K, 0), ntl(e->K, 0);
  std::vector<int64_t> ts;
  for (int b : by_size) {
    st0[b] = (int32_t)tb.size();
    for (int64_t s0 = e->off[b]; s0 < e->off[b + 1]; s0 += e->S) {
      tb.push_back(b);
      ts.push_back(s0);
    }
    ntl[b] = (int32_t)tb.size() - st0[b];
  }
  e->T = (int)tb.size();
  cudaError_t c;
  if ((c = e->tile_b.ensure(tb.size())) || (c = e->tile_s0.ensure(ts.size())) ||
      (c = e->susp_tile0.ensure(st0.size())) || (c = e->susp_ntile.ensure(ntl.size())) ||
      (c = cudaMemcpyAsync(e->susp_ntile.p, ntl.data(), sizeof(int32_t) * ntl.size(),
                           cudaMemcpyHostToDevice, e->stream)) ||
      (c = e->part.ensure((size_t)e->T * kPartKinds * kR)) ||
      (c = e->aux2.ensure((size_t)e->K * kR)) ||
      (c = cudaMemcpyAsync(e->tile_b.p, tb.data(), sizeof(int32_t) * tb.size(),
                           cudaMemcpyHostToDevice, e->stream)) ||
      (c = cudaMemcpyAsync(e->tile_s0.p, ts.data(), sizeof(int64_t) * ts.size(),
                           cudaMemcpyHostToDevice, e->stream)) ||
      (c = cudaMemcpyAsync(e->susp_tile0.p, st0.data(), sizeof(int32_t) * st0.size(),
                           cudaMemcpyHostToDevice, e->stream)) ||
      (c = cudaStreamSynchronize(e->stream)))
    return ecuda(e, c, "series tiles");
  e->tiles_for_S = e->S;
  e->tiles_for_ntot = e->ntot;
  return GGEM_OK;
}

const void *series_kernel(int shape) {
  switch (shape) {
    case 0: return (const void *)k_ens_series<kSeriesShapeThreads[0], kSeriesShapeMinBlocks[0]>;
    case 1: return (const void *)k_ens_series<kSeriesShapeThreads[1], kSeriesShapeMinBlocks[1]>;
    default: return (const void *)k_ens_series<kSeriesShapeThreads[2], kSeriesShapeMinBlocks[2]>;
  }
}

// blocks of the persistent launch: every block resident (cooperative)
int series_grid(ggem_ensemble *e, int shape, int *grid) {
  int sms = 0, per = 0, coop = 0;
  cudaError_t c;
  if ((c = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->device)) ||
      (c = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, e->device)) ||
      (c = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, series_kernel(shape),
                                                          kSeriesShapeThreads[shape], 0)))
    return ecuda(e, c, "series occupancy");
  if (!coop || per < 1) return efail(e, GGEM_ERR_CUDA, "cooperative launch unavailable");
  *grid = sms * per;
  return GGEM_OK;
}

// the whole step of every series in one persistent launch (k_ens_series):
// permute xi in, stage x0's forces, the series, permute dw out
int brownian_persistent(ggem_ensemble *e, int nrhs, int N, const double *eig_min,
                        const double *eig_max, double tol, const double *d_xi, double *d_dw,
                        ggem_cheb_report *rep) {
  const int K = e->K, ldc = N + 1;
  std::vector<double> coef((size_t)K * ldc), da(K), db(K), tda(K), tdb(K);
  for (int b = 0; b < K; ++b) {
    if (!(eig_min[b] >= 0) || !(eig_min[b] < eig_max[b]))
      return efail(e, GGEM_ERR_INVALID_RANGE, "invalid eigenvalue range of suspension " +
                                                  std::to_string(b));
    const double d = eig_max[b] - eig_min[b];
    da[b] = 2.0 / d;
    db[b] = -(eig_max[b] + eig_min[b]) / d;
    tda[b] = 2.0 * da[b];
    tdb[b] = 2.0 * db[b] + tda[b] * e->self_c;
  }
  if (int rc = ensure_tiles(e)) return rc;
  double *x0 = e->v[0].p;
  const unsigned gv = eblocks(e->ntot * kE, 256);
  k_ens_to_slots<<<gv, 256, 0, e->stream>>>(e->ntot, nrhs, e->order_g.p, d_xi, x0);
  if (int rc = elaunch(e, "ensemble permute")) return rc;
  k_ens_stage<<<eblocks(e->ntot * kR, 256), 256, 0, e->stream>>>(e->ntot, x0, e->f4[1].p);
  if (int rc = elaunch(e, "ensemble stage")) return rc;
  // coefficients of all suspensions (chebyshev.C:44-151) while x0 is staged
  cheb_coeffs_host_many(N, K, da.data(), db.data(), GGEM_CHEB_GAUSS, coef.data(), ldc);
  // the pass list: the start, the unchecked stretch up to the predicted
  // degree, then a checked term and its check per term
  const int k_first = std::max(2, e->pred_terms > 0 ? e->pred_terms : 8);
  const int last_unchecked = std::min(k_first - 2, N - 2);
  std::vector<int32_t> ptype{kPassStart}, pterm{0};
  for (int t = 1; t <= last_unchecked; ++t) {
    ptype.push_back(kPassTerm);
    pterm.push_back(t);
  }
  for (int t = std::max(1, last_unchecked + 1); t < N; ++t) {
    ptype.push_back(kPassTermCheck);
    pterm.push_back(t);
    ptype.push_back(kPassCheck);
    pterm.push_back(t);
  }
  const int npass = (int)ptype.size();
  std::vector<uint8_t> act((size_t)K * kR, 0);
  std::vector<ggem_cheb_report> r0((size_t)K * kR, ggem_cheb_report{0, 1, 1, 0.0, 0.0});
  for (int b = 0; b < K; ++b)
    for (int r = 0; r < nrhs; ++r) act[b * kR + r] = 1;
  std::vector<unsigned int> sync0(2 * (size_t)K + 3, 0u);
  sync0[2 * K] = (unsigned)(K * nrhs);  // series still running
  cudaError_t c;
  if ((c = e->coef.ensure((size_t)K * ldc)) || (c = e->pass_type.ensure(npass)) ||
      (c = e->pass_term.ensure(npass)) || (c = e->sync.ensure(sync0.size())) ||
      (c = e->claim.ensure(1)) || (c = e->d_rep.ensure((size_t)K * kR)))
    return ecuda(e, c, "series tables");
  if ((c = cudaMemcpyAsync(e->coef.p, coef.data(), sizeof(double) * K * ldc,
                           cudaMemcpyHostToDevice, e->stream)) ||
      (c = cudaMemcpyAsync(e->da.p, da.data(), sizeof(double) * K, cudaMemcpyHostToDevice,
                           e->stream)) ||
      (c = cudaMemcpyAsync(e->db.p, db.data(), sizeof(double) * K, cudaMemcpyHostToDevice,
                           e->stream)) ||
      (c = cudaMemcpyAsync(e->two_da.p, tda.data(), sizeof(double) * K, cudaMemcpyHostToDevice,
                           e->stream)) ||
      (c = cudaMemcpyAsync(e->c1x.p, tdb.data(), sizeof(double) * K, cudaMemcpyHostToDevice,
                           e->stream)) ||
      (c = cudaMemcpyAsync(e->active.p, act.data(), K * kR, cudaMemcpyHostToDevice, e->stream)) ||
      (c = cudaMemcpyAsync(e->pass_type.p, ptype.data(), sizeof(int32_t) * npass,
                           cudaMemcpyHostToDevice, e->stream)) ||
      (c = cudaMemcpyAsync(e->pass_term.p, pterm.data(), sizeof(int32_t) * npass,
                           cudaMemcpyHostToDevice, e->stream)) ||
      (c = cudaMemcpyAsync(e->sync.p, sync0.data(), sizeof(unsigned int) * sync0.size(),
                           cudaMemcpyHostToDevice, e->stream)) ||
      (c = cudaMemcpyAsync(e->d_rep.p, r0.data(), sizeof(ggem_cheb_report) * r0.size(),
                           cudaMemcpyHostToDevice, e->stream)) ||
      (c = cudaMemsetAsync(e->claim.p, 0, sizeof(unsigned long long), e->stream)))
    return ecuda(e, c, "series tables");
  SeriesArgs a;
  a.ntot = e->ntot;
  a.W = e->W;
  a.K = K;
  a.S = e->S;
  a.T = e->T;
  a.npass = npass;
  a.ldc = ldc;
  a.tol = tol;
  a.self_c = e->self_c;
  a.cnt = e->cnt.p;
  a.list = e->list.p;
  a.ten = e->ten.p;
  a.susp = e->susp.p;
  a.tile_b = e->tile_b.p;
  a.tile_s0 = e->tile_s0.p;
  a.susp_tile0 = e->susp_tile0.p;
  a.susp_ntile = e->susp_ntile.p;
  a.off = e->d_off.p;
  a.pass_type = e->pass_type.p;
  a.pass_term = e->pass_term.p;
  a.X0 = e->v[0].p;
  a.X1 = e->v[1].p;
  a.X2 = e->v[2].p;
  a.dw = e->v[3].p;
  a.dm = e->v[4].p;
  a.F0 = e->f4[0].p;
  a.F1 = e->f4[1].p;
  a.Fdw = e->f4[2].p;
  a.da = e->da.p;
  a.db = e->db.p;
  a.two_da = e->two_da.p;
  a.c1x = e->c1x.p;
  a.coef = e->coef.p;
  a.active = e->active.p;
  a.rep = e->d_rep.p;
  a.part = e->part.p;
  a.aux2 = e->aux2.p;
  a.arrive = e->sync.p;
  a.done = e->sync.p + K;
  a.n_active = reinterpret_cast<int *>(e->sync.p + 2 * K);
  a.all_done = reinterpret_cast<int *>(e->sync.p + 2 * K + 1);
  a.err = reinterpret_cast<int *>(e->sync.p + 2 * K + 2);
  a.claim = e->claim.p;
  a.polls = e->series_polls;
  a.never_ready = e->never_ready;
  int grid = 0;
  const int shape = e->series_shape;
  if (int rc = series_grid(e, shape, &grid)) return rc;
  grid = (int)std::min<int64_t>(grid, (int64_t)e->T * npass);
  void *args[] = {&a};
  if ((c = cudaLaunchCooperativeKernel(series_kernel(shape), dim3(grid),
                                       dim3(kSeriesShapeThreads[shape]), args, 0, e->stream)))
    return ecuda(e, c, "series launch");
  if (int rc = elaunch(e, "series")) return rc;
  k_ens_from_slots<<<gv, 256, 0, e->stream>>>(e->ntot, nrhs, e->order_g.p, e->v[4].p, d_dw);
  if (int rc = elaunch(e, "ensemble permute")) return rc;
  std::vector<ggem_cheb_report> rr((size_t)K * kR);
  unsigned int flags[3] = {0u, 0u, 0u};
  if ((c = cudaMemcpyAsync(rr.data(), e->d_rep.p, sizeof(ggem_cheb_report) * rr.size(),
                           cudaMemcpyDeviceToHost, e->stream)) ||
      (c = cudaMemcpyAsync(flags, e->sync.p + 2 * K, sizeof(flags), cudaMemcpyDeviceToHost,
                           e->stream)) ||
      (c = cudaStreamSynchronize(e->stream)))
    return ecuda(e, c, "series reports");
  if (flags[2] & kErrTimeout)
    return efail(e, GGEM_ERR_TIMEOUT, "a wait of the persistent series ran out");
  // reports; operator applications: the start, one per unchecked term, two
  // per checked term (brownian_system.C:1093, :1117)
  bool all = true;
  int worst = 0;
  const int first_check = last_unchecked + 2;
  bool room = true;
  for (int b = 0; b < K; ++b) {
    const double kap = eig_min[b] > 0 ? eig_max[b] / eig_min[b] : 1e30;
    const double rho = (std::sqrt(kap) - 1.0) / (std::sqrt(kap) + 1.0);
    for (int r = 0; r < nrhs; ++r) {
      ggem_cheb_report R = rr[b * kR + r];
      const int T = R.n_terms;
      const int unchecked = std::min(T - 1, last_unchecked);
      R.n_matvecs = 1 + unchecked + 2 * std::max(0, T - 1 - unchecked);
      rep[b * nrhs + r] = R;
      all = all && R.converged;
      worst = std::max(worst, T);
      room = room && R.err1 <= 0.8 * rho * tol;
    }
  }
  // adaptive schedule, as the launch-per-term path
  if (all) e->pred_terms = (worst == first_check && room) ? std::max(2, worst - 1) : worst;
  return all ? GGEM_OK : efail(e, GGEM_ERR_CHEB_NOT_CONVERGED, "some series did not converge");
}

}  // namespace

extern "C" int ggem_ensemble_set_series_mode(ggem_ensemble *e, int persistent, int slots_per_tile,
                                             uint32_t wait_polls, int never_ready) {
  if (!e || (slots_per_tile != 0 && (slots_per_tile < 8 || slots_per_tile > 1024)))
    return GGEM_ERR_BAD_ARG;
  e->persistent = persistent != 0;
  if (slots_per_tile) e->S = slots_per_tile;
  e->series_polls = wait_polls ? wait_polls : (1u << 26);
  e->never_ready = never_ready != 0;
  return GGEM_OK;
}

extern "C" int ggem_ensemble_autotune_series(ggem_ensemble *e, int nrhs, int N,
                                             const double *eig_min, const double *eig_max,
                                             double tol, const double *d_xi, double *d_dw,
                                             const char *cache_path, int *shape,
                                             int *slots_per_tile, double *ms_per_step) {
  if (!e || nrhs < 1 || nrhs > kR || N < 2 || !eig_min || !eig_max || !d_xi || !d_dw || !shape ||
      !slots_per_tile || !ms_per_step)
    return GGEM_ERR_BAD_ARG;
  if (!e->built) return efail(e, GGEM_ERR_BAD_ARG, "set the ensemble's particles first");
  EnsGuard g(e->device);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, e->device) != cudaSuccess) {
    cudaGetLastError();
    return efail(e, GGEM_ERR_CUDA, "device properties");
  }
  // the cache key: the device, the ensemble's sizes and the right-hand sides
  std::string key = std::string(prop.name) + "|K=" + std::to_string(e->K) +
                    "|beads=" + std::to_string(e->ntot) + "|pairs=" + std::to_string(e->pairs) +
                    "|W=" + std::to_string(e->W) + "|rhs=" + std::to_string(nrhs);
  for (char &ch : key)
    if (ch == ' ') ch = '_';
  if (cache_path) {
    if (FILE *fp = std::fopen(cache_path, "r")) {
      char k[512];
      int sh = 0, S = 0;
      double ms = 0.0;
      bool hit = false;
      while (std::fscanf(fp, "%511s %d %d %lf", k, &sh, &S, &ms) == 4)
        if (key == k && sh >= 0 && sh <= kSeriesShapes && S >= 8 && S <= 1024) {
          e->series_shape = sh;
          e->S = S;
          *shape = sh;
          *slots_per_tile = S;
          *ms_per_step = ms;
          hit = true;
        }
      std::fclose(fp);
      if (hit) {
        e->persistent = e->series_shape < kSeriesShapes;
        if (!e->persistent) e->series_shape = 1;
        return GGEM_OK;
      }
    }
  }
  // time one Brownian step of every series for each launch shape and tile
  // size (tol = 0: every series runs the same N - 1 terms)
  const int tiles[3] = {64, 128, 256};
  const bool keep_pers = e->persistent;
  const int keep_pred = e->pred_terms;
  const int keep_shape = e->series_shape;
  e->persistent = true;
  double best = 1e30;
  int best_sh = e->series_shape, best_S = e->S;
  std::vector<ggem_cheb_report> rep((size_t)e->K * nrhs);
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  int rc = GGEM_OK;
  for (int sh = 0; sh < kSeriesShapes && (rc == GGEM_OK || rc == GGEM_ERR_CHEB_NOT_CONVERGED); ++sh)
    for (int S : tiles) {
      e->series_shape = sh;
      e->S = S;
      e->pred_terms = N;
      rc = brownian_persistent(e, nrhs, N, eig_min, eig_max, 0.0, d_xi, d_dw, rep.data());
      if (rc != GGEM_OK && rc != GGEM_ERR_CHEB_NOT_CONVERGED) break;
      cudaEventRecord(t0, e->stream);
      e->pred_terms = N;
      rc = brownian_persistent(e, nrhs, N, eig_min, eig_max, 0.0, d_xi, d_dw, rep.data());
      cudaEventRecord(t1, e->stream);
      cudaEventSynchronize(t1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, t0, t1);
      if (rc != GGEM_OK && rc != GGEM_ERR_CHEB_NOT_CONVERGED) break;
      if (ms < best) {
        best = ms;
        best_sh = sh;
        best_S = S;
      }
    }
  // and the step as one launch per term (host-side checks; the unchecked
  // stretch as a graph), candidate kSeriesShapes
  if (rc == GGEM_OK || rc == GGEM_ERR_CHEB_NOT_CONVERGED) {
    e->persistent = false;
    for (int k = 0; k < 2; ++k) {
      e->pred_terms = N;
      if (k == 1) cudaEventRecord(t0, e->stream);
      rc = ggem_ensemble_brownian_dev(e, nrhs, N, eig_min, eig_max, 0.0, d_xi, d_dw, rep.data());
      if (rc != GGEM_OK && rc != GGEM_ERR_CHEB_NOT_CONVERGED) break;
    }
    if (rc == GGEM_OK || rc == GGEM_ERR_CHEB_NOT_CONVERGED) {
      cudaEventRecord(t1, e->stream);
      cudaEventSynchronize(t1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, t0, t1);
      if (ms < best) {
        best = ms;
        best_sh = kSeriesShapes;
      }
    }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  e->persistent = keep_pers;
  e->pred_terms = keep_pred;
  if (rc != GGEM_OK && rc != GGEM_ERR_CHEB_NOT_CONVERGED) return rc;
  e->persistent = best_sh < kSeriesShapes;
  e->series_shape = e->persistent ? best_sh : keep_shape;
  e->S = best_S;
  *shape = best_sh;
  *slots_per_tile = best_S;
  *ms_per_step = best;
  if (cache_path) {
    if (FILE *fp = std::fopen(cache_path, "a")) {
      std::fprintf(fp, "%s %d %d %.6f\n", key.c_str(), best_sh, best_S, best);
      std::fclose(fp);
    }
  }
  return GGEM_OK;
}

extern "C" int ggem_ensemble_brownian_dev(ggem_ensemble *e, int nrhs, int N,
                                          const double *eig_min, const double *eig_max,
                                          double tol, const double *d_xi, double *d_dw,
                                          ggem_cheb_report *rep) {
  if (!e || nrhs < 1 || nrhs > kR || N < 2 || !eig_min || !eig_max || !(tol >= 0) || !d_xi ||
      !d_dw || !rep)
    return GGEM_ERR_BAD_ARG;
  if (!e->built) return efail(e, GGEM_ERR_BAD_ARG, "set the ensemble's particles first");
  EnsGuard g(e->device);
  if (e->persistent)
    return brownian_persistent(e, nrhs, N, eig_min, eig_max, tol, d_xi, d_dw, rep);

  const int K = e->K, ldc = N + 1;
  // per suspension: interval (copss.C:1609-1615), coefficients (chebyshev.C:44-151)
  std::vector<double> coef((size_t)K * ldc), da(K), db(K), tda(K), tdb(K);
  for (int b = 0; b < K; ++b) {
    if (!(eig_min[b] >= 0) || !(eig_min[b] < eig_max[b]))
      return efail(e, GGEM_ERR_INVALID_RANGE, "invalid eigenvalue range of suspension " +
                                                  std::to_string(b));
    const double d = eig_max[b] - eig_min[b];
    da[b] = 2.0 / d;
    db[b] = -(eig_max[b] + eig_min[b]) / d;
    tda[b] = 2.0 * da[b];
    tdb[b] = 2.0 * db[b] + tda[b] * e->self_c;  // c1 of the fused term
  }
  double *x0 = e->v[0].p, *x1 = e->v[1].p, *xm = e->v[2].p, *dw = e->v[3].p, *dm = e->v[4].p;
  float4 *fa = e->f4[0].p, *fb = e->f4[1].p, *fc = e->f4[2].p;
  double *aux2 = e->red.p, *q0 = aux2 + K * kR, *q1 = q0 + K * kR, *q2 = q1 + K * kR;
  const unsigned gv = eblocks(e->ntot * kE, 256);
  // x0 = xi; x1 = M x0; aux2 = x1 . x0; x1 = db x0 + da x1; dw = c0 x0 + c1 x1
  k_ens_to_slots<<<gv, 256, 0, e->stream>>>(e->ntot, nrhs, e->order_g.p, d_xi, x0);
  if (int rc = elaunch(e, "ensemble permute")) return rc;
  if (int rc = ens_matvec_slots(e, x0, x1, fa, e->self_c)) return rc;
  if (int rc = ens_dot(e, x1, x0, aux2)) return rc;
  // the coefficients and tables are prepared on the host while the device
  // runs the first matvec (nothing before k_ens_start reads them)
  cheb_coeffs_host_many(N, K, da.data(), db.data(), GGEM_CHEB_GAUSS, coef.data(), ldc);
  std::vector<uint8_t> act((size_t)K * kR, 0);
  for (int b = 0; b < K; ++b)
    for (int r = 0; r < nrhs; ++r) act[b * kR + r] = 1;
  for (int i = 0; i < K * nrhs; ++i) rep[i] = ggem_cheb_report{0, 1, 1, 0.0, 0.0};
  cudaError_t c;
  if (e->coef.count < (size_t)K * ldc) e->drop_graphs();
  if ((c = e->coef.ensure((size_t)K * ldc))) return ecuda(e, c, "coefficients");
  if ((c = cudaMemcpyAsync(e->coef.p, coef.data(), sizeof(double) * K * ldc,
                           cudaMemcpyHostToDevice, e->stream)) ||
      (c = cudaMemcpyAsync(e->da.p, da.data(), sizeof(double) * K, cudaMemcpyHostToDevice,
                           e->stream)) ||
      (c = cudaMemcpyAsync(e->db.p, db.data(), sizeof(double) * K, cudaMemcpyHostToDevice,
                           e->stream)) ||
      (c = cudaMemcpyAsync(e->two_da.p, tda.data(), sizeof(double) * K, cudaMemcpyHostToDevice,
                           e->stream)) ||
      (c = cudaMemcpyAsync(e->c1x.p, tdb.data(), sizeof(double) * K, cudaMemcpyHostToDevice,
                           e->stream)) ||
      (c = cudaMemcpyAsync(e->active.p, act.data(), K * kR, cudaMemcpyHostToDevice, e->stream)))
    return ecuda(e, c, "chebyshev tables");
  k_ens_start<<<gv, 256, 0, e->stream>>>(e->ntot, e->susp.p, e->da.p, e->db.p, e->coef.p, ldc,
                                        x0, x1, dw);
  if (int rc = elaunch(e, "ensemble start")) return rc;
  k_ens_stage<<<eblocks(e->ntot * kR, 256), 256, 0, e->stream>>>(e->ntot, x1, fa);
  if (int rc = elaunch(e, "ensemble stage")) return rc;
  double *h = e->h_red;
  std::vector<double> h_aux2((size_t)K * kR, 0.0);
  bool have_aux2 = false, dm_is_y = false;
  const int k_first = std::max(2, e->pred_terms > 0 ? e->pred_terms : 8);
  int first_check = -1;
  // buffers of term i: (x0, x1, xm) rotate with period 3, forces with period 2
  double *X[3] = {x0, x1, xm};
  float4 *F[2] = {fa, fb};
  int i = 1;
  // terms 1 .. k_first-2 carry no check: one captured graph per stretch
  const int last_unchecked = std::min(k_first - 2, N - 2);
  if (last_unchecked >= 1) {
    e->check_graphs();
    const auto key = std::make_pair(last_unchecked, ldc);
    auto it = e->graphs.find(key);
    if (it == e->graphs.end()) {
      cudaGraph_t graph = nullptr;
      cudaGraphExec_t exec = nullptr;
      if ((c = cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal)))
        return ecuda(e, c, "graph capture");
      int rc = GGEM_OK;
      for (int t = 1; t <= last_unchecked && !rc; ++t)
        rc = ens_term(e, t + 1, ldc, X[(t - 1) % 3], X[t % 3], X[(t + 1) % 3], dw, F[(t - 1) % 2],
                      F[t % 2]);
      c = cudaStreamEndCapture(e->stream, &graph);
      if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
      }
      if (c) return ecuda(e, c, "graph capture");
      c = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (c) return ecuda(e, c, "graph instantiate");
      it = e->graphs.emplace(key, exec).first;
    }
    if ((c = cudaGraphLaunch(it->second, e->stream))) return ecuda(e, c, "graph launch");
    for (int t = 1; t <= last_unchecked; ++t)
      for (int q = 0; q < K * nrhs; ++q) {
        rep[q].n_matvecs += 1;
        rep[q].n_terms = t + 1;
      }
    i = last_unchecked + 1;
  }
  int n_active = K * nrhs;
  for (; i < N && n_active > 0; ++i) {
    double *a0 = X[(i - 1) % 3], *a1 = X[i % 3], *am = X[(i + 1) % 3];
    float4 *fcur = F[(i - 1) % 2], *fnext = F[i % 2];
    // the estimators of this term: |dw| before it, |x_{i+1}|, |M dw| after it
    if (int rc = ens_dot(e, dw, dw, q0)) return rc;
    if (int rc = ens_term(e, i + 1, ldc, a0, a1, am, dw, fcur, fnext)) return rc;
    if (int rc = ens_dot(e, am, am, q1)) return rc;
    if (int rc = ens_matvec_slots(e, dw, dm, fc, e->self_c)) return rc;
    if (int rc = ens_dot(e, dm, dm, q2)) return rc;
    if ((c = cudaMemcpyAsync(h, q0, sizeof(double) * 3 * K * kR, cudaMemcpyDeviceToHost,
                             e->stream)))
      return ecuda(e, c, "estimators");
    if (!have_aux2 &&
        (c = cudaMemcpyAsync(h_aux2.data(), aux2, sizeof(double) * K * kR,
                             cudaMemcpyDeviceToHost, e->stream)))
      return ecuda(e, c, "estimators");
    if ((c = cudaStreamSynchronize(e->stream))) return ecuda(e, c, "estimators");
    have_aux2 = true;
    dm_is_y = true;
    if (first_check < 0) first_check = i + 1;
    bool changed = false;
    for (int b = 0; b < K; ++b)
      for (int r = 0; r < nrhs; ++r) {
        const int q = b * kR, idx = b * nrhs + r;
        if (!act[q + r]) continue;
        ggem_cheb_report &R = rep[idx];
        R.n_matvecs += 2;
        R.n_terms = i + 1;
        const double aux4 = std::sqrt(h[q + r]);
        const double aux3 = std::sqrt(h[K * kR + q + r]) * std::fabs(coef[(size_t)b * ldc + i + 1]);
        const double aux1 = h[2 * K * kR + q + r], a2 = h_aux2[q + r];
        if (a2 != 0.0) R.err1 = std::sqrt(std::fabs(aux1 - a2) / a2);
        if (aux4 != 0.0) R.err2 = aux3 / aux4;
        if (R.err1 <= tol) {  // brownian_system.C:1138-1147
          R.converged = 1;
          act[q + r] = 0;
          changed = true;
        } else if (R.err2 <= 1e-9) {  // :1150
          act[q + r] = 0;
          changed = true;
        }
      }
    if (changed) {
      n_active = 0;
      for (uint8_t a : act) n_active += a;
      if ((c = cudaMemcpyAsync(e->active.p, act.data(), K * kR, cudaMemcpyHostToDevice,
                               e->stream)))
        return ecuda(e, c, "active series");
    }
  }
  // dw = M y: the last check's M dw when no term followed it
  const double *y_out = dm;
  if (!dm_is_y) {
    if (int rc = ens_matvec_slots(e, dw, dm, fc, e->self_c)) return rc;
  }
  k_ens_from_slots<<<gv, 256, 0, e->stream>>>(e->ntot, nrhs, e->order_g.p, y_out, d_dw);
  if (int rc = elaunch(e, "ensemble permute")) return rc;
  if ((c = cudaStreamSynchronize(e->stream))) return ecuda(e, c, "ensemble brownian");
  // adaptive schedule: the next call checks from the degree this one needed
  // (one degree less only when every series passed its first check with
  // room for it: the error shrinks by about rho = (sqrt(k) - 1) / (sqrt(k) + 1)
  // per degree, k = eig_max / eig_min of the suspension; otherwise a steady
  // workload would fail a check, a matvec and a host round trip more, every
  // other call)
  int worst = 0;
  bool all = true, room = true;
  for (int b = 0; b < K; ++b) {
    const double kap = eig_min[b] > 0 ? eig_max[b] / eig_min[b] : 1e30;
    const double rho = (std::sqrt(kap) - 1.0) / (std::sqrt(kap) + 1.0);
    for (int r = 0; r < nrhs; ++r) {
      const ggem_cheb_report &R = rep[b * nrhs + r];
      all = all && R.converged;
      worst = std::max(worst, R.n_terms);
      room = room && R.err1 <= 0.8 * rho * tol;
    }
  }
  if (all) e->pred_terms = (worst == first_check && room) ? std::max(2, worst - 1) : worst;
  return all ? GGEM_OK : efail(e, GGEM_ERR_CHEB_NOT_CONVERGED, "some series did not converge");
}

extern "C" int ggem_ensemble_intervals(ggem_ensemble *e, ggem_surrogate *s,
                                       const double *chain_fraction, double margin_lo,
                                       double margin_hi, double *eig_min, double *eig_max) {
  if (!e || !s || !eig_min || !eig_max || !(margin_lo >= 0) || !(margin_hi >= 0))
    return GGEM_ERR_BAD_ARG;
  if (!e->built) return efail(e, GGEM_ERR_BAD_ARG, "set the ensemble's particles first");
  EnsGuard g(e->device);
  std::vector<float> X((size_t)e->K * GGEM_SUR_FEATURES), Y((size_t)e->K * GGEM_SUR_OUTPUTS);
  for (int b = 0; b < e->K; ++b)
    if (int rc = ggem_surrogate_features(e->sub[b], chain_fraction ? chain_fraction[b] : 0.0,
                                         X.data() + (size_t)b * GGEM_SUR_FEATURES))
      return efail(e, rc, e->sub[b]->last_error);
  // one batched forward pass for all suspensions
  if (int rc = ggem_surrogate_predict(s, X.data(), e->K, Y.data()))
    return efail(e, rc, ggem_surrogate_last_error(s));
  for (int b = 0; b < e->K; ++b) {
    eig_min[b] = std::exp((double)Y[2 * b] - margin_lo);
    eig_max[b] = std::exp((double)Y[2 * b + 1] + margin_hi);
  }
  return GGEM_OK;
}

extern "C" int ggem_ensemble_lanczos(ggem_ensemble *e, int b, int k, uint64_t seed,
                                     double *eig_min, double *eig_max) {
  if (!e || b < 0 || b >= e->K) return GGEM_ERR_BAD_ARG;
  if (!e->built) return efail(e, GGEM_ERR_BAD_ARG, "set the ensemble's particles first");
  if (int rc = ggem_lanczos_bounds(e->sub[b], k, seed, eig_min, eig_max))
    return efail(e, rc, e->sub[b]->last_error);
  return GGEM_OK;
}

extern "C" int ggem_ensemble_autotune(ggem_ensemble *e, int nrhs, int *block_threads,
                                      double *ms_per_term) {
  if (!e || nrhs < 1 || nrhs > kR || !block_threads || !ms_per_term) return GGEM_ERR_BAD_ARG;
  if (!e->built) return efail(e, GGEM_ERR_BAD_ARG, "set the ensemble's particles first");
  EnsGuard g(e->device);
  cudaError_t c;
  // a Chebyshev term of every series on zero-free data: tables for a unit
  // interval, all series active
  const int ldc = 3;
  std::vector<double> coef((size_t)e->K * ldc, 0.5), one(e->K, 1.0);
  std::vector<uint8_t> act((size_t)e->K * kR, 1);
  if (e->coef.count < (size_t)e->K * ldc) e->drop_graphs();
  if ((c = e->coef.ensure((size_t)e->K * ldc)) ||
      (c = cudaMemcpyAsync(e->coef.p, coef.data(), sizeof(double) * coef.size(),
                           cudaMemcpyHostToDevice, e->stream)) ||
      (c = cudaMemcpyAsync(e->two_da.p, one.data(), sizeof(double) * e->K, cudaMemcpyHostToDevice,
                           e->stream)) ||
      (c = cudaMemcpyAsync(e->c1x.p, one.data(), sizeof(double) * e->K, cudaMemcpyHostToDevice,
                           e->stream)) ||
      (c = cudaMemcpyAsync(e->active.p, act.data(), act.size(), cudaMemcpyHostToDevice,
                           e->stream)) ||
      (c = cudaMemsetAsync(e->v[0].p, 0, sizeof(double) * e->ntot * kE, e->stream)) ||
      (c = cudaMemsetAsync(e->v[1].p, 0, sizeof(double) * e->ntot * kE, e->stream)) ||
      (c = cudaMemsetAsync(e->v[3].p, 0, sizeof(double) * e->ntot * kE, e->stream)) ||
      (c = cudaMemsetAsync(e->f4[0].p, 0, sizeof(float4) * e->ntot * kR, e->stream)))
    return ecuda(e, c, "autotune tables");
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int cand[3] = {128, 256, 512};
  double best = 1e30;
  int best_t = 256;
  int rc = GGEM_OK;
  for (int t : cand) {
    e->block = t;
    rc = ens_term(e, 1, ldc, e->v[0].p, e->v[1].p, e->v[2].p, e->v[3].p, e->f4[0].p, e->f4[1].p);
    if (rc) break;
    cudaEventRecord(a, e->stream);
    for (int rep = 0; rep < 5 && !rc; ++rep)
      rc = ens_term(e, 1, ldc, e->v[0].p, e->v[1].p, e->v[2].p, e->v[3].p, e->f4[0].p,
                    e->f4[1].p);
    cudaEventRecord(b, e->stream);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms / 5 < best) {
      best = ms / 5;
      best_t = t;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  if (e->block != best_t) e->drop_graphs();
  e->block = best_t;
  e->drop_graphs();  // the captured graphs used the last candidate's launch shape
  *block_threads = best_t;
  *ms_per_term = best;
  return GGEM_OK;
}
