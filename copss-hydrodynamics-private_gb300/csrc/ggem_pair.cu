// ggem_pair.cu -- Kernel B: the local regularized-Stokeslet pair sums.
//
// u_i = sum_j G(r_ij) f_j + self term, with G the local regularized Green's
// tensor of GGEMStokes::green_tensor_local_regularized (ggem_stokes.C:304-357)
// summed as GGEMStokes::local_solution_bead (ggem_stokes.C:427-503) and the
// self term of PMSystemStokes::compute_point_velocity (pm_system_stokes.C:446-455).
//
// Two arithmetic paths:
//  * FP64 ("plain"): one thread per target slot sweeps the neighbour cells of
//    the stencil, minimum image and cut-off in FP64, erf/exp per pair.
//  * FP32: groups of kGroup lanes share one target and walk its cached CSR
//    pair list (consecutive entries, so the gathered sources of a group sit
//    in the same cells).  The displacement is formed from cell-relative
//    coordinates plus the stencil shift (exact cell offsets);
//    G = A(s) I + B(s) x x^T with A, B = e^{-alpha^2 s} times a polynomial
//    in s (or a cubic table when that fit is not accurate enough); each lane
//    keeps Kahan-compensated FP32 sums; the group reduces them as float-float
//    values in FP32 and forms one FP64 add per output component.
// Algorithmic work per in-cutoff ordered pair: 28 + 19*nrhs flops (FMA = 2,
// rsqrt/exp/erf = 1 each), bound by the FP32 pipe.
#include <cuda_runtime.h>

#include <algorithm>

#include "ggem_ff.cuh"
#include "ggem_internal.cuh"

namespace ggem {
namespace {

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

// green_tensor_local_regularized applied to f: G f = k[(c1+c2) f + (c1-c2)(x.f/r^2) x]
__device__ __forceinline__ void green_apply64(const DevConsts &K, const double x[3], double r,
                                              const double f[3], double out[3]) {
  if (r < K.r_eps) {
#pragma unroll
    for (int a = 0; a < 3; ++a) out[a] = K.coeff_2 * f[a];
    return;
  }
  const double r2 = r * r;
  const double kr = K.ksi * r, kr2 = kr * kr;
  const double ar = K.alpha * r, ar2 = ar * ar;
  const double c1 = (erf(kr) - erf(ar)) / r;
  const double c2 = K.two_ksi_sqrt_pi * exp(-kr2) - K.two_alpha_sqrt_pi * exp(-ar2);
  const double xf = (x[0] * f[0] + x[1] * f[1] + x[2] * f[2]) / r2;
  const double p = (c1 + c2) * K.one_eight_pi_mu, m = (c1 - c2) * xf * K.one_eight_pi_mu;
#pragma unroll
  for (int a = 0; a < 3; ++a) out[a] = p * f[a] + m * x[a];
}

__device__ __forceinline__ void self_term(const DevConsts &K, int self_mode, const double f[3],
                                          double u[3]) {
  if (self_mode == GGEM_SELF_BEAD) {
#pragma unroll
    for (int a = 0; a < 3; ++a) u[a] = (u[a] - K.coeff_1 * f[a]) + f[a];
  } else if (self_mode == GGEM_SELF_LAGRANGIAN) {
#pragma unroll
    for (int a = 0; a < 3; ++a) u[a] = u[a] + K.coeff_2 * f[a];
  }
}

// FP64 plain sweep.  own_first: reference mode (own cell, then the element
// stencil that excludes (0,0,0), no cut-off); otherwise the cut-off stencil.
template <int NR>
__global__ void __launch_bounds__(128) k_matvec_f64(int64_t n, Grid g, DevConsts K,
                                                    const int4 *__restrict__ stencil, int nst,
                                                    int own_first, int use_cutoff, double rc2,
                                                    const int32_t *__restrict__ start,
                                                    const double4_32a *__restrict__ pos64,
                                                    const float4 *__restrict__ pos32,
                                                    const double *__restrict__ f,
                                                    double *__restrict__ u, int self_mode,
                                                    int nrhs_total, int r0) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const double4_32a pi = pos64[s];
  const int32_t cid = __float_as_int(pos32[s].w);
  const int cx = cid % g.nc[0], cy = (cid / g.nc[0]) % g.nc[1], cz = cid / (g.nc[0] * g.nc[1]);
  double acc[NR][3];
#pragma unroll
  for (int r = 0; r < NR; ++r) acc[r][0] = acc[r][1] = acc[r][2] = 0.0;
  const int64_t vstride = 3 * n;
  for (int k = own_first ? -1 : 0; k < nst; ++k) {
    int4 o = (k < 0) ? make_int4(0, 0, 0, 0) : stencil[k];
    int c[3] = {cx + o.x, cy + o.y, cz + o.z};
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (c[d] < 0 || c[d] >= g.nc[d]) {
        if (!g.periodic[d]) ok = false;
        else c[d] = wrap_i(c[d], g.nc[d]);
      }
    }
    if (!ok) continue;
    const int32_t nc = c[0] + g.nc[0] * (c[1] + g.nc[1] * c[2]);
    const int32_t b = start[nc], e = start[nc + 1];
    for (int32_t t = b; t < e; ++t) {
      if (t == s) continue;
      const double4_32a pj = pos64[t];
      double x[3] = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z};
      min_image(g, x);
      if (use_cutoff) {
        const double r2c = __dadd_rn(__dadd_rn(__dmul_rn(x[0], x[0]), __dmul_rn(x[1], x[1])),
                                     __dmul_rn(x[2], x[2]));
        if (!(r2c < rc2)) continue;
      }
      const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
#pragma unroll
      for (int q = 0; q < NR; ++q) {
        const double *fj = f + (int64_t)(r0 + q) * vstride + 3 * (int64_t)t;
        const double fv[3] = {fj[0], fj[1], fj[2]};
        double g3[3];
        green_apply64(K, x, r, fv, g3);
        acc[q][0] += g3[0];
        acc[q][1] += g3[1];
        acc[q][2] += g3[2];
      }
    }
  }
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    const double *fi = f + (int64_t)(r0 + q) * vstride + 3 * s;
    const double fv[3] = {fi[0], fi[1], fi[2]};
    self_term(K, self_mode, fv, acc[q]);
    double *ui = u + (int64_t)(r0 + q) * vstride + 3 * s;
    ui[0] = acc[q][0];
    ui[1] = acc[q][1];
    ui[2] = acc[q][2];
  }
  (void)nrhs_total;
}

// FP64 pair sum over the exact pair list: only the in-cutoff pairs (the
// list is the oracle's), the oracle's arithmetic per pair (minimum image of
// the wrapped FP64 positions, pm_periodic_boundary.C:350-374, and
// green_tensor_local_regularized with erf and exp in FP64,
// ggem_stokes.C:304-357); the tensor's two coefficients are formed once per
// pair and applied to NR right-hand sides.  kGroup lanes per target take
// every kGroup-th entry of its row and add their sums by shuffles.
template <int NR>
__global__ void __launch_bounds__(256) k_pair_list_f64(int64_t n, Grid g, DevConsts K,
                                                       const int32_t *__restrict__ cnt, int W,
                                                       const uint32_t *__restrict__ list,
                                                       const double4_32a *__restrict__ pos64,
                                                       const double *__restrict__ f,
                                                       double *__restrict__ u, int self_mode,
                                                       int r0) {
  const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kGroup;
  const int sub = (int)(threadIdx.x % kGroup);
  const bool act = gid < n;
  const int64_t s = act ? gid : n - 1;
  const double4_32a pi = pos64[s];
  const int64_t vstride = 3 * n;
  double acc[NR][3];
#pragma unroll
  for (int q = 0; q < NR; ++q) acc[q][0] = acc[q][1] = acc[q][2] = 0.0;
  const int m = act ? cnt[s] : 0;
  const uint32_t *row = list + s * (int64_t)W;
  for (int k = sub; k < m; k += kGroup) {
    const int64_t t = (int64_t)(__ldg(row + k) >> kCodeBits);
    const double4_32a pj = pos64[t];
    double x[3] = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z};
    min_image(g, x);
    const double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
    const double r = sqrt(r2);
    if (r < K.r_eps) {
#pragma unroll
      for (int q = 0; q < NR; ++q) {
        const double *fj = f + (int64_t)(r0 + q) * vstride + 3 * t;
        acc[q][0] += K.coeff_2 * fj[0];
        acc[q][1] += K.coeff_2 * fj[1];
        acc[q][2] += K.coeff_2 * fj[2];
      }
      continue;
    }
    const double kr = K.ksi * r, ar = K.alpha * r;
    const double c1 = (erf(kr) - erf(ar)) / r;
    const double c2 = K.two_ksi_sqrt_pi * exp(-kr * kr) - K.two_alpha_sqrt_pi * exp(-ar * ar);
    const double p = (c1 + c2) * K.one_eight_pi_mu, mc = (c1 - c2) * K.one_eight_pi_mu / r2;
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      const double *fj = f + (int64_t)(r0 + q) * vstride + 3 * t;
      const double f0 = fj[0], f1 = fj[1], f2 = fj[2];
      const double xf = (x[0] * f0 + x[1] * f1 + x[2] * f2) * mc;
      acc[q][0] += p * f0 + xf * x[0];
      acc[q][1] += p * f1 + xf * x[1];
      acc[q][2] += p * f2 + xf * x[2];
    }
  }
#pragma unroll
  for (int o = 1; o < kGroup; o <<= 1)
#pragma unroll
    for (int q = 0; q < NR; ++q)
#pragma unroll
      for (int a = 0; a < 3; ++a) acc[q][a] += __shfl_xor_sync(0xffffffffu, acc[q][a], o);
  if (!act || sub != 0) return;
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    const double *fi = f + (int64_t)(r0 + q) * vstride + 3 * s;
    const double fv[3] = {fi[0], fi[1], fi[2]};
    self_term(K, self_mode, fv, acc[q]);
    double *ui = u + (int64_t)(r0 + q) * vstride + 3 * s;
    ui[0] = acc[q][0];
    ui[1] = acc[q][1];
    ui[2] = acc[q][2];
  }
}

__device__ __forceinline__ void kahan_add(float &sum, float &comp, float v) {
  const float y = v - comp;
  const float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

// one 32-byte record per source (cell-relative position, force of the single
// right-hand side): a single 32-byte gather per pair
struct __align__(32) Rec32 {
  float4 a, b;
};

// the analytic tensor, passed by value (constant bank)
// (a_q, b_q) interleaved so that both polynomials advance in one packed
// FP32x2 FMA per degree (Blackwell FFMA2)
struct PolyAB {
  float2 ab[kPolyDeg + 1];
  float x0, x1, e_hi, e_lo;  // x = s x1 + x0; e^{-alpha^2 s} = 2^{s (e_hi + e_lo)}
};

template <bool POLY>
__device__ __forceinline__ void tensor_ab32(float s2, const PolyAB &P,
                                            const Rec32 *__restrict__ tab, float inv_ds,
                                            float &A, float &B) {
  if (POLY) {
    const float x = fmaf(s2, P.x1, P.x0);
    const float2 xx = make_float2(x, x);
    float2 ab = P.ab[kPolyDeg];
#pragma unroll
    for (int q = kPolyDeg - 1; q >= 0; --q) ab = __ffma2_rn(ab, xx, P.ab[q]);
    // e^{-alpha^2 s} = 2^{p + r}: p = s e_hi rounded, r its exact residual plus
    // s e_lo, so the exponent keeps ~1e-7 relative accuracy at s ~ rc^2
    const float p = s2 * P.e_hi;
    const float r = fmaf(s2, P.e_lo, fmaf(s2, P.e_hi, -p));
    const float E0 = exp2f(p);
    const float E = fmaf(E0, r * 0.6931471805599453f, E0);
    ab = __fmul2_rn(ab, make_float2(E, E));
    A = ab.x;
    B = ab.y;
  } else {
    const float uu = s2 * inv_ds;
    const float fi = fminf(floorf(uu), (float)(kTableN - 1));  // last piece extrapolates
    const float t = uu - fi;
    const Rec32 tr = tab[(int)fi];
    A = fmaf(fmaf(fmaf(tr.a.w, t, tr.a.z), t, tr.a.y), t, tr.a.x);
    B = fmaf(fmaf(fmaf(tr.b.w, t, tr.b.z), t, tr.b.y), t, tr.b.x);
  }
}

template <int CD>
__device__ __forceinline__ void decode_shift(uint32_t e, float hx, float hy, float hz, float &sx,
                                             float &sy, float &sz) {
  constexpr int SIDE = 2 * CD + 1;
  const int code = (int)(e & (kMaxCode - 1));
  sx = (float)(code % SIDE - CD) * hx;
  sy = (float)((code / SIDE) % SIDE - CD) * hy;
  sz = (float)(code / (SIDE * SIDE) - CD) * hz;
}

__device__ __forceinline__ void group_ff(float &hi, float &lo) {
#pragma unroll
  for (int o = kGroup / 2; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
    const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
    ff_add(hi, lo, h2, l2);
  }
}

// lanes sub = 0, 1, 2 of a group write component sub of the target:
// u = (hi + lo) + self_c f with the FP64 force of the target
__device__ __forceinline__ void group_store(bool act, int sub, int64_t s, float hx, float lx,
                                            float hy, float ly, float hz, float lz,
                                            double self_c, const double *__restrict__ f,
                                            double *__restrict__ u) {
  if (!act || sub >= 3) return;
  const float h = sub == 0 ? hx : (sub == 1 ? hy : hz);
  const float l = sub == 0 ? lx : (sub == 1 ? ly : lz);
  const double v = f2d_bits(h) + f2d_bits(l);
  u[3 * s + sub] = fma(self_c, f[3 * s + sub], v);
}

__global__ void k_build_src(int64_t n, const float4 *__restrict__ pos32,
                            const double *__restrict__ f, Rec32 *__restrict__ src) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  Rec32 r;
  r.a = pos32[s];
  r.b = make_float4(d2f_bits(f[3 * s]), d2f_bits(f[3 * s + 1]), d2f_bits(f[3 * s + 2]), 0.f);
  src[s] = r;
}

// float-float sum of one target's pair terms
struct PairSum {
  float hx, lx, hy, ly, hz, lz;
};

// 2^x on the special-function unit (PTX ex2.approx.ftz.f32); the argument
// range of the tensor, [-alpha^2 rc^2 log2(e), 0], keeps results normal
__device__ __forceinline__ float ex2_sfu(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// one 32-byte record in a single 256-bit read-only load (sm_100+): the
// position and the force of a source share one sector, so one request per
// warp touches each sector once instead of twice
__device__ __forceinline__ Rec32 ld_rec32(const Rec32 *p) {
  Rec32 r;
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(r.a.x), "=f"(r.a.y), "=f"(r.a.z), "=f"(r.a.w), "=f"(r.b.x), "=f"(r.b.y),
        "=f"(r.b.z), "=f"(r.b.w)
      : "l"(p));
  return r;
}

// the FP32 cell shift of every entry code, staged per block in shared
// memory (one 16-byte load per pair instead of decoding the code); the
// table holds (float)(k h) for offsets |k| <= 2, which equals the FP32
// product k * (float)h that the list build and decode_shift use
__device__ __forceinline__ void stage_shifts(float4 *sh, const float4 *__restrict__ shift) {
  for (int k = threadIdx.x; k < kMaxCode; k += blockDim.x) sh[k] = shift[k];
  __syncthreads();
}

// The series kernels may be launched as programmatic dependents of the
// kernel before them (PTX griddepcontrol): their blocks can start while
// that kernel's last blocks finish, stage the constant shift table, and
// wait here until its results are complete and visible.  Without such a
// launch the wait returns at once.
__device__ __forceinline__ void wait_prior_grid() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// reduce-scatter of the group's float-float sums: afterwards lane sub
// (0, 1, 2) holds component sub of the target's total, summed in the same
// tree as the all-reduce ((lane 0 + lane 2) + (lane 1 + lane 3))
__device__ __forceinline__ void group_scatter3(int sub, const PairSum &r, float &h, float &l) {
  const bool up = sub & 2;
  // lanes 0, 1 keep (x, y) and send z; lanes 2, 3 keep z and send (x, y)
  float k1h = up ? r.hz : r.hx, k1l = up ? r.lz : r.lx;
  float k2h = up ? 0.f : r.hy, k2l = up ? 0.f : r.ly;
  const float s1h = up ? r.hx : r.hz, s1l = up ? r.lx : r.lz;
  const float s2h = up ? r.hy : 0.f, s2l = up ? r.ly : 0.f;
  const float a1h = __shfl_xor_sync(0xffffffffu, s1h, 2), a1l = __shfl_xor_sync(0xffffffffu, s1l, 2);
  const float a2h = __shfl_xor_sync(0xffffffffu, s2h, 2), a2l = __shfl_xor_sync(0xffffffffu, s2l, 2);
  ff_add(k1h, k1l, a1h, a1l);
  ff_add(k2h, k2l, a2h, a2l);
  // lane 0 keeps x, lane 1 keeps y, lane 2 keeps z (lane 3: zero)
  const bool odd = sub & 1;
  h = odd ? k2h : k1h;
  l = odd ? k2l : k1l;
  const float th = odd ? k1h : k2h, tl = odd ? k1l : k2l;
  const float bh = __shfl_xor_sync(0xffffffffu, th, 1), bl = __shfl_xor_sync(0xffffffffu, tl, 1);
  ff_add(h, l, bh, bl);
}

// the pair loop of one target slot s over its list entries (one right-hand
// side, 32-byte source records); lanes sub = 0..kGroup-1 take every
// kGroup-th entry, so a group reads consecutive list words.  The next entry
// of the lane is loaded while the current pair is evaluated.  (Prefetching
// the next source record into registers or L1 as well measured no faster.)
template <bool POLY>
__device__ __forceinline__ PairSum pair_sum_r1(int64_t s, bool act, int sub, const Rec32 &ri,
                                               const Rec32 *__restrict__ src,
                                               const int32_t *__restrict__ cnt, int W,
                                               const uint32_t *__restrict__ list,
                                               const PolyAB &P, const Rec32 *__restrict__ tab,
                                               float inv_ds, const float4 *sh) {
  const uint32_t *lp = list + s * (int64_t)W + sub;
  int left = (act ? cnt[s] : 0) - sub;  // entries lp[0], lp[kGroup], ... while left > 0
  float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  float2 bxy = make_float2(0.f, 0.f);
  float bz = 0.f;
  int blk = 0;
  uint32_t nxt = left > 0 ? __ldg(lp) : 0u;
  while (left > 0) {
    const uint32_t en = nxt;
    left -= kGroup;
    lp += kGroup;
    if (left > 0) nxt = __ldg(lp);
    const Rec32 rj = ld_rec32(src + (en >> kCodeBits));
    const float4 o = sh[en & (kMaxCode - 1)];
    const float dx = (rj.a.x - ri.a.x) + o.x;
    const float dy = (rj.a.y - ri.a.y) + o.y;
    const float dz = (rj.a.z - ri.a.z) + o.z;
    const float s2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    float A, B;
    if (POLY) {
      const float x = fmaf(s2, P.x1, P.x0);
      const float2 xx = make_float2(x, x);
      float2 ab = P.ab[kPolyDeg];
#pragma unroll
      for (int q = kPolyDeg - 1; q >= 0; --q) ab = __ffma2_rn(ab, xx, P.ab[q]);
      // e^{-alpha^2 s} = 2^{p + r}, p = s e_hi rounded, r its residual plus s e_lo
      const float p = s2 * P.e_hi;
      const float r = fmaf(s2, P.e_lo, fmaf(s2, P.e_hi, -p));
      const float E0 = ex2_sfu(p);
      const float E = fmaf(E0, r * 0.6931471805599453f, E0);
      ab = __fmul2_rn(ab, make_float2(E, E));
      A = ab.x;
      B = ab.y;
    } else {
      tensor_ab32<false>(s2, P, tab, inv_ds, A, B);
    }
    // G f = A f + B (x.f) x, the x and y components packed (FFMA2)
    const float2 dxy = make_float2(dx, dy), fxy = make_float2(rj.b.x, rj.b.y);
    const float2 pxy = __fmul2_rn(dxy, fxy);
    const float bxf = B * fmaf(dz, rj.b.z, pxy.x + pxy.y);
    bxy = __fadd2_rn(bxy, __ffma2_rn(make_float2(A, A), fxy,
                                     __fmul2_rn(make_float2(bxf, bxf), dxy)));
    bz += fmaf(A, rj.b.z, bxf * dz);
    if (++blk == 8) {
      kahan_add(sx, cx, bxy.x);
      kahan_add(sy, cy, bxy.y);
      kahan_add(sz, cz, bz);
      bxy = make_float2(0.f, 0.f);
      bz = 0.f;
      blk = 0;
    }
  }
  kahan_add(sx, cx, bxy.x);
  kahan_add(sy, cy, bxy.y);
  kahan_add(sz, cz, bz);
  // Kahan keeps sum = s - c: the float-float value is (s, -c)
  return PairSum{sx, -cx, sy, -cy, sz, -cz};
}

// The fused series' estimator sums (x0 . M x0, |dw|^2, |x_{k+1}|^2, |M dw|^2)
// without FP64 arithmetic (ggem_ff.cuh): float-float products and sums, one
// partial per block (256 threads) written by thread 0.
__device__ __forceinline__ void block_partial_ff(float hi, float lo, double *__restrict__ part) {
  __shared__ float2 sh[32];
  const double v = block_ff_sum(hi, lo, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = v;
}

// ---- symmetric pair sums --------------------------------------------------
// The tensor of a pair is symmetric (G(x) = G(-x)), so each unordered pair is
// evaluated once, from the half list (the row of the smaller slot): the
// target side A f_j + B (x.f_j) x is summed in registers as in pair_sum_r1,
// the source side A f_i + B (x.f_i) x goes to the source's accumulator with
// one 16-byte vector atomic (red.global.add.v4.f32).  The order in which a
// source's contributions arrive varies from run to run, so the FP32 result
// is not bit-reproducible (the FP64 paths and the full-row kernels are).
__device__ __forceinline__ void red_add_v4(float4 *p, float x, float y, float z) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(x), "f"(y),
               "f"(z), "f"(0.f)
               : "memory");
}

template <bool POLY>
__device__ __forceinline__ PairSum pair_sum_sym(int64_t s, bool act, int sub, const Rec32 &ri,
                                                const Rec32 *__restrict__ src,
                                                const int32_t *__restrict__ cnt, int W,
                                                const uint32_t *__restrict__ list,
                                                const PolyAB &P, const Rec32 *__restrict__ tab,
                                                float inv_ds, const float4 *sh,
                                                float4 *__restrict__ acc) {
  const uint32_t *lp = list + s * (int64_t)W + sub;
  int left = (act ? cnt[s] : 0) - sub;
  float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  float2 bxy = make_float2(0.f, 0.f);
  float bz = 0.f;
  int blk = 0;
  const float2 fixy = make_float2(ri.b.x, ri.b.y);
  uint32_t nxt = left > 0 ? __ldg(lp) : 0u;
  while (left > 0) {
    const uint32_t en = nxt;
    left -= kGroup;
    lp += kGroup;
    if (left > 0) nxt = __ldg(lp);
    const uint32_t j = en >> kCodeBits;
    const Rec32 rj = ld_rec32(src + j);
    const float4 o = sh[en & (kMaxCode - 1)];
    const float dx = (rj.a.x - ri.a.x) + o.x;
    const float dy = (rj.a.y - ri.a.y) + o.y;
    const float dz = (rj.a.z - ri.a.z) + o.z;
    const float s2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    float A, B;
    if (POLY) {
      const float x = fmaf(s2, P.x1, P.x0);
      const float2 xx = make_float2(x, x);
      float2 ab = P.ab[kPolyDeg];
#pragma unroll
      for (int q = kPolyDeg - 1; q >= 0; --q) ab = __ffma2_rn(ab, xx, P.ab[q]);
      const float p = s2 * P.e_hi;
      const float r = fmaf(s2, P.e_lo, fmaf(s2, P.e_hi, -p));
      const float E0 = ex2_sfu(p);
      const float E = fmaf(E0, r * 0.6931471805599453f, E0);
      ab = __fmul2_rn(ab, make_float2(E, E));
      A = ab.x;
      B = ab.y;
    } else {
      tensor_ab32<false>(s2, P, tab, inv_ds, A, B);
    }
    const float2 dxy = make_float2(dx, dy);
    // target side: G f_j
    const float2 fxy = make_float2(rj.b.x, rj.b.y);
    const float2 pxy = __fmul2_rn(dxy, fxy);
    const float bxf = B * fmaf(dz, rj.b.z, pxy.x + pxy.y);
    bxy = __fadd2_rn(bxy, __ffma2_rn(make_float2(A, A), fxy,
                                     __fmul2_rn(make_float2(bxf, bxf), dxy)));
    bz += fmaf(A, rj.b.z, bxf * dz);
    // source side: G f_i into the source's accumulator
    const float2 qxy = __fmul2_rn(dxy, fixy);
    const float bxi = B * fmaf(dz, ri.b.z, qxy.x + qxy.y);
    const float2 vxy = __ffma2_rn(make_float2(A, A), fixy, __fmul2_rn(make_float2(bxi, bxi), dxy));
    red_add_v4(acc + j, vxy.x, vxy.y, fmaf(A, ri.b.z, bxi * dz));
    if (++blk == 8) {
      kahan_add(sx, cx, bxy.x);
      kahan_add(sy, cy, bxy.y);
      kahan_add(sz, cz, bz);
      bxy = make_float2(0.f, 0.f);
      bz = 0.f;
      blk = 0;
    }
  }
  kahan_add(sx, cx, bxy.x);
  kahan_add(sy, cy, bxy.y);
  kahan_add(sz, cz, bz);
  return PairSum{sx, -cx, sy, -cy, sz, -cz};
}

// the target sides of the half rows: part[3 s + c] (FP64 of the group's
// float-float sum); the source sides accumulate in acc
template <bool POLY>
__global__ void __launch_bounds__(256, 6) k_pair_sym(
    int64_t n, const Rec32 *__restrict__ src, const int32_t *__restrict__ cnt, int W,
    const uint32_t *__restrict__ list, PolyAB P, const Rec32 *__restrict__ tab, float inv_ds,
    const float4 *__restrict__ shift, float4 *__restrict__ acc, double *__restrict__ part) {
  __shared__ float4 sh[kMaxCode];
  stage_shifts(sh, shift);
  const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kGroup;
  const int sub = (int)(threadIdx.x % kGroup);
  const bool act = gid < n;
  const int64_t s = act ? gid : n - 1;
  const Rec32 ri = src[s];
  const PairSum r = pair_sum_sym<POLY>(s, act, sub, ri, src, cnt, W, list, P, tab, inv_ds, sh,
                                       acc);
  float h, l;
  group_scatter3(sub, r, h, l);
  if (act && sub < 3) part[3 * s + sub] = f2d_bits(h) + f2d_bits(l);
}

// u = part + acc + self term; acc is cleared for the next use
__global__ void k_sym_finish(int64_t n, const double *__restrict__ part, float4 *__restrict__ acc,
                             double self_c, const double *__restrict__ f, double *__restrict__ u) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const float4 a = acc[s];
  acc[s] = make_float4(0.f, 0.f, 0.f, 0.f);
  const float v[3] = {a.x, a.y, a.z};
#pragma unroll
  for (int c = 0; c < 3; ++c)
    u[3 * s + c] = fma(self_c, f[3 * s + c], part[3 * s + c] + f2d_bits(v[c]));
}

// the per-matvec-tensor kernel shapes the autotuner chooses from: blocks of
// 256 threads per SM that the register cap allows (6 at 40 registers, with a
// few spilled epilogue values in some kernels; 5 at 48 without)
constexpr int kComputedMinBlocks[] = {6, 5};
constexpr int kNumComputedVariants = 2;

// u = M f, single right-hand side; with ORIG, u is written in the caller's
// particle order (u[order[s]]) instead of slot order
template <bool POLY, int V, bool ORIG>
__global__ void __launch_bounds__(256, kComputedMinBlocks[V]) k_pair_r1(
    int64_t n, const Rec32 *__restrict__ src, const int32_t *__restrict__ cnt, int W,
    const uint32_t *__restrict__ list, PolyAB P, const Rec32 *__restrict__ tab, float inv_ds,
    const float4 *__restrict__ shift, double self_c, const double *__restrict__ f,
    double *__restrict__ u, const int32_t *__restrict__ order, double *__restrict__ part) {
  __shared__ float4 sh[kMaxCode];
  stage_shifts(sh, shift);
  wait_prior_grid();
  const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kGroup;
  const int sub = (int)(threadIdx.x % kGroup);
  const bool act = gid < n;
  const int64_t s = act ? gid : n - 1;
  const Rec32 ri = src[s];
  const PairSum r = pair_sum_r1<POLY>(s, act, sub, ri, src, cnt, W, list, P, tab, inv_ds, sh);
  float h, l;
  group_scatter3(sub, r, h, l);
  float qh = 0.f, ql = 0.f;
  if (act && sub < 3) {
    const int64_t k = 3 * s + sub;
    const double v = fma(self_c, f[k], f2d_bits(h) + f2d_bits(l));
    if (ORIG) u[3 * (int64_t)order[s] + sub] = v;
    else u[k] = v;
    if (part) sq_ff(v, qh, ql);
  }
  if (part) block_partial_ff(qh, ql, part);  // |u|^2 (uniform branch)
}

// The first Chebyshev step in one pass (brownian_system.C:1036-1056 for one
// right-hand side): m = M x0 (src holds the records of x0, m is kept for
// the dot xi . M xi), x1 = db x0 + da m, dw = c0 x0 + c1 x1, and the 32-byte
// records of x1 for the first term.  (The estimator sums stay in separate
// vector kernels: a block-wide FP64 reduction here costs more than the
// launch it saves, FP64 being 1/64 of the FP32 rate.)
template <bool POLY, int V>
__global__ void __launch_bounds__(256, kComputedMinBlocks[V]) k_pair_first(
    int64_t n, const Rec32 *__restrict__ src, const int32_t *__restrict__ cnt, int W,
    const uint32_t *__restrict__ list, PolyAB P, const Rec32 *__restrict__ tab, float inv_ds,
    const float4 *__restrict__ shift, double self_c, double da, double db, double c0, double c1,
    const double *__restrict__ x0, double *__restrict__ m, double *__restrict__ x1,
    double *__restrict__ dw, Rec32 *__restrict__ next, double *__restrict__ part) {
  __shared__ float4 sh[kMaxCode];
  stage_shifts(sh, shift);
  wait_prior_grid();
  const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kGroup;
  const int sub = (int)(threadIdx.x % kGroup);
  const bool act = gid < n;
  const int64_t s = act ? gid : n - 1;
  const Rec32 ri = src[s];
  const PairSum r = pair_sum_r1<POLY>(s, act, sub, ri, src, cnt, W, list, P, tab, inv_ds, sh);
  float h, l;
  group_scatter3(sub, r, h, l);
  float qh = 0.f, ql = 0.f;
  if (act) {
    float *nf = reinterpret_cast<float *>(next + s);
    if (sub < 3) {
      const int64_t k = 3 * s + sub;
      const double xk = x0[k];
      const double mk = fma(self_c, xk, f2d_bits(h) + f2d_bits(l));
      m[k] = mk;
      const double x1k = db * xk + da * mk;
      x1[k] = x1k;
      dw[k] = c0 * xk + c1 * x1k;
      nf[4 + sub] = d2f_bits(x1k);
      if (part) dot_ff(xk, mk, qh, ql);
    } else {
      reinterpret_cast<float4 *>(nf)[0] = ri.a;
      nf[7] = 0.f;
    }
  }
  if (part) block_partial_ff(qh, ql, part);  // x0 . M x0 (aux2; uniform branch)
}

// One Chebyshev term with the pair sum (brownian_system.C:1091-1108 for one
// right-hand side, without the norms of the error estimators):
//   m = M x1 (pair sum + self term),  xm = (2db x1 + 2da m) - x0,
//   dw += coef xm,  and the 32-byte records of xm for the next term.
// With c1 = 2db + 2da self_c this is xm = 2da (pair sum) + (c1 x1 - x0).
// src holds the records of x1; next must be a different buffer.
template <bool POLY, int V, bool NORMS>
__global__ void __launch_bounds__(256, kComputedMinBlocks[V]) k_pair_cheb(
    int64_t n, const Rec32 *__restrict__ src, const int32_t *__restrict__ cnt, int W,
    const uint32_t *__restrict__ list, PolyAB P, const Rec32 *__restrict__ tab, float inv_ds,
    const float4 *__restrict__ shift, double two_da, double c1, double coef,
    const double *__restrict__ x0, const double *__restrict__ x1, double *__restrict__ xm,
    double *__restrict__ dw, Rec32 *__restrict__ next, double *__restrict__ part,
    int64_t nw, Rec32 *__restrict__ dw_next) {
  __shared__ float4 sh[kMaxCode];
  stage_shifts(sh, shift);
  wait_prior_grid();
  const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kGroup;
  const int sub = (int)(threadIdx.x % kGroup);
  const bool act = gid < n;
  const int64_t s = act ? gid : n - 1;
  const Rec32 ri = src[s];
  const PairSum r = pair_sum_r1<POLY>(s, act, sub, ri, src, cnt, W, list, P, tab, inv_ds, sh);
  float h, l;
  group_scatter3(sub, r, h, l);
  float q0h = 0.f, q0l = 0.f, q1h = 0.f, q1l = 0.f;
  if (act) {
    float *nf = reinterpret_cast<float *>(next + s);
    float *df = reinterpret_cast<float *>(dw_next + s);
    if (sub < 3) {
      const int64_t k = 3 * s + sub;
      const double v = fma(two_da, f2d_bits(h) + f2d_bits(l), fma(c1, x1[k], -x0[k]));
      xm[k] = v;
      const double y = dw[k];
      const double yn = fma(coef, v, y);
      dw[k] = yn;
      nf[4 + sub] = d2f_bits(v);
      if (NORMS) {
        sq_ff(y, q0h, q0l);  // |dw|^2 before the term
        sq_ff(v, q1h, q1l);  // |x_{k+1}|^2
        df[4 + sub] = d2f_bits(yn);
      }
    } else {
      reinterpret_cast<float4 *>(nf)[0] = ri.a;  // the target's position record
      nf[7] = 0.f;
      if (NORMS) {
        reinterpret_cast<float4 *>(df)[0] = ri.a;
        df[7] = 0.f;
      }
    }
  }
  if (NORMS) {  // the estimators' two norms (the records of dw are written)
    block_partial_ff(q0h, q0l, part);
    __syncthreads();  // the shared partials are reused
    block_partial_ff(q1h, q1l, part + nw);
  }
}

// xi (caller order) into slot order and the 32-byte records of it
__global__ void k_to_slots_rec(int64_t n, const int32_t *__restrict__ order,
                               const float4 *__restrict__ pos32, const double *__restrict__ xi,
                               double *__restrict__ x0, Rec32 *__restrict__ rec) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int64_t i = order[s];
  const double a = xi[3 * i], b = xi[3 * i + 1], c = xi[3 * i + 2];
  x0[3 * s] = a;
  x0[3 * s + 1] = b;
  x0[3 * s + 2] = c;
  Rec32 r;
  r.a = pos32[s];
  r.b = make_float4((float)a, (float)b, (float)c, 0.f);
  rec[s] = r;
}

// ---- precomputed pair tensors ---------------------------------------------
//
// Once per configuration (after the list build), every listed pair's tensor
// is stored as t = (A, sqrt(B) x) in the list's row layout, valid when
// B >= 0 on [0, rc^2] (checked at context creation).  A matvec then streams
// 20 B per pair (entry + tensor, evict-first) and gathers a 16-byte force:
// G f = A f + (x~ . f) x~ with x~ = sqrt(B) x, no position gathers and no
// polynomial per pair and matvec.
template <int CD, bool POLY>
__global__ void __launch_bounds__(256) k_pair_tensor(
    int64_t n, const float4 *__restrict__ pos32, const int32_t *__restrict__ cnt, int W,
    const uint32_t *__restrict__ list, PolyAB P, const Rec32 *__restrict__ tab, float inv_ds,
    float hx, float hy, float hz, float4 *__restrict__ ten) {
  const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kGroup;
  const int sub = (int)(threadIdx.x % kGroup);
  if (gid >= n) return;
  const int64_t s = gid;
  const float4 pi = pos32[s];
  const int64_t b = s * (int64_t)W, e = b + cnt[s];
  for (int64_t m = b + sub; m < e; m += 2 * kGroup) {
    const bool two = m + kGroup < e;
    const uint32_t en0 = __ldg(list + m), en1 = two ? __ldg(list + m + kGroup) : en0;
    const float4 pj0 = __ldg(pos32 + (en0 >> kCodeBits)), pj1 = __ldg(pos32 + (en1 >> kCodeBits));
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q == 1 && !two) break;
      const uint32_t en = q ? en1 : en0;
      const float4 pj = q ? pj1 : pj0;
      float ox, oy, oz;
      decode_shift<CD>(en, hx, hy, hz, ox, oy, oz);
      const float dx = (pj.x - pi.x) + ox, dy = (pj.y - pi.y) + oy, dz = (pj.z - pi.z) + oz;
      const float s2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
      float A, B;
      tensor_ab32<POLY>(s2, P, tab, inv_ds, A, B);
      const float w = sqrtf(fmaxf(B, 0.f));
      __stcs(ten + m + q * kGroup, make_float4(A, w * dx, w * dy, w * dz));
    }
  }
}

// forces of one right-hand side as one float4 per slot (w = 0)
__global__ void k_stage_f4(int64_t n, const double *__restrict__ f, float4 *__restrict__ f4) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  f4[s] = make_float4(d2f_bits(f[3 * s]), d2f_bits(f[3 * s + 1]), d2f_bits(f[3 * s + 2]), 0.f);
}

// float-float sum over the G lanes of a target's group
template <int G>
__device__ __forceinline__ void group_ff_g(float &hi, float &lo) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
    const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
    ff_add(hi, lo, h2, l2);
  }
}

// blk += G f over one entry: A f + (x~ . f) x~, x and y packed (FFMA2)
__device__ __forceinline__ void tensor_apply(const float4 &t, const float4 &fj, float2 &bxy,
                                             float &bz) {
  const float2 txy = make_float2(t.y, t.z), fxy = make_float2(fj.x, fj.y);
  const float2 p = __fmul2_rn(txy, fxy);
  const float d = fmaf(t.w, fj.z, p.x + p.y);
  bxy = __fadd2_rn(bxy, __ffma2_rn(make_float2(t.x, t.x), fxy, __fmul2_rn(make_float2(d, d), txy)));
  bz += fmaf(t.x, fj.z, d * t.w);
}

// The pair loop over stored tensors for one target slot s (cf. pair_sum_r1):
// G lanes share the target and take every G-th entry, U entries per lane and
// iteration are loaded before any is used (an entry past the row end reads a
// zero tensor and adds exactly zero).  PIPE: the streamed entries and tensors
// of the next iteration are requested before the current iteration's force
// gathers are used, so that the HBM latency of the stream overlaps the L2
// latency of the gathers.  Variants are picked by ggem_autotune_pair_storage.
template <int G, int U, bool PIPE>
__device__ __forceinline__ PairSum pair_sum_tv(int64_t s, bool act, int sub,
                                               const float4 *__restrict__ f4,
                                               const int32_t *__restrict__ cnt, int W,
                                               const uint32_t *__restrict__ list,
                                               const float4 *__restrict__ ten) {
  constexpr int FLUSH = (8 + U - 1) / U;  // iterations per Kahan flush (~8 entries)
  const int64_t b = s * (int64_t)W, e = act ? b + cnt[s] : b;
  float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  float2 bxy = make_float2(0.f, 0.f);
  float bz = 0.f;
  int blk = 0;
  uint32_t en[U];
  float4 t[U];
  int64_t m = b + sub;
  if (PIPE) {
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int64_t mq = m + q * G;
      const bool ok = mq < e;
      en[q] = ok ? __ldcs(list + mq) : 0u;
      t[q] = ok ? __ldcs(ten + mq) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  for (; m < e; m += U * G) {
    if (!PIPE) {
#pragma unroll
      for (int q = 0; q < U; ++q) {
        const int64_t mq = m + q * G;
        const bool ok = mq < e;
        en[q] = ok ? __ldcs(list + mq) : 0u;
        t[q] = ok ? __ldcs(ten + mq) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    float4 fj[U];
#pragma unroll
    for (int q = 0; q < U; ++q) fj[q] = __ldg(f4 + (en[q] >> kCodeBits));
    float4 tc[U];
#pragma unroll
    for (int q = 0; q < U; ++q) tc[q] = t[q];
    if (PIPE) {
#pragma unroll
      for (int q = 0; q < U; ++q) {
        const int64_t mq = m + U * G + q * G;
        const bool ok = mq < e;
        en[q] = ok ? __ldcs(list + mq) : 0u;
        t[q] = ok ? __ldcs(ten + mq) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
#pragma unroll
    for (int q = 0; q < U; ++q) tensor_apply(tc[q], fj[q], bxy, bz);
    if (++blk == FLUSH) {
      kahan_add(sx, cx, bxy.x);
      kahan_add(sy, cy, bxy.y);
      kahan_add(sz, cz, bz);
      bxy = make_float2(0.f, 0.f);
      bz = 0.f;
      blk = 0;
    }
  }
  kahan_add(sx, cx, bxy.x);
  kahan_add(sy, cy, bxy.y);
  kahan_add(sz, cz, bz);
  PairSum r{sx, -cx, sy, -cy, sz, -cz};
  group_ff_g<G>(r.hx, r.lx);
  group_ff_g<G>(r.hy, r.ly);
  group_ff_g<G>(r.hz, r.lz);
  return r;
}

// u = M f from stored tensors, single right-hand side
template <int G, int U, bool PIPE>
__global__ void __launch_bounds__(256) k_pair_r1tv(int64_t n, const float4 *__restrict__ f4,
                                                   const int32_t *__restrict__ cnt, int W,
                                                   const uint32_t *__restrict__ list,
                                                   const float4 *__restrict__ ten, double self_c,
                                                   const double *__restrict__ f,
                                                   double *__restrict__ u) {
  const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int sub = (int)(threadIdx.x % G);
  const bool act = gid < n;
  const int64_t s = act ? gid : n - 1;
  const PairSum r = pair_sum_tv<G, U, PIPE>(s, act, sub, f4, cnt, W, list, ten);
  group_store(act, sub, s, r.hx, r.lx, r.hy, r.ly, r.hz, r.lz, self_c, f, u);
}

// one Chebyshev term from stored tensors (cf. k_pair_cheb); f4 holds the
// FP32 forces of x1, next receives those of xm
template <int G, int U, bool PIPE>
__global__ void __launch_bounds__(256) k_pair_cheb_tv(
    int64_t n, const float4 *__restrict__ f4, const int32_t *__restrict__ cnt, int W,
    const uint32_t *__restrict__ list, const float4 *__restrict__ ten, double self_c,
    double two_da, double two_db, double coef, const double *__restrict__ x0,
    const double *__restrict__ x1, double *__restrict__ xm, double *__restrict__ dw,
    float4 *__restrict__ next) {
  const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int sub = (int)(threadIdx.x % G);
  const bool act = gid < n;
  const int64_t s = act ? gid : n - 1;
  const PairSum r = pair_sum_tv<G, U, PIPE>(s, act, sub, f4, cnt, W, list, ten);
  if (!act) return;
  float *nf = reinterpret_cast<float *>(next + s);
  if (sub < 3) {
    const float h = sub == 0 ? r.hx : (sub == 1 ? r.hy : r.hz);
    const float l = sub == 0 ? r.lx : (sub == 1 ? r.ly : r.lz);
    const int64_t k = 3 * s + sub;
    const double xk = x1[k];
    const double m = fma(self_c, xk, f2d_bits(h) + f2d_bits(l));
    double v = two_db * xk + two_da * m;
    v -= x0[k];
    xm[k] = v;
    dw[k] = dw[k] + coef * v;
    nf[sub] = d2f_bits(v);
  } else if (sub == 3) {
    nf[3] = 0.f;
  }
}

// the stored-tensor variants the autotuner chooses from: lanes per target,
// entries in flight per lane, pipelined stream
struct StoredVariant {
  int G, U;
  bool pipe;
};
constexpr StoredVariant kStoredVariants[] = {{4, 4, false}, {4, 2, true}, {8, 2, true}, {8, 4, false}};
constexpr int kNumStoredVariants = 4;

template <int V>
void launch_stored_r1(ggem_ctx *c, const float4 *f4, double self_c, const double *f, double *u) {
  constexpr StoredVariant sv = kStoredVariants[V];
  const int64_t threads = c->n * sv.G;
  k_pair_r1tv<sv.G, sv.U, sv.pipe><<<(unsigned)((threads + 255) / 256), 256, 0, c->stream>>>(
      c->n, f4, c->nb_cnt.p, c->nb_w, c->nb_list.p, c->pair_ten.p, self_c, f, u);
}

template <int V>
void launch_stored_cheb(ggem_ctx *c, const float4 *f4, double self_c, double two_da,
                        double two_db, double coef, const double *x0, const double *x1,
                        double *xm, double *dw, float4 *next) {
  constexpr StoredVariant sv = kStoredVariants[V];
  const int64_t threads = c->n * sv.G;
  k_pair_cheb_tv<sv.G, sv.U, sv.pipe><<<(unsigned)((threads + 255) / 256), 256, 0, c->stream>>>(
      c->n, f4, c->nb_cnt.p, c->nb_w, c->nb_list.p, c->pair_ten.p, self_c, two_da, two_db, coef,
      x0, x1, xm, dw, next);
}

void dispatch_stored_r1(ggem_ctx *c, const float4 *f4, double self_c, const double *f, double *u) {
  switch (c->stored_variant) {
    case 1: launch_stored_r1<1>(c, f4, self_c, f, u); break;
    case 2: launch_stored_r1<2>(c, f4, self_c, f, u); break;
    case 3: launch_stored_r1<3>(c, f4, self_c, f, u); break;
    default: launch_stored_r1<0>(c, f4, self_c, f, u); break;
  }
}

void dispatch_stored_cheb(ggem_ctx *c, const float4 *f4, double self_c, double two_da,
                          double two_db, double coef, const double *x0, const double *x1,
                          double *xm, double *dw, float4 *next) {
  switch (c->stored_variant) {
    case 1: launch_stored_cheb<1>(c, f4, self_c, two_da, two_db, coef, x0, x1, xm, dw, next); break;
    case 2: launch_stored_cheb<2>(c, f4, self_c, two_da, two_db, coef, x0, x1, xm, dw, next); break;
    case 3: launch_stored_cheb<3>(c, f4, self_c, two_da, two_db, coef, x0, x1, xm, dw, next); break;
    default: launch_stored_cheb<0>(c, f4, self_c, two_da, two_db, coef, x0, x1, xm, dw, next); break;
  }
}

// NR right-hand sides r0 .. r0+NR-1: f32 is [r][n] float4, u [r][n][3]
template <int CD, bool POLY, int NR>
__global__ void __launch_bounds__(256) k_pair_nr(
    int64_t n, const float4 *__restrict__ pos32, const float4 *__restrict__ f32,
    const int32_t *__restrict__ cnt, int W, const uint32_t *__restrict__ list, PolyAB P,
    const Rec32 *__restrict__ tab, float inv_ds, float hx, float hy, float hz, double self_c,
    const double *__restrict__ f, double *__restrict__ u, int r0) {
  const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kGroup;
  const int sub = (int)(threadIdx.x % kGroup);
  const bool act = gid < n;
  const int64_t s = act ? gid : n - 1;
  const int64_t b = s * (int64_t)W, e = act ? b + cnt[s] : b;
  const float4 pi = pos32[s];
  float sx[NR], sy[NR], sz[NR], cx[NR], cy[NR], cz[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) sx[q] = sy[q] = sz[q] = cx[q] = cy[q] = cz[q] = 0.f;
  for (int64_t m = b + sub; m < e; m += kGroup) {
    const uint32_t en = __ldg(list + m);
    const uint32_t j = en >> kCodeBits;
    const float4 pj = __ldg(pos32 + j);
    float ox, oy, oz;
    decode_shift<CD>(en, hx, hy, hz, ox, oy, oz);
    const float dx = (pj.x - pi.x) + ox;
    const float dy = (pj.y - pi.y) + oy;
    const float dz = (pj.z - pi.z) + oz;
    const float s2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    float A, B;
    tensor_ab32<POLY>(s2, P, tab, inv_ds, A, B);
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      const float4 fj = __ldg(f32 + (int64_t)(r0 + q) * n + j);
      const float bxf = B * fmaf(dz, fj.z, fmaf(dy, fj.y, dx * fj.x));
      kahan_add(sx[q], cx[q], fmaf(A, fj.x, bxf * dx));
      kahan_add(sy[q], cy[q], fmaf(A, fj.y, bxf * dy));
      kahan_add(sz[q], cz[q], fmaf(A, fj.z, bxf * dz));
    }
  }
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    cx[q] = -cx[q];
    cy[q] = -cy[q];
    cz[q] = -cz[q];
    group_ff(sx[q], cx[q]);
    group_ff(sy[q], cy[q]);
    group_ff(sz[q], cz[q]);
    const int64_t roff = (int64_t)(r0 + q) * n * 3;
    group_store(act, sub, s, sx[q], cx[q], sy[q], cy[q], sz[q], cz[q], self_c, f + roff,
                u + roff);
  }
}

// ---- batched right-hand sides: 64 per pass, lanes over right-hand sides ----
//
// Forces of a pass are staged as FP32 [slot][3][64] (768 B per source, the
// pair (2l, 2l+1) of right-hand sides at float2 index l), so the 32 lanes of
// a warp read one source's forces with three coalesced 256-byte loads.  A
// warp owns one target slot: its lanes first evaluate the tensors of 32
// entries of the target's row at once (one entry per lane) into shared
// memory, then walk those entries with every lane updating its two
// right-hand sides in packed FP32x2 arithmetic.  Block-Kahan sums per lane;
// the CTA transposes the float-float results through shared memory so that
// the FP64 velocities [r][slot][3] (self term added in FP64) are written
// coalesced.
constexpr int kBatchR = 64;      // right-hand sides per pass
constexpr int kBatchMinRhs = 16; // fewer go through k_pair_nr in chunks of 8
constexpr int kBatchWarps = 8;   // target slots per CTA

__global__ void __launch_bounds__(256) k_stage_b64(int64_t n, int nr, const double *__restrict__ f,
                                                   float *__restrict__ fb) {
  // block: 32 slots x 64 right-hand sides; smem [r][96 + 1]
  __shared__ float t[kBatchR][97];
  const int64_t s0 = blockIdx.x * 32LL;
  const int ns = (int)(n - s0 < 32 ? n - s0 : 32);
  for (int k = threadIdx.x; k < kBatchR * 96; k += blockDim.x) {
    const int r = k / 96, q = k - r * 96;
    t[r][q] = (r < nr && q < 3 * ns) ? d2f_bits(f[((int64_t)r * n + s0) * 3 + q]) : 0.f;
  }
  __syncthreads();
  float *out = fb + s0 * 3 * kBatchR;
  for (int k = threadIdx.x; k < ns * 3 * kBatchR; k += blockDim.x) {
    const int sc = k / kBatchR, r = k - sc * kBatchR;
    out[k] = t[r][sc];
  }
}

// xi (caller order, [r][i][3]) into slot order (x0) and its batched FP32
// staging in one pass: k_to_slots followed by k_stage_b64
__global__ void __launch_bounds__(256) k_to_slots_b64(int64_t n, int nr,
                                                      const int32_t *__restrict__ order,
                                                      const double *__restrict__ xi,
                                                      double *__restrict__ x0,
                                                      float *__restrict__ fb) {
  __shared__ float t[kBatchR][97];
  const int64_t s0 = blockIdx.x * 32LL;
  const int ns = (int)(n - s0 < 32 ? n - s0 : 32);
  for (int k = threadIdx.x; k < kBatchR * 96; k += blockDim.x) {
    const int r = k / 96, q = k - r * 96;
    float v = 0.f;
    if (r < nr && q < 3 * ns) {
      const int sl = q / 3, c = q - 3 * sl;
      const double x = xi[((int64_t)r * n + order[s0 + sl]) * 3 + c];
      x0[((int64_t)r * n + s0) * 3 + q] = x;
      v = d2f_bits(x);
    }
    t[r][q] = v;
  }
  __syncthreads();
  float *out = fb + s0 * 3 * kBatchR;
  for (int k = threadIdx.x; k < ns * 3 * kBatchR; k += blockDim.x) {
    const int sc = k / kBatchR, r = k - sc * kBatchR;
    out[k] = t[r][sc];
  }
}

// The first step of a batched series in one pass (brownian_system.C:1041,
// 1050-1056): x1 = db x0 + da x1 (x1 holds M x0 on entry), dw = c0 x0 +
// c1 x1, and the batched FP32 staging of x1 for the first fused term
__global__ void __launch_bounds__(256) k_cheb_start_b64(int64_t n, int nr, double da, double db,
                                                        double c0, double c1,
                                                        const double *__restrict__ x0,
                                                        double *__restrict__ x1,
                                                        double *__restrict__ dw,
                                                        float *__restrict__ fb) {
  __shared__ float t[kBatchR][97];
  const int64_t s0 = blockIdx.x * 32LL;
  const int ns = (int)(n - s0 < 32 ? n - s0 : 32);
  for (int k = threadIdx.x; k < kBatchR * 96; k += blockDim.x) {
    const int r = k / 96, q = k - r * 96;
    float v = 0.f;
    if (r < nr && q < 3 * ns) {
      const int64_t idx = ((int64_t)r * n + s0) * 3 + q;
      const double x = x0[idx];
      const double y = db * x + da * x1[idx];
      x1[idx] = y;
      const double c0x = c0 * x;
      dw[idx] = c0x + c1 * y;
      v = d2f_bits(y);
    }
    t[r][q] = v;
  }
  __syncthreads();
  float *out = fb + s0 * 3 * kBatchR;
  for (int k = threadIdx.x; k < ns * 3 * kBatchR; k += blockDim.x) {
    const int sc = k / kBatchR, r = k - sc * kBatchR;
    out[k] = t[r][sc];
  }
}

// forces of row entry q (clamped to the last one) for the two right-hand
// sides of this lane: fw = fb + lane, jw = the warp's source slots
__device__ __forceinline__ void b64_fetch(const float2 *__restrict__ fw, const uint32_t *jw, int q,
                                          int np, float2 &x, float2 &y, float2 &z) {
  const float2 *fp = fw + (int64_t)jw[min(q, np - 1)] * (3 * 32);
  x = __ldg(fp);
  y = __ldg(fp + 32);
  z = __ldg(fp + 64);
}

// blk += A f + B (x.f) x for both right-hand sides of the lane (packed)
__device__ __forceinline__ void b64_accumulate(const float4 &g0, const float4 &g1,
                                               const float2 &g2, const float2 &fx,
                                               const float2 &fy, const float2 &fz, float2 &b0,
                                               float2 &b1, float2 &b2) {
  const float2 dx2 = make_float2(g0.x, g0.y), dy2 = make_float2(g0.z, g0.w);
  const float2 dz2 = make_float2(g1.x, g1.y), A2 = make_float2(g1.z, g1.w);
  float2 d = __ffma2_rn(dz2, fz, __ffma2_rn(dy2, fy, __fmul2_rn(dx2, fx)));
  d = __fmul2_rn(g2, d);
  b0 = __ffma2_rn(d, dx2, __ffma2_rn(A2, fx, b0));
  b1 = __ffma2_rn(d, dy2, __ffma2_rn(A2, fy, b1));
  b2 = __ffma2_rn(d, dz2, __ffma2_rn(A2, fz, b2));
}

// block sums into the Kahan pairs, blocks cleared
__device__ __forceinline__ void b64_flush(float2 (&sum)[3], float2 (&cmp)[3], float2 &b0,
                                          float2 &b1, float2 &b2) {
  kahan_add(sum[0].x, cmp[0].x, b0.x);
  kahan_add(sum[0].y, cmp[0].y, b0.y);
  kahan_add(sum[1].x, cmp[1].x, b1.x);
  kahan_add(sum[1].y, cmp[1].y, b1.y);
  kahan_add(sum[2].x, cmp[2].x, b2.x);
  kahan_add(sum[2].y, cmp[2].y, b2.y);
  b0 = b1 = b2 = make_float2(0.f, 0.f);
}

// per right-hand side Chebyshev coefficient of a fused batched term (0 for
// a right-hand side whose series has stopped)
struct BatchCoef {
  double c[kBatchR];
};

// With CHEB the kernel is one unchecked Chebyshev term for up to 64
// right-hand sides (brownian_system.C:1091-1108, the order of k_cheb_term):
// u is x_{k+1}: u = (2db x1 + 2da M x1) - x0, dw += c_r u, and fb_next
// receives the FP32 staging of u for the next term.
template <int CD, bool POLY, bool CHEB>
__global__ void __launch_bounds__(32 * kBatchWarps, 4) k_pair_b64(
    int64_t n, int nr, const float4 *__restrict__ pos32, const float2 *__restrict__ fb,
    const int32_t *__restrict__ cnt, int W, const uint32_t *__restrict__ list, PolyAB P,
    const Rec32 *__restrict__ tab, float inv_ds, float hx, float hy, float hz, float self_hi,
    float self_lo, double *__restrict__ u, double two_da, double two_db, BatchCoef cf,
    const double *__restrict__ x0, const double *__restrict__ x1, double *__restrict__ dw,
    float *__restrict__ fb_next) {
  // per entry, pre-duplicated for the packed arithmetic:
  // g0 = (dx, dx, dy, dy), g1 = (dz, dz, A, A), g2 = (B, B), source slot
  __shared__ float4 s_g0[kBatchWarps][32], s_g1[kBatchWarps][32];
  __shared__ float2 s_g2[kBatchWarps][32];
  __shared__ uint32_t s_j[kBatchWarps][32];
  __shared__ float2 s_out[kBatchWarps][kBatchR][3];  // float-float results
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t s = blockIdx.x * (int64_t)kBatchWarps + w;
  const bool act = s < n;
  float2 sum[3], cmp[3];
  float2 blk0 = make_float2(0.f, 0.f), blk1 = blk0, blk2 = blk0;
#pragma unroll
  for (int c = 0; c < 3; ++c) sum[c] = cmp[c] = make_float2(0.f, 0.f);
  if (act) {
    // self term from the target's own staged forces, as a float-float
    // product with self_c = self_hi + self_lo
    {
      const float2 *fo = fb + s * (3 * 32);
      const float2 ch = make_float2(self_hi, self_hi), cl = make_float2(self_lo, self_lo);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float2 v = __ldg(fo + 32 * c + lane);
        const float2 pr = __fmul2_rn(ch, v);
        const float2 er = __ffma2_rn(cl, v, __ffma2_rn(ch, v, make_float2(-pr.x, -pr.y)));
        sum[c] = pr;
        cmp[c] = make_float2(-er.x, -er.y);  // Kahan keeps value = sum - cmp
      }
    }
    const float4 pi = pos32[s];
    const int64_t b = s * (int64_t)W;
    const int e = cnt[s];
    int nb = 0;
    for (int m0 = 0; m0 < e; m0 += 32) {
      const int np = min(32, e - m0);
      if (lane < np) {
        const uint32_t en = __ldg(list + b + m0 + lane);
        const uint32_t j = en >> kCodeBits;
        const float4 pj = __ldg(pos32 + j);
        float ox, oy, oz;
        decode_shift<CD>(en, hx, hy, hz, ox, oy, oz);
        const float dx = (pj.x - pi.x) + ox, dy = (pj.y - pi.y) + oy, dz = (pj.z - pi.z) + oz;
        const float s2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        float A, B;
        tensor_ab32<POLY>(s2, P, tab, inv_ds, A, B);
        s_g0[w][lane] = make_float4(dx, dx, dy, dy);
        s_g1[w][lane] = make_float4(dz, dz, A, A);
        s_g2[w][lane] = make_float2(B, B);
        s_j[w][lane] = j;
      }
      __syncwarp();
      // three force slots in flight: each is refilled with the entry three
      // ahead right after its own entry is used (no register rotation)
      const float2 *fw = fb + lane;
      const uint32_t *jw = s_j[w];
      float2 ax, ay, az, bx, by, bz, cx, cy, cz;
      b64_fetch(fw, jw, 0, np, ax, ay, az);
      b64_fetch(fw, jw, 1, np, bx, by, bz);
      b64_fetch(fw, jw, 2, np, cx, cy, cz);
      for (int p = 0; p < np; p += 3) {
        b64_accumulate(s_g0[w][p], s_g1[w][p], s_g2[w][p], ax, ay, az, blk0, blk1, blk2);
        b64_fetch(fw, jw, p + 3, np, ax, ay, az);
        if (p + 1 < np) {
          b64_accumulate(s_g0[w][p + 1], s_g1[w][p + 1], s_g2[w][p + 1], bx, by, bz, blk0, blk1,
                         blk2);
          b64_fetch(fw, jw, p + 4, np, bx, by, bz);
        }
        if (p + 2 < np) {
          b64_accumulate(s_g0[w][p + 2], s_g1[w][p + 2], s_g2[w][p + 2], cx, cy, cz, blk0, blk1,
                         blk2);
          b64_fetch(fw, jw, p + 5, np, cx, cy, cz);
        }
        if (++nb == 3) {  // every 9 entries into the compensated sums
          b64_flush(sum, cmp, blk0, blk1, blk2);
          nb = 0;
        }
      }
      __syncwarp();
    }
  }
  b64_flush(sum, cmp, blk0, blk1, blk2);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    s_out[w][2 * lane][c] = make_float2(sum[c].x, -cmp[c].x);
    s_out[w][2 * lane + 1][c] = make_float2(sum[c].y, -cmp[c].y);
  }
  __syncthreads();
  // coalesced FP64 write-out: per right-hand side, the CTA's targets'
  // 3 components are consecutive doubles; one FP64 add per value
  const int64_t s0 = blockIdx.x * (int64_t)kBatchWarps;
  const int ns = (int)(n - s0 < kBatchWarps ? n - s0 : kBatchWarps);
  constexpr int kRow = 3 * kBatchWarps;
  for (int k = threadIdx.x; k < nr * kRow; k += blockDim.x) {
    const int r = k / kRow, q = k - r * kRow;
    const int t = q / 3, c = q - t * 3;
    if (t >= ns) continue;
    const float2 v = s_out[t][r][c];
    const int64_t idx = ((int64_t)r * n + s0) * 3 + q;
    double m = f2d_bits(v.x) + f2d_bits(v.y);
    if (CHEB) {
      // x_{k+1} = 2da M x_k + (2db x_k - x_{k-1}), dw += c x_{k+1}: four
      // FP64 operations per element with the add above (FP64 issues at a
      // small fraction of the FP32 rate on this GPU)
      const double x = fma(two_da, m, fma(two_db, x1[idx], -x0[idx]));
      dw[idx] = fma(cf.c[r], x, dw[idx]);
      m = x;
      // FP32 staging of x_{k+1}, transposed through shared memory below
      reinterpret_cast<float *>(&s_out[t][r][c])[0] = d2f_bits(x);
    }
    u[idx] = m;
  }
  if (CHEB) {
    __syncthreads();
    // staging layout [slot][3][64], right-hand sides fastest
    float *out = fb_next + s0 * 3 * kBatchR;
    for (int k = threadIdx.x; k < ns * 3 * kBatchR; k += blockDim.x) {
      const int sc = k / kBatchR, r = k - sc * kBatchR;
      const int t = sc / 3, c = sc - t * 3;
      out[k] = r < nr ? reinterpret_cast<const float *>(&s_out[t][r][c])[0] : 0.f;
    }
  }
}

__global__ void k_slots_to_f32(int64_t n, int nrhs, const double *__restrict__ f,
                               float4 *__restrict__ f32) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n * nrhs) return;
  const double *p = f + 3 * k;
  f32[k] = make_float4((float)p[0], (float)p[1], (float)p[2], 0.f);
}

// orig [r][n][3] -> slots [r][n][3]
__global__ void k_to_slots(int64_t n, int nrhs, const int32_t *__restrict__ order,
                           const double *__restrict__ orig, double *__restrict__ slot) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n * nrhs) return;
  const int64_t r = k / n, s = k - r * n;
  const int64_t i = order[s];
  const double *src = orig + (r * n + i) * 3;
  double *dst = slot + (r * n + s) * 3;
  dst[0] = src[0];
  dst[1] = src[1];
  dst[2] = src[2];
}

__global__ void k_from_slots(int64_t n, int nrhs, const int32_t *__restrict__ rank,
                             const double *__restrict__ slot, double *__restrict__ orig) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n * nrhs) return;
  const int64_t r = k / n, i = k - r * n;
  const int64_t s = rank[i];
  const double *src = slot + (r * n + s) * 3;
  double *dst = orig + (r * n + i) * 3;
  dst[0] = src[0];
  dst[1] = src[1];
  dst[2] = src[2];
}

template <int NR>
int launch_f64(ggem_ctx *c, const double *f, double *u, int self_mode, int r0) {
  if (c->f64_list && c->list_built) {
    const int64_t threads = c->n * kGroup;
    kt_start(c, kKPairF64);
    k_pair_list_f64<NR><<<(unsigned)((threads + 255) / 256), 256, 0, c->stream>>>(
        c->n, c->grid, c->dc, c->nb_cnt.p, c->nb_w, c->nb_list.p, c->pos64.p, f, u, self_mode,
        r0);
    kt_stop(c, kKPairF64);
    return check_launch(c, "matvec f64 list");
  }
  const int T = 128;
  const unsigned bn = (unsigned)((c->n + T - 1) / T);
  const bool ref = c->prm.nb_mode == GGEM_NB_REFERENCE;
  kt_start(c, kKPairF64);
  k_matvec_f64<NR><<<bn, T, 0, c->stream>>>(c->n, c->grid, c->dc, c->d_stencil.p,
                                             (int)c->stencil.size(), ref ? 1 : 0, ref ? 0 : 1,
                                             c->rc2, c->cell_start.p, c->pos64.p, c->pos32.p, f,
                                             u, self_mode, 0, r0);
  kt_stop(c, kKPairF64);
  return check_launch(c, "matvec f64");
}

PolyAB poly_of(const ggem_ctx *c) {
  PolyAB P;
  for (int q = 0; q <= kPolyDeg; ++q) P.ab[q] = make_float2(c->poly_a[q], c->poly_b[q]);
  P.x0 = c->poly_x0;
  P.x1 = c->poly_x1;
  P.e_hi = c->poly_e[0];
  P.e_lo = c->poly_e[1];
  return P;
}

// a series kernel launched as a programmatic dependent of the kernel
// before it on the stream (its first global reads wait in wait_prior_grid);
// measured at N = 200k: the reference-faithful series (a vector kernel
// between pair kernels) 777-781 -> 795-797 steps/s, the host-buffer leg
// 1492-1496 -> 1512-1519, the device-resident fused series unchanged
template <typename... KArgs, typename... Args>
void launch_dependent(void (*kern)(KArgs...), unsigned grid, unsigned block, cudaStream_t st,
                      Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, args...);
}

template <bool POLY, int V, bool ORIG>
void launch_r1(ggem_ctx *c, const Rec32 *src, const double *f, double *u, double self_c,
               double *part) {
  launch_dependent(k_pair_r1<POLY, V, ORIG>, (unsigned)pair_grid_blocks(c), 256u, c->stream,
                   c->n, src, (const int32_t *)c->nb_cnt.p, c->nb_w, (const uint32_t *)c->nb_list.p,
                   poly_of(c), reinterpret_cast<const Rec32 *>(c->tab.p), c->tab_inv_ds,
                   (const float4 *)c->d_shift.p, self_c, f, u, (const int32_t *)c->order.p, part);
}

template <bool POLY, bool ORIG = false>
void dispatch_r1(ggem_ctx *c, const Rec32 *src, const double *f, double *u, double self_c,
                 double *part = nullptr) {
  if (c->computed_variant == 1) launch_r1<POLY, 1, ORIG>(c, src, f, u, self_c, part);
  else launch_r1<POLY, 0, ORIG>(c, src, f, u, self_c, part);
}

// single right-hand side: records from FP64 slot-order f, then the pair sum
// u = M f for one right-hand side from the half list (k_pair_sym +
// k_sym_finish); src holds the records of f
int launch_sym_r1(ggem_ctx *c, const Rec32 *src, const double *f, double *u, double self_c) {
  const int64_t n = c->n;
  cudaError_t e;
  if (c->sym_acc.count < (size_t)n) {
    if ((e = c->sym_acc.ensure((size_t)n)) ||
        (e = cudaMemsetAsync(c->sym_acc.p, 0, sizeof(float4) * c->sym_acc.count, c->stream)))
      return cuda_fail(c, e, "symmetric accumulators");
  }
  if ((e = c->sym_part.ensure(3 * (size_t)n))) return cuda_fail(c, e, "symmetric sums");
  const unsigned nb = (unsigned)((n * kGroup + 255) / 256);
  kt_start(c, kKPairF32);
  if (c->use_poly)
    k_pair_sym<true><<<nb, 256, 0, c->stream>>>(
        n, src, c->nb_cnt_h.p, c->nb_w, c->nb_list_h.p, poly_of(c),
        reinterpret_cast<const Rec32 *>(c->tab.p), c->tab_inv_ds, c->d_shift.p, c->sym_acc.p,
        c->sym_part.p);
  else
    k_pair_sym<false><<<nb, 256, 0, c->stream>>>(
        n, src, c->nb_cnt_h.p, c->nb_w, c->nb_list_h.p, poly_of(c),
        reinterpret_cast<const Rec32 *>(c->tab.p), c->tab_inv_ds, c->d_shift.p, c->sym_acc.p,
        c->sym_part.p);
  if (int rc = check_launch(c, "pair f32 symmetric")) return rc;
  k_sym_finish<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, c->sym_part.p, c->sym_acc.p,
                                                                  self_c, f, u);
  kt_stop(c, kKPairF32);
  return check_launch(c, "pair f32 symmetric finish");
}

int launch_f32_r1(ggem_ctx *c, const double *f, double *u, double self_c) {
  const int64_t n = c->n;
  cudaError_t e;
  if (c->pretensor_ok) {
    if ((e = c->w_f4[0].ensure((size_t)n))) return cuda_fail(c, e, "pair forces");
    k_stage_f4<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, f, c->w_f4[0].p);
    if (int rc = check_launch(c, "pair forces")) return rc;
    kt_start(c, kKPairF32);
    dispatch_stored_r1(c, c->w_f4[0].p, self_c, f, u);
    kt_stop(c, kKPairF32);
    return check_launch(c, "pair f32 r1 (tensors)");
  }
  if ((e = c->w_src.ensure(2 * (size_t)n))) return cuda_fail(c, e, "pair records");
  Rec32 *src = reinterpret_cast<Rec32 *>(c->w_src.p);
  k_build_src<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, c->pos32.p, f, src);
  if (int rc = check_launch(c, "pair records")) return rc;
  if (c->sym_pairs && c->nb_list_h.p) return launch_sym_r1(c, src, f, u, self_c);
  kt_start(c, kKPairF32);
  if (c->use_poly) dispatch_r1<true>(c, src, f, u, self_c);
  else dispatch_r1<false>(c, src, f, u, self_c);
  kt_stop(c, kKPairF32);
  return check_launch(c, "pair f32 r1");
}

// c1 = 2db + 2da self_c folds the self term into the x1 coefficient
template <bool POLY, int V, bool NORMS>
void launch_cheb(ggem_ctx *c, const Rec32 *src, Rec32 *next, double two_da, double c1,
                 double coef, const double *x0, const double *x1, double *xm, double *dw,
                 double *part, Rec32 *dw_next) {
  launch_dependent(k_pair_cheb<POLY, V, NORMS>, (unsigned)pair_grid_blocks(c), 256u, c->stream,
                   c->n, src, (const int32_t *)c->nb_cnt.p, c->nb_w, (const uint32_t *)c->nb_list.p,
                   poly_of(c), reinterpret_cast<const Rec32 *>(c->tab.p), c->tab_inv_ds,
                   (const float4 *)c->d_shift.p, two_da, c1, coef, x0, x1, xm, dw, next, part,
                   pair_partials(c), dw_next);
}

// with part (and dw_next) the term also leaves the estimators' two norms as
// per-block partials and the records of the new dw
template <bool POLY>
void dispatch_cheb(ggem_ctx *c, const Rec32 *src, Rec32 *next, double two_da, double c1,
                   double coef, const double *x0, const double *x1, double *xm, double *dw,
                   double *part, Rec32 *dw_next) {
  const bool v1 = c->computed_variant == 1;
  if (part) {
    if (v1) launch_cheb<POLY, 1, true>(c, src, next, two_da, c1, coef, x0, x1, xm, dw, part, dw_next);
    else launch_cheb<POLY, 0, true>(c, src, next, two_da, c1, coef, x0, x1, xm, dw, part, dw_next);
  } else {
    if (v1) launch_cheb<POLY, 1, false>(c, src, next, two_da, c1, coef, x0, x1, xm, dw, part, dw_next);
    else launch_cheb<POLY, 0, false>(c, src, next, two_da, c1, coef, x0, x1, xm, dw, part, dw_next);
  }
}

template <bool POLY, int V>
void launch_first(ggem_ctx *c, const Rec32 *src, Rec32 *next, double self_c, double da,
                  double db, double c0, double c1, const double *x0, double *m, double *x1,
                  double *dw, double *part) {
  launch_dependent(k_pair_first<POLY, V>, (unsigned)pair_grid_blocks(c), 256u, c->stream, c->n,
                   src, (const int32_t *)c->nb_cnt.p, c->nb_w, (const uint32_t *)c->nb_list.p,
                   poly_of(c), reinterpret_cast<const Rec32 *>(c->tab.p), c->tab_inv_ds,
                   (const float4 *)c->d_shift.p, self_c, da, db, c0, c1, x0, m, x1, dw, next,
                   part);
}

template <int CD, bool POLY>
void launch_b64_t(ggem_ctx *c, int nr, const double *f, double *u, double self_c) {
  const Grid &g = c->grid;
  const unsigned grid = (unsigned)((c->n + kBatchWarps - 1) / kBatchWarps);
  k_pair_b64<CD, POLY, false><<<grid, 32 * kBatchWarps, 0, c->stream>>>(
      c->n, nr, c->pos32.p, reinterpret_cast<const float2 *>(c->w_fb.p), c->nb_cnt.p, c->nb_w,
      c->nb_list.p, poly_of(c), reinterpret_cast<const Rec32 *>(c->tab.p), c->tab_inv_ds,
      g.h32[0], g.h32[1], g.h32[2], (float)self_c, (float)(self_c - (double)(float)self_c), u,
      0.0, 0.0, BatchCoef{}, nullptr, nullptr, nullptr, nullptr);
}

template <int CD, bool POLY>
void launch_b64_cheb(ggem_ctx *c, int nr, const float *fb, float *fb_next, double self_c,
                     double two_da, double two_db, const BatchCoef &cf, const double *x0,
                     const double *x1, double *xm, double *dw) {
  const Grid &g = c->grid;
  const unsigned grid = (unsigned)((c->n + kBatchWarps - 1) / kBatchWarps);
  k_pair_b64<CD, POLY, true><<<grid, 32 * kBatchWarps, 0, c->stream>>>(
      c->n, nr, c->pos32.p, reinterpret_cast<const float2 *>(fb), c->nb_cnt.p, c->nb_w,
      c->nb_list.p, poly_of(c), reinterpret_cast<const Rec32 *>(c->tab.p), c->tab_inv_ds,
      g.h32[0], g.h32[1], g.h32[2], (float)self_c, (float)(self_c - (double)(float)self_c), xm,
      two_da, two_db, cf, x0, x1, dw, fb_next);
}

// many right-hand sides: passes of 64 (k_stage_b64 + k_pair_b64)
// (staged: w_fb already holds the FP32 staging of f, one pass of at most 64)
int matvec_b64(ggem_ctx *c, int nrhs, const double *f, double *u, double self_c,
               bool staged = false) {
  const int64_t n = c->n;
  cudaError_t e = c->w_fb.ensure((size_t)n * 3 * kBatchR);
  if (e) return cuda_fail(c, e, "batched staging");
  const bool cd2 = c->prm.cell_div == 2;
  for (int r0 = 0; r0 < nrhs; r0 += kBatchR) {
    const int nr = std::min(kBatchR, nrhs - r0);
    const double *fr = f + (int64_t)r0 * n * 3;
    double *ur = u + (int64_t)r0 * n * 3;
    if (!staged) {
      k_stage_b64<<<(unsigned)((n + 31) / 32), 256, 0, c->stream>>>(n, nr, fr, c->w_fb.p);
      if (int rc = check_launch(c, "batched staging")) return rc;
    }
    kt_start(c, kKPairF32);
    if (c->use_poly) cd2 ? launch_b64_t<2, true>(c, nr, fr, ur, self_c)
                         : launch_b64_t<1, true>(c, nr, fr, ur, self_c);
    else cd2 ? launch_b64_t<2, false>(c, nr, fr, ur, self_c)
             : launch_b64_t<1, false>(c, nr, fr, ur, self_c);
    kt_stop(c, kKPairF32);
    if (int rc = check_launch(c, "pair f32 batched")) return rc;
  }
  return GGEM_OK;
}

template <int CD, bool POLY, int NR>
void launch_nr_t(ggem_ctx *c, const double *f, double *u, double self_c, int r0) {
  const int64_t threads = c->n * kGroup;
  const Grid &g = c->grid;
  k_pair_nr<CD, POLY, NR><<<(unsigned)((threads + 255) / 256), 256, 0, c->stream>>>(
      c->n, c->pos32.p, c->w_f32.p, c->nb_cnt.p, c->nb_w, c->nb_list.p, poly_of(c),
      reinterpret_cast<const Rec32 *>(c->tab.p), c->tab_inv_ds, g.h32[0], g.h32[1], g.h32[2],
      self_c, f, u, r0);
}

template <int NR>
int launch_nr(ggem_ctx *c, const double *f, double *u, double self_c, int r0) {
  const bool cd2 = c->prm.cell_div == 2;
  kt_start(c, kKPairF32);
  if (c->use_poly) {
    if (cd2) launch_nr_t<2, true, NR>(c, f, u, self_c, r0);
    else launch_nr_t<1, true, NR>(c, f, u, self_c, r0);
  } else {
    if (cd2) launch_nr_t<2, false, NR>(c, f, u, self_c, r0);
    else launch_nr_t<1, false, NR>(c, f, u, self_c, r0);
  }
  kt_stop(c, kKPairF32);
  return check_launch(c, "pair f32");
}

}  // namespace

int permute_to_slots(ggem_ctx *c, int nrhs, const double *d_orig, double *d_slot) {
  const int64_t tot = c->n * nrhs;
  if (tot == 0) return GGEM_OK;
  k_to_slots<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(c->n, nrhs, c->order.p,
                                                                   d_orig, d_slot);
  return check_launch(c, "to slots");
}

int permute_from_slots(ggem_ctx *c, int nrhs, const double *d_slot, double *d_orig) {
  const int64_t tot = c->n * nrhs;
  if (tot == 0) return GGEM_OK;
  k_from_slots<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(c->n, nrhs, c->rank.p,
                                                                     d_slot, d_orig);
  return check_launch(c, "from slots");
}

// One fused Chebyshev term on the FP32 single-RHS path (k_pair_cheb).
// records_fresh: c->w_rec[c->rec_cur] already holds the records of x1 (the
// previous fused term wrote them); otherwise they are built here first.
int pair_cheb_term(ggem_ctx *c, bool records_fresh, const double *x0, const double *x1,
                   double *xm, double *dw, double two_da, double two_db, double coef,
                   int self_mode, double *norms) {
  const int64_t n = c->n;
  if (n == 0) return GGEM_OK;
  cudaError_t e;
  const double self_c0 = self_coefficient(c, self_mode);
  if (c->pretensor_ok) {
    if (norms) return fail(c, GGEM_ERR_BAD_ARG, "fused norms need per-matvec pair tensors");
    if ((e = c->w_f4[0].ensure((size_t)n)) || (e = c->w_f4[1].ensure((size_t)n)))
      return cuda_fail(c, e, "chebyshev forces");
    float4 *cur = c->w_f4[c->rec_cur].p, *nxt = c->w_f4[c->rec_cur ^ 1].p;
    if (!records_fresh) {
      k_stage_f4<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, x1, cur);
      if (int rc = check_launch(c, "chebyshev forces")) return rc;
    }
    kt_start(c, kKPairCheb);
    dispatch_stored_cheb(c, cur, self_c0, two_da, two_db, coef, x0, x1, xm, dw, nxt);
    kt_stop(c, kKPairCheb);
    c->rec_cur ^= 1;
    return check_launch(c, "pair chebyshev term (tensors)");
  }
  if ((e = c->w_rec[0].ensure(2 * (size_t)n)) || (e = c->w_rec[1].ensure(2 * (size_t)n)))
    return cuda_fail(c, e, "chebyshev records");
  Rec32 *cur = reinterpret_cast<Rec32 *>(c->w_rec[c->rec_cur].p);
  Rec32 *nxt = reinterpret_cast<Rec32 *>(c->w_rec[c->rec_cur ^ 1].p);
  if (!records_fresh) {
    k_build_src<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, c->pos32.p, x1, cur);
    if (int rc = check_launch(c, "chebyshev records")) return rc;
  }
  const double c1 = two_db + two_da * self_c0;
  // a checked term leaves the records of the new dw in w_src for the check
  // matvec (matvec_dw_records)
  Rec32 *dwr = nullptr;
  if (norms) {
    if ((e = c->w_src.ensure(2 * (size_t)n))) return cuda_fail(c, e, "pair records");
    dwr = reinterpret_cast<Rec32 *>(c->w_src.p);
  }
  kt_start(c, kKPairCheb);
  if (c->use_poly) dispatch_cheb<true>(c, cur, nxt, two_da, c1, coef, x0, x1, xm, dw, norms, dwr);
  else dispatch_cheb<false>(c, cur, nxt, two_da, c1, coef, x0, x1, xm, dw, norms, dwr);
  kt_stop(c, kKPairCheb);
  c->rec_cur ^= 1;
  return check_launch(c, "pair chebyshev term");
}

// (the batched kernels evaluate their tensors per pair whether or not the
// single-RHS path stores them)
bool batch_term_fusable(const ggem_ctx *c, int nrhs) {
  return nrhs >= kBatchMinRhs && nrhs <= kBatchR && c->prm.precision == GGEM_FP32 &&
         c->prm.nb_mode == GGEM_NB_CUTOFF;
}

// One unchecked Chebyshev term for 16 .. 64 right-hand sides in one kernel
// (k_pair_b64 with the recurrence in its write-out).  staged_fresh:
// c->w_fb holds the FP32 staging of x1 (the previous fused term wrote it);
// otherwise it is staged here first.  coef[r] is 0 for a stopped series.
int batch_cheb_term(ggem_ctx *c, int nrhs, bool staged_fresh, const double *x0, const double *x1,
                    double *xm, double *dw, double two_da, double two_db, const double *coef,
                    int self_mode) {
  const int64_t n = c->n;
  if (n == 0) return GGEM_OK;
  cudaError_t e;
  if ((e = c->w_fb.ensure((size_t)n * 3 * kBatchR)) || (e = c->w_fb2.ensure((size_t)n * 3 * kBatchR)))
    return cuda_fail(c, e, "batched staging");
  if (!staged_fresh) {
    k_stage_b64<<<(unsigned)((n + 31) / 32), 256, 0, c->stream>>>(n, nrhs, x1, c->w_fb.p);
    if (int rc = check_launch(c, "batched staging")) return rc;
  }
  BatchCoef cf{};
  for (int r = 0; r < nrhs; ++r) cf.c[r] = coef[r];
  const double self_c = self_coefficient(c, self_mode);
  const bool cd2 = c->prm.cell_div == 2;
  kt_start(c, kKPairCheb);
  if (c->use_poly) {
    if (cd2) launch_b64_cheb<2, true>(c, nrhs, c->w_fb.p, c->w_fb2.p, self_c, two_da, two_db, cf, x0, x1, xm, dw);
    else launch_b64_cheb<1, true>(c, nrhs, c->w_fb.p, c->w_fb2.p, self_c, two_da, two_db, cf, x0, x1, xm, dw);
  } else {
    if (cd2) launch_b64_cheb<2, false>(c, nrhs, c->w_fb.p, c->w_fb2.p, self_c, two_da, two_db, cf, x0, x1, xm, dw);
    else launch_b64_cheb<1, false>(c, nrhs, c->w_fb.p, c->w_fb2.p, self_c, two_da, two_db, cf, x0, x1, xm, dw);
  }
  kt_stop(c, kKPairCheb);
  std::swap(c->w_fb.p, c->w_fb2.p);  // the staging of x_{k+1} is the next term's x1
  std::swap(c->w_fb.count, c->w_fb2.count);
  return check_launch(c, "pair chebyshev term (batched)");
}

int pair_grid_blocks(const ggem_ctx *c) {
  return (int)std::max<int64_t>(1, (c->n * kGroup + 255) / 256);
}

int64_t pair_partials(const ggem_ctx *c) { return pair_grid_blocks(c); }

// The first step of a fused series: xi (caller order) into slot order (x0)
// with its records, then k_pair_first (m = M x0, x1, dw and the records of
// x1 for the first term).
int cheb_start_fused(ggem_ctx *c, const double *xi, double *x0, double *m, double *x1,
                     double *dw, double da, double db, double c0, double c1, int self_mode,
                     double *aux2) {
  const int64_t n = c->n;
  if (n == 0) return GGEM_OK;
  if (c->pretensor_ok) return fail(c, GGEM_ERR_BAD_ARG, "fused start needs per-matvec pair tensors");
  cudaError_t e;
  if ((e = c->w_rec[0].ensure(2 * (size_t)n)) || (e = c->w_rec[1].ensure(2 * (size_t)n)))
    return cuda_fail(c, e, "chebyshev records");
  Rec32 *cur = reinterpret_cast<Rec32 *>(c->w_rec[c->rec_cur].p);
  Rec32 *nxt = reinterpret_cast<Rec32 *>(c->w_rec[c->rec_cur ^ 1].p);
  k_to_slots_rec<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, c->order.p, c->pos32.p,
                                                                     xi, x0, cur);
  if (int rc = check_launch(c, "to slots + records")) return rc;
  const double self_c = self_coefficient(c, self_mode);
  kt_start(c, kKPairF32);
  const bool v1 = c->computed_variant == 1;
  if (c->use_poly) {
    if (v1) launch_first<true, 1>(c, cur, nxt, self_c, da, db, c0, c1, x0, m, x1, dw, aux2);
    else launch_first<true, 0>(c, cur, nxt, self_c, da, db, c0, c1, x0, m, x1, dw, aux2);
  } else {
    if (v1) launch_first<false, 1>(c, cur, nxt, self_c, da, db, c0, c1, x0, m, x1, dw, aux2);
    else launch_first<false, 0>(c, cur, nxt, self_c, da, db, c0, c1, x0, m, x1, dw, aux2);
  }
  kt_stop(c, kKPairF32);
  c->rec_cur ^= 1;
  return check_launch(c, "pair first step");
}

// u = M dw after a checked fused term: the term left the records of dw in
// w_src, so the check matvec is one launch, and |u|^2 leaves as per-block
// partials (norm)
int matvec_dw_records(ggem_ctx *c, const double *dw, double *u, int self_mode, double *norm) {
  return matvec_records(c, c->w_src.p, dw, u, self_mode, norm);
}

// u = M f from the 32-byte records of f already staged in rec (2 float4 per
// slot: the cell-relative position, then the FP32 force), f in slot order
int matvec_records(ggem_ctx *c, const float4 *rec, const double *f, double *u, int self_mode,
                   double *norm) {
  if (c->n == 0) return GGEM_OK;
  const Rec32 *src = reinterpret_cast<const Rec32 *>(rec);
  const double self_c = self_coefficient(c, self_mode);
  kt_start(c, kKPairF32);
  if (c->use_poly) dispatch_r1<true>(c, src, f, u, self_c, norm);
  else dispatch_r1<false>(c, src, f, u, self_c, norm);
  kt_stop(c, kKPairF32);
  return check_launch(c, "pair f32 r1");
}

// u = M f for one right-hand side with f and u in the caller's particle
// order (FP32 list, per-matvec tensors): the slot permutation of f is fused
// with its records (k_to_slots_rec) and the pair kernel writes u in caller
// order, so a matvec is two launches.  f_slot receives f in slot order (the
// self term reads it).
int matvec_orig_fused(ggem_ctx *c, const double *f, double *u, double *f_slot, int self_mode) {
  const int64_t n = c->n;
  if (n == 0) return GGEM_OK;
  if (c->pretensor_ok) return fail(c, GGEM_ERR_BAD_ARG, "fused matvec needs per-matvec pair tensors");
  cudaError_t e = c->w_src.ensure(2 * (size_t)n);
  if (e) return cuda_fail(c, e, "pair records");
  Rec32 *src = reinterpret_cast<Rec32 *>(c->w_src.p);
  k_to_slots_rec<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, c->order.p, c->pos32.p,
                                                                     f, f_slot, src);
  if (int rc = check_launch(c, "to slots + records")) return rc;
  const double self_c = self_coefficient(c, self_mode);
  kt_start(c, kKPairF32);
  if (c->use_poly) dispatch_r1<true, true>(c, src, f_slot, u, self_c);
  else dispatch_r1<false, true>(c, src, f_slot, u, self_c);
  kt_stop(c, kKPairF32);
  return check_launch(c, "pair f32 r1");
}

// the per-pair tensors of the current list (k_pair_tensor)
int build_pair_tensors(ggem_ctx *c) {
  c->pretensor_ok = false;
  if (!c->use_pretensor || !c->allow_pretensor || !c->list_built) return GGEM_OK;
  const int64_t n = c->n;
  if (n == 0) {
    c->pretensor_ok = true;
    return GGEM_OK;
  }
  cudaError_t e = c->pair_ten.ensure((size_t)n * c->nb_w);
  if (e) {
    // no room for the tensors: the pair kernels evaluate them on the fly
    cudaGetLastError();
    return GGEM_OK;
  }
  const Grid &g = c->grid;
  const int64_t threads = n * kGroup;
  const unsigned grid = (unsigned)((threads + 255) / 256);
  const bool cd2 = c->prm.cell_div == 2;
  const Rec32 *tab = reinterpret_cast<const Rec32 *>(c->tab.p);
  kt_start(c, kKListBuild);
  if (c->use_poly) {
    if (cd2)
      k_pair_tensor<2, true><<<grid, 256, 0, c->stream>>>(n, c->pos32.p, c->nb_cnt.p, c->nb_w,
                                                          c->nb_list.p, poly_of(c), tab, c->tab_inv_ds,
                                                          g.h32[0], g.h32[1], g.h32[2], c->pair_ten.p);
    else
      k_pair_tensor<1, true><<<grid, 256, 0, c->stream>>>(n, c->pos32.p, c->nb_cnt.p, c->nb_w,
                                                          c->nb_list.p, poly_of(c), tab, c->tab_inv_ds,
                                                          g.h32[0], g.h32[1], g.h32[2], c->pair_ten.p);
  } else {
    if (cd2)
      k_pair_tensor<2, false><<<grid, 256, 0, c->stream>>>(n, c->pos32.p, c->nb_cnt.p, c->nb_w,
                                                           c->nb_list.p, poly_of(c), tab, c->tab_inv_ds,
                                                           g.h32[0], g.h32[1], g.h32[2], c->pair_ten.p);
    else
      k_pair_tensor<1, false><<<grid, 256, 0, c->stream>>>(n, c->pos32.p, c->nb_cnt.p, c->nb_w,
                                                           c->nb_list.p, poly_of(c), tab, c->tab_inv_ds,
                                                           g.h32[0], g.h32[1], g.h32[2], c->pair_ten.p);
  }
  kt_stop(c, kKListBuild);
  if (int rc = check_launch(c, "pair tensors")) return rc;
  c->pretensor_ok = true;
  return GGEM_OK;
}

double self_coefficient(const ggem_ctx *c, int self_mode) {
  if (self_mode == GGEM_SELF_BEAD) return 1.0 - c->cst.coeff_1;
  if (self_mode == GGEM_SELF_LAGRANGIAN) return c->cst.coeff_2;
  return 0.0;
}

// u = M f on slot-ordered FP64 vectors [r][n][3]
int matvec_slots(ggem_ctx *c, int nrhs, const double *f, double *u, int self_mode) {
  if (c->n == 0) return GGEM_OK;
  if (c->prm.precision == GGEM_FP64) {
    int r0 = 0;
    while (r0 < nrhs) {
      const int left = nrhs - r0;
      int rc;
      if (left >= 4) rc = launch_f64<4>(c, f, u, self_mode, r0), r0 += 4;
      else if (left >= 2) rc = launch_f64<2>(c, f, u, self_mode, r0), r0 += 2;
      else rc = launch_f64<1>(c, f, u, self_mode, r0), r0 += 1;
      if (rc) return rc;
    }
    return GGEM_OK;
  }
  if (nrhs == 1) return launch_f32_r1(c, f, u, self_coefficient(c, self_mode));
  if (nrhs >= kBatchMinRhs) return matvec_b64(c, nrhs, f, u, self_coefficient(c, self_mode));
  cudaError_t e = c->w_f32.ensure((size_t)c->n * nrhs);
  if (e) return cuda_fail(c, e, "f32 staging");
  const int64_t tot = c->n * nrhs;
  k_slots_to_f32<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(c->n, nrhs, f,
                                                                       c->w_f32.p);
  if (int rc = check_launch(c, "to f32")) return rc;
  return matvec_f32_staged(c, nrhs, f, u, self_mode);
}

// xi (caller order) into slot order x0 and, for a batched series, x0's
// staging in w_fb (then matvec_slots_prestaged); false: nothing done
bool to_slots_staged(ggem_ctx *c, int nrhs, const double *xi, double *x0, int *rc) {
  *rc = GGEM_OK;
  if (c->n == 0 || !batch_term_fusable(c, nrhs)) return false;
  const int64_t n = c->n;
  cudaError_t e = c->w_fb.ensure((size_t)n * 3 * kBatchR);
  if (e) {
    *rc = cuda_fail(c, e, "batched staging");
    return true;
  }
  k_to_slots_b64<<<(unsigned)((n + 31) / 32), 256, 0, c->stream>>>(n, nrhs, c->order.p, xi, x0,
                                                                  c->w_fb.p);
  *rc = check_launch(c, "to slots + staging");
  return true;
}

// the batched series' first step with x1's staging left in w_fb (see
// k_cheb_start_b64; 16 .. 64 right-hand sides)
int cheb_start_staged(ggem_ctx *c, int nrhs, double da, double db, double c0, double c1,
                      const double *x0, double *x1, double *dw) {
  const int64_t n = c->n;
  if (n == 0) return GGEM_OK;
  cudaError_t e = c->w_fb.ensure((size_t)n * 3 * kBatchR);
  if (e) return cuda_fail(c, e, "batched staging");
  k_cheb_start_b64<<<(unsigned)((n + 31) / 32), 256, 0, c->stream>>>(n, nrhs, da, db, c0, c1, x0,
                                                                    x1, dw, c->w_fb.p);
  return check_launch(c, "cheb start + staging");
}

// u = M f when the batched staging of f is already in w_fb (the last fused
// batched term wrote it): the batched kernel without the staging pass
int matvec_slots_prestaged(ggem_ctx *c, int nrhs, const double *f, double *u, int self_mode) {
  if (c->n == 0) return GGEM_OK;
  if (!batch_term_fusable(c, nrhs)) return matvec_slots(c, nrhs, f, u, self_mode);
  return matvec_b64(c, nrhs, f, u, self_coefficient(c, self_mode), true);
}

// FP32 pair sum from the already staged c->w_f32 ([r][n] float4); f is the
// FP64 slot-order force of the self term
int matvec_f32_staged(ggem_ctx *c, int nrhs, const double *f, double *u, int self_mode) {
  const double self_c = self_coefficient(c, self_mode);
  int r0 = 0;
  while (r0 < nrhs) {
    const int left = nrhs - r0;
    int rc;
    if (left >= 8) rc = launch_nr<8>(c, f, u, self_c, r0), r0 += 8;
    else if (left >= 4) rc = launch_nr<4>(c, f, u, self_c, r0), r0 += 4;
    else if (left >= 2) rc = launch_nr<2>(c, f, u, self_c, r0), r0 += 2;
    else rc = launch_nr<1>(c, f, u, self_c, r0), r0 += 1;
    if (rc) return rc;
  }
  return GGEM_OK;
}

}  // namespace ggem


using namespace ggem;

extern "C" int ggem_set_symmetric_pairs(ggem_ctx *ctx, int enable) {
  if (!ctx) return GGEM_ERR_BAD_ARG;
  if (ctx->prm.precision != GGEM_FP32 || ctx->prm.nb_mode != GGEM_NB_CUTOFF)
    return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "symmetric pair sums need a GGEM_FP32 cutoff context");
  ctx->sym_pairs = enable != 0;
  ctx->cells_built = false;  // the next ggem_build_cells writes (or drops) the half list
  ctx->list_built = false;
  return GGEM_OK;
}

extern "C" int ggem_set_pair_variant(ggem_ctx *ctx, int computed, int stored) {
  if (!ctx || computed < 0 || computed >= kNumComputedVariants || stored < 0 ||
      stored >= kNumStoredVariants)
    return GGEM_ERR_BAD_ARG;
  ctx->computed_variant = computed;
  ctx->stored_variant = stored;
  return GGEM_OK;
}

extern "C" int ggem_autotune_pair_storage(ggem_ctx *ctx, int reps, double matvecs_per_build,
                                          int *use_stored, double *ms_computed,
                                          double *ms_stored, int *variants) {
  if (!ctx || reps < 1 || !(matvecs_per_build > 0) || !use_stored || !ms_computed ||
      !ms_stored || !variants)
    return GGEM_ERR_BAD_ARG;
  if (int rc = settle_list(ctx)) return rc;
  if (ctx->prm.precision != GGEM_FP32 || !ctx->list_built)
    return fail(ctx, GGEM_ERR_BAD_ARG, "autotune needs a built FP32 pair list");
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != ctx->device) cudaSetDevice(ctx->device);
  const int64_t n = ctx->n;
  cudaError_t e;
  if ((e = ctx->w_in.ensure((size_t)3 * std::max<int64_t>(n, 1))) ||
      (e = ctx->w_out.ensure((size_t)3 * std::max<int64_t>(n, 1))))
    return cuda_fail(ctx, e, "autotune buffers");
  if (n > 0 && (e = cudaMemsetAsync(ctx->w_in.p, 0, sizeof(double) * 3 * n, ctx->stream)))
    return cuda_fail(ctx, e, "autotune buffers");
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const bool timing = ctx->timing;
  ctx->timing = false;
  auto time_matvecs = [&](double *ms) -> int {
    if (int rc = matvec_slots(ctx, 1, ctx->w_in.p, ctx->w_out.p, GGEM_SELF_BEAD)) return rc;
    cudaEventRecord(a, ctx->stream);
    for (int r = 0; r < reps; ++r)
      if (int rc = matvec_slots(ctx, 1, ctx->w_in.p, ctx->w_out.p, GGEM_SELF_BEAD)) return rc;
    cudaEventRecord(b, ctx->stream);
    cudaEventSynchronize(b);
    float t = 0.f;
    cudaEventElapsedTime(&t, a, b);
    *ms = t / reps;
    return GGEM_OK;
  };
  int rc = GGEM_OK;
  double t_comp = 0.0, t_store = 1e30;
  const bool allow = ctx->allow_pretensor;
  // tensors evaluated per pair and matvec, each loop shape; the fastest stays
  ctx->pretensor_ok = false;
  {
    int best_v = 0;
    t_comp = 1e30;
    for (int v = 0; v < kNumComputedVariants && !rc; ++v) {
      ctx->computed_variant = v;
      double t_mv = 0.0;
      rc = time_matvecs(&t_mv);
      if (!rc && t_mv < t_comp) {
        t_comp = t_mv;
        best_v = v;
      }
    }
    ctx->computed_variant = best_v;
  }
  if (!rc && ctx->use_pretensor) {
    ctx->allow_pretensor = true;
    cudaEventRecord(a, ctx->stream);
    rc = build_pair_tensors(ctx);
    cudaEventRecord(b, ctx->stream);
    cudaEventSynchronize(b);
    float t_pass = 0.f;
    cudaEventElapsedTime(&t_pass, a, b);
    if (!rc && ctx->pretensor_ok) {
      // every stored-tensor kernel shape; the fastest stays selected
      int best_v = 0;
      double best_mv = 1e30;
      for (int v = 0; v < kNumStoredVariants && !rc; ++v) {
        ctx->stored_variant = v;
        double t_mv = 0.0;
        rc = time_matvecs(&t_mv);
        if (!rc && t_mv < best_mv) {
          best_mv = t_mv;
          best_v = v;
        }
      }
      ctx->stored_variant = best_v;
      t_store = best_mv + t_pass / matvecs_per_build;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  ctx->timing = timing;
  if (rc) {
    ctx->allow_pretensor = allow;
    if (dev != ctx->device) cudaSetDevice(dev);
    return rc;
  }
  const bool stored = t_store < t_comp;
  ctx->allow_pretensor = stored;
  if (!stored) ctx->pretensor_ok = false;  // the stored tensors stay allocated but unused
  *use_stored = stored ? 1 : 0;
  *ms_computed = t_comp;
  *ms_stored = ctx->use_pretensor ? t_store : -1.0;
  variants[0] = ctx->computed_variant;
  variants[1] = ctx->stored_variant;
  if (dev != ctx->device) cudaSetDevice(dev);
  return GGEM_OK;
}
