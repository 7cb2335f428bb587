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

extern "C" int ggem_ensemble_brownian_dev(ggem_ensemble *e, int nrhs, int N,
                                          const double *eig_min, const double *eig_max,
                                          double tol, const double *d_xi, double *d_dw,
                                          ggem_cheb_report *rep) {
  if (!e || nrhs < 1 || nrhs > kR || N < 2 || !eig_min || !eig_max || !(tol >= 0) || !d_xi ||
      !d_dw || !rep)
    return GGEM_ERR_BAD_ARG;
  if (!e->built) return efail(e, GGEM_ERR_BAD_ARG, "set the ensemble's particles first");
  EnsGuard g(e->device);
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
