// ggem_surrogate.cu -- the learned eigen-interval surrogate: a BF16 MLP
// (35 features -> 3 hidden layers of 128 SiLU units -> log lambda_min,
// log lambda_max) trained and evaluated on the GPU by this file's kernels.
//
// It stands in for the spectral-bound estimate of the Brownian step,
// BrownianSystem::compute_eigenvalue(s) (brownian_system.C:527-657, SLEPc
// Krylov-Schur, widened by eig_factor in copss.C:1598-1639): the network
// predicts the interval from configuration features, the FP64 Chebyshev
// error check judges every prediction, and Lanczos stays the fallback.
//
// Every matrix product (forward, both backward products) is one tcgen05
// kernel: BF16 operands staged in shared memory in the K-major core-matrix
// layout, one thread issues 128 x N x 16 MMAs accumulating FP32 in TMEM,
// completion arrives on an mbarrier (bounded wait), and four warps read the
// 128 TMEM lanes back.  Bias, SiLU, the loss gradient, the bias gradients
// and Adam are small fused elementwise kernels.  Master weights stay FP32;
// the products use BF16 copies (K-major W^T for the forward product, W for
// the input-gradient product).
//
// Layer shapes (rows = batch B, a multiple of 128):
//   X  [B x 48]   (35 standardised features, zero padded)
//   Z1 = X  W1^T + b1 [B x 128], H1 = silu(Z1)
//   Z2 = H1 W2^T + b2,           H2 = silu(Z2)
//   Z3 = H2 W3^T + b3,           H3 = silu(Z3)
//   Y  = H3 W4^T + b4, outputs 0, 1 of 128 (W4 rows >= 2 stay zero)
// Loss: mean over the batch of the squared error of the two standardised
// outputs.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ggem_internal.cuh"
#include "ggem_surrogate.h"
#include "ggem_tc.cuh"

namespace ggem {
namespace sur {

constexpr int kIn = 35;      // features
constexpr int kInPad = 48;   // padded input width (K multiple of 16)
constexpr int kHid = 128;    // hidden width, also the padded output width
constexpr int kOut = 2;      // log lambda_min, log lambda_max
constexpr int kLayers = 4;
constexpr int kRowBlock = 128;
constexpr uint32_t kMaxPolls = 1u << 22;  // bounded mbarrier wait (~0.3 s)
constexpr double kPiS = 3.14159265358979323846;

using bf16 = __nv_bfloat16;

// ---- C[M x N] = A[M x K] * Bt[N x K]^T on the tensor cores ---------------
// A, Bt BF16 row-major with K contiguous (lda, ldb multiples of 8 elements,
// 16-byte aligned rows); C FP32 row-major.  M % 128 == 0, N % 16 == 0 with
// 16 <= N <= 128, K % 16 == 0, K > 0.  One CTA of 4 warps per 128-row block.
constexpr int kKChunk = 64;

__global__ void __launch_bounds__(128) k_gemm_bf16(const bf16 *__restrict__ A, int lda,
                                                   const bf16 *__restrict__ Bt, int ldb,
                                                   float *__restrict__ C, int ldc, int N, int K,
                                                   uint32_t polls, int *__restrict__ err) {
  // K-major core-matrix tiles: offset(row, k) = ((row/8)*8 + k/8)*128 +
  // (row%8)*16 + (k%8)*2, so core matrices adjacent along K are 128 B apart
  // (leading byte offset) and 8-row groups 1024 B apart (stride byte offset)
  __shared__ __align__(1024) uint8_t sA[kRowBlock * kKChunk * 2];
  __shared__ __align__(1024) uint8_t sB[kHid * kKChunk * 2];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t m0 = (int64_t)blockIdx.x * kRowBlock;
  const uint32_t ncols = tc::tmem_cols(N);
  if (warp == 0) tc::tmem_alloc(&tslot, ncols);
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_fence_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tslot;
  const uint32_t idesc = tc::idesc_bf16_f32(kRowBlock, N);
  uint32_t phase = 0;
  bool ok = true;
  for (int k0 = 0; k0 < K && ok; k0 += kKChunk) {
    const int kw = min(kKChunk, K - k0);
    const int pieces = kw >> 3;  // 16-byte pieces per row
    for (int c = tid; c < kRowBlock * pieces; c += blockDim.x) {
      const int row = c / pieces, kb = c - row * pieces;
      const uint4 v = *reinterpret_cast<const uint4 *>(A + (m0 + row) * lda + k0 + kb * 8);
      *reinterpret_cast<uint4 *>(sA + ((row >> 3) * 8 + kb) * 128 + (row & 7) * 16) = v;
    }
    for (int c = tid; c < N * pieces; c += blockDim.x) {
      const int row = c / pieces, kb = c - row * pieces;
      const uint4 v = *reinterpret_cast<const uint4 *>(Bt + (int64_t)row * ldb + k0 + kb * 8);
      *reinterpret_cast<uint4 *>(sB + ((row >> 3) * 8 + kb) * 128 + (row & 7) * 16) = v;
    }
    tc::fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
      for (int s = 0; s < (kw >> 4); ++s) {
        const uint64_t ad = tc::smem_desc(a0 + s * 256, 128, 1024);
        const uint64_t bd = tc::smem_desc(b0 + s * 256, 128, 1024);
        tc::mma_bf16(tmem, ad, bd, idesc, (k0 > 0 || s > 0) ? 1u : 0u);
      }
      tc::mma_commit(&bar);
    }
    // the tiles are reused only after the MMAs that read them completed
    // (polls bounds this wait; the drain below keeps the full window)
    const bool done = tc::mbar_wait_bounded(&bar, phase, polls);
    phase ^= 1u;
    ok = __syncthreads_and(done) != 0;
  }
  if (!ok) {
    if (tid == 0) atomicOr(err, kErrTimeout);
    // give MMAs still in flight a second bounded window before TMEM is freed
    tc::mbar_wait_bounded(&bar, phase ^ 1u, kMaxPolls);
  } else {
    tc::fence_after_sync();
    // warp w owns TMEM lanes 32w .. 32w+31 = rows m0 + 32w + lane
    float *dst = C + (m0 + warp * 32 + lane) * ldc;
    for (int c0 = 0; c0 < N; c0 += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 8; ++i) dst[c0 + i] = v[i];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, ncols);
  }
}

// ---- the whole forward pass in one kernel (inference) ----------------------
// One CTA of 4 warps per 128 rows.  All four BF16 weight matrices W^T stay in
// shared memory (K-major core-matrix tiles) for the CTA's lifetime; the
// activations of a layer are written back into one shared tile that the
// next product reads, so nothing but the raw features and the two outputs
// touches global memory.  Per layer: one thread issues the 128 x N x 16 MMA
// steps into a TMEM accumulator of 128 columns, commits to an mbarrier, all
// threads wait (bounded) and thread t reads TMEM lane t (its row), adds the
// bias, applies SiLU and stores the BF16 row into the activation tile.  The
// arithmetic is the layer-by-layer path's (same products in the same K
// order, same bias, SiLU and BF16 rounding), so the outputs agree bit for bit.
// Tile of R rows x KP 16-byte pieces: offset(row, piece) =
// ((row / 8) * KP + piece) * 128 + (row % 8) * 16; LBO 128 B, SBO KP * 128 B.
constexpr int kOutN = 16;  // N of the last product (outputs 0, 1 used)
constexpr size_t kMlpActBytes = (size_t)kRowBlock * kHid * 2;
constexpr size_t kMlpW0 = kMlpActBytes;
constexpr size_t kMlpW1 = kMlpW0 + (size_t)kHid * kInPad * 2;
constexpr size_t kMlpW2 = kMlpW1 + (size_t)kHid * kHid * 2;
constexpr size_t kMlpW3 = kMlpW2 + (size_t)kHid * kHid * 2;
constexpr size_t kMlpBias = kMlpW3 + (size_t)kOutN * kHid * 2;  // hidden layers' biases
constexpr size_t kMlpSmem = kMlpBias + (size_t)(kLayers - 1) * kHid * 4;

// offset of layer l's bias in the flat parameter vector (W1^T [128 x 48],
// b1, then [128 x 128] weights and 128 biases per layer)
__host__ __device__ constexpr int bias_off_d(int l) {
  return l == 0 ? kHid * kInPad
                : kHid * kInPad + kHid + (l - 1) * (kHid * kHid + kHid) + kHid * kHid;
}

__device__ __forceinline__ uint32_t tile_off(int row, int piece, int kp) {
  return (uint32_t)(((row >> 3) * kp + piece) * 128 + (row & 7) * 16);
}

// W^T [rows x K] into its tile with 16-byte asynchronous copies (cp.async:
// every copy of the thread in flight at once; completed by cp_async_wait)
__device__ __forceinline__ void stage_wt(uint8_t *dst, const bf16 *__restrict__ W, int rows,
                                         int K) {
  const int kp = K >> 3;
  for (int c = threadIdx.x; c < rows * kp; c += blockDim.x) {
    const int row = c / kp, kb = c - row * kp;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                     tc::smem_u32(dst + tile_off(row, kb, kp))),
                 "l"(W + (int64_t)row * K + kb * 8)
                 : "memory");
  }
}

__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}

// this thread's copies complete but for the N most recent groups
template <int N>
__device__ __forceinline__ void cp_async_wait_upto() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// 4 * n floats (16-byte pieces) with asynchronous copies
__device__ __forceinline__ void stage_f32(float *dst, const float *__restrict__ src, int n4) {
  for (int c = threadIdx.x; c < n4; c += blockDim.x)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_u32(dst + 4 * c)),
                 "l"(src + 4 * c)
                 : "memory");
}

// the logistic function on the special-function unit (ex2 and a correctly
// rounded reciprocal): a few ulp from 1 / (1 + e^-z), far below the BF16
// rounding of the activations; every kernel of the network uses this one
__device__ __forceinline__ float sigmoid_sfu(float z) { return __frcp_rn(1.f + __expf(-z)); }
__device__ __forceinline__ float silu_f(float z) { return z * sigmoid_sfu(z); }

constexpr int kMlpThreads = 1024;  // 32 warps: warp w reads TMEM lanes 32 (w % 4) .. + 31,
                                   // columns 16 (w / 4) .. + 15
constexpr int kMlpCols = kHid / (kMlpThreads / 128);  // hidden columns per thread

// The whole forward pass of one 128-row tile in one CTA.  The weights of the
// four layers (and the hidden biases) arrive by asynchronous copies in one
// group per layer, so that the first product starts once its own weights
// are in.  Each product is one tcgen05.mma chain by one thread into TMEM;
// the epilogue (bias, SiLU, BF16 into the next product's A tile) is spread
// over 32 warps, 16 columns per thread, and warps whose 32 rows are all
// past the last row of the batch skip it: rows of a product never mix, so
// those rows' stale activations reach no output.
__global__ void __launch_bounds__(kMlpThreads) k_mlp_forward(
    const float *__restrict__ x, int n, const float *__restrict__ mean,
    const float *__restrict__ inv_std, const bf16 *__restrict__ w0, const bf16 *__restrict__ w1,
    const bf16 *__restrict__ w2, const bf16 *__restrict__ w3, const float *__restrict__ params,
    float *__restrict__ Y, uint32_t polls, int *__restrict__ err) {
  extern __shared__ __align__(1024) uint8_t mlp_smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  uint8_t *sA = mlp_smem;
  float *s_bias = reinterpret_cast<float *>(mlp_smem + kMlpBias);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quarter = warp & 3, cb = warp >> 2;
  const int row = quarter * 32 + lane;  // this thread's row = its TMEM lane
  const int64_t row_g = (int64_t)blockIdx.x * kRowBlock + row;
  // a warp whose 32 rows all lie past the batch has no epilogue to run
  const bool live = (int64_t)blockIdx.x * kRowBlock + quarter * 32 < n;
  if (warp == 0) tc::tmem_alloc(&tslot, (uint32_t)kHid);
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_fence_init();
  }
  // weights and hidden biases, one copy group per layer
  stage_wt(mlp_smem + kMlpW0, w0, kHid, kInPad);
  stage_f32(s_bias, params + bias_off_d(0), kHid / 4);
  cp_async_commit();
  stage_wt(mlp_smem + kMlpW1, w1, kHid, kHid);
  stage_f32(s_bias + kHid, params + bias_off_d(1), kHid / 4);
  cp_async_commit();
  stage_wt(mlp_smem + kMlpW2, w2, kHid, kHid);
  stage_f32(s_bias + 2 * kHid, params + bias_off_d(2), kHid / 4);
  cp_async_commit();
  stage_wt(mlp_smem + kMlpW3, w3, kOutN, kHid);
  cp_async_commit();
  // meanwhile the standardised input rows (48 BF16, zero padded)
  if (warp < 4) {
#pragma unroll
    for (int kb = 0; kb < kInPad / 8; ++kb) {
      __align__(16) bf16 h[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int c = kb * 8 + i;
        const float v =
            (row_g < n && c < kIn) ? (x[row_g * kIn + c] - mean[c]) * inv_std[c] : 0.f;
        h[i] = __float2bfloat16_rn(v);
      }
      *reinterpret_cast<uint4 *>(sA + tile_off(row, kb, kInPad / 8)) =
          *reinterpret_cast<const uint4 *>(h);
    }
  }
  cp_async_wait_upto<3>();  // layer 0's weights and bias
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tslot;
  const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16);
  const size_t woff[kLayers] = {kMlpW0, kMlpW1, kMlpW2, kMlpW3};
  bool ok = true;
  uint32_t phase = 0;
  for (int l = 0; l < kLayers && ok; ++l) {
    const int K = l == 0 ? kInPad : kHid, N = l == kLayers - 1 ? kOutN : kHid;
    if (tid == 0) {
      const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(mlp_smem + woff[l]);
      const uint32_t idesc = tc::idesc_bf16_f32(kRowBlock, N);
      for (int s = 0; s < K / 16; ++s) {
        const uint64_t ad = tc::smem_desc(a0 + s * 256, 128, (uint32_t)(K / 8) * 128);
        const uint64_t bd = tc::smem_desc(b0 + s * 256, 128, (uint32_t)(K / 8) * 128);
        tc::mma_bf16(tmem, ad, bd, idesc, s > 0 ? 1u : 0u);
      }
      tc::mma_commit(&bar);
    }
    const bool done = tc::mbar_wait_bounded(&bar, phase, polls);
    phase ^= 1u;
    ok = __syncthreads_and(done) != 0;
    if (!ok) break;
    tc::fence_after_sync();
    if (l < kLayers - 1) {
      // H = silu(Z + b) into the activation tile (the product that read it
      // has completed)
      if (live) {
        const int c0 = cb * kMlpCols;
        const float *bias = s_bias + l * kHid + c0;
        float v[16];
        tc::tmem_ld16(lane_base + (uint32_t)c0, v);
#pragma unroll
        for (int h8 = 0; h8 < kMlpCols / 8; ++h8) {
          __align__(16) bf16 h[8];
#pragma unroll
          for (int i = 0; i < 8; ++i)
            h[i] = __float2bfloat16_rn(silu_f(v[8 * h8 + i] + bias[8 * h8 + i]));
          *reinterpret_cast<uint4 *>(sA + tile_off(row, (c0 >> 3) + h8, kHid / 8)) =
              *reinterpret_cast<const uint4 *>(h);
        }
      }
      // the next layer's weights are in (at most the later groups pending)
      if (l == 0) cp_async_wait_upto<2>();
      else if (l == 1) cp_async_wait_upto<1>();
      else cp_async_wait_upto<0>();
      tc::fence_proxy_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
    } else if (warp < 4 && live) {
      float v[8];
      tc::tmem_ld8(lane_base, v);
      if (row_g < n) {
        const float *bias = params + bias_off_d(l);
        Y[row_g * kOut] = v[0] + bias[0];
        Y[row_g * kOut + 1] = v[1] + bias[1];
      }
    }
  }
  if (!ok) {
    if (tid == 0) atomicOr(err, kErrTimeout);
    // the product still in flight completes before TMEM is freed
    tc::mbar_wait_bounded(&bar, phase ^ 1u, kMaxPolls);
  }
  cp_async_wait_upto<0>();  // no copy outlives the block (the timeout path)
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, (uint32_t)kHid);
  }
}

// ---- elementwise pieces ---------------------------------------------------
__device__ __forceinline__ float sigmoidf(float z) { return sigmoid_sfu(z); }

// standardised, zero-padded inputs: X [B x 48] and X^T [48 x B] (BF16);
// rows >= n (batch padding) are zero
__global__ void k_stage_inputs(const float *__restrict__ x, const int32_t *__restrict__ idx,
                               int n, int B, const float *__restrict__ mean,
                               const float *__restrict__ inv_std, bf16 *__restrict__ X,
                               bf16 *__restrict__ Xt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= B * kInPad) return;
  const int r = k / kInPad, c = k - r * kInPad;
  float v = 0.f;
  if (r < n && c < kIn) {
    const int src = idx ? idx[r] : r;
    v = (x[(int64_t)src * kIn + c] - mean[c]) * inv_std[c];
  }
  const bf16 b = __float2bfloat16_rn(v);
  X[k] = b;
  Xt[(int64_t)c * B + r] = b;
}

// Z += bias; hidden layers: H = silu(Z) as BF16 [B x 128] and H^T, Z kept
// for the backward pass; output layer: Y[:, 0:2] = Z + b (FP32)
__global__ void k_bias_act(float *__restrict__ Z, const float *__restrict__ bias, int B,
                           int hidden, bf16 *__restrict__ H, bf16 *__restrict__ Ht,
                           float *__restrict__ Y) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= B * kHid) return;
  const int r = k / kHid, c = k - r * kHid;
  const float z = Z[k] + bias[c];
  Z[k] = z;
  if (hidden) {
    const bf16 h = __float2bfloat16_rn(silu_f(z));
    H[k] = h;
    Ht[(int64_t)c * B + r] = h;
  } else if (c < kOut) {
    Y[(int64_t)r * kOut + c] = z;
  }
}

// dL/dY for L = mean_r sum_c (Y - T)^2 over the n valid rows, as the output
// layer's dZ (FP32 for the bias gradient, BF16 and its transpose for the
// products); partial sums of the loss per block
__global__ void k_loss_grad(const float *__restrict__ Y, const float *__restrict__ T,
                            const int32_t *__restrict__ idx, int n, int B,
                            float *__restrict__ dZf, bf16 *__restrict__ dZ,
                            bf16 *__restrict__ dZt, float *__restrict__ loss_part) {
  __shared__ float sh[256];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (k < B * kHid) {
    const int r = k / kHid, c = k - r * kHid;
    float g = 0.f;
    if (r < n && c < kOut) {
      const int src = idx ? idx[r] : r;
      const float e = Y[(int64_t)r * kOut + c] - T[(int64_t)src * kOut + c];
      l = e * e;
      g = 2.f * e / (float)n;
    }
    dZf[k] = g;
    const bf16 b = __float2bfloat16_rn(g);
    dZ[k] = b;
    dZt[(int64_t)c * B + r] = b;
  }
  sh[threadIdx.x] = l;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_part[blockIdx.x] = sh[0];
}

// dZ = dH * silu'(Z)
__global__ void k_act_back(const float *__restrict__ dH, const float *__restrict__ Z, int B,
                           float *__restrict__ dZf, bf16 *__restrict__ dZ,
                           bf16 *__restrict__ dZt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= B * kHid) return;
  const int r = k / kHid, c = k - r * kHid;
  const float z = Z[k], s = sigmoidf(z);
  const float g = dH[k] * s * (1.f + z * (1.f - s));
  dZf[k] = g;
  const bf16 b = __float2bfloat16_rn(g);
  dZ[k] = b;
  dZt[(int64_t)c * B + r] = b;
}

// db[c] = sum_r dZ[r][c], fixed order per column
__global__ void k_colsum(const float *__restrict__ dZf, int B, float *__restrict__ db) {
  __shared__ float sh[128];
  const int c = blockIdx.x;
  float acc = 0.f;
  for (int r = threadIdx.x; r < B; r += blockDim.x) acc += dZf[(int64_t)r * kHid + c];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) db[c] = sh[0];
}

// acc[0] += sum of count partials, fixed order (one block)
__global__ void k_sum_parts(const float *__restrict__ parts, int count, float *__restrict__ acc) {
  __shared__ float sh[128];
  float a = 0.f;
  for (int i = threadIdx.x; i < count; i += blockDim.x) a += parts[i];
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) acc[0] += sh[0];
}

// Adam (Kingma & Ba) on the FP32 master parameters; weights [out x in] also
// refresh their BF16 copies W^T [out x in] and W [in x out]
__global__ void k_adam(int64_t count, float *__restrict__ p, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, float lr, float b1, float b2,
                       float eps, float c1, float c2, int in_dim, bf16 *__restrict__ Wt,
                       bf16 *__restrict__ W) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= count) return;
  const float gk = g[k];
  const float mk = b1 * m[k] + (1.f - b1) * gk;
  const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
  m[k] = mk;
  v[k] = vk;
  const float pk = p[k] - lr * (mk * c1) / (sqrtf(vk * c2) + eps);
  p[k] = pk;
  if (Wt) {
    const bf16 b = __float2bfloat16_rn(pk);
    const int64_t o = k / in_dim, i = k - o * in_dim;
    Wt[k] = b;
    W[i * kHid + o] = b;
  }
}

__global__ void k_to_bf16_pair(int64_t count, const float *__restrict__ p, int in_dim,
                               bf16 *__restrict__ Wt, bf16 *__restrict__ W) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= count) return;
  const bf16 b = __float2bfloat16_rn(p[k]);
  const int64_t o = k / in_dim, i = k - o * in_dim;
  Wt[k] = b;
  W[i * kHid + o] = b;
}

}  // namespace sur
}  // namespace ggem

// ---- pair-distance histogram of the FP32 pair list -------------------------
namespace ggem {
namespace sur {

__global__ void k_pair_hist(int64_t n, const float4 *__restrict__ pos32,
                            const int32_t *__restrict__ cnt, int W,
                            const uint32_t *__restrict__ list, const float4 *__restrict__ shift,
                            float r_lo, float inv_dr, int nb, unsigned long long *__restrict__ hist) {
  __shared__ unsigned int sh[GGEM_SUR_HIST_BINS];
  if (threadIdx.x < GGEM_SUR_HIST_BINS) sh[threadIdx.x] = 0u;
  __syncthreads();
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x) {
    const float4 pi = pos32[s];
    const int e = cnt[s];
    for (int m = 0; m < e; ++m) {
      const uint32_t en = list[s * (int64_t)W + m];
      const float4 pj = pos32[en >> kCodeBits];
      const float4 o = shift[en & (kMaxCode - 1)];
      const float dx = (pj.x - pi.x) + o.x, dy = (pj.y - pi.y) + o.y, dz = (pj.z - pi.z) + o.z;
      const float r = sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
      const int b = (int)floorf((r - r_lo) * inv_dr);
      if (b >= 0 && b < nb) atomicAdd(&sh[b], 1u);
    }
  }
  __syncthreads();
  if (threadIdx.x < nb && sh[threadIdx.x]) atomicAdd(&hist[threadIdx.x], (unsigned long long)sh[threadIdx.x]);
}

constexpr int kWOff[kLayers] = {0, 128 * 48 + 128, 128 * 48 + 128 + 128 * 128 + 128,
                                128 * 48 + 128 + 2 * (128 * 128 + 128)};
constexpr int kInDim[kLayers] = {kInPad, kHid, kHid, kHid};
inline int bias_off(int l) { return kWOff[l] + kHid * kInDim[l]; }
static_assert(bias_off_d(0) == kWOff[0] + kHid * kInDim[0] &&
                  bias_off_d(1) == kWOff[1] + kHid * kInDim[1] &&
                  bias_off_d(2) == kWOff[2] + kHid * kInDim[2] &&
                  bias_off_d(3) == kWOff[3] + kHid * kInDim[3],
              "bias offsets");

// seeded host generator (SplitMix64) for initialisation and shuffles
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
};

}  // namespace sur
}  // namespace ggem

using namespace ggem;
using namespace ggem::sur;

struct ggem_surrogate {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  DevBuf<float> p, m, v, g;               // master parameters, Adam moments, gradient
  DevBuf<bf16> wt[kLayers], w[kLayers];   // BF16 W^T [out x in] and W [in x out]
  float norm[GGEM_SUR_NORM] = {0};
  DevBuf<float> d_mean, d_inv_std;
  int cap = 0;                            // batch capacity (rows)
  DevBuf<bf16> X, Xt, H[3], Ht[3], dZ, dZt;
  DevBuf<float> Z[kLayers], Y, dZf, dH, loss_part, loss_acc;
  DevBuf<float> xin, yin;
  DevBuf<int32_t> idx;
  DevBuf<int> flag;
  DevBuf<float> yout;                     // fused forward outputs [n x 2]
  int64_t adam_t = 0;
  uint32_t polls = kMaxPolls;             // first-wait poll budget of the products
};

namespace {

struct SurDeviceGuard {
  int prev = -1;
  explicit SurDeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~SurDeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

int sfail(ggem_surrogate *s, int code, const std::string &msg) {
  s->err = msg;
  return code;
}
int scuda(ggem_surrogate *s, cudaError_t e, const char *what) {
  cudaGetLastError();
  s->err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? GGEM_ERR_OOM : GGEM_ERR_CUDA;
}
int slaunch(ggem_surrogate *s, const char *what) {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GGEM_OK : scuda(s, e, what);
}

int ensure_cap(ggem_surrogate *s, int B) {
  if (B <= s->cap) return GGEM_OK;
  cudaError_t e = cudaSuccess;
  const size_t b = (size_t)B;
  if ((e = s->X.ensure(b * kInPad)) || (e = s->Xt.ensure(b * kInPad)) ||
      (e = s->dZ.ensure(b * kHid)) || (e = s->dZt.ensure(b * kHid)) ||
      (e = s->Y.ensure(b * kOut)) || (e = s->dZf.ensure(b * kHid)) ||
      (e = s->dH.ensure(b * kHid)) || (e = s->loss_part.ensure(b * kHid / 256 + 1)))
    return scuda(s, e, "surrogate activations");
  for (int l = 0; l < kLayers; ++l)
    if ((e = s->Z[l].ensure(b * kHid))) return scuda(s, e, "surrogate activations");
  for (int l = 0; l < 3; ++l)
    if ((e = s->H[l].ensure(b * kHid)) || (e = s->Ht[l].ensure(b * kHid)))
      return scuda(s, e, "surrogate activations");
  s->cap = B;
  return GGEM_OK;
}

int gemm(ggem_surrogate *s, const bf16 *A, int lda, const bf16 *Bt, int ldb, float *C, int ldc,
         int M, int N, int K) {
  if (M % kRowBlock || N % 16 || N < 16 || N > kHid || K % 16 || K <= 0 || lda % 8 || ldb % 8)
    return sfail(s, GGEM_ERR_BAD_ARG, "surrogate product shape");
  k_gemm_bf16<<<M / kRowBlock, 128, 0, s->stream>>>(A, lda, Bt, ldb, C, ldc, N, K, s->polls,
                                                    s->flag.p);
  return slaunch(s, "tensor-core product");
}

// raw device features d_x [n x 35] through the fused forward kernel into
// d_y [n x 2] (standardised outputs)
int forward_fused(ggem_surrogate *s, const float *d_x, int64_t n, float *d_y) {
  cudaError_t e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kMlpSmem);
  if (e) return scuda(s, e, "network attributes");
  k_mlp_forward<<<(unsigned)((n + kRowBlock - 1) / kRowBlock), kMlpThreads, kMlpSmem,
                  s->stream>>>(
      d_x, (int)n, s->d_mean.p, s->d_inv_std.p, s->wt[0].p, s->wt[1].p, s->wt[2].p, s->wt[3].p,
      s->p.p, d_y, s->polls, s->flag.p);
  return slaunch(s, "network forward");
}

unsigned blocks(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// the staged batch X, Xt (B rows) through the four layers into s->Y
int forward(ggem_surrogate *s, int B) {
  const bf16 *in = s->X.p;
  int in_dim = kInPad;
  for (int l = 0; l < kLayers; ++l) {
    if (int rc = gemm(s, in, in_dim, s->wt[l].p, in_dim, s->Z[l].p, kHid, B, kHid, in_dim))
      return rc;
    const bool hidden = l < kLayers - 1;
    k_bias_act<<<blocks((int64_t)B * kHid), 256, 0, s->stream>>>(
        s->Z[l].p, s->p.p + bias_off(l), B, hidden ? 1 : 0, hidden ? s->H[l].p : nullptr,
        hidden ? s->Ht[l].p : nullptr, s->Y.p);
    if (int rc = slaunch(s, "bias/activation")) return rc;
    if (hidden) {
      in = s->H[l].p;
      in_dim = kHid;
    }
  }
  return GGEM_OK;
}

// gradient of the loss over n valid rows of the staged batch into s->g
int backward(ggem_surrogate *s, int B, int n, const int32_t *d_idx, const float *d_T,
             float *d_loss) {
  const unsigned nb = blocks((int64_t)B * kHid);
  k_loss_grad<<<nb, 256, 0, s->stream>>>(s->Y.p, d_T, d_idx, n, B, s->dZf.p, s->dZ.p, s->dZt.p,
                                         s->loss_part.p);
  if (int rc = slaunch(s, "loss gradient")) return rc;
  if (d_loss) {
    k_sum_parts<<<1, 128, 0, s->stream>>>(s->loss_part.p, (int)nb, d_loss);
    if (int rc = slaunch(s, "loss sum")) return rc;
  }
  for (int l = kLayers - 1; l >= 0; --l) {
    const int in_dim = kInDim[l];
    const bf16 *prevT = l > 0 ? s->Ht[l - 1].p : s->Xt.p;
    // dW^T [128 x in] = dZ^T [128 x B] * prev [B x in]
    if (int rc = gemm(s, s->dZt.p, B, prevT, B, s->g.p + kWOff[l], in_dim, kHid, in_dim, B))
      return rc;
    k_colsum<<<kHid, 128, 0, s->stream>>>(s->dZf.p, B, s->g.p + bias_off(l));
    if (int rc = slaunch(s, "bias gradient")) return rc;
    if (l == 0) break;
    // dH [B x in] = dZ [B x 128] * W [in x 128]^T
    if (int rc = gemm(s, s->dZ.p, kHid, s->w[l].p, kHid, s->dH.p, kHid, B, in_dim, kHid))
      return rc;
    k_act_back<<<nb, 256, 0, s->stream>>>(s->dH.p, s->Z[l - 1].p, B, s->dZf.p, s->dZ.p,
                                          s->dZt.p);
    if (int rc = slaunch(s, "activation gradient")) return rc;
  }
  return GGEM_OK;
}

}  // namespace

namespace {

int upload_bf16_copies(ggem_surrogate *s) {
  for (int l = 0; l < kLayers; ++l) {
    const int64_t cnt = (int64_t)kHid * kInDim[l];
    k_to_bf16_pair<<<blocks(cnt), 256, 0, s->stream>>>(cnt, s->p.p + kWOff[l], kInDim[l],
                                                       s->wt[l].p, s->w[l].p);
    if (int rc = slaunch(s, "bf16 weights")) return rc;
  }
  return GGEM_OK;
}

int upload_norm(ggem_surrogate *s) {
  float inv[kIn];
  for (int c = 0; c < kIn; ++c) {
    const float sd = s->norm[kIn + c];
    inv[c] = sd > 0.f ? 1.f / sd : 1.f;
  }
  cudaError_t e;
  if ((e = cudaMemcpyAsync(s->d_mean.p, s->norm, sizeof(float) * kIn, cudaMemcpyHostToDevice,
                           s->stream)) ||
      (e = cudaMemcpyAsync(s->d_inv_std.p, inv, sizeof(float) * kIn, cudaMemcpyHostToDevice,
                           s->stream)) ||
      (e = cudaStreamSynchronize(s->stream)))
    return scuda(s, e, "normalisation");
  return GGEM_OK;
}

int check_flag(ggem_surrogate *s) {
  int f = 0;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(&f, s->flag.p, sizeof(int), cudaMemcpyDeviceToHost, s->stream)) ||
      (e = cudaStreamSynchronize(s->stream)))
    return scuda(s, e, "surrogate status");
  if (f & kErrTimeout) return sfail(s, GGEM_ERR_TIMEOUT, "tensor-core product timed out");
  return GGEM_OK;
}

// stage rows [0, n) of device features x (through idx when given) as batch B
int stage(ggem_surrogate *s, const float *d_x, const int32_t *d_idx, int n, int B) {
  k_stage_inputs<<<blocks((int64_t)B * kInPad), 256, 0, s->stream>>>(
      d_x, d_idx, n, B, s->d_mean.p, s->d_inv_std.p, s->X.p, s->Xt.p);
  return slaunch(s, "stage inputs");
}

int round_rows(int64_t n) { return (int)((n + kRowBlock - 1) / kRowBlock * kRowBlock); }

}  // namespace

extern "C" ggem_surrogate *ggem_surrogate_create(int device, uint64_t seed) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    return nullptr;
  }
  SurDeviceGuard dg(device);
  ggem_surrogate *s = new ggem_surrogate();
  s->device = device;
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) ||
      (e = s->p.ensure(GGEM_SUR_PARAMS)) || (e = s->m.ensure(GGEM_SUR_PARAMS)) ||
      (e = s->v.ensure(GGEM_SUR_PARAMS)) || (e = s->g.ensure(GGEM_SUR_PARAMS)) ||
      (e = s->d_mean.ensure(kIn)) || (e = s->d_inv_std.ensure(kIn)) ||
      (e = s->flag.ensure(1)) || (e = s->loss_acc.ensure(4096))) {
    cudaGetLastError();
    ggem_surrogate_destroy(s);
    return nullptr;
  }
  (void)e;
  for (int l = 0; l < kLayers; ++l) {
    if ((e = s->wt[l].ensure((size_t)kHid * kInDim[l])) ||
        (e = s->w[l].ensure((size_t)kHid * kInDim[l]))) {
      cudaGetLastError();
      ggem_surrogate_destroy(s);
      return nullptr;
    }
  }
  // Glorot-uniform weights over the real fan-in / fan-out, zero biases and
  // zero padding (input columns >= 35, output rows >= 2)
  std::vector<float> p(GGEM_SUR_PARAMS, 0.f);
  Rng rng(seed);
  for (int l = 0; l < kLayers; ++l) {
    const int fin = l == 0 ? kIn : kHid, fout = l == kLayers - 1 ? kOut : kHid;
    const double lim = std::sqrt(6.0 / (fin + fout));
    for (int o = 0; o < fout; ++o)
      for (int i = 0; i < fin; ++i)
        p[kWOff[l] + o * kInDim[l] + i] = (float)((2.0 * rng.uniform() - 1.0) * lim);
  }
  for (int c = 0; c < kIn; ++c) s->norm[kIn + c] = 1.f;
  s->norm[2 * kIn + 2] = s->norm[2 * kIn + 3] = 1.f;
  if (ggem_surrogate_set_params(s, p.data()) || upload_norm(s) ||
      cudaMemsetAsync(s->flag.p, 0, sizeof(int), s->stream)) {
    ggem_surrogate_destroy(s);
    return nullptr;
  }
  return s;
}

extern "C" void ggem_surrogate_destroy(ggem_surrogate *s) {
  if (!s) return;
  {
    SurDeviceGuard dg(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    s->p.release();
    s->m.release();
    s->v.release();
    s->g.release();
    for (int l = 0; l < kLayers; ++l) {
      s->wt[l].release();
      s->w[l].release();
      s->Z[l].release();
    }
    for (int l = 0; l < 3; ++l) {
      s->H[l].release();
      s->Ht[l].release();
    }
    s->X.release();
    s->Xt.release();
    s->dZ.release();
    s->dZt.release();
    s->Y.release();
    s->dZf.release();
    s->dH.release();
    s->loss_part.release();
    s->loss_acc.release();
    s->xin.release();
    s->yin.release();
    s->idx.release();
    s->flag.release();
    s->yout.release();
    s->d_mean.release();
    s->d_inv_std.release();
    if (s->stream) cudaStreamDestroy(s->stream);
  }
  delete s;
}

extern "C" const char *ggem_surrogate_last_error(const ggem_surrogate *s) {
  return s ? s->err.c_str() : "null surrogate";
}

extern "C" int ggem_surrogate_set_norm(ggem_surrogate *s, const float *norm) {
  if (!s || !norm) return GGEM_ERR_BAD_ARG;
  SurDeviceGuard dg(s->device);
  std::memcpy(s->norm, norm, sizeof(s->norm));
  return upload_norm(s);
}

extern "C" int ggem_surrogate_get_norm(const ggem_surrogate *s, float *norm) {
  if (!s || !norm) return GGEM_ERR_BAD_ARG;
  std::memcpy(norm, s->norm, sizeof(s->norm));
  return GGEM_OK;
}

extern "C" int ggem_surrogate_set_params(ggem_surrogate *s, const float *params) {
  if (!s || !params) return GGEM_ERR_BAD_ARG;
  SurDeviceGuard dg(s->device);
  cudaError_t e;
  if ((e = cudaMemcpyAsync(s->p.p, params, sizeof(float) * GGEM_SUR_PARAMS,
                           cudaMemcpyHostToDevice, s->stream)) ||
      (e = cudaMemsetAsync(s->m.p, 0, sizeof(float) * GGEM_SUR_PARAMS, s->stream)) ||
      (e = cudaMemsetAsync(s->v.p, 0, sizeof(float) * GGEM_SUR_PARAMS, s->stream)))
    return scuda(s, e, "parameters");
  s->adam_t = 0;
  if (int rc = upload_bf16_copies(s)) return rc;
  if ((e = cudaStreamSynchronize(s->stream))) return scuda(s, e, "parameters");
  return GGEM_OK;
}

extern "C" int ggem_surrogate_get_params(ggem_surrogate *s, float *params) {
  if (!s || !params) return GGEM_ERR_BAD_ARG;
  SurDeviceGuard dg(s->device);
  cudaError_t e;
  if ((e = cudaMemcpyAsync(params, s->p.p, sizeof(float) * GGEM_SUR_PARAMS,
                           cudaMemcpyDeviceToHost, s->stream)) ||
      (e = cudaStreamSynchronize(s->stream)))
    return scuda(s, e, "parameters");
  return GGEM_OK;
}

namespace {

// standardised targets (n x 2) and raw features (n x 35) on the device
int upload_data(ggem_surrogate *s, const float *X, const float *Y, int64_t n) {
  std::vector<float> t(Y ? (size_t)n * kOut : 0);
  for (int64_t r = 0; r < (Y ? n : 0); ++r)
    for (int c = 0; c < kOut; ++c) {
      const float sd = s->norm[2 * kIn + kOut + c];
      t[r * kOut + c] = (Y[r * kOut + c] - s->norm[2 * kIn + c]) / (sd > 0.f ? sd : 1.f);
    }
  cudaError_t e;
  if ((e = s->xin.ensure((size_t)n * kIn)) ||
      (Y && (e = s->yin.ensure((size_t)n * kOut))))
    return scuda(s, e, "surrogate data");
  if ((e = cudaMemcpyAsync(s->xin.p, X, sizeof(float) * n * kIn, cudaMemcpyHostToDevice,
                           s->stream)))
    return scuda(s, e, "surrogate data");
  if (Y && (e = cudaMemcpyAsync(s->yin.p, t.data(), sizeof(float) * n * kOut,
                                cudaMemcpyHostToDevice, s->stream)))
    return scuda(s, e, "surrogate data");
  if ((e = cudaStreamSynchronize(s->stream))) return scuda(s, e, "surrogate data");
  return GGEM_OK;
}

int adam_step(ggem_surrogate *s, float lr) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  s->adam_t += 1;
  const float c1 = 1.f / (1.f - std::pow(b1, (float)s->adam_t));
  const float c2 = 1.f / (1.f - std::pow(b2, (float)s->adam_t));
  for (int l = 0; l < kLayers; ++l) {
    const int64_t cw = (int64_t)kHid * kInDim[l];
    k_adam<<<blocks(cw), 256, 0, s->stream>>>(cw, s->p.p + kWOff[l], s->g.p + kWOff[l],
                                              s->m.p + kWOff[l], s->v.p + kWOff[l], lr, b1, b2,
                                              eps, c1, c2, kInDim[l], s->wt[l].p, s->w[l].p);
    k_adam<<<1, kHid, 0, s->stream>>>(kHid, s->p.p + bias_off(l), s->g.p + bias_off(l),
                                      s->m.p + bias_off(l), s->v.p + bias_off(l), lr, b1, b2,
                                      eps, c1, c2, 1, nullptr, nullptr);
  }
  return slaunch(s, "adam");
}

}  // namespace

extern "C" int ggem_surrogate_train(ggem_surrogate *s, const float *X, const float *Y, int64_t n,
                                    int epochs, int batch, float lr, uint64_t seed, float *loss) {
  if (!s || !X || !Y || n <= 0 || epochs < 1 || batch < kRowBlock || batch % kRowBlock ||
      !(lr > 0.f) || n > (int64_t)1 << 30)
    return s ? sfail(s, GGEM_ERR_BAD_ARG, "train: bad arguments (batch a multiple of 128)")
             : GGEM_ERR_BAD_ARG;
  SurDeviceGuard dg(s->device);
  if (int rc = ensure_cap(s, batch)) return rc;
  if (int rc = upload_data(s, X, Y, n)) return rc;
  cudaError_t e;
  if ((e = s->idx.ensure((size_t)n)) || (e = s->loss_acc.ensure((size_t)epochs)))
    return scuda(s, e, "train buffers");
  if ((e = cudaMemsetAsync(s->loss_acc.p, 0, sizeof(float) * epochs, s->stream)) ||
      (e = cudaMemsetAsync(s->flag.p, 0, sizeof(int), s->stream)))
    return scuda(s, e, "train buffers");
  std::vector<int32_t> perm((size_t)n);
  for (int64_t i = 0; i < n; ++i) perm[i] = (int32_t)i;
  Rng rng(seed);
  const int64_t steps_per_epoch = (n + batch - 1) / batch;
  const double total = (double)steps_per_epoch * epochs;
  int64_t step = 0;
  for (int ep = 0; ep < epochs; ++ep) {
    for (int64_t i = n - 1; i > 0; --i) std::swap(perm[i], perm[rng.next() % (uint64_t)(i + 1)]);
    if ((e = cudaMemcpyAsync(s->idx.p, perm.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice,
                             s->stream)) ||
        (e = cudaStreamSynchronize(s->stream)))
      return scuda(s, e, "shuffle");
    for (int64_t b0 = 0; b0 < n; b0 += batch, ++step) {
      const int nb = (int)std::min<int64_t>(batch, n - b0);
      const int B = round_rows(nb);
      const int32_t *ib = s->idx.p + b0;
      if (int rc = stage(s, s->xin.p, ib, nb, B)) return rc;
      if (int rc = forward(s, B)) return rc;
      if (int rc = backward(s, B, nb, ib, s->yin.p, s->loss_acc.p + ep)) return rc;
      // cosine decay to lr / 20
      const float f = (float)(0.05 + 0.95 * 0.5 * (1.0 + std::cos(kPiS * step / total)));
      if (int rc = adam_step(s, lr * f)) return rc;
    }
  }
  if (int rc = check_flag(s)) return rc;
  if (loss) {
    std::vector<float> acc((size_t)epochs);
    if ((e = cudaMemcpyAsync(acc.data(), s->loss_acc.p, sizeof(float) * epochs,
                             cudaMemcpyDeviceToHost, s->stream)) ||
        (e = cudaStreamSynchronize(s->stream)))
      return scuda(s, e, "loss readback");
    // each batch adds sum(err^2); the mean over rows of the per-row sum
    for (int ep = 0; ep < epochs; ++ep) loss[ep] = acc[ep] / (float)n;
  }
  return GGEM_OK;
}

extern "C" int ggem_surrogate_predict(ggem_surrogate *s, const float *X, int64_t n, float *Y) {
  if (!s || !X || !Y || n <= 0 || n > (int64_t)1 << 30) return GGEM_ERR_BAD_ARG;
  SurDeviceGuard dg(s->device);
  if (int rc = upload_data(s, X, nullptr, n)) return rc;
  cudaError_t e;
  if ((e = s->yout.ensure((size_t)n * kOut)) ||
      (e = cudaMemsetAsync(s->flag.p, 0, sizeof(int), s->stream)))
    return scuda(s, e, "predict");
  // one launch: all layers, weights resident in shared memory
  if (int rc = forward_fused(s, s->xin.p, n, s->yout.p)) return rc;
  std::vector<float> out((size_t)n * kOut);
  if ((e = cudaMemcpyAsync(out.data(), s->yout.p, sizeof(float) * n * kOut,
                           cudaMemcpyDeviceToHost, s->stream)) ||
      (e = cudaStreamSynchronize(s->stream)))
    return scuda(s, e, "predict readback");
  if (int rc = check_flag(s)) return rc;
  for (int64_t r = 0; r < n; ++r)
    for (int c = 0; c < kOut; ++c)
      Y[r * kOut + c] = out[r * kOut + c] * s->norm[2 * kIn + kOut + c] + s->norm[2 * kIn + c];
  return GGEM_OK;
}

extern "C" int ggem_surrogate_predict_layers(ggem_surrogate *s, const float *X, int64_t n,
                                             float *Y) {
  if (!s || !X || !Y || n <= 0 || n > (int64_t)1 << 30) return GGEM_ERR_BAD_ARG;
  SurDeviceGuard dg(s->device);
  const int cap = std::max(s->cap, std::min(round_rows(n), 4096));
  if (int rc = ensure_cap(s, cap)) return rc;
  if (int rc = upload_data(s, X, nullptr, n)) return rc;
  cudaError_t e;
  if ((e = cudaMemsetAsync(s->flag.p, 0, sizeof(int), s->stream))) return scuda(s, e, "predict");
  std::vector<float> out((size_t)cap * kOut);
  for (int64_t r0 = 0; r0 < n; r0 += cap) {
    const int nb = (int)std::min<int64_t>(cap, n - r0);
    const int B = round_rows(nb);
    if (int rc = stage(s, s->xin.p + r0 * kIn, nullptr, nb, B)) return rc;
    if (int rc = forward(s, B)) return rc;
    if ((e = cudaMemcpyAsync(out.data(), s->Y.p, sizeof(float) * nb * kOut,
                             cudaMemcpyDeviceToHost, s->stream)) ||
        (e = cudaStreamSynchronize(s->stream)))
      return scuda(s, e, "predict readback");
    for (int r = 0; r < nb; ++r)
      for (int c = 0; c < kOut; ++c)
        Y[(r0 + r) * kOut + c] =
            out[r * kOut + c] * s->norm[2 * kIn + kOut + c] + s->norm[2 * kIn + c];
  }
  return check_flag(s);
}

extern "C" int ggem_surrogate_set_poll_budget(ggem_surrogate *s, uint32_t polls) {
  if (!s) return GGEM_ERR_BAD_ARG;
  s->polls = polls;
  return GGEM_OK;
}

extern "C" int ggem_surrogate_time_forward(ggem_surrogate *s, int64_t n, int reps, double *ms) {
  if (!s || n <= 0 || n > (int64_t)1 << 20 || reps < 1 || !ms) return GGEM_ERR_BAD_ARG;
  SurDeviceGuard dg(s->device);
  cudaError_t e;
  if ((e = s->xin.ensure((size_t)n * kIn)) || (e = s->yout.ensure((size_t)n * kOut)) ||
      (e = cudaMemsetAsync(s->xin.p, 0, sizeof(float) * n * kIn, s->stream)) ||
      (e = cudaMemsetAsync(s->flag.p, 0, sizeof(int), s->stream)))
    return scuda(s, e, "forward timing");
  if (int rc = forward_fused(s, s->xin.p, n, s->yout.p)) return rc;  // warm-up
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, s->stream);
  int rc = GGEM_OK;
  for (int r = 0; r < reps && !rc; ++r) rc = forward_fused(s, s->xin.p, n, s->yout.p);
  cudaEventRecord(b, s->stream);
  cudaEventSynchronize(b);
  float t = 0.f;
  cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  *ms = t / reps;
  return check_flag(s);
}

extern "C" int ggem_surrogate_gradient(ggem_surrogate *s, const float *X, const float *Y,
                                       int64_t n, float *loss, float *grad) {
  if (!s || !X || !Y || n <= 0 || n > 4096 || !grad) return GGEM_ERR_BAD_ARG;
  SurDeviceGuard dg(s->device);
  const int B = round_rows(n);
  if (int rc = ensure_cap(s, B)) return rc;
  if (int rc = upload_data(s, X, Y, n)) return rc;
  cudaError_t e;
  if ((e = cudaMemsetAsync(s->flag.p, 0, sizeof(int), s->stream)) ||
      (e = cudaMemsetAsync(s->loss_acc.p, 0, sizeof(float), s->stream)))
    return scuda(s, e, "gradient");
  if (int rc = stage(s, s->xin.p, nullptr, (int)n, B)) return rc;
  if (int rc = forward(s, B)) return rc;
  if (int rc = backward(s, B, (int)n, nullptr, s->yin.p, s->loss_acc.p)) return rc;
  float l = 0.f;
  if ((e = cudaMemcpyAsync(grad, s->g.p, sizeof(float) * GGEM_SUR_PARAMS, cudaMemcpyDeviceToHost,
                           s->stream)) ||
      (e = cudaMemcpyAsync(&l, s->loss_acc.p, sizeof(float), cudaMemcpyDeviceToHost, s->stream)) ||
      (e = cudaStreamSynchronize(s->stream)))
    return scuda(s, e, "gradient readback");
  if (loss) *loss = l / (float)n;
  return check_flag(s);
}

extern "C" int ggem_surrogate_features(ggem_ctx *ctx, double chain_fraction, float *features) {
  if (!ctx || !features) return GGEM_ERR_BAD_ARG;
  if (int rc = ggem::settle_list(ctx)) return rc;
  if (ctx->prm.precision != GGEM_FP32 || !ctx->list_built)
    return fail(ctx, GGEM_ERR_BAD_ARG, "features need the FP32 pair list (build cells first)");
  SurDeviceGuard dg(ctx->device);
  const double a = ctx->prm.br0 > 0 ? ctx->prm.br0 : 1.0;
  const double r_lo = 2.0 * a, r_hi = std::sqrt(ctx->rc2);
  const Grid &g = ctx->grid;
  const double vol = g.L[0] * g.L[1] * g.L[2];
  const int64_t n = ctx->n;
  std::vector<unsigned long long> hist(GGEM_SUR_HIST_BINS, 0ull);
  if (n > 0) {
    DevBuf<unsigned long long> d_hist;
    cudaError_t e;
    if ((e = d_hist.ensure(GGEM_SUR_HIST_BINS)) ||
        (e = cudaMemsetAsync(d_hist.p, 0, sizeof(unsigned long long) * GGEM_SUR_HIST_BINS,
                             ctx->stream)))
      return cuda_fail(ctx, e, "histogram");
    const float inv_dr = (float)(GGEM_SUR_HIST_BINS / (r_hi - r_lo));
    const unsigned nblk = (unsigned)std::min<int64_t>((n + 255) / 256, 4096);
    k_pair_hist<<<nblk, 256, 0, ctx->stream>>>(n, ctx->pos32.p, ctx->nb_cnt.p, ctx->nb_w,
                                               ctx->nb_list.p, ctx->d_shift.p, (float)r_lo,
                                               inv_dr, GGEM_SUR_HIST_BINS, d_hist.p);
    if (int rc = check_launch(ctx, "histogram")) return rc;
    if ((e = cudaMemcpyAsync(hist.data(), d_hist.p, sizeof(unsigned long long) * GGEM_SUR_HIST_BINS,
                             cudaMemcpyDeviceToHost, ctx->stream)) ||
        (e = cudaStreamSynchronize(ctx->stream)))
      return cuda_fail(ctx, e, "histogram");
  }
  const double rho = vol > 0 ? (double)n / vol : 0.0;
  features[0] = (float)(n * 4.0 / 3.0 * kPiS * a * a * a / (vol > 0 ? vol : 1.0));
  features[1] = (float)std::log((double)std::max<int64_t>(n, 1));
  const double dr = (r_hi - r_lo) / GGEM_SUR_HIST_BINS;
  for (int b = 0; b < GGEM_SUR_HIST_BINS; ++b) {
    const double r0 = r_lo + b * dr, r1 = r0 + dr;
    const double ideal = n * rho * 4.0 / 3.0 * kPiS * (r1 * r1 * r1 - r0 * r0 * r0);
    features[2 + b] = (float)(ideal > 0 ? hist[b] / ideal : 0.0);
  }
  features[2 + GGEM_SUR_HIST_BINS] = (float)chain_fraction;
  return GGEM_OK;
}

extern "C" int ggem_surrogate_interval(ggem_ctx *ctx, ggem_surrogate *s, double chain_fraction,
                                       double margin_lo, double margin_hi, double *eig_min,
                                       double *eig_max) {
  if (!ctx || !s || !eig_min || !eig_max || !(margin_lo >= 0) || !(margin_hi >= 0))
    return GGEM_ERR_BAD_ARG;
  float f[GGEM_SUR_FEATURES], y[GGEM_SUR_OUTPUTS];
  if (int rc = ggem_surrogate_features(ctx, chain_fraction, f)) return rc;
  if (int rc = ggem_surrogate_predict(s, f, 1, y)) return fail(ctx, rc, s->err);
  *eig_min = std::exp((double)y[0] - margin_lo);
  *eig_max = std::exp((double)y[1] + margin_hi);
  return GGEM_OK;
}
