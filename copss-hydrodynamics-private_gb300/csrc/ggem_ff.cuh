// ggem_ff.cuh -- float-float arithmetic for the device code.
//
// GB300 issues FP64 at a small fraction of the FP32 rate.  These helpers
// keep sums and products of FP64 values accurate to ~47 bits with FP32 and
// integer instructions only: error-free transformations (Knuth's TwoSum,
// products with fused multiply-adds) and integer splitting of doubles.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "ggem_internal.cuh"

namespace ggem {

// s + e == a + b exactly (Knuth's TwoSum)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (hi, lo) += (h2, l2), renormalised so that |lo| <= ulp(hi) / 2
__device__ __forceinline__ void ff_add(float &hi, float &lo, float h2, float l2) {
  float s, e;
  two_sum(hi, h2, s, e);
  e += lo + l2;
  hi = s + e;
  lo = e - (hi - s);
}

// float -> double from the bit fields with integer operations (exact for
// normal floats; subnormals, below 1.2e-38, become signed zero)
__device__ __forceinline__ double f2d_bits(float x) {
  const uint32_t b = __float_as_uint(x);
  const uint32_t sign = b & 0x80000000u, ex = (b >> 23) & 0xffu, m = b & 0x7fffffu;
  if (ex == 0u) return __hiloint2double((int)sign, 0);
  const uint32_t e64 = ex == 0xffu ? 0x7ffu : ex + (1023u - 127u);
  return __hiloint2double((int)(sign | (e64 << 20) | (m >> 3)), (int)(m << 29));
}

// A double split with integer operations into a truncated float and the
// float of its remaining 29 mantissa bits (about 47 bits in all).
__device__ __forceinline__ void split_f64(double v, float &hi, float &lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ffu) - 1023;
  if (e < -126 || e > 127) {  // zero, tiny, huge or not finite: one float
    hi = d2f_bits(v);
    lo = 0.f;
    return;
  }
  hi = __uint_as_float(sign | ((uint32_t)(e + 127) << 23) | (uint32_t)((b >> 29) & 0x7fffffu));
  // the rest: (low 29 mantissa bits) x 2^(e - 52), zero below the float range
  const float scale = e - 52 >= -126 ? __uint_as_float((uint32_t)(e - 52 + 127) << 23) : 0.f;
  const float r = (float)(uint32_t)(b & 0x1fffffffu) * scale;
  lo = sign ? -r : r;
}

// (ah + al)(bh + bl) as a float-float value (the al bl term is below it)
__device__ __forceinline__ void ff_prod(float ah, float al, float bh, float bl, float &ph,
                                        float &pl) {
  ph = ah * bh;
  pl = fmaf(ah, bl, fmaf(al, bh, fmaf(ah, bh, -ph)));
}

// a . b for doubles, as a float-float value
__device__ __forceinline__ void dot_ff(double a, double b, float &ph, float &pl) {
  float ah, al, bh, bl;
  split_f64(a, ah, al);
  split_f64(b, bh, bl);
  ff_prod(ah, al, bh, bl, ph, pl);
}

__device__ __forceinline__ void sq_ff(double a, float &ph, float &pl) {
  float ah, al;
  split_f64(a, ah, al);
  ff_prod(ah, al, ah, al, ph, pl);
}


// float-float sum over the warp by a fixed butterfly (every lane receives
// the same value: TwoSum's error term is exact, so both lanes of a pair
// compute the same sum)
__device__ __forceinline__ void warp_ff_sum(float &hi, float &lo) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
    const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
    ff_add(hi, lo, h2, l2);
  }
}

// float-float sum over the block (blockDim.x a multiple of 32, at most
// 1024): warp butterflies, then the warps' sums in order; the value as a
// double is returned to thread 0.  Every thread calls it; sh holds 32
// float2 and is free again when it returns.
__device__ __forceinline__ double block_ff_sum(float hi, float lo, float2 *sh) {
  warp_ff_sum(hi, lo);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = make_float2(hi, lo);
  __syncthreads();
  double out = 0.0;
  if (threadIdx.x == 0) {
    float th = sh[0].x, tl = sh[0].y;
    const int nw = (int)(blockDim.x >> 5);
    for (int w = 1; w < nw; ++w) ff_add(th, tl, sh[w].x, sh[w].y);
    out = f2d_bits(th) + f2d_bits(tl);
  }
  __syncthreads();
  return out;
}

}  // namespace ggem
