// ggem_spread_elem.cu -- the Gaussian force spreading onto the quadrature
// points of every element of the mesh, brick by brick.
//
// rho(q) = sum_j g_alpha(q - x_j) f_j with
// g_alpha(r) = alpha^3 pi^{-3/2} e^{-alpha^2 r^2} (2.5 - alpha^2 r^2)
// (GGEMStokes::smoothed_force_exp, ggem_stokes.C:117-128), summed for each
// quadrature point of element e over the particles of e's element
// neighbour list (AssembleStokes::compute_element_rhs,
// assemble_stokes.C:645-662; the list of point_mesh.C:652-799: the
// particles of every element whose centroid lies within search_radius_e of
// e's centroid, e itself included).
//
// Reference mode only: elements are the cells of the context's grid and a
// particle belongs to e's list exactly when the offset between its element
// and e lies in the element stencil (the host's centroid test), so the
// list test is integer arithmetic on element coordinates.
//
// One CTA takes a brick of B x B x B elements.  It stages every particle of
// the brick's stencil-dilated region (contiguous slot ranges, one per row of
// elements along x) into shared memory once; each warp then takes one
// element at a time: its lanes test the staged particles' element offsets
// against the stencil bitmap and compact the members into a per-warp list,
// then 32 / nq lanes per quadrature point sum g f over the members.  The
// gathers of a particle are shared by the brick's 64 elements instead of
// being repeated per element, and the ~1000 stencil elements of each
// element (most of them empty) are never visited one by one.
//
// Two arithmetic paths over the same lists:
//  * FP64: the oracle's arithmetic (minimum-image point_vector in FP64,
//    exp in FP64);
//  * FP32: positions relative to the element centres (|x| <= h/2), the
//    element offset as an exact FP32 shift, e^{-alpha^2 s} on the
//    special-function unit with the exponent split into hi + lo parts,
//    block-Kahan sums per lane and a float-float combine of the lanes.
// Algorithmic work per (quadrature point, listed particle): 20 flops + 1 exp.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ggem_ff.cuh"
#include "ggem_internal.cuh"

namespace ggem {
namespace {

constexpr int kSpThreads = 256;
constexpr int kSpWarps = kSpThreads / 32;
constexpr int kSpCap32 = 512;    // staged particles per pass (FP32 records, 32 B)
constexpr int kSpCap64 = 256;    // staged particles per pass (FP64 records, 64 B)
constexpr int kSpMaxSeg = 2048;  // contiguous slot ranges of one dilated brick
constexpr int kSpMaxExt = 32;    // dilated brick extent per axis (5-bit coordinates)
constexpr size_t kSpRecBytes = 16384;
constexpr int kSpMaxWords = 1024;  // stencil bitmap words (32768 element offsets)
constexpr int kSpQueue = 64;      // queued members per warp (< 32 left + 32 new)
constexpr size_t kSpShared = kSpRecBytes + kSpWarps * (32 * sizeof(float4) + kSpQueue * sizeof(uint32_t)) +
                             2 * (kSpMaxSeg + 1) * sizeof(int32_t) +
                             kSpMaxWords * sizeof(uint32_t);

struct SpreadGeo {
  Grid g;
  int lo[3], hi[3], dim[3];  // element-offset range of the stencil bitmap
  int nwords;                // 32-bit words of the bitmap
  int pad;                   // padded bitmap: bit (i + B - 1) + 32 (j + B - 1) + 1024 (k + B - 1)
                             // for the stencil offset index (i, j, k), read with the packed
                             // frame coordinates of a particle minus one value per element
  int B;                     // brick edge in elements
  int nb[3];                 // bricks per axis
  int nq;                    // quadrature points per element (<= 32)
  int lq;                    // lanes per quadrature point (32 / next power of two >= nq)
  float shift[3][kSpMaxExt]; // (float)(d h) for d in [lo, hi], per axis
  float L32[3];
  // FP32 constants: e^{-alpha^2 s} = 2^{s (e_hi + e_lo)}, g = E (c25 - c1 s)
  float e_hi, e_lo, c25, c1;
};

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ void kahan_acc(float &sum, float &comp, float v) {
  const float y = v - comp;
  const float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

// the brick's dilated frame along one axis: start F (unwrapped) and extent E;
// full = the frame covers the whole periodic axis (coordinates absolute,
// offsets wrapped)
struct Frame {
  int F, E, full;
};

__device__ __forceinline__ Frame brick_frame(const SpreadGeo &sg, int d, int b0, int b1) {
  Frame f;
  const int nc = sg.g.nc[d];
  const int ext = (b1 - b0) + (sg.hi[d] - sg.lo[d]);
  if (sg.g.periodic[d] && ext >= nc) {
    f.F = 0;
    f.E = nc;
    f.full = 1;
  } else if (sg.g.periodic[d]) {
    f.F = b0 + sg.lo[d];
    f.E = ext;
    f.full = 0;
  } else {
    const int a = max(0, b0 + sg.lo[d]), z = min(nc - 1, b1 - 1 + sg.hi[d]);
    f.F = a;
    f.E = z - a + 1;
    f.full = 0;
  }
  return f;
}

__device__ __forceinline__ int wrap_cell(int k, int n) {
  k %= n;
  return k < 0 ? k + n : k;
}

// offset d (frame coordinates) of a staged particle from the element, or
// a value outside [lo, hi] when it is no stencil offset
__device__ __forceinline__ int axis_offset(const SpreadGeo &sg, int d, int us, int ue, int full) {
  int o = us - ue;
  if (full) {
    const int nc = sg.g.nc[d];
    if (o > nc / 2) o -= nc;
    else if (o < -((nc - 1) / 2)) o += nc;
  }
  return o;
}

// ANYFULL: some brick frame spans a whole periodic axis (small meshes);
// without it the wrapped-offset and minimum-image code is compiled out
template <bool F32, bool ANYFULL, bool PAD>
__global__ void __launch_bounds__(kSpThreads, F32 ? 4 : 1) k_spread_brick(
    SpreadGeo sg, DevConsts K, const int32_t *__restrict__ start,
    const float4 *__restrict__ pos32, const double4_32a *__restrict__ pos64,
    const double *__restrict__ f_slot, const float4 *__restrict__ q_rel,
    const double *__restrict__ q_xyz, const uint32_t *__restrict__ bits,
    double *__restrict__ rho, unsigned long long *__restrict__ pairs) {
  extern __shared__ __align__(16) unsigned char sp_smem[];
  constexpr int CAP = F32 ? kSpCap32 : kSpCap64;
  // FP32 records as two arrays, positions [CAP] then forces [CAP]: the 16-byte
  // stride spreads the four members a warp reads at once over more banks
  // than 32-byte records would
  float4 *rec32 = reinterpret_cast<float4 *>(sp_smem);        // [2][CAP]
  double4_32a *rec64 = reinterpret_cast<double4_32a *>(sp_smem);  // [CAP][2]
  float4 *batch = reinterpret_cast<float4 *>(sp_smem + kSpRecBytes);       // [warps][32]
  uint32_t *queue = reinterpret_cast<uint32_t *>(batch + kSpWarps * 32);  // [warps][kSpQueue]
  int32_t *seg_begin = reinterpret_cast<int32_t *>(queue + kSpWarps * kSpQueue);
  int32_t *seg_pre = seg_begin + kSpMaxSeg + 1;
  uint32_t *s_bits = reinterpret_cast<uint32_t *>(seg_pre + kSpMaxSeg + 1);
  // the element-offset shifts and the stencil bitmap in shared memory: lanes
  // index them with different offsets (divergent constant-bank reads would
  // serialise)
  __shared__ float s_shift[3][kSpMaxExt];
  __shared__ int s_total;
  for (int k = threadIdx.x; k < 3 * kSpMaxExt; k += kSpThreads)
    s_shift[k / kSpMaxExt][k % kSpMaxExt] = sg.shift[k / kSpMaxExt][k % kSpMaxExt];
  for (int k = threadIdx.x; k < sg.nwords; k += kSpThreads) s_bits[k] = bits[k];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int B = sg.B;
  int bid = blockIdx.x;
  const int bx = bid % sg.nb[0];
  bid /= sg.nb[0];
  const int by = bid % sg.nb[1];
  const int bz = bid / sg.nb[1];
  const int e0[3] = {bx * B, by * B, bz * B};
  const int e1[3] = {min(e0[0] + B, sg.g.nc[0]), min(e0[1] + B, sg.g.nc[1]),
                     min(e0[2] + B, sg.g.nc[2])};
  Frame fr[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    fr[d] = brick_frame(sg, d, e0[d], e1[d]);
    if (!ANYFULL) fr[d].full = 0;  // the host found no frame that spans an axis
  }
  // x segments per row: a periodic frame that is not the whole axis may
  // wrap once; others are one range
  const int xa = fr[0].F, xz = fr[0].F + fr[0].E - 1;
  const int nseg_x = (!fr[0].full && sg.g.periodic[0] && (xa < 0 || xz >= sg.g.nc[0])) ? 2 : 1;
  const int nrow = fr[1].E * fr[2].E;
  const int nseg = nrow * nseg_x;  // <= kSpMaxSeg (checked on the host)
  // slot range of every segment and the running prefix (block scan)
  for (int s0 = 0; s0 < nseg; s0 += kSpThreads) {
    const int s = s0 + threadIdx.x;
    int b = 0, cnt = 0;
    if (s < nseg) {
      const int row = s / nseg_x, k = s - row * nseg_x;
      const int uy = row % fr[1].E, uz = row / fr[1].E;
      const int cy = fr[1].full ? uy : (sg.g.periodic[1] ? wrap_cell(fr[1].F + uy, sg.g.nc[1])
                                                          : fr[1].F + uy);
      const int cz = fr[2].full ? uz : (sg.g.periodic[2] ? wrap_cell(fr[2].F + uz, sg.g.nc[2])
                                                          : fr[2].F + uz);
      int x0, x1;  // absolute cells [x0, x1]
      if (nseg_x == 1) {
        x0 = fr[0].full ? 0 : (sg.g.periodic[0] ? wrap_cell(xa, sg.g.nc[0]) : xa);
        x1 = x0 + fr[0].E - 1;
      } else if (k == 0) {
        x0 = wrap_cell(xa, sg.g.nc[0]);
        x1 = sg.g.nc[0] - 1;
      } else {
        x0 = 0;
        x1 = wrap_cell(xz, sg.g.nc[0]);
      }
      const int64_t rowc = (int64_t)sg.g.nc[0] * (cy + (int64_t)sg.g.nc[1] * cz);
      b = start[rowc + x0];
      cnt = start[rowc + x1 + 1] - b;
    }
    // block exclusive scan of cnt
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    __shared__ int wsum[kSpWarps];
    const int carry = (s0 == 0) ? 0 : seg_pre[s0];  // written before the last barrier
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    int before = carry;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    if (s < nseg) {
      seg_begin[s] = b;
      seg_pre[s] = before + incl - cnt;
    }
    if (threadIdx.x == kSpThreads - 1) seg_pre[min(s0 + kSpThreads, nseg)] = before + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) s_total = seg_pre[nseg];
  __syncthreads();
  const int total = s_total;
  // elements of this brick, one warp at a time
  const int ebx = e1[0] - e0[0], eby = e1[1] - e0[1], ebz = e1[2] - e0[2];
  const int nel = ebx * eby * ebz;
  const int nq = sg.nq, lq = sg.lq;
  const int qi = lane / lq, sub = lane - qi * lq;
  unsigned long long my_pairs = 0;
  // the warp's member queue: per member its staged index (10 bits) and its
  // element offset (the padded bitmap index, or three 5-bit offsets); each
  // batch of 32 becomes positions in the element's frame (FP32: the staged
  // position plus the offset's shift, formed once per member instead of
  // once per point, one member per lane) with the staged index in .w
  uint32_t *mq = queue + warp * kSpQueue;
  float4 *mb = batch + warp * 32;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int c0 = 0; c0 < total; c0 += CAP) {
    const int cn = min(CAP, total - c0);
    // stage particles [c0, c0 + cn): segment by binary search
    for (int k = threadIdx.x; k < cn; k += kSpThreads) {
      const int v = c0 + k;
      int lo = 0, hi = nseg - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (seg_pre[mid] <= v) lo = mid;
        else hi = mid - 1;
      }
      const int slot = seg_begin[lo] + (v - seg_pre[lo]);
      const int row = lo / nseg_x, kk = lo - row * nseg_x;
      const int uy = row % fr[1].E, uz = row / fr[1].E;
      const float4 p = pos32[slot];
      const int cid = __float_as_int(p.w);
      const int cx = cid % sg.g.nc[0];
      int ux;
      if (fr[0].full) ux = cx;
      else if (!sg.g.periodic[0]) ux = cx - fr[0].F;
      else if (nseg_x == 1) ux = cx - wrap_cell(xa, sg.g.nc[0]);
      else ux = kk == 0 ? cx - wrap_cell(xa, sg.g.nc[0]) : cx + (sg.g.nc[0] - wrap_cell(xa, sg.g.nc[0]));
      const uint32_t u = (uint32_t)ux | ((uint32_t)uy << 5) | ((uint32_t)uz << 10);
      const double *fp = f_slot + 3 * (int64_t)slot;
      if (F32) {
        rec32[k] = make_float4(p.x, p.y, p.z, __uint_as_float(u));
        rec32[kSpCap32 + k] = make_float4(d2f_bits(fp[0]), d2f_bits(fp[1]), d2f_bits(fp[2]), 0.f);
      } else {
        const double4_32a q = pos64[slot];
        rec64[2 * k] = make_double4_32a(q.x, q.y, q.z, __longlong_as_double((long long)u));
        rec64[2 * k + 1] = make_double4_32a(fp[0], fp[1], fp[2], 0.0);
      }
    }
    __syncthreads();
    for (int le = warp; le < nel; le += kSpWarps) {
      const int lx = le % ebx, ly = (le / ebx) % eby, lz = le / (ebx * eby);
      const int ex = e0[0] + lx, ey = e0[1] + ly, ez = e0[2] + lz;
      const int64_t e = ex + (int64_t)sg.g.nc[0] * (ey + (int64_t)sg.g.nc[1] * ez);
      const int uex = fr[0].full ? ex : ex - fr[0].F;
      const int uey = fr[1].full ? ey : ey - fr[1].F;
      const int uez = fr[2].full ? ez : ez - fr[2].F;
      // with the padded bitmap, the packed frame coordinates u of a staged
      // particle minus qe index the bitmap directly (each 5-bit field stays
      // in [0, 32) for every particle of the brick's frame)
      const int qe = (uex + sg.lo[0] - B + 1) + 32 * (uey + sg.lo[1] - B + 1) +
                     1024 * (uez + sg.lo[2] - B + 1);
      const bool qok = qi < nq;
      const int64_t qg = e * nq + (qok ? qi : 0);
      float4 qr = make_float4(0.f, 0.f, 0.f, 0.f);
      double q0 = 0.0, q1 = 0.0, q2 = 0.0;
      if (F32) {
        qr = q_rel[qg];
      } else {
        q0 = q_xyz[3 * qg];
        q1 = q_xyz[3 * qg + 1];
        q2 = q_xyz[3 * qg + 2];
      }
      float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
      float bx_ = 0.f, by_ = 0.f, bz_ = 0.f;
      int blk = 0;
      double ax = 0.0, ay = 0.0, az = 0.0;
      // members: staged particles whose element offset is a stencil offset,
      // queued in staging order and summed 32 at a time; lane (qi, sub)
      // takes members sub, sub + lq, ... of each batch, so every lane sees its
      // members in the order of one pass over the whole member list
      int queued = 0;  // warp-uniform
      for (int k0 = 0; k0 < cn; k0 += 32) {
        const int k = k0 + lane;
        bool in = false;
        uint32_t item = 0;
        if (k < cn) {
          const uint32_t u = F32 ? __float_as_uint(rec32[k].w)
                                 : (uint32_t)__double_as_longlong(rec64[2 * k].w);
          if (PAD) {
            const int idx = (int)u - qe;
            in = (s_bits[idx >> 5] >> (idx & 31)) & 1u;
            item = (uint32_t)k | ((uint32_t)idx << 10);
          } else {
            const int ix =
                axis_offset(sg, 0, (int)(u & 31u), uex, ANYFULL && fr[0].full) - sg.lo[0];
            const int iy =
                axis_offset(sg, 1, (int)((u >> 5) & 31u), uey, ANYFULL && fr[1].full) - sg.lo[1];
            const int iz =
                axis_offset(sg, 2, (int)(u >> 10), uez, ANYFULL && fr[2].full) - sg.lo[2];
            if ((unsigned)ix < (unsigned)sg.dim[0] && (unsigned)iy < (unsigned)sg.dim[1] &&
                (unsigned)iz < (unsigned)sg.dim[2]) {
              const int idx = (iz * sg.dim[1] + iy) * sg.dim[0] + ix;
              in = (s_bits[idx >> 5] >> (idx & 31)) & 1u;
              item = (uint32_t)k | ((uint32_t)ix << 10) | ((uint32_t)iy << 15) |
                     ((uint32_t)iz << 20);
            }
          }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, in);
        if (in) mq[queued + __popc(bal & lt_mask)] = item;
        queued += __popc(bal);
        my_pairs += (unsigned long long)__popc(bal);
        const bool last = k0 + 32 >= cn;
        while (queued >= 32 || (last && queued > 0)) {
          __syncwarp();
          const int m = min(queued, 32);
          if (F32 && lane < m) {
            const uint32_t en = mq[lane];
            const int kk = (int)(en & 1023u);
            float4 v = make_float4(0.f, 0.f, 0.f, __uint_as_float((uint32_t)kk));
            if (F32) {
              int ix, iy, iz;
              if (PAD) {
                const int idx = (int)(en >> 10);
                ix = (idx & 31) - (B - 1);
                iy = ((idx >> 5) & 31) - (B - 1);
                iz = (idx >> 10) - (B - 1);
              } else {
                ix = (int)((en >> 10) & 31u);
                iy = (int)((en >> 15) & 31u);
                iz = (int)(en >> 20);
              }
              const float4 a = rec32[kk];
              v.x = a.x + s_shift[0][ix];
              v.y = a.y + s_shift[1][iy];
              v.z = a.z + s_shift[2][iz];
            }
            mb[lane] = v;
          }
          __syncwarp();
          // one (point, member) term of the FP32 sum into the block sums
          auto term32 = [&](const float4 &mp) {
            const float4 fb = rec32[kSpCap32 + (int)__float_as_uint(mp.w)];
            float dx = mp.x - qr.x;
            float dy = mp.y - qr.y;
            float dz = mp.z - qr.z;
            // minimum image (pm_periodic_boundary.C:350-374); only an axis
            // whose frame is the whole box can produce |d| > L/2
            if (ANYFULL && fr[0].full) {
              if (dx <= -0.5f * sg.L32[0]) dx += sg.L32[0];
              if (dx > 0.5f * sg.L32[0]) dx -= sg.L32[0];
            }
            if (ANYFULL && fr[1].full) {
              if (dy <= -0.5f * sg.L32[1]) dy += sg.L32[1];
              if (dy > 0.5f * sg.L32[1]) dy -= sg.L32[1];
            }
            if (ANYFULL && fr[2].full) {
              if (dz <= -0.5f * sg.L32[2]) dz += sg.L32[2];
              if (dz > 0.5f * sg.L32[2]) dz -= sg.L32[2];
            }
            const float s2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            const float p = s2 * sg.e_hi;
            const float r = fmaf(s2, sg.e_lo, fmaf(s2, sg.e_hi, -p));
            const float E0 = ex2_approx(p);
            const float E = fmaf(E0, r * 0.6931471805599453f, E0);
            const float gv = E * fmaf(-sg.c1, s2, sg.c25);
            bx_ = fmaf(gv, fb.x, bx_);
            by_ = fmaf(gv, fb.y, by_);
            bz_ = fmaf(gv, fb.z, bz_);
          };
          auto flush32 = [&]() {  // the block sums into the compensated sums
            kahan_acc(sx, cx, bx_);
            kahan_acc(sy, cy, by_);
            kahan_acc(sz, cz, bz_);
            bx_ = by_ = bz_ = 0.f;
            blk = 0;
          };
          if (F32 && lq == 4 && m == 32 && qok) {
            // a full batch with four lanes per point: eight members per
            // lane, which is one block of the compensated sums (blk is 0
            // here: every earlier batch was full)
#pragma unroll
            for (int t = 0; t < 8; ++t) term32(mb[sub + 4 * t]);
            flush32();
          } else {
            for (int j = sub; j < m && qok; j += lq) {
              if (F32) {
                term32(mb[j]);
                if (++blk == 8) flush32();  // every 8 pairs into the compensated sums
              } else {
                const int kk = (int)(mq[j] & 1023u);
                const double4_32a a = rec64[2 * kk], fb = rec64[2 * kk + 1];
                // point_vector(q, x_j) with the minimum image (pm_periodic_boundary.C:350-374)
                double x[3] = {a.x - q0, a.y - q1, a.z - q2};
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                  if (sg.g.periodic[d]) {
                    const double xs = sg.g.L[d];
                    if (x[d] <= -xs / 2.0) x[d] += xs;
                    if (x[d] > xs / 2.0) x[d] -= xs;
                  }
                }
                // smoothed_force_exp (ggem_stokes.C:117-128)
                const double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
                const double a2r2 = K.alpha2 * r2;
                const double gv = K.alpha3_pi_23 * exp(-a2r2) * (2.5 - a2r2);
                ax += gv * fb.x;
                ay += gv * fb.y;
                az += gv * fb.z;
              }
            }
          }
          // the rest of the queue to its front
          const int rest = queued - m;
          const uint32_t rv = lane < rest ? mq[32 + lane] : 0u;
          __syncwarp();
          if (lane < rest) mq[lane] = rv;
          queued = rest;
        }
      }
      __syncwarp();
      double out[3];
      if (F32) {
        kahan_acc(sx, cx, bx_);
        kahan_acc(sy, cy, by_);
        kahan_acc(sz, cz, bz_);
        float h[3] = {sx, sy, sz}, l[3] = {-cx, -cy, -cz};
        for (int o = 1; o < lq; o <<= 1) {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const float h2 = __shfl_xor_sync(0xffffffffu, h[c], o);
            const float l2 = __shfl_xor_sync(0xffffffffu, l[c], o);
            ff_add(h[c], l[c], h2, l2);
          }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) out[c] = f2d_bits(h[c]) + f2d_bits(l[c]);
      } else {
        out[0] = ax;
        out[1] = ay;
        out[2] = az;
        for (int o = 1; o < lq; o <<= 1) {
#pragma unroll
          for (int c = 0; c < 3; ++c) out[c] += __shfl_xor_sync(0xffffffffu, out[c], o);
        }
      }
      if (qok && sub == 0) {
        double *dst = rho + 3 * qg;
        if (c0 == 0) {
          dst[0] = out[0];
          dst[1] = out[1];
          dst[2] = out[2];
        } else {  // a brick staged in several passes adds each pass's sums
          dst[0] += out[0];
          dst[1] += out[1];
          dst[2] += out[2];
        }
      }
      __syncwarp();  // the member list is rebuilt for the next element
    }
    __syncthreads();  // the staged particles are replaced
  }
  if (pairs) {
    if (lane == 0 && my_pairs) atomicAdd(pairs, my_pairs * (unsigned long long)nq);
  }
}

// quadrature points relative to their element centre (FP64 difference,
// rounded once to FP32); w = 0
__global__ void k_qp_rel(int64_t nqt, int nq, Grid g, const double *__restrict__ q,
                         float4 *__restrict__ rel) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nqt) return;
  const int64_t e = t / nq;
  const int ex = (int)(e % g.nc[0]), ey = (int)((e / g.nc[0]) % g.nc[1]),
            ez = (int)(e / ((int64_t)g.nc[0] * g.nc[1]));
  const double cx = g.lo[0] + (ex + 0.5) * g.h[0];
  const double cy = g.lo[1] + (ey + 0.5) * g.h[1];
  const double cz = g.lo[2] + (ez + 0.5) * g.h[2];
  rel[t] = make_float4((float)(q[3 * t] - cx), (float)(q[3 * t + 1] - cy),
                       (float)(q[3 * t + 2] - cz), 0.f);
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

// the stencil bitmap (own element included) and the brick geometry
int spread_geometry(ggem_ctx *c, SpreadGeo *sg) {
  std::memset(sg, 0, sizeof(*sg));
  sg->g = c->grid;
  const Grid &g = c->grid;
  for (int d = 0; d < 3; ++d) sg->lo[d] = sg->hi[d] = 0;
  for (const int4 &o : c->stencil) {
    const int v[3] = {o.x, o.y, o.z};
    for (int d = 0; d < 3; ++d) {
      sg->lo[d] = std::min(sg->lo[d], v[d]);
      sg->hi[d] = std::max(sg->hi[d], v[d]);
    }
  }
  int B = 4;
  for (; B >= 1; B /= 2) {
    bool ok = true;
    int rows = 1, xs = 1;
    for (int d = 0; d < 3; ++d) {
      int ext = B + sg->hi[d] - sg->lo[d];
      if (g.periodic[d] && ext >= g.nc[d]) ext = g.nc[d];
      if (ext > kSpMaxExt) ok = false;
      if (d > 0) rows *= std::min(ext, g.nc[d]);
      else xs = (g.periodic[0] && ext < g.nc[0]) ? 2 : 1;
    }
    if (ok && rows * xs <= kSpMaxSeg) break;
  }
  if (B < 1)
    return fail(c, GGEM_ERR_BAD_ARG,
                "element stencil too wide for the brick spread (more than 28 elements across)");
  sg->B = B;
  for (int d = 0; d < 3; ++d) {
    sg->dim[d] = sg->hi[d] - sg->lo[d] + 1;
    sg->nb[d] = (g.nc[d] + B - 1) / B;
    for (int k = 0; k < kSpMaxExt; ++k) {
      const int off = sg->lo[d] + k;
      sg->shift[d][k] = off <= sg->hi[d] ? (float)(off * g.h[d]) : 0.f;
    }
    sg->L32[d] = (float)g.L[d];
  }
  // the padded layout needs every frame offset field in [0, 32): offsets
  // run over [-(B - 1), dim + B - 2] per axis, so dim + 2B - 2 <= 32; a
  // frame spanning a whole periodic axis wraps its offsets and keeps the
  // compact layout
  bool any_full = false;
  sg->pad = 1;
  for (int d = 0; d < 3; ++d) {
    any_full = any_full || (g.periodic[d] && B + sg->hi[d] - sg->lo[d] >= g.nc[d]);
    if (sg->dim[d] + 2 * B - 2 > 32) sg->pad = 0;
  }
  if (any_full) sg->pad = 0;
  const int nbits = sg->pad ? 1024 * (sg->dim[2] + 2 * B - 2)
                            : sg->dim[0] * sg->dim[1] * sg->dim[2];
  sg->nwords = (nbits + 31) / 32;
  if (sg->nwords > kSpMaxWords)
    return fail(c, GGEM_ERR_BAD_ARG, "element stencil bitmap too large for the brick spread");
  std::vector<uint32_t> bits(sg->nwords, 0u);
  auto set = [&](int x, int y, int z) {
    const int i = x - sg->lo[0], j = y - sg->lo[1], k = z - sg->lo[2];
    const int idx = sg->pad ? (i + B - 1) + 32 * (j + B - 1) + 1024 * (k + B - 1)
                            : (k * sg->dim[1] + j) * sg->dim[0] + i;
    bits[idx >> 5] |= 1u << (idx & 31);
  };
  set(0, 0, 0);  // the element's own particles come first in its list
  for (const int4 &o : c->stencil) set(o.x, o.y, o.z);
  cudaError_t e = c->sp_bits.ensure(bits.size());
  if (e) return cuda_fail(c, e, "spread stencil");
  if ((e = cudaMemcpyAsync(c->sp_bits.p, bits.data(), sizeof(uint32_t) * bits.size(),
                           cudaMemcpyHostToDevice, c->stream)))
    return cuda_fail(c, e, "spread stencil");
  // e^{-alpha^2 s} = 2^{s k}, k = -alpha^2 log2(e) split into hi + lo floats
  const double k = -c->cst.alpha2 * 1.4426950408889634;
  sg->e_hi = (float)k;
  sg->e_lo = (float)(k - (double)sg->e_hi);
  sg->c25 = (float)(2.5 * c->cst.alpha3_pi_23);
  sg->c1 = (float)(c->cst.alpha2 * c->cst.alpha3_pi_23);
  sg->nq = c->q_per_elem;
  int p2 = 1;
  while (p2 < sg->nq) p2 <<= 1;
  sg->lq = 32 / p2;
  return GGEM_OK;
}

int spread_elements(ggem_ctx *c, int precision, const double *d_f_slot, double *d_rho,
                    unsigned long long *d_pairs) {
  SpreadGeo sg;
  if (int rc = spread_geometry(c, &sg)) return rc;
  const unsigned nblk = (unsigned)((int64_t)sg.nb[0] * sg.nb[1] * sg.nb[2]);
  cudaError_t e;
  // does any brick frame span a whole periodic axis? (brick_frame: the
  // frame of a brick of at most B elements spans B + hi - lo)
  bool any_full = false;
  for (int d = 0; d < 3; ++d)
    any_full = any_full || (sg.g.periodic[d] && sg.B + sg.hi[d] - sg.lo[d] >= sg.g.nc[d]);
  auto launch = [&](auto kernel) -> int {
    // (the attribute is per device; setting it costs microseconds)
    if ((e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kSpShared)))
      return cuda_fail(c, e, "spread attributes");
    kernel<<<nblk, kSpThreads, kSpShared, c->stream>>>(
        sg, c->dc, c->cell_start.p, c->pos32.p, c->pos64.p, d_f_slot, c->q_rel.p, c->q_xyz.p,
        c->sp_bits.p, d_rho, d_pairs);
    return GGEM_OK;
  };
  int rc;
  if (precision == GGEM_FP32)
    rc = any_full   ? launch(k_spread_brick<true, true, false>)
         : sg.pad   ? launch(k_spread_brick<true, false, true>)
                    : launch(k_spread_brick<true, false, false>);
  else
    rc = any_full   ? launch(k_spread_brick<false, true, false>)
         : sg.pad   ? launch(k_spread_brick<false, false, true>)
                    : launch(k_spread_brick<false, false, false>);
  if (rc) return rc;
  return check_launch(c, "spread bricks");
}

int quadrature_common(ggem_ctx *c, int nq) {
  if (c->prm.nb_mode != GGEM_NB_REFERENCE)
    return fail(c, GGEM_ERR_BAD_ARG, "the element spread needs reference mode (elements = cells)");
  if (nq < 1 || nq > 32)
    return fail(c, GGEM_ERR_BAD_ARG, "quadrature points per element must be in [1, 32]");
  const int64_t nqt = c->grid.ncell * nq;
  cudaError_t e;
  if ((e = c->q_xyz.ensure(3 * nqt)) || (e = c->q_rel.ensure(nqt)))
    return cuda_fail(c, e, "quadrature buffers");
  c->q_per_elem = 0;
  return GGEM_OK;
}

int quadrature_finish(ggem_ctx *c, int nq) {
  const int64_t nqt = c->grid.ncell * nq;
  k_qp_rel<<<(unsigned)((nqt + 255) / 256), 256, 0, c->stream>>>(nqt, nq, c->grid, c->q_xyz.p,
                                                                 c->q_rel.p);
  if (int rc = check_launch(c, "quadrature")) return rc;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e) return cuda_fail(c, e, "quadrature");
  c->q_per_elem = nq;
  return GGEM_OK;
}

}  // namespace
}  // namespace ggem

using namespace ggem;

extern "C" int ggem_set_quadrature(ggem_ctx *ctx, int nq_per_elem, const double *qxyz) {
  if (!ctx || (!qxyz && ctx->grid.ncell > 0)) return GGEM_ERR_BAD_ARG;
  DeviceGuard dg(ctx->device);
  if (int rc = quadrature_common(ctx, nq_per_elem)) return rc;
  const int64_t nqt = ctx->grid.ncell * nq_per_elem;
  cudaError_t e = cudaMemcpyAsync(ctx->q_xyz.p, qxyz, sizeof(double) * 3 * nqt,
                                  cudaMemcpyHostToDevice, ctx->stream);
  if (e) return cuda_fail(ctx, e, "quadrature h2d");
  return quadrature_finish(ctx, nq_per_elem);
}

extern "C" int ggem_set_quadrature_dev(ggem_ctx *ctx, int nq_per_elem, const double *d_qxyz) {
  if (!ctx || (!d_qxyz && ctx->grid.ncell > 0)) return GGEM_ERR_BAD_ARG;
  DeviceGuard dg(ctx->device);
  if (int rc = quadrature_common(ctx, nq_per_elem)) return rc;
  const int64_t nqt = ctx->grid.ncell * nq_per_elem;
  cudaError_t e = cudaMemcpyAsync(ctx->q_xyz.p, d_qxyz, sizeof(double) * 3 * nqt,
                                  cudaMemcpyDeviceToDevice, ctx->stream);
  if (e) return cuda_fail(ctx, e, "quadrature copy");
  return quadrature_finish(ctx, nq_per_elem);
}

extern "C" int ggem_spread_elements_dev(ggem_ctx *ctx, int precision, const double *d_f,
                                        double *d_rho, int64_t *pairs) {
  if (!ctx || (precision != GGEM_FP32 && precision != GGEM_FP64) || !d_rho ||
      (ctx->n > 0 && !d_f))
    return GGEM_ERR_BAD_ARG;
  if (!ctx->cells_built) return fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_build_cells first");
  if (ctx->q_per_elem < 1) return fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_set_quadrature first");
  DeviceGuard dg(ctx->device);
  const size_t n3 = (size_t)ctx->n * 3;
  cudaError_t e;
  if ((e = ctx->w_in.ensure(std::max<size_t>(n3, 1))) || (e = ctx->sp_pairs.ensure(1)))
    return cuda_fail(ctx, e, "spread buffers");
  if (n3) {
    if (int rc = permute_to_slots(ctx, 1, d_f, ctx->w_in.p)) return rc;
  }
  unsigned long long *d_pairs = nullptr;
  if (pairs) {
    d_pairs = ctx->sp_pairs.p;
    if ((e = cudaMemsetAsync(d_pairs, 0, sizeof(unsigned long long), ctx->stream)))
      return cuda_fail(ctx, e, "memset");
  }
  if (int rc = spread_elements(ctx, precision, ctx->w_in.p, d_rho, d_pairs)) return rc;
  if (pairs) {
    unsigned long long h = 0;
    if ((e = cudaMemcpyAsync(&h, d_pairs, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream)) ||
        (e = cudaStreamSynchronize(ctx->stream)))
      return cuda_fail(ctx, e, "spread pairs");
    *pairs = (int64_t)h;
  }
  return GGEM_OK;
}

extern "C" int ggem_spread_elements(ggem_ctx *ctx, int precision, const double *f, double *rho) {
  if (!ctx || !rho || (ctx->n > 0 && !f)) return GGEM_ERR_BAD_ARG;
  if (ctx->q_per_elem < 1) return fail(ctx, GGEM_ERR_BAD_ARG, "call ggem_set_quadrature first");
  DeviceGuard dg(ctx->device);
  const size_t n3 = (size_t)ctx->n * 3;
  const size_t nr = (size_t)ctx->grid.ncell * ctx->q_per_elem * 3;
  cudaError_t e;
  if ((e = ctx->w_a.ensure(std::max<size_t>(n3, 1))) || (e = ctx->w_d.ensure(std::max<size_t>(nr, 1))))
    return cuda_fail(ctx, e, "spread buffers");
  if (n3 && (e = cudaMemcpyAsync(ctx->w_a.p, f, 8 * n3, cudaMemcpyHostToDevice, ctx->stream)))
    return cuda_fail(ctx, e, "forces h2d");
  if (int rc = ggem_spread_elements_dev(ctx, precision, ctx->w_a.p, ctx->w_d.p, nullptr)) return rc;
  if ((e = cudaMemcpyAsync(rho, ctx->w_d.p, 8 * nr, cudaMemcpyDeviceToHost, ctx->stream)) ||
      (e = cudaStreamSynchronize(ctx->stream)))
    return cuda_fail(ctx, e, "rho d2h");
  return GGEM_OK;
}
