// ggem_cells.cu -- Kernel A: the sorted cell list and the cached FP32 pair
// list.
//
// Replaces PointMesh::reinit (point_mesh.C:245-289): the element-point
// containing list (:573-648) becomes a counting sort of particles by cell,
// and the per-particle neighbour lists (:652-848) with their stored
// displacement vectors (:220-241) become either an on-the-fly cell stencil
// sweep (FP64 path) or fixed-width rows of (source slot, stencil code)
// entries (FP32 path), built in one pass per configuration.
//
// Bound: HBM.  Algorithmic bytes per particle of the cell build: 24 (read
// xyz) + 4 (cell id) + 4 (order) + 4 (rank) + 32 (pos64) + 16 (pos32) plus
// the scatter re-reads; the list build writes 4 B per listed pair once.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "ggem_internal.cuh"

namespace ggem {
namespace {

__device__ __forceinline__ int wrap_index(int k, int n) {
  k %= n;
  return k < 0 ? k + n : k;
}

// cell coordinate along one axis, as the oracle and the reference's element
// search would compute it: floor((x - lo) / h), periodic axes wrapped first
__global__ void k_assign(int64_t n, const double *__restrict__ xyz, Grid g,
                         int32_t *__restrict__ cell_of, int32_t *__restrict__ count,
                         double4_32a *__restrict__ wrapped, int *__restrict__ err) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double p[3];
  int c[3];
  bool bad = false, nonfinite = false;
  for (int d = 0; d < 3; ++d) {
    double x = xyz[3 * i + d];
    // common case without FP64 arithmetic (GB300 issues FP64 at a small
    // fraction of the FP32 rate): inside the box away from its faces and
    // away from the cell faces, the FP32 index is the FP64 one
    {
      const float t = d2f_bits(x) - g.lo32[d];  // NaN and infinities fail below
      if (t > g.margin32[d] && t < g.L32[d] - g.margin32[d]) {
        const float q = t * g.inv_h32[d];
        const float fq = floorf(q);
        if (q - fq > g.band32[d] && (fq + 1.f) - q > g.band32[d]) {
          const int k = (int)fq;
          p[d] = x;
          c[d] = k < 0 ? 0 : (k >= g.nc[d] ? g.nc[d] - 1 : k);
          continue;
        }
      }
    }
    if (!isfinite(x)) {  // reported as a bad argument; the cell index stays in range
      nonfinite = true;
      x = g.lo[d];
    }
    double t = x - g.lo[d];
    // (FP64 runs at a small fraction of the FP32 rate: fmod and the division
    // are taken only where they can change the result)
    if (g.periodic[d]) {
      // inside, fmod(t, L) == t; a bead inside the box whose x - lo rounded
      // up to L keeps t = L and so the last cell (the element search's
      // closed upper face, point_mesh.C) instead of wrapping to cell 0
      if (!(t >= 0.0 && t < g.L[d]) && !(x >= g.lo[d] && x < g.lo[d] + g.L[d])) {
        t = fmod(t, g.L[d]);
        if (t < 0) t += g.L[d];
        if (t >= g.L[d]) t = 0.0;
        x = g.lo[d] + t;  // a caller's value inside the box is kept as it is
      }
    } else if (!(t >= 0.0 && t <= g.L[d])) {
      bad = true;
    }
    p[d] = x;
    // floor(t / h): t * (1/h) is within a few ulps of t / h, so its floor is
    // the same unless it lies within 1e-9 of an integer (|t / h| < 1e6)
    const double q = t * g.inv_h[d];
    double fq = floor(q);
    if (q - fq < 1e-9 || (fq + 1.0) - q < 1e-9 || !(fabs(q) < 1e6)) fq = floor(t / g.h[d]);
    int k = (int)fq;
    c[d] = k < 0 ? 0 : (k >= g.nc[d] ? g.nc[d] - 1 : k);
  }
  if (bad) atomicOr(err, kErrOutOfDomain);
  if (nonfinite) atomicOr(err, kErrNonFinite);
  const int32_t id = c[0] + g.nc[0] * (c[1] + g.nc[1] * c[2]);
  cell_of[i] = id;
  atomicAdd(&count[id], 1);
  wrapped[i] = make_double4_32a(p[0], p[1], p[2], 0.0);
}

// ---- exclusive scan (warp shuffles, 1024-element blocks) ----------------
template <typename T>
__global__ void k_scan_block(const T *__restrict__ in, T *__restrict__ out,
                             int64_t *__restrict__ block_sums, int64_t n) {
  __shared__ T warp_tot[32];
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T v = (i < n) ? in[i] : T(0);
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    T w = (lane < nw) ? warp_tot[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) warp_tot[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  const T base = warp ? warp_tot[warp - 1] : T(0);
  if (i < n) out[i] = base + x - v;
  if (threadIdx.x == blockDim.x - 1 && block_sums) block_sums[blockIdx.x] = (int64_t)(base + x);
}

template <typename T>
__global__ void k_scan_add(T *__restrict__ out, const int64_t *__restrict__ block_off, int64_t n,
                           const T *__restrict__ in, T *__restrict__ total_slot) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    out[i] += (T)block_off[blockIdx.x];
    if (i == n - 1 && total_slot) *total_slot = out[i] + in[i];
  }
}

template <typename T>
__global__ void k_scan_total(T *__restrict__ out, const T *__restrict__ in, int64_t n) {
  if (threadIdx.x == 0 && blockIdx.x == 0) out[n] = (n > 0) ? out[n - 1] + in[n - 1] : T(0);
}

template <typename T>
int scan_impl(ggem_ctx *c, const T *in, T *out, int64_t n, int level) {
  const int B = 1024;
  const int64_t nb = (n + B - 1) / B;
  if (n <= 0) {
    k_scan_total<T><<<1, 1, 0, c->stream>>>(out, in, 0);
    return check_launch(c, "scan");
  }
  if ((int)c->scan_scratch.size() <= 2 * level + 1) {
    c->scan_scratch.resize(2 * level + 2, nullptr);
  }
  for (int k = 0; k < 2; ++k)
    if (!c->scan_scratch[2 * level + k]) c->scan_scratch[2 * level + k] = new DevBuf<int64_t>();
  DevBuf<int64_t> &sums = *c->scan_scratch[2 * level];
  DevBuf<int64_t> &offs = *c->scan_scratch[2 * level + 1];
  cudaError_t e = sums.ensure(nb + 1);
  if (e == cudaSuccess) e = offs.ensure(nb + 1);
  if (e != cudaSuccess) return cuda_fail(c, e, "scan scratch");
  k_scan_block<T><<<(unsigned)nb, B, 0, c->stream>>>(in, out, sums.p, n);
  int rc = check_launch(c, "scan block");
  if (rc) return rc;
  if (nb > 1) {
    rc = scan_impl<int64_t>(c, sums.p, offs.p, nb, level + 1);
    if (rc) return rc;
    k_scan_add<T><<<(unsigned)nb, B, 0, c->stream>>>(out, offs.p, n, in, out + n);
    return check_launch(c, "scan add");
  }
  k_scan_total<T><<<1, 1, 0, c->stream>>>(out, in, n);
  return check_launch(c, "scan total");
}

// the cell list's exclusive scan in one block when the grid is small
// enough: tiles of 4096 counts (four consecutive counts per thread), all
// loaded before the first tile is scanned, then one block-wide scan of the
// threads' sums per tile with a running carry; start[0..ncell].  The counts
// are zeroed as they are read, ready for the next build's k_assign, and so
// are the pair-list statistics (stat, when given) that the list build of
// the same configuration accumulates.
constexpr int kScanTiles = 8;
constexpr int64_t kScanCellsMax = 4096 * kScanTiles;

__global__ void __launch_bounds__(1024) k_scan_cells(int32_t *__restrict__ count,
                                                     int32_t *__restrict__ start, int64_t n,
                                                     unsigned long long *__restrict__ stat) {
  __shared__ int32_t warp_tot[2][32];
  if (stat && threadIdx.x < 2) stat[threadIdx.x] = 0ull;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int tiles = (int)((n + 4095) / 4096);
  int32_t v[kScanTiles][4];
#pragma unroll
  for (int k = 0; k < kScanTiles; ++k)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t i = (int64_t)k * 4096 + 4 * threadIdx.x + j;
      v[k][j] = (k < tiles && i < n) ? count[i] : 0;
    }
#pragma unroll
  for (int k = 0; k < kScanTiles; ++k)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t i = (int64_t)k * 4096 + 4 * threadIdx.x + j;
      if (k < tiles && i < n) count[i] = 0;
    }
  int32_t carry = 0;
#pragma unroll
  for (int k = 0; k < kScanTiles; ++k) {
    if (k < tiles) {
      const int32_t tsum = (v[k][0] + v[k][1]) + (v[k][2] + v[k][3]);
      int32_t x = tsum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      int32_t *wt = warp_tot[k & 1];  // alternate buffers: one barrier per tile
      if (lane == 31) wt[warp] = x;
      __syncthreads();
      int32_t w = wt[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      // every warp scans the 32 warp totals itself (no second barrier)
      const int32_t before = __shfl_sync(0xffffffffu, w, (warp + 31) & 31);
      const int32_t total = __shfl_sync(0xffffffffu, w, 31);
      int32_t run = carry + (warp ? before : 0) + x - tsum;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t i = (int64_t)k * 4096 + 4 * threadIdx.x + j;
        if (i < n) start[i] = run;
        run += v[k][j];
      }
      carry += total;
    }
  }
  if (threadIdx.x == 0) start[n] = carry;
}

__global__ void k_scatter(int64_t n, const int32_t *__restrict__ cell_of,
                          const int32_t *__restrict__ start, int32_t *__restrict__ fill,
                          int32_t *__restrict__ order) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t cid = cell_of[i];
  const int32_t slot = start[cid] + atomicAdd(&fill[cid], 1);
  order[slot] = (int32_t)i;
}

// ascending particle id inside each cell (deterministic slot order, and the
// order of build_elem_point_containing_list, point_mesh.C:585-631): cells of
// up to 16 particles are sorted in registers by an odd-even transposition
// network, larger ones by insertion in place.  The cell's fill counter is
// zeroed for the next build.
__global__ void k_sort_cells(int64_t ncell, const int32_t *__restrict__ start,
                             int32_t *__restrict__ order, int32_t *__restrict__ fill) {
  const int64_t cidx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (cidx >= ncell) return;
  fill[cidx] = 0;  // scattered; ready for the next build
  const int32_t b = start[cidx], e = start[cidx + 1];
  const int32_t m = e - b;
  if (m <= 1) return;
  if (m <= 16) {
    int32_t v[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = k < m ? order[b + k] : 0x7fffffff;
#pragma unroll
    for (int r = 0; r < 16; ++r) {
#pragma unroll
      for (int k = r & 1; k + 1 < 16; k += 2) {
        const int32_t lo = min(v[k], v[k + 1]), hi = max(v[k], v[k + 1]);
        v[k] = lo;
        v[k + 1] = hi;
      }
    }
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (k < m) order[b + k] = v[k];
    return;
  }
  for (int32_t k = b + 1; k < e; ++k) {
    const int32_t v = order[k];
    int32_t m = k - 1;
    while (m >= b && order[m] > v) {
      order[m + 1] = order[m];
      --m;
    }
    order[m + 1] = v;
  }
}

__global__ void k_gather_sorted(int64_t n, Grid g, const int32_t *__restrict__ order,
                                const int32_t *__restrict__ cell_of,
                                const double4_32a *__restrict__ wrapped,
                                int32_t *__restrict__ rank, double4_32a *__restrict__ pos64,
                                float4 *__restrict__ pos32) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int32_t i = order[s];
  rank[i] = (int32_t)s;
  const double4_32a p = wrapped[i];
  pos64[s] = p;
  const int32_t cid = cell_of[i];
  const int cx = cid % g.nc[0], cy = (cid / g.nc[0]) % g.nc[1], cz = cid / (g.nc[0] * g.nc[1]);
  // position relative to the cell centre: |rel| <= h/2 keeps FP32 exact to
  // ~1e-7 of h whatever the box size
  const double rx = p.x - (g.lo[0] + (cx + 0.5) * g.h[0]);
  const double ry = p.y - (g.lo[1] + (cy + 0.5) * g.h[1]);
  const double rz = p.z - (g.lo[2] + (cz + 0.5) * g.h[2]);
  pos32[s] = make_float4((float)rx, (float)ry, (float)rz, __int_as_float(cid));
}

// neighbour cell of cell coordinate (cx,cy,cz) shifted by o; -1 if outside a
// non-periodic axis
__device__ __forceinline__ int32_t shifted_cell(const Grid &g, int cx, int cy, int cz, int4 o) {
  int c[3] = {cx + o.x, cy + o.y, cz + o.z};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (c[d] < 0 || c[d] >= g.nc[d]) {
      if (!g.periodic[d]) return -1;
      c[d] = wrap_index(c[d], g.nc[d]);
    }
  }
  return c[0] + g.nc[0] * (c[1] + g.nc[1] * c[2]);
}

// exact FP64 cut-off decision, the oracle's predicate: minimum-image vector
// (pm_periodic_boundary.C:350-374) and (dx*dx + dy*dy) + dz*dz < rc^2
// without contraction
__device__ __forceinline__ bool exact_within(const Grid &g, double4_32a a, double4_32a b, double rc2) {
  double d[3] = {b.x - a.x, b.y - a.y, b.z - a.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (g.periodic[k]) {
      const double xs = g.L[k];
      if (d[k] <= -xs / 2.0) d[k] += xs;
      if (d[k] > xs / 2.0) d[k] -= xs;
    }
  }
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])),
                              __dmul_rn(d[2], d[2]));
  return r2 < rc2;
}

// Warp-per-cell pair list, one pass into fixed-width rows.  The candidates
// of a target cell are the concatenation of its stencil cells (stencil
// order, slot order inside a cell).  For each chunk of up to 32 targets the
// lanes first take 32 consecutive candidates at a time with coalesced loads
// and keep those within reach of the chunk's bounding box; the kept ones
// queue in shared memory, in candidate order, and every 32 of them are
// tested against the chunk's targets, which are broadcast one at a time from
// shared memory; a ballot prefix places each accepted candidate.  Entries
// therefore come out in exactly the per-target order of a sequential sweep.
// Row s holds entries [s*W, s*W + cnt[s]); a row longer than W is counted
// but not stored: the kernel records the longest row and sets
// kErrListCapacity, and the host rebuilds with a wider W.
// One warp per block, one block per cell: cells hold different numbers of
// targets, and a block of several cell-warps held its resources until its
// longest cell was done (N = 200k, phi = 0.1: 92 us against 101 us with 8
// warps per block, and against 97 us with 8-warp blocks claiming cells from
// a counter).
constexpr int kMaxStencil = 128;  // stencil cells per target cell
constexpr int kListQueue = 64;    // queued candidates per warp (< 32 left + 32 new)

// FP32 distance of a candidate from the targets' box, formed like the pair
// test's r2 below (the same subtractions, squares and fused adds, each
// monotone in its operands), so that it never exceeds the r2 of any target
// inside the box: a candidate whose box distance is above rc2_hi is above it
// for every target and would be rejected there without the exact test
__device__ __forceinline__ float box_r2(float qx, float qy, float qz, float3 lo, float3 hi) {
  const float bx = qx > hi.x ? qx - hi.x : (qx < lo.x ? lo.x - qx : 0.f);
  const float by = qy > hi.y ? qy - hi.y : (qy < lo.y ? lo.y - qy : 0.f);
  const float bz = qz > hi.z ? qz - hi.z : (qz < lo.z ? lo.z - qz : 0.f);
  return fmaf(bz, bz, fmaf(by, by, bx * bx));
}

__global__ void __launch_bounds__(32, 32) k_pair_list_warp(
    Grid g, const int4 *__restrict__ stencil, int nst, const float4 *__restrict__ shift,
    const int32_t *__restrict__ start, const float4 *__restrict__ pos32,
    const double4_32a *__restrict__ pos64, float rc2_lo, float rc2_hi, double rc2, int W,
    int32_t *__restrict__ count, uint32_t *__restrict__ list,
    unsigned long long *__restrict__ stat, int *__restrict__ err,
    int32_t *__restrict__ count_h, uint32_t *__restrict__ list_h) {
  __shared__ int32_t s_base[kMaxStencil];
  __shared__ int32_t s_pre[kMaxStencil + 1];
  __shared__ int32_t s_code[kMaxStencil];
  __shared__ float4 s_pi[32];          // the targets of the current chunk
  __shared__ float4 s_q[kListQueue];   // kept candidates: frame position, entry
  __shared__ int s_mark[32];           // stencil cell starting at each lane of a chunk
  const int lane = threadIdx.x;
  s_mark[lane] = -1;
  const int64_t C = blockIdx.x;
  const int32_t tb = start[C], te = start[C + 1];
  if (te <= tb) return;
  const int cx = (int)(C % g.nc[0]), cy = (int)((C / g.nc[0]) % g.nc[1]),
            cz = (int)(C / ((int64_t)g.nc[0] * g.nc[1]));
  // stencil cell ranges and their running prefix (warp scan over chunks)
  int32_t carry = 0;
  for (int k0 = 0; k0 < nst; k0 += 32) {
    const int k = k0 + lane;
    int32_t cnt = 0, base = 0, code = 0;
    if (k < nst) {
      const int4 o = stencil[k];
      const int32_t nc = shifted_cell(g, cx, cy, cz, o);
      code = o.w;
      if (nc >= 0) {
        base = start[nc];
        cnt = start[nc + 1] - base;
      }
    }
    int32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (k < nst) {
      s_base[k] = base;
      s_code[k] = code;
      s_pre[k] = carry + incl - cnt;
    }
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) s_pre[nst] = carry;
  __syncwarp();
  const int32_t V = carry;
  const unsigned lt_mask = (1u << lane) - 1u;
  unsigned long long cell_total = 0;
  int32_t cell_max = 0;
  for (int32_t t0 = tb; t0 < te; t0 += 32) {
    const int ntc = min(32, te - t0);
    const int32_t own = t0 + lane;
    const bool own_ok = lane < ntc;
    __syncwarp();  // the previous chunk's targets are no longer read
    const float4 mine = own_ok ? pos32[own] : make_float4(0.f, 0.f, 0.f, 0.f);
    s_pi[lane] = mine;
    // the chunk's bounding box (FP32 min / max of the targets' own values)
    float3 blo = own_ok ? make_float3(mine.x, mine.y, mine.z)
                        : make_float3(INFINITY, INFINITY, INFINITY);
    float3 bhi = own_ok ? make_float3(mine.x, mine.y, mine.z)
                        : make_float3(-INFINITY, -INFINITY, -INFINITY);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      blo.x = fminf(blo.x, __shfl_xor_sync(0xffffffffu, blo.x, o));
      blo.y = fminf(blo.y, __shfl_xor_sync(0xffffffffu, blo.y, o));
      blo.z = fminf(blo.z, __shfl_xor_sync(0xffffffffu, blo.z, o));
      bhi.x = fmaxf(bhi.x, __shfl_xor_sync(0xffffffffu, bhi.x, o));
      bhi.y = fmaxf(bhi.y, __shfl_xor_sync(0xffffffffu, bhi.y, o));
      bhi.z = fmaxf(bhi.z, __shfl_xor_sync(0xffffffffu, bhi.z, o));
    }
    __syncwarp();
    int32_t own_cnt = 0, own_cnt_h = 0;
    int queued = 0;  // warp-uniform
    int kcur = -1;   // warp-uniform: the stencil cell of candidate v0 - 1
    for (int32_t v0 = 0; v0 < V; v0 += 32) {
      const int32_t v = v0 + lane;
      const bool valid = v < V;
      // stencil cell of candidate v, the last k with s_pre[k] <= v: the
      // cells after kcur that start inside this chunk mark their first lane
      // (the largest k wins, skipping empty cells), and a max-scan over the
      // lanes carries each cell forward
      for (int kk = kcur + 1;; kk += 32) {
        const int k = kk + lane;
        const int p = k < nst ? s_pre[k] - v0 : 32;
        if (p < 32) atomicMax(&s_mark[p], k);
        if (__shfl_sync(0xffffffffu, p, 31) >= 32) break;
      }
      __syncwarp();
      int lo = max(s_mark[lane], kcur);
      s_mark[lane] = -1;  // ready for the next chunk
      __syncwarp();
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, lo, o);
        if (lane >= o) lo = max(lo, y);
      }
      kcur = __shfl_sync(0xffffffffu, lo, 31);
      const int32_t t = valid ? s_base[lo] + (v - s_pre[lo]) : 0;
      const int code = s_code[lo];
      const float4 sh = shift[code];
      const float4 pj = valid ? pos32[t] : make_float4(0.f, 0.f, 0.f, 0.f);
      // the candidate in the target cell's frame (the shift added once per
      // candidate; the filter's band absorbs the different rounding)
      const float qx = pj.x + sh.x, qy = pj.y + sh.y, qz = pj.z + sh.z;
      const bool keep = valid && !(box_r2(qx, qy, qz, blo, bhi) > rc2_hi);
      const unsigned kb = __ballot_sync(0xffffffffu, keep);
      if (keep)
        s_q[queued + __popc(kb & lt_mask)] =
            make_float4(qx, qy, qz, __uint_as_float(((uint32_t)t << kCodeBits) | (uint32_t)code));
      queued += __popc(kb);
      const bool last = v0 + 32 >= V;
      // test the queue 32 at a time (a partial batch only after the last
      // candidates); at most two batches per pass
      while (queued >= 32 || (last && queued > 0)) {
        __syncwarp();
        const int m = min(queued, 32);
        // lanes past the batch carry a far point: r2 overflows, never accepted
        const float4 c = lane < m ? s_q[lane] : make_float4(1e30f, 1e30f, 1e30f, 0.f);
        const uint32_t en = __float_as_uint(c.w);
        const int32_t tj = (int32_t)(en >> kCodeBits);
        for (int i = 0; i < ntc; ++i) {
          const float4 pi = s_pi[i];  // one broadcast read
          const int32_t ti = t0 + i;
          const float dx = c.x - pi.x;
          const float dy = c.y - pi.y;
          const float dz = c.z - pi.z;
          const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
          // accepted below rc2_lo, rejected above rc2_hi; in between (FP32
          // rounding of |r| = rc) the exact FP64 test decides, behind a
          // warp-uniform branch so that the common case carries none of it
          bool in = tj != ti && !(r2 > rc2_hi);
          const bool band = in && !(r2 < rc2_lo);
          if (__any_sync(0xffffffffu, band)) {
            if (band) in = exact_within(g, pos64[ti], pos64[tj], rc2);
          }
          const unsigned bal = __ballot_sync(0xffffffffu, in);
          const int32_t at = __shfl_sync(0xffffffffu, own_cnt, i);
          if (in) {
            const int32_t k = at + __popc(bal & lt_mask);
            if (k < W) list[(int64_t)ti * W + k] = en;
          }
          if (lane == i) own_cnt += __popc(bal);
          if (list_h) {
            // the half list: each unordered pair once, in the row of its
            // smaller slot (the full list is symmetric, its predicate exact)
            const bool in_h = in && tj > ti;
            const unsigned bal_h = __ballot_sync(0xffffffffu, in_h);
            const int32_t at_h = __shfl_sync(0xffffffffu, own_cnt_h, i);
            if (in_h) {
              const int32_t k = at_h + __popc(bal_h & lt_mask);
              if (k < W) list_h[(int64_t)ti * W + k] = en;
            }
            if (lane == i) own_cnt_h += __popc(bal_h);
          }
        }
        // move the rest of the queue to its front
        const int rest = queued - m;
        const float4 r = lane < rest ? s_q[32 + lane] : c;
        __syncwarp();
        if (lane < rest) s_q[lane] = r;
        queued = rest;
      }
    }
    if (own_ok) {
      if (count_h) count_h[own] = min(own_cnt_h, W);
      count[own] = min(own_cnt, W);  // the stored entries; the full length goes to stat
      cell_total += (unsigned long long)own_cnt;
      cell_max = max(cell_max, own_cnt);
    }
  }
  // one atomic per warp (per cell) for the list statistics
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    cell_total += __shfl_xor_sync(0xffffffffu, cell_total, o);
    cell_max = max(cell_max, __shfl_xor_sync(0xffffffffu, cell_max, o));
  }
  if (lane == 0) {
    atomicAdd(&stat[0], cell_total);
    atomicMax(&stat[1], (unsigned long long)cell_max);
    if (cell_max > W) atomicOr(err, kErrListCapacity);
  }
}

}  // namespace

int device_exclusive_scan_i32(ggem_ctx *c, const int32_t *in, int32_t *out, int64_t n) {
  return scan_impl<int32_t>(c, in, out, n, 0);
}
int device_exclusive_scan_i64(ggem_ctx *c, const int64_t *in, int64_t *out, int64_t n) {
  return scan_impl<int64_t>(c, in, out, n, 0);
}

int build_cells(ggem_ctx *c, bool defer_flags) {
  const int64_t n = c->n;
  const Grid &g = c->grid;
  cudaError_t e = cudaSuccess;
  if ((e = c->cell_of.ensure(n)) || (e = c->cell_count.ensure(g.ncell)) ||
      (e = c->cell_fill.ensure(g.ncell)) || (e = c->cell_start.ensure(g.ncell + 1)) ||
      (e = c->order.ensure(n)) || (e = c->rank.ensure(n)) || (e = c->wrapped.ensure(n)) ||
      (e = c->pos64.ensure(n)) || (e = c->pos32.ensure(n)))
    return cuda_fail(c, e, "cell buffers");
  cudaStream_t st = c->stream;
  // the cell counters are left at zero by the previous build (the
  // single-block scan zeroes the counts, k_sort_cells the fills); they are
  // cleared here only after a reallocation, an interrupted build or on
  // grids too large for the single-block scan
  const bool small = g.ncell <= kScanCellsMax;
  const bool clean = small && c->cell_counters_zero && c->cell_count.p == c->cell_counters_at;
  c->cell_counters_zero = false;
  if ((!clean && ((e = cudaMemsetAsync(c->cell_count.p, 0, sizeof(int32_t) * g.ncell, st)) ||
                  (e = cudaMemsetAsync(c->cell_fill.p, 0, sizeof(int32_t) * g.ncell, st)))) ||
      (e = cudaMemsetAsync(c->err.p, 0, sizeof(int), st)))
    return cuda_fail(c, e, "cell memset");
  const int T = 256;
  const unsigned bn = (unsigned)((n + T - 1) / T);
  if (n > 0) {
    k_assign<<<bn, T, 0, st>>>(n, c->xyz_in.p, g, c->cell_of.p, c->cell_count.p, c->wrapped.p,
                               c->err.p);
    if (int rc = check_launch(c, "assign")) return rc;
  }
  c->list_stat_zero = false;
  if (small) {
    k_scan_cells<<<1, 1024, 0, st>>>(c->cell_count.p, c->cell_start.p, g.ncell, c->nb_stat.p);
    if (int rc = check_launch(c, "scan cells")) return rc;
    c->list_stat_zero = c->nb_stat.p != nullptr;
  } else if (int rc = device_exclusive_scan_i32(c, c->cell_count.p, c->cell_start.p, g.ncell)) {
    return rc;
  }
  if (n > 0) {
    k_scatter<<<bn, T, 0, st>>>(n, c->cell_of.p, c->cell_start.p, c->cell_fill.p, c->order.p);
    if (int rc = check_launch(c, "scatter")) return rc;
  }
  // (for n = 0 only the fill counters are cleared)
  k_sort_cells<<<(unsigned)((g.ncell + T - 1) / T), T, 0, st>>>(g.ncell, c->cell_start.p,
                                                                 c->order.p, c->cell_fill.p);
  if (int rc = check_launch(c, "sort cells")) return rc;
  if (n > 0) {
    k_gather_sorted<<<bn, T, 0, st>>>(n, g, c->order.p, c->cell_of.p, c->wrapped.p, c->rank.p,
                                      c->pos64.p, c->pos32.p);
    if (int rc = check_launch(c, "gather sorted")) return rc;
  }
  c->cell_counters_zero = small;
  c->cell_counters_at = c->cell_count.p;
  c->cells_built = false;
  c->list_built = false;
  c->pretensor_ok = false;
  if (!defer_flags) {
    int flags = 0;
    if (int rc = read_error_flags(c, &flags)) return rc;
    if (int rc = cell_flag_error(c, flags)) return rc;
  }
  c->cells_built = true;
  return GGEM_OK;
}

int cell_flag_error(ggem_ctx *c, int flags) {
  if (flags & kErrNonFinite) {
    c->cells_built = false;
    return fail(c, GGEM_ERR_BAD_ARG, "non-finite position");
  }
  if (flags & kErrOutOfDomain) {
    c->cells_built = false;
    return fail(c, GGEM_ERR_OUT_OF_DOMAIN,
                "a particle lies outside the box on a non-periodic axis "
                "(point_mesh.C:602-613: no element contains it)");
  }
  return GGEM_OK;
}

void launch_pair_list(ggem_ctx *c, int nst, int W, cudaStream_t st) {
  k_pair_list_warp<<<(unsigned)c->grid.ncell, 32, 0, st>>>(
      c->grid, c->d_stencil.p, nst, c->d_shift.p, c->cell_start.p, c->pos32.p, c->pos64.p,
      c->rc2_lo, c->rc2_hi, c->rc2, W, c->nb_cnt.p, c->nb_list.p, c->nb_stat.p, c->err.p,
      c->sym_pairs ? c->nb_cnt_h.p : nullptr, c->sym_pairs ? c->nb_list_h.p : nullptr);
}

int build_pair_list(ggem_ctx *c) {
  const int64_t n = c->n;
  cudaError_t e = cudaSuccess;
  if ((e = c->nb_cnt.ensure(n)) || (e = c->nb_stat.ensure(2)))
    return cuda_fail(c, e, "pair list buffers");
  cudaStream_t st = c->stream;
  if (c->nb_w <= 0) {
    // first build: twice the mean row length of a uniform suspension plus slack
    const Grid &g = c->grid;
    const double vol = g.L[0] * g.L[1] * g.L[2];
    const double mean = vol > 0 ? (double)n / vol * 4.18879020478639 * c->rc2 * std::sqrt(c->rc2)
                                : 0.0;
    c->nb_w = (int)std::min<double>(((int64_t)(2.0 * mean) + 16 + 7) / 8 * 8, 1 << 20);
  }
  if (n == 0) {
    c->n_pairs = 0;
    c->cells_built = true;
    c->list_built = true;
    return GGEM_OK;
  }
  const int nst = (int)c->stencil.size();
  if (nst > kMaxStencil) return fail(c, GGEM_ERR_BAD_ARG, "stencil too large for the list builder");
  if (c->defer_checks && c->list_checked_once) {
    // keep the width of the previous build; a longer row is stored clipped
    // (counts never exceed W) and found when the statistics are read
    if ((e = c->nb_list.ensure((size_t)n * c->nb_w))) return cuda_fail(c, e, "pair list");
    // (the statistics were zeroed by this configuration's cell scan)
    if (!c->list_stat_zero &&
        (e = cudaMemsetAsync(c->nb_stat.p, 0, 2 * sizeof(unsigned long long), st)))
      return cuda_fail(c, e, "memset");
    c->list_stat_zero = false;
    kt_start(c, kKListBuild);
    if (c->sym_pairs && ((e = c->nb_list_h.ensure((size_t)n * c->nb_w)) ||
                         (e = c->nb_cnt_h.ensure(n))))
      return cuda_fail(c, e, "half pair list");
    launch_pair_list(c, nst, c->nb_w, st);
    kt_stop(c, kKListBuild);
    if (int rc = check_launch(c, "pair list")) return rc;
    c->cells_built = true;
    c->list_built = true;
    c->list_unchecked = true;
    c->n_pairs = -1;
    return GGEM_OK;
  }
  // The error word still holds the cell build's flags; they come back with
  // the list statistics in one host synchronisation.  A row longer than the
  // current width makes the host widen the rows and fill once more.
  unsigned long long *h = reinterpret_cast<unsigned long long *>(c->h_red);
  c->list_stat_zero = false;
  for (int attempt = 0; attempt < 2; ++attempt) {
    const int W = c->nb_w;
    if ((e = c->nb_list.ensure((size_t)n * W))) return cuda_fail(c, e, "pair list");
    if ((e = cudaMemsetAsync(c->nb_stat.p, 0, 2 * sizeof(unsigned long long), st)))
      return cuda_fail(c, e, "memset");
    if (c->sym_pairs && ((e = c->nb_list_h.ensure((size_t)n * W)) || (e = c->nb_cnt_h.ensure(n))))
      return cuda_fail(c, e, "half pair list");
    if (attempt == 0) kt_start(c, kKListBuild);
    launch_pair_list(c, nst, W, st);
    if (attempt == 0) kt_stop(c, kKListBuild);  // a widened refill is left out
    if (int rc = check_launch(c, "pair list")) return rc;
    h[2] = 0;
    if ((e = cudaMemcpyAsync(h, c->nb_stat.p, 2 * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, st)) ||
        (e = cudaMemcpyAsync(&h[2], c->err.p, sizeof(int), cudaMemcpyDeviceToHost, st)) ||
        (e = cudaStreamSynchronize(st)))
      return cuda_fail(c, e, "list statistics");
    const int flags = (int)h[2];
    if (int rc = cell_flag_error(c, flags)) return rc;
    c->cells_built = true;
    if (!(flags & kErrListCapacity)) {
      c->n_pairs = (int64_t)h[0];
      c->list_built = true;
      c->list_checked_once = true;
      return GGEM_OK;
    }
    const unsigned long long longest = h[1];
    c->nb_w = (int)std::min<unsigned long long>((longest + longest / 8 + 8 + 7) / 8 * 8, 1u << 24);
    if ((e = cudaMemsetAsync(c->err.p, 0, sizeof(int), st))) return cuda_fail(c, e, "memset");
  }
  return fail(c, GGEM_ERR_CELL_OVERFLOW, "pair list rows exceeded their width twice");
}

int enqueue_list_check(ggem_ctx *c) {
  if (!c->list_unchecked) return GGEM_OK;
  unsigned long long *h = reinterpret_cast<unsigned long long *>(c->h_red + kListStatSlot);
  h[2] = 0;
  cudaError_t e = cudaMemcpyAsync(h, c->nb_stat.p, 2 * sizeof(unsigned long long),
                                  cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&h[2], c->err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e) return cuda_fail(c, e, "list statistics");
  return GGEM_OK;
}

int finish_list_check(ggem_ctx *c, unsigned long long total, unsigned long long longest, int flags,
                      bool *rebuilt) {
  if (rebuilt) *rebuilt = false;
  if (!c->list_unchecked) return GGEM_OK;
  c->list_unchecked = false;
  if (int rc = cell_flag_error(c, flags)) {
    c->list_built = false;
    return rc;
  }
  if (!(flags & kErrListCapacity)) {
    c->n_pairs = (int64_t)total;
    return GGEM_OK;
  }
  // rows overflowed: widen them and rebuild with the synchronous path
  c->nb_w = (int)std::min<unsigned long long>((longest + longest / 8 + 8 + 7) / 8 * 8, 1u << 24);
  cudaError_t e = cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream);
  if (e) return cuda_fail(c, e, "memset");
  const bool defer = c->defer_checks;
  c->defer_checks = false;
  int rc = build_pair_list(c);
  c->defer_checks = defer;
  if (rc) return rc;
  if ((rc = build_pair_tensors(c))) return rc;
  if (rebuilt) *rebuilt = true;
  return GGEM_OK;
}

int settle_list(ggem_ctx *c) {
  if (!c->list_unchecked) return GGEM_OK;
  if (int rc = enqueue_list_check(c)) return rc;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e) return cuda_fail(c, e, "list statistics");
  const unsigned long long *h = reinterpret_cast<unsigned long long *>(c->h_red + kListStatSlot);
  return finish_list_check(c, h[0], h[1], (int)h[2], nullptr);
}

}  // namespace ggem
