// ggem_noalloc.cu -- the local mobility matvec for callers that cannot
// allocate device memory.
//
// Some callers cannot call cudaMalloc: their device memory is entirely held
// by another allocator (a framework's caching pool or a solver's own
// arena), they run where an allocation would block or is not allowed (a
// solver callback, a real-time loop), or their build budgets device memory
// statically.  ggem_local_matvec_noalloc serves them: it runs the FP64
// cut-off cell-list pair sweep (the same arithmetic as the context path of
// ggem_local_matvec_dev with GGEM_FP64) with all of its scratch -- cell
// counts, the sorted cell list and slot-ordered copies of positions and
// forces -- in one fixed device array declared in this file.  Nothing is
// allocated, on the device or the host.
//
// The array is a file-scope __device__ object, so every GPU that loads this
// library holds its kNoAllocScratchBytes until the process exits.  All calls
// share it and it keeps the last call's contents; each call clears the cell
// counters it relies on.  Calls that overlap on the GPU (on any streams or
// from several host threads) race on the array and must be serialised by
// the caller.  The first call on a device looks up the array's device
// address with cudaGetSymbolAddress while that device is current; make that
// first call before any stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "ggem_internal.cuh"
#include "ggem_noalloc.h"

namespace ggem {
namespace {

constexpr int64_t kNaMaxParticles = GGEM_NOALLOC_MAX_PARTICLES;
constexpr int64_t kNaMaxCells = GGEM_NOALLOC_MAX_CELLS;
constexpr int kNaMaxDevices = 64;

// section sizes in bytes, each rounded up to 256
constexpr size_t al256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kOffCellOf = 0;                                              // int32[n]
constexpr size_t kOffCount = kOffCellOf + al256(4 * kNaMaxParticles);         // int32[ncell]
constexpr size_t kOffFill = kOffCount + al256(4 * kNaMaxCells);               // int32[ncell]
constexpr size_t kOffStart = kOffFill + al256(4 * kNaMaxCells);               // int32[ncell+1]
constexpr size_t kOffOrder = kOffStart + al256(4 * (kNaMaxCells + 1));        // int32[n]
constexpr size_t kOffSlotCell = kOffOrder + al256(4 * kNaMaxParticles);       // int32[n]
constexpr size_t kOffPos = kOffSlotCell + al256(4 * kNaMaxParticles);         // double4[n]
constexpr size_t kOffF = kOffPos + al256(32 * kNaMaxParticles);               // double[3n]
constexpr size_t kScratchBytes = kOffF + al256(24 * kNaMaxParticles);
static_assert(kScratchBytes == GGEM_NOALLOC_SCRATCH_BYTES, "header and layout disagree");

// the scratch of every call, on every device that loads the library
__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

unsigned char *g_scratch_dev[kNaMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;

struct NaBufs {
  int32_t *cell_of, *count, *fill, *start, *order, *slot_cell;
  double4_32a *pos;
  double *f;
};

NaBufs carve(unsigned char *base) {
  NaBufs b;
  b.cell_of = reinterpret_cast<int32_t *>(base + kOffCellOf);
  b.count = reinterpret_cast<int32_t *>(base + kOffCount);
  b.fill = reinterpret_cast<int32_t *>(base + kOffFill);
  b.start = reinterpret_cast<int32_t *>(base + kOffStart);
  b.order = reinterpret_cast<int32_t *>(base + kOffOrder);
  b.slot_cell = reinterpret_cast<int32_t *>(base + kOffSlotCell);
  b.pos = reinterpret_cast<double4_32a *>(base + kOffPos);
  b.f = reinterpret_cast<double *>(base + kOffF);
  return b;
}

__global__ void k_na_clear(int64_t ncell, NaBufs b, int *err) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < ncell) {
    b.count[k] = 0;
    b.fill[k] = 0;
  }
  if (k == 0) *err = 0;
}

// cell of each particle, floor((x - lo) / h) with the context path's rules:
// a coordinate outside [lo, lo + L) on a periodic axis is wrapped, one
// inside keeps its value (a bead whose x - lo rounds up to L stays in the
// last cell, the element search's closed upper face); a NaN or infinite
// coordinate sets the non-finite status bit and takes cell 0 on that axis
__global__ void k_na_assign(int64_t n, const double *__restrict__ xyz, Grid g, NaBufs b,
                            int *err) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c[3];
  bool bad = false, nonfinite = false;
  for (int d = 0; d < 3; ++d) {
    double x = xyz[3 * i + d];
    if (!isfinite(x)) {
      nonfinite = true;
      x = g.lo[d];
    }
    double t = x - g.lo[d];
    if (g.periodic[d]) {
      if (!(t >= 0.0 && t < g.L[d]) && !(x >= g.lo[d] && x < g.lo[d] + g.L[d])) {
        t = fmod(t, g.L[d]);
        if (t < 0) t += g.L[d];
        if (t >= g.L[d]) t = 0.0;
      }
    } else if (!(t >= 0.0 && t <= g.L[d])) {
      bad = true;
    }
    const int k = (int)floor(t / g.h[d]);
    c[d] = k < 0 ? 0 : (k >= g.nc[d] ? g.nc[d] - 1 : k);
  }
  if (bad) atomicOr(err, GGEM_NOALLOC_STATUS_OUT_OF_BOX);
  if (nonfinite) atomicOr(err, GGEM_NOALLOC_STATUS_NON_FINITE);
  const int32_t id = c[0] + g.nc[0] * (c[1] + g.nc[1] * c[2]);
  b.cell_of[i] = id;
  atomicAdd(&b.count[id], 1);
}

// exclusive scan of the cell counts by one block (ncell <= kNaMaxCells)
__global__ void __launch_bounds__(1024) k_na_scan(int64_t ncell, NaBufs b) {
  __shared__ int32_t warp_tot[32];
  __shared__ int32_t carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < ncell; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const int32_t v = (i < ncell) ? b.count[i] : 0;
    int32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int32_t w = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warp_tot[lane] = w;
    }
    __syncthreads();
    const int32_t excl = carry + (warp ? warp_tot[warp - 1] : 0) + x - v;
    if (i < ncell) b.start[i] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) b.start[ncell] = carry;
}

__global__ void k_na_scatter(int64_t n, NaBufs b) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t c = b.cell_of[i];
  b.order[b.start[c] + atomicAdd(&b.fill[c], 1)] = (int32_t)i;
}

__global__ void k_na_sort(int64_t ncell, NaBufs b) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int32_t lo = b.start[c], hi = b.start[c + 1];
  for (int32_t k = lo + 1; k < hi; ++k) {
    const int32_t v = b.order[k];
    int32_t m = k - 1;
    while (m >= lo && b.order[m] > v) {
      b.order[m + 1] = b.order[m];
      --m;
    }
    b.order[m + 1] = v;
  }
}

// slot-ordered positions (wrapped as the context path does), cells, forces
__global__ void k_na_gather(int64_t n, Grid g, const double *__restrict__ xyz,
                            const double *__restrict__ f, NaBufs b) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int32_t i = b.order[s];
  double p[3];
  for (int d = 0; d < 3; ++d) {
    double x = xyz[3 * (int64_t)i + d];
    if (g.periodic[d] && !(x >= g.lo[d] && x < g.lo[d] + g.L[d])) {
      double t = fmod(x - g.lo[d], g.L[d]);
      if (t < 0) t += g.L[d];
      if (t >= g.L[d]) t = 0.0;
      x = g.lo[d] + t;
    }
    p[d] = x;
  }
  b.pos[s] = make_double4_32a(p[0], p[1], p[2], 0.0);
  b.slot_cell[s] = b.cell_of[i];
  for (int d = 0; d < 3; ++d) b.f[3 * s + d] = f[3 * (int64_t)i + d];
}

// the FP64 cut-off pair sweep over the 27 neighbouring cells, written
// straight to the caller's particle order
__global__ void __launch_bounds__(128) k_na_sweep(int64_t n, Grid g, DevConsts K, double rc2,
                                                  int self_mode, NaBufs b,
                                                  double *__restrict__ u) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const double4_32a pi = b.pos[s];
  const int32_t cid = b.slot_cell[s];
  const int cx = cid % g.nc[0], cy = (cid / g.nc[0]) % g.nc[1], cz = cid / (g.nc[0] * g.nc[1]);
  double acc[3] = {0.0, 0.0, 0.0};
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        int c[3] = {cx + dx, cy + dy, cz + dz};
        bool ok = true;
        for (int d = 0; d < 3; ++d) {
          if (c[d] < 0 || c[d] >= g.nc[d]) {
            if (!g.periodic[d]) ok = false;
            else c[d] = (c[d] + g.nc[d]) % g.nc[d];
          }
        }
        if (!ok) continue;
        const int32_t cell = c[0] + g.nc[0] * (c[1] + g.nc[1] * c[2]);
        for (int32_t t = b.start[cell]; t < b.start[cell + 1]; ++t) {
          if (t == s) continue;
          const double4_32a pj = b.pos[t];
          double x[3] = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z};
          for (int k = 0; k < 3; ++k) {
            if (g.periodic[k]) {
              if (x[k] <= -g.L[k] / 2.0) x[k] += g.L[k];
              if (x[k] > g.L[k] / 2.0) x[k] -= g.L[k];
            }
          }
          const double r2c = __dadd_rn(__dadd_rn(__dmul_rn(x[0], x[0]), __dmul_rn(x[1], x[1])),
                                       __dmul_rn(x[2], x[2]));
          if (!(r2c < rc2)) continue;
          const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
          const double *fj = b.f + 3 * (int64_t)t;
          if (r < K.r_eps) {
            for (int a = 0; a < 3; ++a) acc[a] += K.coeff_2 * fj[a];
            continue;
          }
          // green_tensor_local_regularized (ggem_stokes.C:304-357) applied to f_j
          const double rr = r * r;
          const double kr = K.ksi * r, ar = K.alpha * r;
          const double c1 = (erf(kr) - erf(ar)) / r;
          const double c2 = K.two_ksi_sqrt_pi * exp(-kr * kr) - K.two_alpha_sqrt_pi * exp(-ar * ar);
          const double xf = (x[0] * fj[0] + x[1] * fj[1] + x[2] * fj[2]) / rr;
          const double pp = (c1 + c2) * K.one_eight_pi_mu, mm = (c1 - c2) * xf * K.one_eight_pi_mu;
          for (int a = 0; a < 3; ++a) acc[a] += pp * fj[a] + mm * x[a];
        }
      }
  const double *fi = b.f + 3 * s;
  double *ui = u + 3 * (int64_t)b.order[s];
  for (int a = 0; a < 3; ++a) {
    double v = acc[a];
    if (self_mode == GGEM_SELF_BEAD) v = (v - K.coeff_1 * fi[a]) + fi[a];
    else if (self_mode == GGEM_SELF_LAGRANGIAN) v = v + K.coeff_2 * fi[a];
    ui[a] = v;
  }
}

// the device address of the scratch array on the current device, looked up
// once per device
int scratch_for_current_device(unsigned char **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return GGEM_ERR_CUDA;
  if (dev < 0 || dev >= kNaMaxDevices) return GGEM_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_dev[dev]) {
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
      cudaGetLastError();
      return GGEM_ERR_CUDA;
    }
    g_scratch_dev[dev] = static_cast<unsigned char *>(ptr);
  }
  *out = g_scratch_dev[dev];
  return GGEM_OK;
}

}  // namespace
}  // namespace ggem

using namespace ggem;

extern "C" int ggem_local_matvec_noalloc(const ggem_params *p, int64_t n, const double *d_xyz,
                                         const double *d_f, double *d_u, int self_mode,
                                         int *d_status, void *stream) {
  if (!p || n < 0 || self_mode < 0 || self_mode > 2 || !d_status) return GGEM_ERR_BAD_ARG;
  if (n > 0 && (!d_xyz || !d_f || !d_u)) return GGEM_ERR_BAD_ARG;
  if (n > kNaMaxParticles) return GGEM_ERR_BAD_ARG;  // beyond GGEM_NOALLOC_MAX_PARTICLES
  if (p->nb_mode != GGEM_NB_CUTOFF) return GGEM_ERR_BAD_ARG;
  if (!(p->mu > 0) || !(p->alpha > 0) || !(p->br0 > 0) || p->point_type < 0 ||
      p->point_type > 2 || !(p->rc > 0) || !std::isfinite(p->rc))
    return GGEM_ERR_BAD_ARG;
  if (p->point_type == GGEM_LAGRANGIAN_POINT && !(p->ibm_beta > 0 && p->hmin > 0))
    return GGEM_ERR_BAD_ARG;
  ggem_constants cst;
  compute_constants(*p, &cst);
  if (!(cst.ksi > p->alpha)) return GGEM_ERR_BAD_ARG;
  const DevConsts K{cst.one_eight_pi_mu, cst.alpha, cst.alpha2, cst.alpha3_pi_23,
                    cst.two_alpha_sqrt_pi, cst.coeff_1, cst.ksi, cst.two_ksi_sqrt_pi,
                    cst.coeff_2, cst.r_eps};
  Grid g;
  std::memset(&g, 0, sizeof(g));
  for (int d = 0; d < 3; ++d) {
    if (!std::isfinite(p->box_lo[d]) || !std::isfinite(p->box_hi[d]) ||
        !(p->box_hi[d] > p->box_lo[d]))
      return GGEM_ERR_BAD_ARG;
    g.lo[d] = p->box_lo[d];
    g.L[d] = p->box_hi[d] - p->box_lo[d];
    g.periodic[d] = p->periodic[d] ? 1 : 0;
    int nc = (int)std::floor(g.L[d] / p->rc);
    nc = nc < 1 ? 1 : (nc > 2048 ? 2048 : nc);
    if (g.periodic[d] && nc < 3) return GGEM_ERR_BAD_ARG;  // edge >= 3 rc
    g.nc[d] = nc;
    g.h[d] = g.L[d] / nc;
    g.h32[d] = (float)g.h[d];
  }
  g.ncell = (int64_t)g.nc[0] * g.nc[1] * g.nc[2];
  if (g.ncell > kNaMaxCells) return GGEM_ERR_BAD_ARG;  // beyond GGEM_NOALLOC_MAX_CELLS
  unsigned char *base = nullptr;
  if (int rc = scratch_for_current_device(&base)) return rc;
  const NaBufs b = carve(base);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int T = 256;
  const unsigned bn = (unsigned)((n + T - 1) / T);
  const unsigned bc = (unsigned)((g.ncell + T - 1) / T);
  k_na_clear<<<bc, T, 0, st>>>(g.ncell, b, d_status);
  if (n > 0) {
    k_na_assign<<<bn, T, 0, st>>>(n, d_xyz, g, b, d_status);
    k_na_scan<<<1, 1024, 0, st>>>(g.ncell, b);
    k_na_scatter<<<bn, T, 0, st>>>(n, b);
    k_na_sort<<<bc, T, 0, st>>>(g.ncell, b);
    k_na_gather<<<bn, T, 0, st>>>(n, g, d_xyz, d_f, b);
    k_na_sweep<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(n, g, K, p->rc * p->rc, self_mode,
                                                          b, d_u);
  }
  if (cudaGetLastError() != cudaSuccess) return GGEM_ERR_CUDA;
  return GGEM_OK;
}
