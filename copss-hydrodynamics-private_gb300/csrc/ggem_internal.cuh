// ggem_internal.cuh -- shared declarations of the GB300 GGEM library.
//
// Data layout in HBM (all per context):
//   xyz_in     double[3n]   caller positions, original particle order
//   cell_of    int32[n]     cell (element) id of each particle
//   cell_start int32[ncell+1] sorted cell list (exclusive scan of counts)
//   order      int32[n]     slot -> original id, ascending within a cell
//   rank       int32[n]     original id -> slot
//   pos64      double4_32a[n]   wrapped positions in slot order (FP64 paths)
//   pos32      float4[n]    position relative to its cell centre (x,y,z) and
//                           the cell id bits (w), slot order (FP32 path)
//   pair list  uint32[n][W] fixed-width rows in slot order (row s holds
//                           nb_cnt[s] entries), entry =
//                           (source slot << 7) | stencil code, built in one
//                           pass per configuration with an FP32 filter and
//                           an exact FP64 decision in the rounding band
//   tab        float4[2*kTableN] cubic pieces of A(s), B(s), s = r^2, with
//                           G(x) = A I + B x x^T (FP32 path)
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "ggem_gb300.h"

namespace ggem {

constexpr int kTableN = 512;       // cubic pieces of the FP32 tensor table
constexpr int kCodeBits = 7;       // stencil code bits of a pair entry
constexpr int kMaxCode = 1 << kCodeBits;
constexpr int kMaxRhsChunk = 8;    // right-hand sides per pair-kernel pass
constexpr int kPolyDeg = 13;       // degree of the analytic tensor polynomials
constexpr int kGroup = 4;          // lanes per target in the pair kernel

// device error bits
enum : int {
  kErrOutOfDomain = 1,
  kErrListOverflow = 2,
  kErrTimeout = 4,
  kErrBadIndex = 8,
  kErrListCapacity = 16,  // speculative list fill ran past the allocated list
  kErrNonFinite = 32,     // a particle position is NaN or infinite
};

// derived GGEM constants (ggem_stokes.C:39-114) in FP64
struct DevConsts {
  double one_eight_pi_mu, alpha, alpha2, alpha3_pi_23, two_alpha_sqrt_pi, coeff_1;
  double ksi, two_ksi_sqrt_pi, coeff_2, r_eps;
};

// uniform cell grid over the box (cells == elements in reference mode)
struct Grid {
  double lo[3], L[3], h[3];
  double inv_h[3];  // 1 / h, for the fast path of the cell index
  float h32[3];
  // the cell index in FP32 away from the box faces and the cell faces:
  // lo, L and 1/h as floats, and the margins (box, in length; cell, in
  // units of h) beyond which FP32 rounding cannot change the FP64 result
  float lo32[3], L32[3], inv_h32[3], margin32[3], band32[3];
  int nc[3];
  int periodic[3];
  int64_t ncell;
};

template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t count = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    count = 0;
  }
  // grows (never shrinks); contents are not preserved
  cudaError_t ensure(size_t n) {
    if (n <= count && p) return cudaSuccess;
    release();
    size_t want = n ? n : 1;
    cudaError_t e = cudaMalloc(&p, want * sizeof(T));
    if (e == cudaSuccess) count = want;
    else p = nullptr;
    return e;
  }
};

}  // namespace ggem

struct ggem_ctx {
  ggem_params prm{};
  ggem_constants cst{};
  ggem::DevConsts dc{};
  ggem::Grid grid{};
  int device = 0;
  cudaStream_t stream = nullptr;      // active stream
  cudaStream_t own_stream = nullptr;  // created by the library
  std::string last_error;

  // stencils: offsets (dx,dy,dz,0); code k = index into the list
  std::vector<int4> stencil;          // neighbour cells (excludes (0,0,0) in reference mode)
  ggem::DevBuf<int4> d_stencil;
  ggem::DevBuf<float4> d_shift;       // FP32 offset * h for each stencil code
  float rc2_lo = 0.f, rc2_hi = 0.f;   // FP32 rounding band of the cutoff test
  double rc2 = 0.0;
  double search_radius_e = 0.0;

  // particles
  int64_t n = 0;
  bool cells_built = false;
  ggem::DevBuf<double> xyz_in;
  ggem::DevBuf<int32_t> cell_of, cell_count, cell_start, cell_fill, order, rank;
  // the cell counters were left at zero by the last build (and still live
  // at cell_counters_at)
  bool cell_counters_zero = false;
  const int32_t *cell_counters_at = nullptr;
  ggem::DevBuf<double4_32a> wrapped, pos64;
  ggem::DevBuf<float4> pos32;
  ggem::DevBuf<int> err;

  // FP32 pair list (built for GGEM_FP64 contexts too when f64_list is set:
  // the FP64 pair kernel then walks the exact list instead of sweeping cells)
  bool list_built = false;
  bool f64_list = false;
  // symmetric pair sums (ggem_set_symmetric_pairs): the list build also
  // writes the half list (each unordered pair once, in the row of its smaller
  // slot, same row width) and single-RHS FP32 matvecs evaluate each tensor
  // once, scattering the source side into sym_acc (FP32, zero between uses)
  bool sym_pairs = false;
  ggem::DevBuf<int32_t> nb_cnt_h;
  ggem::DevBuf<uint32_t> nb_list_h;
  ggem::DevBuf<float4> sym_acc;
  ggem::DevBuf<double> sym_part;
  // deferred checks (ggem_set_deferred_checks): a build after the first one
  // keeps the row width and leaves its statistics and error word on the
  // device; the next synchronising call reads them (list_unchecked)
  bool defer_checks = false;
  bool list_checked_once = false;
  bool list_unchecked = false;
  bool list_stat_zero = false;  // the cell scan of this configuration zeroed nb_stat
  int64_t n_pairs = 0;
  ggem::DevBuf<int32_t> nb_cnt;       // entries per target row
  ggem::DevBuf<unsigned long long> nb_stat;  // [0] total entries, [1] longest row
  int nb_w = 0;                       // row width (multiple of 8)
  ggem::DevBuf<uint32_t> nb_list;
  ggem::DevBuf<float4> tab;
  float tab_inv_ds = 0.f;
  double tab_max_err = 0.0;
  // analytic tensor: A = e^{-alpha^2 s} a(x), B = e^{-alpha^2 s} b(x),
  // x = s * poly_x1 + poly_x0, a and b monomials of degree kPolyDeg
  bool use_poly = false;
  float poly_a[16] = {0}, poly_b[16] = {0};
  float poly_x0 = 0.f, poly_x1 = 0.f, poly_e[2] = {0.f, 0.f};  // exponent hi + lo
  double poly_max_err = 0.0;
  // single-RHS pair kernel: 32-byte source records (2 float4 per slot):
  // w_src for plain matvecs, w_rec[2] for the fused Chebyshev chain (the
  // records of x_k in w_rec[rec_cur], those of x_{k+1} written to the other)
  ggem::DevBuf<float4> w_src;
  ggem::DevBuf<float4> w_rec[2];
  // per-pair tensors (A, sqrt(B) x) in the list's row layout, computed once
  // per configuration when B >= 0 on [0, rc^2]; forces then travel as one
  // float4 per slot (w_f4, w_f4n for the fused Chebyshev chain)
  bool use_pretensor = false;   // B >= 0 holds for these constants
  bool allow_pretensor = true;  // ggem_set_pair_tensors
  bool pretensor_ok = false;
  int stored_variant = 0;         // shape of the stored-tensor pair kernels (autotuned)
  int computed_variant = 0;       // loop shape of the per-matvec-tensor kernels (autotuned)
  ggem::DevBuf<float4> pair_ten;
  ggem::DevBuf<float4> w_f4[2];
  int rec_cur = 0;
  int cheb_pred_terms = 0;             // degree the last adaptive Chebyshev needed
  // polymer bonds as a per-bead adjacency (caller ids, bond order)
  int64_t bond_n = -1;                 // particle count the bonds were set for
  ggem::DevBuf<int64_t> bond_off;      // [n+1]
  ggem::DevBuf<int32_t> bond_nbr;      // [2m]

  // element-major quadrature points of the mesh (ggem_set_quadrature,
  // reference mode): FP64 as given and FP32 relative to the element centre;
  // the spread's element-offset bitmap and its pair counter
  int q_per_elem = 0;
  ggem::DevBuf<double> q_xyz;
  ggem::DevBuf<float4> q_rel;
  ggem::DevBuf<uint32_t> sp_bits;
  ggem::DevBuf<unsigned long long> sp_pairs;

  // scan scratch (one per recursion level)
  std::vector<ggem::DevBuf<int64_t> *> scan_scratch;

  // vector workspaces (FP64 slot order) and FP32 staging
  ggem::DevBuf<double> w_in, w_out, w_a, w_b, w_c, w_d, w_e, w_y;
  ggem::DevBuf<float4> w_f32;
  ggem::DevBuf<float> w_fb;     // batched forces [slot][3][64] FP32
  ggem::DevBuf<float> w_fb2;    // the next term's staging in a fused batched series
  ggem::DevBuf<double> w_red;   // reduction partials
  ggem::DevBuf<double> lz_Q;    // Lanczos basis
  double *h_red = nullptr;      // pinned host mirror of reductions
  cudaEvent_t ev_readback = nullptr;  // recorded behind the reductions' readback
  // host inputs of ggem_brownian_displacement: copied on their own stream
  // into a buffer no other call uses
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_copy = nullptr;
  ggem::DevBuf<double> w_hin;
  double *h_stage = nullptr;    // pinned host staging
  size_t h_stage_bytes = 0;

  // measurement hooks (ggem_diag.h)
  int64_t launches = 0;
  bool timing = false;
  struct KTimer {
    std::vector<cudaEvent_t> ev;  // start/stop pairs
    std::vector<int> n;           // launches inside each closed pair
    double total_ms = 0.0;
    int64_t count = 0;
  } ktimer[5];
  unsigned timing_mask = 0x1fu;  // kernel kinds timed while timing is on
  // The fused single-RHS series' prefix (first step, unchecked terms, the
  // first checked term and its check's device half) as one CUDA graph:
  // built when the same key comes back, replayed while it holds.
  // Three graphs: the first step, the fused terms, the check; the kernel
  // timer's span around the fused terms is recorded between them.
  bool series_graphs = true;
  cudaGraphExec_t sg_exec[3] = {nullptr, nullptr, nullptr};
  std::vector<uint64_t> sg_key;
  int64_t sg_launches = 0;  // kernel launches inside the three
  int64_t sg_captures = 0, sg_replays = 0;
  // an open span (kt_span_begin): one event pair around consecutive
  // launches of one kind, which then record no events of their own
  int span_kind = -1;
  int span_n = 0;
  std::vector<cudaEvent_t> ev_pool;
  // launch trace (ggem_set_launch_trace): one event after every launch
  bool trace = false;
  std::vector<std::pair<const char *, cudaEvent_t>> trace_ev;

  ~ggem_ctx();
};

namespace ggem {

#ifdef __CUDACC__
// double -> float rounded to nearest even, from the IEEE 754 bit fields
// with integer operations only (GB300 runs FP64 conversions at the FP64
// rate, 1/64 of FP32); results below the float normal range (|x| < 2^-126)
// take the hardware conversion.  Checked bit for bit against
// __double2float_rn (ggem_diag_convert_f32).
__device__ __forceinline__ float d2f_bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int ex = (int)((b >> 52) & 0x7ffu);
  const unsigned long long m = b & 0xfffffffffffffull;
  if (ex == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x400000u : 0u));
  const int e32 = ex - 1023 + 127;
  if (e32 >= 255) return __uint_as_float(sign | 0x7f800000u);
  if (e32 <= 0) return __double2float_rn(x);
  unsigned long long keep = m >> 29;
  const unsigned long long rem = m & 0x1fffffffull, half = 0x10000000ull;
  keep += (rem > half || (rem == half && (keep & 1ull))) ? 1ull : 0ull;
  // a carry out of the mantissa moves into the exponent (up to infinity)
  return __uint_as_float(sign | (uint32_t)(((unsigned long long)e32 << 23) + keep));
}
#endif

// kernel kinds of the timing hooks
enum : int { kKPairF32 = 0, kKPairF64 = 1, kKChebTerm = 2, kKListBuild = 3, kKPairCheb = 4 };

void kt_start(ggem_ctx *c, int kind);
void kt_stop(ggem_ctx *c, int kind);
// one event pair around a run of consecutive launches of one kind (kt_start
// / kt_stop of that kind inside the run only count launches); the run must
// contain no launch of another kernel
void kt_span_begin(ggem_ctx *c, int kind);
void kt_span_end(ggem_ctx *c);
bool kt_enabled(const ggem_ctx *c, int kind);
void trace_mark(ggem_ctx *c, const char *what);

int fail(ggem_ctx *c, int code, const std::string &msg);
int cuda_fail(ggem_ctx *c, cudaError_t e, const char *what);
int check_launch(ggem_ctx *c, const char *what);
int read_error_flags(ggem_ctx *c, int *flags);
int ensure_host_stage(ggem_ctx *c, size_t bytes);

// host-side helpers (ggem_host.cpp)
void compute_constants(const ggem_params &p, ggem_constants *c);
int fit_tensor_table(const ggem_constants &c, double s_max, int nt, std::vector<float4> &tab,
                     double *max_err);
int fit_tensor_poly(const ggem_constants &c, double s_max, float *a, float *b, float *x0,
                    float *x1, float *e_coef, double *max_err);
bool tensor_b_nonnegative(const ggem_constants &c, double s_max);
void tridiag_extremes(int k, const double *a, const double *b, double *lmin, double *lmax);
void cheb_coeffs_host(int N, double da, double db, int method, double *coef);
void cheb_coeffs_host_many(int N, int K, const double *da, const double *db, int method,
                           double *coef, int ldc);

// cell build and pair list (ggem_cells.cu)
// defer_flags: leave the device error word unread (build_pair_list reads it)
int build_cells(ggem_ctx *c, bool defer_flags = false);
int cell_flag_error(ggem_ctx *c, int flags);
int build_pair_list(ggem_ctx *c);
// deferred builds: copy the list statistics and the error word to the host
// mirror (asynchronous), then, after the stream has synchronised, evaluate
// them; *rebuilt is set when the rows had overflowed and the list (and the
// stored pair tensors) were rebuilt wider: results computed since the
// build are void.  settle_list does both with its own synchronisation.
int enqueue_list_check(ggem_ctx *c);
int finish_list_check(ggem_ctx *c, unsigned long long total, unsigned long long longest, int flags,
                      bool *rebuilt);
int settle_list(ggem_ctx *c);
constexpr int kListStatSlot = 4088;  // h_red[4088 .. 4090]: deferred list statistics
int device_exclusive_scan_i32(ggem_ctx *c, const int32_t *in, int32_t *out, int64_t n);
int device_exclusive_scan_i64(ggem_ctx *c, const int64_t *in, int64_t *out, int64_t n);

// pair sums (ggem_pair.cu); vectors in slot order, [r][slot][3] doubles
int matvec_slots(ggem_ctx *c, int nrhs, const double *d_f_slot, double *d_u_slot,
                 int self_mode);
int matvec_f32_staged(ggem_ctx *c, int nrhs, const double *d_f_slot, double *d_u_slot,
                      int self_mode);
// the batched series' first step (x1 = db x0 + da x1, dw = c0 x0 + c1 x1)
// with x1's FP32 staging left in w_fb (16 .. 64 right-hand sides)
int cheb_start_staged(ggem_ctx *c, int nrhs, double da, double db, double c0, double c1,
                      const double *x0, double *x1, double *dw);
// xi (caller order) into slot order x0 with its batched FP32 staging in w_fb
// (16 .. 64 right-hand sides; returns false and does nothing otherwise)
bool to_slots_staged(ggem_ctx *c, int nrhs, const double *xi, double *x0, int *rc);
// u = M f for 16 .. 64 right-hand sides whose batched FP32 staging a fused
// batched term left in w_fb (other counts: matvec_slots)
int matvec_slots_prestaged(ggem_ctx *c, int nrhs, const double *d_f_slot, double *d_u_slot,
                           int self_mode);
double self_coefficient(const ggem_ctx *c, int self_mode);
int build_pair_tensors(ggem_ctx *c);
int pair_cheb_term(ggem_ctx *c, bool records_fresh, const double *x0, const double *x1,
                   double *xm, double *dw, double two_da, double two_db, double coef,
                   int self_mode, double *norms = nullptr);
// an unchecked Chebyshev term for this many right-hand sides can run as one
// batched kernel (batch_cheb_term)
bool batch_term_fusable(const ggem_ctx *c, int nrhs);
int batch_cheb_term(ggem_ctx *c, int nrhs, bool staged_fresh, const double *x0, const double *x1,
                    double *xm, double *dw, double two_da, double two_db, const double *coef,
                    int self_mode);
// blocks of the single-RHS pair kernels, and the partial sums a fused
// series' estimator sums leave (one per block)
int pair_grid_blocks(const ggem_ctx *c);
int64_t pair_partials(const ggem_ctx *c);
// u = M dw from the dw records a checked fused term left (norms given to
// pair_cheb_term); |u|^2 as per-block partials into norm
int matvec_dw_records(ggem_ctx *c, const double *dw, double *u, int self_mode, double *norm);
int matvec_records(ggem_ctx *c, const float4 *rec, const double *f, double *u, int self_mode,
                   double *norm);
// u = M f, one right-hand side, caller order in and out (FP32 list with
// per-matvec tensors only); f_slot receives f in slot order
int matvec_orig_fused(ggem_ctx *c, const double *f, double *u, double *f_slot, int self_mode);
// the fused first step of a series (xi in caller order; m = M x0 is kept)
int cheb_start_fused(ggem_ctx *c, const double *xi, double *x0, double *m, double *x1,
                     double *dw, double da, double db, double c0, double c1, int self_mode,
                     double *aux2 = nullptr);
int permute_to_slots(ggem_ctx *c, int nrhs, const double *d_orig, double *d_slot);
int permute_from_slots(ggem_ctx *c, int nrhs, const double *d_slot, double *d_orig);

}  // namespace ggem
