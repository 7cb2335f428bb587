// ggem_host.cpp -- host-side parts of the GGEM library: constants, the FP32
// tensor table, Chebyshev coefficients, the tridiagonal eigen solver of the
// Lanczos bounds, the reference noise stream and synthetic workloads.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "ggem_internal.cuh"
#include "ggem_workloads.h"

namespace ggem {

// libMesh::pi as a double (libmesh_common.h)
static const double kPi = 3.14159265358979323846264338327950288;

// GGEMStokes::set_mu, set_alpha, set_ksi (ggem_stokes.C:39-114)
void compute_constants(const ggem_params &p, ggem_constants *c) {
  const double sqrt_pi = std::sqrt(kPi);
  const double pi_23 = std::pow(kPi, 3. / 2.);
  std::memset(c, 0, sizeof(*c));
  c->r_eps = 1e-6;
  c->mu = p.mu;
  c->one_eight_pi_mu = 1. / (8. * kPi * p.mu);
  c->alpha = p.alpha;
  c->alpha2 = p.alpha * p.alpha;
  c->alpha3 = c->alpha2 * p.alpha;
  c->alpha3_pi_23 = c->alpha3 / pi_23;
  c->two_alpha_sqrt_pi = 2. * p.alpha / sqrt_pi;
  c->coeff_1 = c->one_eight_pi_mu * 4.0 * p.alpha / sqrt_pi;
  c->br0 = p.br0;
  if (p.point_type == GGEM_LAGRANGIAN_POINT) c->ksi = 1.0 / (p.ibm_beta * p.hmin);
  else c->ksi = sqrt_pi / (3. * p.br0);
  c->ksi2 = c->ksi * c->ksi;
  c->ksi3 = c->ksi2 * c->ksi;
  c->ksi3_pi_23 = c->ksi3 / pi_23;
  c->two_ksi_sqrt_pi = 2. * c->ksi / sqrt_pi;
  c->coeff_2 = c->one_eight_pi_mu * 4.0 * (c->ksi - p.alpha) / sqrt_pi;
}

// A(s) = k (c1 + c2), B(s) = k (c1 - c2) / s with s = r^2, so that
// G(x) = A I + B x x^T equals green_tensor_local_regularized
// (ggem_stokes.C:304-357): (I + xx/r^2) c1 + (I - xx/r^2) c2.
static void tensor_ab(const ggem_constants &c, double s, double *A, double *B,
                      double *scale) {
  const double k = c.one_eight_pi_mu;
  const double two_sqrt_pi = 2.0 / std::sqrt(kPi);
  if (s < 0.5) {
    // Taylor series in s of erf(z)/r and z exp(-z^2)/r (z = a r): both are
    // (2/sqrt(pi)) sum_n (-1)^n a^(2n+1) s^n / n! * {1/(2n+1), 1}
    double sum_p = 0.0, sum_m = 0.0, term_s = 1.0, fact = 1.0;
    double kp = c.ksi, ap = c.alpha;  // a^(2n+1)
    for (int n = 0; n < 40; ++n) {
      if (n > 0) {
        fact *= n;
        term_s *= s;
        kp *= c.ksi * c.ksi;
        ap *= c.alpha * c.alpha;
      }
      const double sign = (n % 2) ? -1.0 : 1.0;
      const double d = (kp - ap) * term_s / fact * sign;
      const double c1n = d / (2.0 * n + 1.0);
      const double c2n = d;
      sum_p += c1n + c2n;
      // (c1 - c2)/s: the n = 0 terms cancel exactly
      if (n > 0) sum_m += (c1n - c2n) / s;
    }
    if (s == 0.0) {
      // limit of (c1 - c2)/s: (2/3)(ksi^3 - alpha^3)
      sum_m = (2.0 / 3.0) * (c.ksi3 - c.alpha3);
    }
    *A = k * two_sqrt_pi * sum_p;
    *B = k * two_sqrt_pi * sum_m;
    *scale = std::fabs(*A) + std::fabs(*B) * s + 1e-300;
    return;
  }
  const double r = std::sqrt(s);
  const double c1 = (std::erf(c.ksi * r) - std::erf(c.alpha * r)) / r;
  const double c2 = c.two_ksi_sqrt_pi * std::exp(-c.ksi2 * s) -
                    c.two_alpha_sqrt_pi * std::exp(-c.alpha2 * s);
  *A = k * (c1 + c2);
  *B = k * (c1 - c2) / s;
  *scale = k * (std::fabs(c1) + std::fabs(c2)) + 1e-300;
}

// Piecewise cubic fit of A and B on nt equal pieces of [0, s_max]; piece i
// holds monomial coefficients in t = s/ds - i for A (tab[2i]) and B
// (tab[2i+1]).  Interpolation at the four Chebyshev points of each piece.
int fit_tensor_table(const ggem_constants &c, double s_max, int nt, std::vector<float4> &tab,
                     double *max_err) {
  tab.assign(2 * nt, make_float4(0.f, 0.f, 0.f, 0.f));
  const double ds = s_max / nt;
  double worst = 0.0;
  for (int i = 0; i < nt; ++i) {
    double tn[4], fa[4], fb[4];
    for (int k = 0; k < 4; ++k) {
      tn[k] = 0.5 - 0.5 * std::cos((2.0 * k + 1.0) * kPi / 8.0);
      double sc;
      tensor_ab(c, (i + tn[k]) * ds, &fa[k], &fb[k], &sc);
    }
    // Newton divided differences -> monomial coefficients
    double ca[4], cb[4];
    for (int which = 0; which < 2; ++which) {
      double d[4];
      for (int k = 0; k < 4; ++k) d[k] = which ? fb[k] : fa[k];
      for (int lvl = 1; lvl < 4; ++lvl)
        for (int k = 3; k >= lvl; --k) d[k] = (d[k] - d[k - 1]) / (tn[k] - tn[k - lvl]);
      // p(t) = d0 + d1 (t-t0) + d2 (t-t0)(t-t1) + d3 (t-t0)(t-t1)(t-t2)
      double m[4] = {d[3], 0, 0, 0};  // Horner expansion into monomials
      double deg = 0;
      for (int k = 2; k >= 0; --k) {
        // m(t) = m(t) * (t - tn[k]) + d[k]
        double nm[4] = {0, 0, 0, 0};
        for (int q = 0; q <= deg; ++q) {
          nm[q + 1] += m[q];
          nm[q] -= m[q] * tn[k];
        }
        nm[0] += d[k];
        std::memcpy(m, nm, sizeof(m));
        deg += 1;
      }
      // m[q] is the coefficient of t^q
      double *dst = which ? cb : ca;
      for (int q = 0; q < 4; ++q) dst[q] = m[q];
    }
    tab[2 * i] = make_float4((float)ca[0], (float)ca[1], (float)ca[2], (float)ca[3]);
    tab[2 * i + 1] = make_float4((float)cb[0], (float)cb[1], (float)cb[2], (float)cb[3]);
    for (int q = 0; q <= 16; ++q) {
      const double t = q / 16.0;
      double A, B, sc;
      tensor_ab(c, (i + t) * ds, &A, &B, &sc);
      const double pa = ((ca[3] * t + ca[2]) * t + ca[1]) * t + ca[0];
      const double pb = ((cb[3] * t + cb[2]) * t + cb[1]) * t + cb[0];
      const double s = (i + t) * ds;
      const double e = (std::fabs(pa - A) + std::fabs(pb - B) * s) / sc;
      worst = std::max(worst, e);
    }
  }
  if (max_err) *max_err = worst;
  return (worst < 1e-5) ? 0 : -1;
}

// Analytic form of the FP32 tensor: A(s) = e^{-alpha^2 s} a(s) and
// B(s) = e^{-alpha^2 s} b(s).  a and b are entire in s (the 1/r singularities
// of the two erf terms cancel), so one Chebyshev interpolant of degree
// kPolyDeg on [0, s_max] reaches ~1e-9; it is stored as monomials in
// x = 2 s / s_max - 1 for FP32 Horner evaluation.  The returned max_err is
// measured with FP32 arithmetic (fused multiply-adds, as on the device) on a
// dense grid, relative to |A| + |B| s; the caller falls back to the table when
// it is too large.
// B(s) >= 0 on [0, s_max] (sampled densely in FP64): the condition under
// which a pair's tensor packs as (A, sqrt(B) x)
bool tensor_b_nonnegative(const ggem_constants &c, double s_max) {
  const int m = 20000;
  for (int k = 0; k <= m; ++k) {
    double A, B, sc;
    tensor_ab(c, s_max * k / m, &A, &B, &sc);
    if (!(B >= 0.0)) return false;
  }
  return true;
}

int fit_tensor_poly(const ggem_constants &c, double s_max, float *a, float *b, float *x0,
                    float *x1, float *e_coef, double *max_err) {
  const int deg = kPolyDeg;
  const double al2 = c.alpha2;
  std::vector<double> fa(deg + 1), fb(deg + 1);
  for (int j = 0; j <= deg; ++j) {
    const double xj = std::cos(kPi * (j + 0.5) / (deg + 1));
    const double s = (xj + 1.0) * 0.5 * s_max;
    double A, B, sc;
    tensor_ab(c, s, &A, &B, &sc);
    fa[j] = A * std::exp(al2 * s);
    fb[j] = B * std::exp(al2 * s);
  }
  std::vector<double> ca(deg + 1), cb(deg + 1);
  for (int k = 0; k <= deg; ++k) {
    double sa = 0.0, sb = 0.0;
    for (int j = 0; j <= deg; ++j) {
      const double t = std::cos(k * kPi * (j + 0.5) / (deg + 1));
      sa += fa[j] * t;
      sb += fb[j] * t;
    }
    ca[k] = sa * 2.0 / (deg + 1);
    cb[k] = sb * 2.0 / (deg + 1);
  }
  ca[0] *= 0.5;
  cb[0] *= 0.5;
  // Chebyshev -> monomial coefficients (T_k expanded by the recurrence)
  std::vector<std::vector<double>> T(deg + 1, std::vector<double>(deg + 1, 0.0));
  T[0][0] = 1.0;
  if (deg >= 1) T[1][1] = 1.0;
  for (int k = 2; k <= deg; ++k)
    for (int q = 0; q <= k; ++q) T[k][q] = (q > 0 ? 2.0 * T[k - 1][q - 1] : 0.0) - T[k - 2][q];
  for (int q = 0; q < 16; ++q) {
    a[q] = 0.f;
    b[q] = 0.f;
  }
  for (int q = 0; q <= deg; ++q) {
    double ma = 0.0, mb = 0.0;
    for (int k = 0; k <= deg; ++k) {
      ma += ca[k] * T[k][q];
      mb += cb[k] * T[k][q];
    }
    a[q] = (float)ma;
    b[q] = (float)mb;
  }
  *x1 = (float)(2.0 / s_max);
  *x0 = -1.0f;
  // exponent coefficient split into two floats (hi + lo)
  const double ecoef = -al2 / std::log(2.0);
  e_coef[0] = (float)ecoef;
  e_coef[1] = (float)(ecoef - (double)e_coef[0]);
  double worst = 0.0;
  const int samples = 20000;
  for (int i = 0; i <= samples; ++i) {
    const double s = s_max * i / samples;
    const float s32 = (float)s;
    const float x = std::fmaf(s32, *x1, *x0);
    float pa = a[deg], pb = b[deg];
    for (int q = deg - 1; q >= 0; --q) {
      pa = std::fmaf(pa, x, a[q]);
      pb = std::fmaf(pb, x, b[q]);
    }
    const float pe = s32 * e_coef[0];
    const float re = std::fmaf(s32, e_coef[1], std::fmaf(s32, e_coef[0], -pe));
    const float E0 = std::exp2f(pe);
    const float E = std::fmaf(E0, re * 0.6931471805599453f, E0);
    double A, B, sc;
    tensor_ab(c, (double)s32, &A, &B, &sc);
    const double e = (std::fabs((double)(pa * E) - A) + std::fabs((double)(pb * E) - B) * s) / sc;
    worst = std::max(worst, e);
  }
  if (max_err) *max_err = worst;
  return (worst <= 1e-6) ? 0 : -1;
}

// smallest / largest eigenvalue of a symmetric tridiagonal matrix (diagonal
// a, off-diagonal b) by Sturm-sequence bisection
static int sturm_below(int k, const double *a, const double *b, double x) {
  int cnt = 0;
  double d = 1.0;
  for (int i = 0; i < k; ++i) {
    const double bb = (i > 0) ? b[i - 1] * b[i - 1] : 0.0;
    d = a[i] - x - (i > 0 ? bb / d : 0.0);
    if (d == 0.0) d = -1e-300;
    if (d < 0) ++cnt;
  }
  return cnt;
}

void tridiag_extremes(int k, const double *a, const double *b, double *lmin, double *lmax) {
  double lo = a[0], hi = a[0];
  for (int i = 0; i < k; ++i) {
    const double r = (i > 0 ? std::fabs(b[i - 1]) : 0.) + (i < k - 1 ? std::fabs(b[i]) : 0.);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  const double pad = 1e-12 * (std::fabs(lo) + std::fabs(hi)) + 1e-300;
  for (int which = 0; which < 2; ++which) {
    double l = lo - pad, h = hi + pad;
    const int target = which ? k - 1 : 0;
    for (int it = 0; it < 200; ++it) {
      const double mid = 0.5 * (l + h);
      if (mid == l || mid == h) break;
      if (sturm_below(k, a, b, mid) > target) h = mid;
      else l = mid;
    }
    (which ? *lmax : *lmin) = 0.5 * (l + h);
  }
}

// Chebyshev::chebyshev_coefficients and its three quadratures
// (chebyshev.C:44-190).  The expressions keep the reference's evaluation
// order so that the coefficients agree bit for bit.
// K intervals at once (the ensemble's suspensions): the quadrature nodes,
// weights and cos(tmpt) depend only on N and the method, so they are formed
// once; each coefficient keeps the reference's expression and summation
// order (acc += w_j cos(tmpt) f_j over j), so the values are the same bits
// as one interval at a time.  coef of interval b starts at coef + b * ldc.
// c_k of every interval from the nodes x_j and the table w_j cos(tmpt(k, j))
static void cheb_coeffs_from_table(int N, int K, const double *__restrict__ da,
                                   const double *__restrict__ db, const double *__restrict__ x,
                                   const double *__restrict__ wc, double *__restrict__ coef,
                                   int ldc) {
  const double PI = kPi;
  std::vector<double> fjv(N + 1);
  double *__restrict__ fj = fjv.data();
  for (int b = 0; b < K; ++b) {
    for (int j = 0; j <= N; ++j) fj[j] = 1.0 / std::sqrt((x[j] - db[b]) / da[b]);
    double *cb = coef + (size_t)b * ldc;
    // four coefficients at a time: four independent sums, each in j order
    int k = 0;
    for (; k + 3 <= N; k += 4) {
      const double *r0 = wc + (size_t)k * (N + 1), *r1 = r0 + (N + 1), *r2 = r1 + (N + 1),
                   *r3 = r2 + (N + 1);
      double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      for (int j = 0; j <= N; ++j) {
        const double f = fj[j];
        a0 += r0[j] * f;
        a1 += r1[j] * f;
        a2 += r2[j] * f;
        a3 += r3[j] * f;
      }
      cb[k] = a0 * (2. / (PI * (k == 0 ? 2.0 : 1.0)));
      cb[k + 1] = a1 * (2. / PI);
      cb[k + 2] = a2 * (2. / PI);
      cb[k + 3] = a3 * (2. / PI);
    }
    for (; k <= N; ++k) {
      const double *row = wc + (size_t)k * (N + 1);
      double acc = 0.0;
      for (int j = 0; j <= N; ++j) acc += row[j] * fj[j];
      const double ck = (k == 0) ? 2.0 : 1.0;
      cb[k] = acc * (2. / (PI * ck));
    }
  }
}

void cheb_coeffs_host_many(int N, int K, const double *da, const double *db, int method,
                           double *coef, int ldc) {
  // the nodes and the w_j cos(tmpt(k, j)) table depend on (N, method) only:
  // kept per thread for the next call
  struct Table {
    int N = -1, method = -1;
    std::vector<double> x, wc;
  };
  thread_local Table T;
  const double PI = kPi;
  if (T.N == N && T.method == method) {
    cheb_coeffs_from_table(N, K, da, db, T.x.data(), T.wc.data(), coef, ldc);
    return;
  }
  std::vector<double> x(N + 1), w(N + 1);
  for (int i = 0; i <= N; ++i) {
    const double j = (double)i;
    if (method == GGEM_CHEB_GAUSS_LOBATTO) {
      x[i] = std::cos(PI * j / (double)N);
      w[i] = PI / (double)N;
    } else if (method == GGEM_CHEB_GAUSS_RADAU) {
      x[i] = std::cos(2. * PI * j / (2. * (double)N + 1.));
      w[i] = 2. * PI / (2. * (double)N + 1.);
    } else {
      x[i] = std::cos((2. * j + 1.) * PI / (2. * (double)N + 2.));
      w[i] = PI / ((double)N + 1.);
    }
  }
  if (method == GGEM_CHEB_GAUSS_LOBATTO) {
    w[0] = PI / (2. * (double)N);
    w[N] = PI / (2. * (double)N);
  } else if (method == GGEM_CHEB_GAUSS_RADAU) {
    w[0] = PI / (2. * (double)N + 1.);
  }
  const double RN = (double)N;
  std::vector<double> wc((size_t)(N + 1) * (N + 1));  // w_j cos(tmpt(k, j))
  for (int k = 0; k <= N; ++k)
    for (int j = 0; j <= N; ++j) {
      double tmpt;
      if (method == GGEM_CHEB_GAUSS_LOBATTO) tmpt = PI * (double)((size_t)k * (size_t)j) / RN;
      else if (method == GGEM_CHEB_GAUSS_RADAU)
        tmpt = 2. * PI * (double)((size_t)k * (size_t)j) / (2. * RN + 1.);
      else tmpt = PI * (double)(2. * j + 1.) * (double)k / (2. * RN + 2.);
      wc[(size_t)k * (N + 1) + j] = w[j] * std::cos(tmpt);
    }
  cheb_coeffs_from_table(N, K, da, db, x.data(), wc.data(), coef, ldc);
  T.x = std::move(x);
  T.wc = std::move(wc);
  T.N = N;
  T.method = method;
}

void cheb_coeffs_host(int N, double da, double db, int method, double *coef) {
  cheb_coeffs_host_many(N, 1, &da, &db, method, coef, N + 1);
}

}  // namespace ggem

extern "C" int ggem_cheb_coeffs(int N, double da, double db, int method, double *coef) {
  if (N < 1 || !coef || method < 0 || method > 2 || !(da > 0.0) || !std::isfinite(db))
    return GGEM_ERR_BAD_ARG;
  ggem::cheb_coeffs_host(N, da, db, method, coef);
  return GGEM_OK;
}

// random_generator.C:43-67 and brownian_system.C:434-472: a default engine
// seeded once, a fresh normal_distribution per vector.
extern "C" int ggem_std_random_vector(uint64_t seed, int64_t skip_vectors, int64_t n,
                                      double mean, double stddev, double *out) {
  if (n < 0 || skip_vectors < 0 || !(stddev >= 0.0) || (n > 0 && !out)) return GGEM_ERR_BAD_ARG;
  std::default_random_engine gen;
  gen.seed(static_cast<std::size_t>(seed));
  for (int64_t v = 0; v <= skip_vectors; ++v) {
    std::normal_distribution<double> dist(mean, stddev);
    dist.reset();
    for (int64_t i = 0; i < n; ++i) {
      const double x = dist(gen);
      if (v == skip_vectors) out[i] = x;
    }
  }
  return GGEM_OK;
}

// ---------------------------------------------------------------------------
// Synthetic workloads (seeded): random sequential non-overlapping placement
// and self-avoiding bead-spring chains in a periodic cube.
// ---------------------------------------------------------------------------
namespace {

struct SplitMix {
  uint64_t s;
  explicit SplitMix(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return ((next() >> 11) + 0.5) * 0x1.0p-53; }
  double normal() {
    const double u1 = uniform(), u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * ggem::kPi * u2);
  }
};

// hash grid of cell side >= min_sep for overlap tests in a periodic cube
struct OverlapGrid {
  double L, h;
  int nc;
  std::vector<std::vector<int64_t>> cells;
  const double *xyz;
  OverlapGrid(double L_, double min_sep, const double *p) : L(L_), xyz(p) {
    nc = std::max(1, std::min(512, (int)std::floor(L / min_sep)));
    h = L / nc;
    cells.resize((size_t)nc * nc * nc);
  }
  int coord(double x) const {
    double t = std::fmod(x, L);
    if (t < 0) t += L;
    int c = (int)(t / h);
    return std::min(std::max(c, 0), nc - 1);
  }
  bool overlaps(const double *p, double min2, int64_t skip) const {
    const int cx = coord(p[0]), cy = coord(p[1]), cz = coord(p[2]);
    const int span = nc >= 3 ? 1 : 0;
    for (int dz = -span; dz <= span; ++dz)
      for (int dy = -span; dy <= span; ++dy)
        for (int dx = -span; dx <= span; ++dx) {
          const int ix = (cx + dx + nc) % nc, iy = (cy + dy + nc) % nc, iz = (cz + dz + nc) % nc;
          for (int64_t j : cells[((size_t)iz * nc + iy) * nc + ix]) {
            if (j == skip) continue;
            double r2 = 0;
            for (int d = 0; d < 3; ++d) {
              double v = xyz[3 * j + d] - p[d];
              v -= L * std::nearbyint(v / L);
              r2 += v * v;
            }
            if (r2 < min2) return true;
          }
        }
    return false;
  }
  void insert(int64_t i) {
    const double *p = xyz + 3 * i;
    cells[((size_t)coord(p[2]) * nc + coord(p[1])) * nc + coord(p[0])].push_back(i);
  }
};

}  // namespace

namespace {

// grows n_chains self-avoiding random-walk chains (bond length `bond`,
// beads closer than sqrt(min2) rejected, the bonded predecessor skipped) at
// indices [base, base + n_chains * beads); a chain that runs into a dead end
// is removed and grown again
int grow_chains(SplitMix &rng, OverlapGrid &g, double *xyz, double L, int64_t base0,
                int64_t n_chains, int beads_per_chain, double bond, double min2) {
  for (int64_t c = 0; c < n_chains; ++c) {
    const int64_t base = base0 + c * beads_per_chain;
    int64_t restarts = 0;
  restart:
    if (++restarts > 10000) return GGEM_ERR_BAD_ARG;
    for (int b = 0; b < beads_per_chain; ++b) {
      const int64_t i = base + b;
      int tries = 0;
      for (;;) {
        if (++tries > 2000) {
          // dead end: remove this chain's beads and grow it again
          for (int q = 0; q < b; ++q) {
            const int64_t k = base + q;
            auto &cell = g.cells[((size_t)g.coord(xyz[3 * k + 2]) * g.nc + g.coord(xyz[3 * k + 1])) *
                                     g.nc +
                                 g.coord(xyz[3 * k])];
            cell.erase(std::remove(cell.begin(), cell.end(), k), cell.end());
          }
          goto restart;
        }
        if (b == 0) {
          for (int d = 0; d < 3; ++d) xyz[3 * i + d] = rng.uniform() * L;
        } else {
          double v[3], nv = 0;
          do {
            nv = 0;
            for (int d = 0; d < 3; ++d) {
              v[d] = rng.normal();
              nv += v[d] * v[d];
            }
          } while (nv < 1e-12);
          nv = std::sqrt(nv);
          for (int d = 0; d < 3; ++d) {
            double x = xyz[3 * (i - 1) + d] + bond * v[d] / nv;
            x -= L * std::floor(x / L);
            if (x >= L) x -= L;
            xyz[3 * i + d] = x;
          }
        }
        if (!g.overlaps(xyz + 3 * i, min2, b > 0 ? i - 1 : -1)) break;
      }
      g.insert(i);
    }
  }
  return GGEM_OK;
}

// random sequential addition of free beads at indices [base, base + count)
int place_free(SplitMix &rng, OverlapGrid &g, double *xyz, double L, int64_t base, int64_t count,
               double min2) {
  for (int64_t i = base; i < base + count; ++i) {
    int64_t tries = 0;
    for (;;) {
      if (++tries > 1000000) return GGEM_ERR_BAD_ARG;
      for (int d = 0; d < 3; ++d) xyz[3 * i + d] = rng.uniform() * L;
      if (!g.overlaps(xyz + 3 * i, min2, -1)) break;
    }
    g.insert(i);
  }
  return GGEM_OK;
}

}  // namespace

extern "C" int ggem_make_suspension(uint64_t seed, int64_t n, double phi, double radius,
                                    double *xyz, double *box_length) {
  if (n <= 0 || !(phi > 0.0 && phi < 0.35) || !(radius > 0) || !xyz || !box_length)
    return GGEM_ERR_BAD_ARG;
  const double L = std::cbrt((double)n * 4.0 / 3.0 * ggem::kPi * radius * radius * radius / phi);
  *box_length = L;
  SplitMix rng(seed);
  const double min_sep = 2.0 * radius, min2 = min_sep * min_sep;
  OverlapGrid g(L, min_sep, xyz);
  if (g.nc < 3) {
    // tiny boxes: brute force
    for (int64_t i = 0; i < n; ++i) {
      int64_t tries = 0;
      for (;;) {
        if (++tries > 1000000) return GGEM_ERR_BAD_ARG;
        for (int d = 0; d < 3; ++d) xyz[3 * i + d] = rng.uniform() * L;
        bool ok = true;
        for (int64_t j = 0; j < i && ok; ++j) {
          double r2 = 0;
          for (int d = 0; d < 3; ++d) {
            double v = xyz[3 * j + d] - xyz[3 * i + d];
            v -= L * std::nearbyint(v / L);
            r2 += v * v;
          }
          ok = r2 >= min2;
        }
        if (ok) break;
      }
    }
    return GGEM_OK;
  }
  return place_free(rng, g, xyz, L, 0, n, min2);
}

extern "C" int ggem_make_chains(uint64_t seed, int64_t n_chains, int beads_per_chain,
                                double bond, double phi, double radius, double *xyz,
                                double *box_length) {
  if (n_chains <= 0 || beads_per_chain <= 0 || !(bond > 0) || !(phi > 0.0 && phi < 0.35) ||
      !(radius > 0) || !xyz || !box_length)
    return GGEM_ERR_BAD_ARG;
  const int64_t n = n_chains * (int64_t)beads_per_chain;
  const double L = std::cbrt((double)n * 4.0 / 3.0 * ggem::kPi * radius * radius * radius / phi);
  *box_length = L;
  SplitMix rng(seed);
  const double min_sep = 2.0 * radius;
  // beads closer than min_sep are rejected; the bonded predecessor sits at
  // exactly `bond` and is skipped in the test
  const double min2 = min_sep * min_sep * (1.0 - 1e-12);
  OverlapGrid g(L, min_sep, xyz);
  if (g.nc < 3) return GGEM_ERR_BAD_ARG;
  return grow_chains(rng, g, xyz, L, 0, n_chains, beads_per_chain, bond, min2);
}

extern "C" int ggem_make_mixture(uint64_t seed, int64_t n_chains, int beads_per_chain,
                                 int64_t n_free, double bond, double phi, double radius,
                                 double *xyz, double *box_length) {
  if (n_chains < 0 || n_free < 0 || n_chains + n_free <= 0 ||
      (n_chains > 0 && beads_per_chain <= 0) || !(bond > 0) || !(phi > 0.0 && phi < 0.35) ||
      !(radius > 0) || !xyz || !box_length)
    return GGEM_ERR_BAD_ARG;
  const int64_t nc_beads = n_chains * (int64_t)std::max(beads_per_chain, 0);
  const int64_t n = nc_beads + n_free;
  const double L = std::cbrt((double)n * 4.0 / 3.0 * ggem::kPi * radius * radius * radius / phi);
  *box_length = L;
  SplitMix rng(seed);
  const double min_sep = 2.0 * radius;
  OverlapGrid g(L, min_sep, xyz);
  if (g.nc < 3) return GGEM_ERR_BAD_ARG;
  if (int rc = grow_chains(rng, g, xyz, L, 0, n_chains, beads_per_chain, bond,
                           min_sep * min_sep * (1.0 - 1e-12)))
    return rc;
  return place_free(rng, g, xyz, L, nc_beads, n_free, min_sep * min_sep);
}

extern "C" int ggem_make_normals(uint64_t seed, int64_t n, double *out) {
  if (n < 0 || (n > 0 && !out)) return GGEM_ERR_BAD_ARG;
  SplitMix rng(seed ^ 0xA5A5A5A5DEADBEEFull);
  for (int64_t i = 0; i < n; ++i) out[i] = rng.normal();
  return GGEM_OK;
}
