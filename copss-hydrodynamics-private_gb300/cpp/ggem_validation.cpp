// ggem_validation.cpp -- the reference's GGEM point-force validation run
// (PMSystemStokes::test_velocity_profile, pm_system_stokes.C:620-740) on the
// GB300 library: velocity profiles along the x, y and z axes through the
// box centre, written as output_velocity_profile_{x,y,z}_<NP>P.csv with the
// reference's 13 columns (pm_system_stokes.C:669-674).  The global (FEM)
// columns are 0: the FEM solve stays with libMesh/PETSc and is not part of
// this library, so u_total = u_local here.  The exact columns are the
// unbounded xi-smoothed solution (analytical_solution_stokes.C:66-102).
//
// usage: ggem_validation alpha lo hi ns_x ns_y ns_z search_radius outdir
//                         x y z fx fy fz [x y z fx fy fz ...]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "ggem_copss.hpp"

using ggem_copss::Point;

static Point exact_unbounded(const ggem_constants &c, const std::vector<double> &xyz,
                             const std::vector<double> &f, const Point &p) {
  const double pi = 3.14159265358979323846264338327950288;
  const double a = c.ksi, k = c.one_eight_pi_mu;
  Point u{0, 0, 0};
  for (size_t i = 0; i < xyz.size() / 3; ++i) {
    const double x[3] = {p[0] - xyz[3 * i], p[1] - xyz[3 * i + 1], p[2] - xyz[3 * i + 2]};
    const double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    double G[3][3];
    if (r < c.r_eps) {
      const double c0 = k * 4.0 * a / std::sqrt(pi);
      for (int m = 0; m < 3; ++m)
        for (int n = 0; n < 3; ++n) G[m][n] = m == n ? c0 : 0.0;
    } else {
      const double c1 = std::erf(a * r) / r;
      const double c2 = 2. * a / std::sqrt(pi) * std::exp(-a * a * r * r);
      for (int m = 0; m < 3; ++m)
        for (int n = 0; n < 3; ++n) {
          const double d = m == n ? 1.0 : 0.0, xx = x[m] * x[n] / (r * r);
          G[m][n] = ((d + xx) * c1 + (d - xx) * c2) * k;
        }
    }
    for (int m = 0; m < 3; ++m)
      for (int n = 0; n < 3; ++n) u[m] += G[m][n] * f[3 * i + n];
  }
  return u;
}

int main(int argc, char **argv) {
  if (argc < 15 || (argc - 9) % 6 != 0) {
    std::fprintf(stderr,
                 "usage: %s alpha lo hi ns_x ns_y ns_z search_radius outdir "
                 "x y z fx fy fz [...]\n",
                 argv[0]);
    return 2;
  }
  const double alpha = std::atof(argv[1]), lo = std::atof(argv[2]), hi = std::atof(argv[3]);
  const int ns[3] = {std::atoi(argv[4]), std::atoi(argv[5]), std::atoi(argv[6])};
  const double radius = std::atof(argv[7]);
  const std::string outdir = argv[8];
  std::vector<double> xyz, f;
  for (int k = 9; k + 5 < argc; k += 6) {
    for (int d = 0; d < 3; ++d) xyz.push_back(std::atof(argv[k + d]));
    for (int d = 0; d < 3; ++d) f.push_back(std::atof(argv[k + 3 + d]));
  }
  ggem_params p;
  ggem_default_params(&p);
  p.alpha = alpha;
  for (int d = 0; d < 3; ++d) {
    p.box_lo[d] = lo;
    p.box_hi[d] = hi;
    p.periodic[d] = 0;  // slit box, periodicity 'false false false'
  }
  p.nb_mode = GGEM_NB_CUTOFF;
  p.rc = radius > 0 ? radius : 4.0 / alpha;  // search_radius_p, copss.C:1074
  p.precision = GGEM_FP64;
  try {
    ggem_copss::ParticleSystem ps(p);
    ps.reinit(xyz);
    ggem_copss::GGEMStokes ggem(ps);
    const size_t NP = xyz.size() / 3;
    const char *names[3] = {"x", "y", "z"};
    for (int dim = 0; dim < 3; ++dim) {
      const double ds = (hi - lo) / ns[dim];
      std::vector<double> pts;
      for (int i = 0; i <= ns[dim]; ++i) {
        Point pt{0, 0, 0};
        pt[dim] = lo + i * ds;
        pts.insert(pts.end(), pt.begin(), pt.end());
      }
      const std::vector<double> ul = ggem.local_solution_field(pts, f);
      const std::string fn = outdir + "/output_velocity_profile_" + names[dim] + "_" +
                             std::to_string(NP) + "P.csv";
      FILE *out = std::fopen(fn.c_str(), "w");
      if (!out) {
        std::perror(fn.c_str());
        return 1;
      }
      std::fprintf(out, "%s,u_total,v_total,w_total,u_global,v_global,w_global,"
                        "u_local,v_local,w_local,u_exact,v_exact,w_exact\n", names[dim]);
      for (int i = 0; i <= ns[dim]; ++i) {
        const Point pt{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        const Point ue = exact_unbounded(ggem.constants(), xyz, f, pt);
        const double *u = &ul[3 * i];
        std::fprintf(out, "%.9f,%.9f,%.9f,%.9f,0,0,0,%.12e,%.12e,%.12e,%.12e,%.12e,%.12e\n",
                     pt[dim], u[0], u[1], u[2], u[0], u[1], u[2], ue[0], ue[1], ue[2]);
      }
      std::fclose(out);
    }
  } catch (const ggem_copss::Error &e) {
    std::fprintf(stderr, "ggem_validation: %s\n", e.what());
    return 1;
  }
  return 0;
}
