/*
 * ggem_oracle.c -- FP64 CPU oracle for the GGEM particle-side hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library and the timed
 * CPU baseline.  Nothing in the shipped library links or calls this file.
 *
 * Every function restates the reference algorithm it cites (paths relative
 * to the COPSS-Hydrodynamics source tree).  Arithmetic is plain IEEE double
 * with libm erf/exp/sqrt, in the same order as the reference where that
 * order is visible.
 */
#include "ggem_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* libMesh::pi (libmesh_common.h) as a double */
static const double ORC_PI = 3.14159265358979323846264338327950288;

/* ----------------------------------------------------------------------
 * constants: ggem_stokes.C:39-114, ggem_system.h:107-116
 * -------------------------------------------------------------------- */
int orc_set_constants(double mu, double alpha, double br0, int point_type,
                      double ibm_beta, double hmin, orc_consts *c) {
  const double sqrt_pi = sqrt(ORC_PI);
  const double pi_23 = pow(ORC_PI, 3. / 2.);
  memset(c, 0, sizeof(*c));
  c->r_eps = 1e-6;
  /* set_mu, ggem_stokes.C:39-47 */
  c->mu = mu;
  c->one_eight_pi_mu = 1. / (8. * ORC_PI * mu);
  /* set_alpha, ggem_stokes.C:50-62 */
  c->alpha = alpha;
  c->alpha2 = alpha * alpha;
  c->alpha3 = c->alpha2 * alpha;
  c->alpha3_pi_23 = c->alpha3 / pi_23;
  c->two_alpha_sqrt_pi = 2. * alpha / sqrt_pi;
  c->coeff_1 = c->one_eight_pi_mu * 4.0 * alpha / sqrt_pi;
  /* set_ksi, ggem_stokes.C:65-114 */
  c->br0 = br0;
  switch (point_type) {
    case ORC_POLYMER_BEAD:
    case ORC_POINT_PARTICLE:
      c->ksi = sqrt_pi / (3. * br0);
      break;
    case ORC_LAGRANGIAN_POINT:
      c->ksi = 1.0 / (ibm_beta * hmin);
      break;
    default:
      return -1;
  }
  c->ksi2 = c->ksi * c->ksi;
  c->ksi3 = c->ksi2 * c->ksi;
  c->ksi3_pi_23 = c->ksi3 / pi_23;
  c->two_ksi_sqrt_pi = 2. * c->ksi / sqrt_pi;
  c->coeff_2 = c->one_eight_pi_mu * 4.0 * (c->ksi - alpha) / sqrt_pi;
  return 0;
}

/* green_tensor_local_regularized, ggem_stokes.C:304-357 */
void orc_green_local(const orc_consts *c, const double x[3], double G[9]) {
  const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  if (r < c->r_eps) {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) G[3 * i + j] = (i == j) ? c->coeff_2 : 0.0;
    return;
  }
  const double r2 = r * r;
  const double kr = c->ksi * r, kr2 = kr * kr;
  const double ar = c->alpha * r, ar2 = ar * ar;
  const double c1 = (erf(kr) - erf(ar)) / r;
  const double c2 = c->two_ksi_sqrt_pi * exp(-kr2) - c->two_alpha_sqrt_pi * exp(-ar2);
  for (int i = 0; i < 3; ++i) {
    for (int j = i; j < 3; ++j) {
      const double d = (i == j) ? 1.0 : 0.0;
      const double xixj_r2 = x[i] * x[j] / r2;
      G[3 * i + j] = ((d + xixj_r2) * c1 + (d - xixj_r2) * c2) * c->one_eight_pi_mu;
    }
    for (int j = i - 1; j >= 0; --j) G[3 * i + j] = G[3 * j + i];
  }
}

/* green_tensor_unbounded_smoothed, ggem_stokes.C:201-251 */
void orc_green_unbounded_smoothed(const orc_consts *c, const double x[3],
                                  double a, double G[9]) {
  const double sqrt_pi = sqrt(ORC_PI);
  const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  if (r < c->r_eps) {
    const double c0 = c->one_eight_pi_mu * 4.0 * a / sqrt_pi;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) G[3 * i + j] = (i == j) ? c0 : 0.0;
    return;
  }
  const double r2 = r * r;
  const double c1 = erf(a * r) / r;
  const double c2 = 2. * a / sqrt_pi * exp(-a * a * r2);
  for (int i = 0; i < 3; ++i) {
    for (int j = i; j < 3; ++j) {
      const double d = (i == j) ? 1.0 : 0.0;
      const double xixj_r2 = x[i] * x[j] / r2;
      G[3 * i + j] = ((d + xixj_r2) * c1 + (d - xixj_r2) * c2) * c->one_eight_pi_mu;
    }
    for (int j = i - 1; j >= 0; --j) G[3 * i + j] = G[3 * j + i];
  }
}

/* smoothed_force_exp, ggem_stokes.C:117-128 */
double orc_smoothed_force_exp(const orc_consts *c, const double r[3]) {
  const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  const double a2r2 = c->alpha2 * r2;
  return c->alpha3_pi_23 * exp(-a2r2) * (2.5 - a2r2);
}

/* point_vector, pm_periodic_boundary.C:350-374: p1 - p0 with minimum image */
void orc_point_vector(const orc_box *b, const double p0[3], const double p1[3],
                      double out[3]) {
  for (int i = 0; i < 3; ++i) {
    double d = p1[i] - p0[i];
    if (b->periodic[i]) {
      const double xsize = b->hi[i] - b->lo[i];
      if (d <= -xsize / 2.0) d += xsize;
      if (d > xsize / 2.0) d -= xsize;
    }
    out[i] = d;
  }
}

void orc_free_nblist(orc_nblist *l) {
  free(l->offsets);
  free(l->ids);
  l->offsets = NULL;
  l->ids = NULL;
  l->n = 0;
}

static int cmp_i32(const void *a, const void *b) {
  const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

/* ----------------------------------------------------------------------
 * Cut-off neighbour lists: {j != i : |point_vector(x_i, x_j)| < rc},
 * each list in ascending j.  Cells of side >= rc; every distinct
 * neighbouring cell is visited once (so boxes with < 3 cells per axis are
 * handled by de-duplicating the stencil).
 * -------------------------------------------------------------------- */
typedef struct cellgrid {
  int nc[3];
  double h[3];
  int64_t *start; /* ncell + 1 */
  int32_t *items;
} cellgrid;

static int cell_coord(const orc_box *b, const cellgrid *g, int d, double x) {
  const double L = b->hi[d] - b->lo[d];
  double t = x - b->lo[d];
  if (b->periodic[d]) {
    t = fmod(t, L);
    if (t < 0) t += L;
  }
  int c = (int)floor(t / g->h[d]);
  if (c < 0) c = 0;
  if (c >= g->nc[d]) c = g->nc[d] - 1;
  return c;
}

static int build_cellgrid(const orc_box *b, int64_t n, const double *xyz,
                          double rc, cellgrid *g) {
  for (int d = 0; d < 3; ++d) {
    const double L = b->hi[d] - b->lo[d];
    int nc = (int)floor(L / rc);
    if (nc < 1) nc = 1;
    if (nc > 1024) nc = 1024;
    g->nc[d] = nc;
    g->h[d] = L / nc;
  }
  const int64_t ncell = (int64_t)g->nc[0] * g->nc[1] * g->nc[2];
  g->start = (int64_t *)calloc((size_t)ncell + 1, sizeof(int64_t));
  g->items = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  int32_t *cid = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  if (!g->start || !g->items || !cid) return -1;
  for (int64_t i = 0; i < n; ++i) {
    const int cx = cell_coord(b, g, 0, xyz[3 * i]);
    const int cy = cell_coord(b, g, 1, xyz[3 * i + 1]);
    const int cz = cell_coord(b, g, 2, xyz[3 * i + 2]);
    cid[i] = cx + g->nc[0] * (cy + g->nc[1] * cz);
    g->start[cid[i] + 1]++;
  }
  for (int64_t c = 0; c < ncell; ++c) g->start[c + 1] += g->start[c];
  int64_t *fill = (int64_t *)calloc((size_t)ncell, sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) {
    g->items[g->start[cid[i]] + fill[cid[i]]++] = (int32_t)i;
  }
  free(fill);
  free(cid);
  return 0;
}

static void free_cellgrid(cellgrid *g) {
  free(g->start);
  free(g->items);
}

/* distinct neighbouring cells of (cx,cy,cz); returns count, writes ids */
static int neighbor_cells(const orc_box *b, const cellgrid *g, int cx, int cy,
                          int cz, int64_t out[27]) {
  int cnt = 0;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        int c[3] = {cx + dx, cy + dy, cz + dz};
        int ok = 1;
        for (int d = 0; d < 3; ++d) {
          if (c[d] < 0 || c[d] >= g->nc[d]) {
            if (b->periodic[d]) {
              c[d] = (c[d] + g->nc[d]) % g->nc[d];
            } else {
              ok = 0;
            }
          }
        }
        if (!ok) continue;
        const int64_t id = c[0] + (int64_t)g->nc[0] * (c[1] + (int64_t)g->nc[1] * c[2]);
        int dup = 0;
        for (int k = 0; k < cnt; ++k)
          if (out[k] == id) dup = 1;
        if (!dup) out[cnt++] = id;
      }
  return cnt;
}

int orc_build_neighbors_cutoff(const orc_box *b, int64_t n, const double *xyz,
                               double rc, orc_nblist *out) {
  cellgrid g;
  if (build_cellgrid(b, n, xyz, rc, &g)) return -1;
  out->n = n;
  out->offsets = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
  int64_t cap = n * 16 + 16, used = 0;
  out->ids = (int32_t *)malloc(sizeof(int32_t) * (size_t)cap);
  const double rc2 = rc * rc;
  for (int64_t i = 0; i < n; ++i) {
    const double *pi = xyz + 3 * i;
    const int cx = cell_coord(b, &g, 0, pi[0]);
    const int cy = cell_coord(b, &g, 1, pi[1]);
    const int cz = cell_coord(b, &g, 2, pi[2]);
    int64_t cells[27];
    const int nn = neighbor_cells(b, &g, cx, cy, cz, cells);
    const int64_t begin = used;
    for (int k = 0; k < nn; ++k) {
      for (int64_t s = g.start[cells[k]]; s < g.start[cells[k] + 1]; ++s) {
        const int32_t j = g.items[s];
        if (j == i) continue;
        double x[3];
        orc_point_vector(b, pi, xyz + 3 * (int64_t)j, x);
        /* |x| < rc is decided as (x0*x0 + x1*x1) + x2*x2 < rc*rc, without
         * fused multiply-adds, so the device list build can reproduce the
         * same set bit for bit */
        const double r2 = (x[0] * x[0] + x[1] * x[1]) + x[2] * x[2];
        if (r2 < rc2) {
          if (used == cap) {
            cap *= 2;
            out->ids = (int32_t *)realloc(out->ids, sizeof(int32_t) * (size_t)cap);
          }
          out->ids[used++] = j;
        }
      }
    }
    qsort(out->ids + begin, (size_t)(used - begin), sizeof(int32_t), cmp_i32);
    out->offsets[i + 1] = used;
  }
  free_cellgrid(&g);
  return 0;
}

/* ----------------------------------------------------------------------
 * Reference neighbour mode (element-as-cell), point_mesh.C:293-848.
 * Elements are the cells of a structured n_mesh grid on the box
 * (MeshTools::Generation::build_cube, copss.C:994-1004), element id
 * ix + nx*(iy + ny*iz), centroid at the cell centre.
 * -------------------------------------------------------------------- */
int orc_elem_of_point(const orc_box *b, const orc_mesh *m, const double p[3]) {
  const int n[3] = {m->nx, m->ny, m->nz};
  int c[3];
  for (int d = 0; d < 3; ++d) {
    const double h = (b->hi[d] - b->lo[d]) / n[d];
    int k = (int)floor((p[d] - b->lo[d]) / h);
    if (k < 0 || k >= n[d]) {
      if (k == n[d] && p[d] <= b->hi[d]) k = n[d] - 1; /* closed upper face */
      else return -1;
    }
    c[d] = k;
  }
  return c[0] + m->nx * (c[1] + m->ny * c[2]);
}

static void elem_centroid(const orc_box *b, const orc_mesh *m, int e, double c[3]) {
  const int n[3] = {m->nx, m->ny, m->nz};
  const int ix = e % m->nx, iy = (e / m->nx) % m->ny, iz = e / (m->nx * m->ny);
  const int k[3] = {ix, iy, iz};
  for (int d = 0; d < 3; ++d) {
    const double h = (b->hi[d] - b->lo[d]) / n[d];
    c[d] = b->lo[d] + (k[d] + 0.5) * h;
  }
}

/* build_elem_elem_neighbor_list, point_mesh.C:293-443: every element i != e
 * whose centroid is within search_radius_e (min image) of e's centroid.  The
 * reference loops over all n_elem; this visits only the bounding range of
 * element indices that can pass the same test, which yields the same set. */
static int elem_elem_list(const orc_box *b, const orc_mesh *m, int e,
                          int32_t *out, unsigned char *mark) {
  const int n[3] = {m->nx, m->ny, m->nz};
  double ce[3];
  elem_centroid(b, m, e, ce);
  int range[3];
  for (int d = 0; d < 3; ++d) {
    const double h = (b->hi[d] - b->lo[d]) / n[d];
    range[d] = (int)ceil(m->search_radius_e / h) + 1;
    if (2 * range[d] + 1 > n[d]) range[d] = n[d]; /* covers everything */
  }
  const int ix = e % m->nx, iy = (e / m->nx) % m->ny, iz = e / (m->nx * m->ny);
  int cnt = 0;
  for (int dz = -range[2]; dz <= range[2]; ++dz)
    for (int dy = -range[1]; dy <= range[1]; ++dy)
      for (int dx = -range[0]; dx <= range[0]; ++dx) {
        int c[3] = {ix + dx, iy + dy, iz + dz};
        int ok = 1;
        for (int d = 0; d < 3; ++d) {
          if (c[d] < 0 || c[d] >= n[d]) {
            if (b->periodic[d]) c[d] = ((c[d] % n[d]) + n[d]) % n[d];
            else ok = 0;
          }
        }
        if (!ok) continue;
        const int i = c[0] + m->nx * (c[1] + m->ny * c[2]);
        if (i == e || mark[i]) continue;
        double ci[3], pt[3];
        elem_centroid(b, m, i, ci);
        orc_point_vector(b, ce, ci, pt);
        if (sqrt(pt[0] * pt[0] + pt[1] * pt[1] + pt[2] * pt[2]) < m->search_radius_e) {
          mark[i] = 1;
          out[cnt++] = i;
        }
      }
  for (int k = 0; k < cnt; ++k) mark[out[k]] = 0;
  qsort(out, (size_t)cnt, sizeof(int32_t), cmp_i32); /* ascending like :333 */
  return cnt;
}

/* build_elem_point_containing_list + build_elem_point_neighbor_list,
 * point_mesh.C:573-799: per element, its own points then the points of each
 * neighbour element in ascending element order; points of one element in
 * ascending particle id. */
int orc_build_elem_lists(const orc_box *b, const orc_mesh *m, int64_t n,
                         const double *xyz, orc_nblist *elem_nb,
                         int32_t *elem_of_particle) {
  const int64_t ne = (int64_t)m->nx * m->ny * m->nz;
  int64_t *cstart = (int64_t *)calloc((size_t)ne + 1, sizeof(int64_t));
  int32_t *citems = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  int32_t *eop = elem_of_particle;
  for (int64_t i = 0; i < n; ++i) {
    eop[i] = orc_elem_of_point(b, m, xyz + 3 * i);
    if (eop[i] < 0) {
      free(cstart);
      free(citems);
      return -2; /* point_mesh.C:602-613: point outside every element */
    }
    cstart[eop[i] + 1]++;
  }
  for (int64_t e = 0; e < ne; ++e) cstart[e + 1] += cstart[e];
  int64_t *fill = (int64_t *)calloc((size_t)ne, sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) citems[cstart[eop[i]] + fill[eop[i]]++] = (int32_t)i;
  free(fill);

  unsigned char *mark = (unsigned char *)calloc((size_t)ne, 1);
  int32_t *enb = (int32_t *)malloc(sizeof(int32_t) * (size_t)ne);
  elem_nb->n = ne;
  elem_nb->offsets = (int64_t *)calloc((size_t)ne + 1, sizeof(int64_t));
  int64_t cap = n * 64 + 64, used = 0;
  elem_nb->ids = (int32_t *)malloc(sizeof(int32_t) * (size_t)cap);
  for (int64_t e = 0; e < ne; ++e) {
    const int cnt = elem_elem_list(b, m, (int)e, enb, mark);
    /* own points first (point_mesh.C:696-699) */
    int64_t need = used + (cstart[e + 1] - cstart[e]);
    for (int k = 0; k < cnt; ++k) need += cstart[enb[k] + 1] - cstart[enb[k]];
    while (need > cap) {
      cap *= 2;
      elem_nb->ids = (int32_t *)realloc(elem_nb->ids, sizeof(int32_t) * (size_t)cap);
    }
    for (int64_t s = cstart[e]; s < cstart[e + 1]; ++s) elem_nb->ids[used++] = citems[s];
    for (int k = 0; k < cnt; ++k)
      for (int64_t s = cstart[enb[k]]; s < cstart[enb[k] + 1]; ++s)
        elem_nb->ids[used++] = citems[s];
    elem_nb->offsets[e + 1] = used;
  }
  free(mark);
  free(enb);
  free(cstart);
  free(citems);
  return 0;
}

/* build_point_point_neighbor_list, point_mesh.C:803-848: the element list of
 * the particle's element with the particle itself removed (order kept). */
int orc_build_neighbors_reference(const orc_box *b, const orc_mesh *m,
                                  int64_t n, const double *xyz, orc_nblist *out) {
  orc_nblist el;
  int32_t *eop = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  int rc = orc_build_elem_lists(b, m, n, xyz, &el, eop);
  if (rc) {
    free(eop);
    return rc;
  }
  out->n = n;
  out->offsets = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
  int64_t total = 0;
  for (int64_t i = 0; i < n; ++i) total += el.offsets[eop[i] + 1] - el.offsets[eop[i]];
  out->ids = (int32_t *)malloc(sizeof(int32_t) * (size_t)(total > 0 ? total : 1));
  int64_t used = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int e = eop[i];
    for (int64_t s = el.offsets[e]; s < el.offsets[e + 1]; ++s)
      if (el.ids[s] != i) out->ids[used++] = el.ids[s];
    out->offsets[i + 1] = used;
  }
  free(eop);
  orc_free_nblist(&el);
  return 0;
}

/* ----------------------------------------------------------------------
 * Local mobility matvec.
 * local_solution_bead, ggem_stokes.C:427-503: u_i = sum_v G(r_iv) f_v with
 * r_iv = point_vector(x_i, x_v) (point_mesh.C:220-241); self terms per
 * pm_system_stokes.C:446-455 and ggem_stokes.C:485-499.
 * -------------------------------------------------------------------- */
typedef struct mv_job {
  const orc_consts *c;
  const orc_box *b;
  int64_t n, i0, i1;
  const double *xyz;
  const orc_nblist *nb;
  int nrhs;
  const double *f;
  double *u;
  int self_mode;
} mv_job;

static void *mv_worker(void *arg) {
  const mv_job *J = (const mv_job *)arg;
  const int64_t dim = 3 * J->n;
  for (int64_t i = J->i0; i < J->i1; ++i) {
    for (int r = 0; r < J->nrhs; ++r) {
      const double *f = J->f + r * dim;
      double u[3] = {0., 0., 0.};
      for (int64_t s = J->nb->offsets[i]; s < J->nb->offsets[i + 1]; ++s) {
        const int64_t j = J->nb->ids[s];
        double x[3], G[9];
        orc_point_vector(J->b, J->xyz + 3 * i, J->xyz + 3 * j, x);
        orc_green_local(J->c, x, G);
        for (int a = 0; a < 3; ++a)
          for (int bb = 0; bb < 3; ++bb) u[a] += G[3 * a + bb] * f[3 * j + bb];
      }
      const double *fi = f + 3 * i;
      double *ui = J->u + r * dim + 3 * i;
      for (int a = 0; a < 3; ++a) {
        if (J->self_mode == ORC_SELF_BEAD) {
          ui[a] = (u[a] - J->c->coeff_1 * fi[a]) + fi[a];
        } else if (J->self_mode == ORC_SELF_LAGRANGIAN) {
          ui[a] = u[a] + J->c->coeff_2 * fi[a];
        } else {
          ui[a] = u[a];
        }
      }
    }
  }
  return NULL;
}

void orc_local_matvec(const orc_consts *c, const orc_box *b, int64_t n,
                      const double *xyz, const orc_nblist *nb, int nrhs,
                      const double *f, double *u, int self_mode, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  mv_job jobs[256];
  pthread_t th[256];
  const int64_t chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; ++t) {
    jobs[t] = (mv_job){c, b, n, t * chunk, (t + 1) * chunk, xyz, nb, nrhs, f, u, self_mode};
    if (jobs[t].i1 > n) jobs[t].i1 = n;
    if (jobs[t].i0 > n) jobs[t].i0 = n;
  }
  if (nthreads == 1) {
    mv_worker(&jobs[0]);
    return;
  }
  for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, mv_worker, &jobs[t]);
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
}

/* local_solution_field, ggem_stokes.C:360-424: target in element e uses the
 * element's point neighbour list, no self exclusion */
void orc_local_field_reference(const orc_consts *c, const orc_box *b,
                               const orc_mesh *m, const orc_nblist *elem_nb,
                               int64_t n, const double *xyz, const double *f,
                               int64_t nt, const double *targets, double *u) {
  (void)n;
  for (int64_t t = 0; t < nt; ++t) {
    const double *pt = targets + 3 * t;
    double acc[3] = {0., 0., 0.};
    const int e = orc_elem_of_point(b, m, pt);
    if (e >= 0) {
      for (int64_t s = elem_nb->offsets[e]; s < elem_nb->offsets[e + 1]; ++s) {
        const int64_t j = elem_nb->ids[s];
        double x[3], G[9];
        orc_point_vector(b, pt, xyz + 3 * j, x);
        orc_green_local(c, x, G);
        for (int a = 0; a < 3; ++a)
          for (int bb = 0; bb < 3; ++bb) acc[a] += G[3 * a + bb] * f[3 * j + bb];
      }
    }
    for (int a = 0; a < 3; ++a) u[3 * t + a] = acc[a];
  }
}

void orc_local_field_cutoff(const orc_consts *c, const orc_box *b, int64_t n,
                            const double *xyz, const double *f, double rc,
                            int64_t nt, const double *targets, double *u) {
  for (int64_t t = 0; t < nt; ++t) {
    const double *pt = targets + 3 * t;
    double acc[3] = {0., 0., 0.};
    for (int64_t j = 0; j < n; ++j) {
      double x[3], G[9];
      orc_point_vector(b, pt, xyz + 3 * j, x);
      if (rc > 0 && !((x[0] * x[0] + x[1] * x[1]) + x[2] * x[2] < rc * rc)) continue;
      orc_green_local(c, x, G);
      for (int a = 0; a < 3; ++a)
        for (int bb = 0; bb < 3; ++bb) acc[a] += G[3 * a + bb] * f[3 * j + bb];
    }
    for (int a = 0; a < 3; ++a) u[3 * t + a] = acc[a];
  }
}

/* exact_solution_infinite_domain, analytical_solution_stokes.C:66-102 */
void orc_exact_unbounded(const orc_consts *c, int64_t n, const double *xyz,
                         const double *f, int64_t nt, const double *targets,
                         double *u) {
  for (int64_t t = 0; t < nt; ++t) {
    double acc[3] = {0., 0., 0.};
    for (int64_t i = 0; i < n; ++i) {
      double x[3], G[9];
      for (int d = 0; d < 3; ++d) x[d] = targets[3 * t + d] - xyz[3 * i + d];
      orc_green_unbounded_smoothed(c, x, c->ksi, G);
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) acc[k] += G[3 * k + l] * f[3 * i + l];
    }
    for (int k = 0; k < 3; ++k) u[3 * t + k] = acc[k];
  }
}

/* ----------------------------------------------------------------------
 * Gaussian spreading, assemble_stokes.C:645-671 with smoothed_force_exp.
 * -------------------------------------------------------------------- */
static void rho_at(const orc_consts *c, const orc_box *b,
                   const orc_nblist *elem_nb, int64_t n, const double *xyz,
                   const double *f, const double *q, int elem, double rc,
                   double rho[3]) {
  rho[0] = rho[1] = rho[2] = 0.;
  if (rc > 0) {
    for (int64_t j = 0; j < n; ++j) {
      double x[3];
      orc_point_vector(b, q, xyz + 3 * j, x);
      if (!((x[0] * x[0] + x[1] * x[1]) + x[2] * x[2] < rc * rc)) continue;
      const double g = orc_smoothed_force_exp(c, x);
      for (int d = 0; d < 3; ++d) rho[d] += g * f[3 * j + d];
    }
    return;
  }
  if (elem < 0) return;
  for (int64_t s = elem_nb->offsets[elem]; s < elem_nb->offsets[elem + 1]; ++s) {
    const int64_t j = elem_nb->ids[s];
    double x[3];
    orc_point_vector(b, q, xyz + 3 * j, x);
    const double g = orc_smoothed_force_exp(c, x);
    for (int d = 0; d < 3; ++d) rho[d] += g * f[3 * j + d];
  }
}

void orc_spread_qp(const orc_consts *c, const orc_box *b,
                   const orc_nblist *elem_nb, int64_t n, const double *xyz,
                   const double *f, int64_t nq, const double *qxyz,
                   const int32_t *qp_elem, double rc, double *rho) {
  for (int64_t q = 0; q < nq; ++q)
    rho_at(c, b, elem_nb, n, xyz, f, qxyz + 3 * q, qp_elem ? qp_elem[q] : -1, rc,
           rho + 3 * q);
}

void orc_element_rhs(const orc_consts *c, const orc_box *b,
                     const orc_nblist *elem_nb, int64_t n, const double *xyz,
                     const double *f, int64_t n_elem, int nq_per_elem, int n_u,
                     const double *qxyz, const double *int_force, double rc,
                     double *Fe) {
  for (int64_t e = 0; e < n_elem; ++e) {
    double *F = Fe + e * 3 * n_u;
    for (int k = 0; k < 3 * n_u; ++k) F[k] = 0.;
    /* assemble_global_F skips elements without neighbouring points,
     * assemble_stokes.C:492-494 */
    if (rc <= 0 && elem_nb->offsets[e + 1] == elem_nb->offsets[e]) continue;
    for (int qp = 0; qp < nq_per_elem; ++qp) {
      double rho[3];
      rho_at(c, b, elem_nb, n, xyz, f, qxyz + 3 * (e * nq_per_elem + qp), (int)e, rc,
             rho);
      const double *IF = int_force + e * (int64_t)n_u * nq_per_elem;
      for (int j = 0; j < 3; ++j)
        for (int l = 0; l < n_u; ++l) F[j * n_u + l] += IF[l * nq_per_elem + qp] * rho[j];
    }
  }
}

/* ----------------------------------------------------------------------
 * Chebyshev coefficients, chebyshev.C:44-190.
 * -------------------------------------------------------------------- */
static double cheb_function(double x, double da, double db) {
  const double fv = sqrt((x - db) / da); /* chebyshev.C:50 */
  return 1.0 / fv;
}

void orc_cheb_coeffs(int N, double da, double db, int method, double *coef) {
  double *x = (double *)malloc(sizeof(double) * (size_t)(N + 1));
  double *w = (double *)malloc(sizeof(double) * (size_t)(N + 1));
  const double PI = ORC_PI;
  for (int i = 0; i <= N; ++i) {
    const double j = (double)i;
    if (method == 2) { /* Gauss_Lobatto, chebyshev.C:173-190 */
      x[i] = cos(PI * j / (double)N);
      w[i] = PI / (double)N;
    } else if (method == 1) { /* Gauss_Radau, chebyshev.C:154-170 */
      x[i] = cos(2. * PI * j / (2. * (double)N + 1.));
      w[i] = 2. * PI / (2. * (double)N + 1.);
    } else { /* Gauss, chebyshev.C:136-151 */
      x[i] = cos((2. * j + 1.) * PI / (2. * (double)N + 2.));
      w[i] = PI / ((double)N + 1.);
    }
  }
  if (method == 2) {
    w[0] = PI / (2. * (double)N);
    w[N] = PI / (2. * (double)N);
  } else if (method == 1) {
    w[0] = PI / (2. * (double)N + 1.);
  }
  const double RN = (double)N;
  for (int k = 0; k <= N; ++k) {
    double ck_sum = 0.0;
    for (int j = 0; j <= N; ++j) {
      double tmpt;
      if (method == 2) tmpt = PI * (double)((size_t)k * (size_t)j) / RN;
      else if (method == 1) tmpt = 2. * PI * (double)((size_t)k * (size_t)j) / (2. * RN + 1.);
      else tmpt = PI * (double)(2. * j + 1.) * (double)k / (2. * RN + 2.);
      const double fj = cheb_function(x[j], da, db);
      ck_sum += w[j] * cos(tmpt) * fj;
    }
    const double ck = (k == 0) ? 2.0 : 1.0;
    coef[k] = ck_sum * (2. / (PI * ck));
  }
  free(x);
  free(w);
}

/* ----------------------------------------------------------------------
 * Chebyshev approximation y ~ M^{-1/2} dw, brownian_system.C:967-1178.
 * -------------------------------------------------------------------- */
static double vdot(int64_t n, const double *a, const double *b) {
  double s = 0.;
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}
static double vnorm(int64_t n, const double *a) { return sqrt(vdot(n, a, a)); }

void orc_cheb_inv_sqrt(orc_op_fn op, void *ctx, int64_t dim, int N,
                       double eig_min, double eig_max, double tol_cheb,
                       double *dw, orc_cheb_report *rep) {
  double *x0 = (double *)malloc(sizeof(double) * (size_t)dim);
  double *x1 = (double *)malloc(sizeof(double) * (size_t)dim);
  double *xm = (double *)malloc(sizeof(double) * (size_t)dim);
  double *dm = (double *)malloc(sizeof(double) * (size_t)dim);
  double *X = (double *)malloc(sizeof(double) * (size_t)(N + 1));
  double err1 = 0., err2 = 0., aux1, aux2, aux3, aux4;
  int conv = 0, nmv = 0, nterms = 1;
  /* :1001-1003 */
  const double d_eig = eig_max - eig_min;
  const double da = 2.0 / d_eig;
  const double db = -(eig_max + eig_min) / d_eig;
  orc_cheb_coeffs(N, da, db, 0, X); /* :1021-1024, "Gauss" */
  /* :1036-1041 */
  memcpy(x0, dw, sizeof(double) * (size_t)dim);
  op(ctx, x0, x1);
  nmv++;
  aux2 = vdot(dim, x1, x0);
  for (int64_t i = 0; i < dim; ++i) x1[i] = db * x0[i] + da * x1[i];
  /* :1050-1056 */
  for (int64_t i = 0; i < dim; ++i) dw[i] = X[0] * x0[i];
  aux4 = vnorm(dim, dw);
  for (int64_t i = 0; i < dim; ++i) dw[i] += X[1] * x1[i];
  aux3 = vnorm(dim, x1);
  aux3 *= fabs(X[1]);
  /* :1064-1072 */
  op(ctx, dw, dm);
  nmv++;
  aux1 = vdot(dim, dm, dm);
  if (aux2 != 0.0) err1 = sqrt(fabs(aux1 - aux2) / aux2);
  if (aux4 != 0.0) err2 = aux3 / aux4;
  /* :1089-1155 */
  for (int i = 1; i < N; ++i) {
    aux4 = vnorm(dim, dw);
    op(ctx, x1, xm);
    nmv++;
    for (int64_t k = 0; k < dim; ++k) xm[k] = 2. * db * x1[k] + 2. * da * xm[k];
    for (int64_t k = 0; k < dim; ++k) xm[k] -= x0[k];
    for (int64_t k = 0; k < dim; ++k) dw[k] += X[i + 1] * xm[k];
    aux3 = vnorm(dim, xm);
    aux3 *= fabs(X[i + 1]);
    op(ctx, dw, dm);
    nmv++;
    aux1 = vdot(dim, dm, dm);
    if (aux2 != 0.0) err1 = sqrt(fabs(aux1 - aux2) / aux2);
    if (aux4 != 0.0) err2 = aux3 / aux4;
    nterms = i + 1;
    if (err1 <= tol_cheb) {
      conv = 1;
      break;
    }
    if (err2 <= 1E-9) break;
    memcpy(x0, x1, sizeof(double) * (size_t)dim);
    memcpy(x1, xm, sizeof(double) * (size_t)dim);
  }
  rep->converged = conv;
  rep->n_terms = nterms;
  rep->n_matvecs = nmv;
  rep->err1 = err1;
  rep->err2 = err2;
  free(x0);
  free(x1);
  free(xm);
  free(dm);
  free(X);
}

/* ----------------------------------------------------------------------
 * Spectral bounds.  The reference uses SLEPc Krylov-Schur
 * (brownian_system.C:527-657, :803-843); this is Lanczos with full
 * reorthogonalisation, whose extreme Ritz values bound the same interval
 * from inside.
 * -------------------------------------------------------------------- */
static int sturm_count(int k, const double *a, const double *b, double x) {
  /* number of eigenvalues < x of the tridiagonal (a diag, b offdiag) */
  int cnt = 0;
  double d = 1.0;
  for (int i = 0; i < k; ++i) {
    const double bb = (i > 0) ? b[i - 1] * b[i - 1] : 0.0;
    d = a[i] - x - (i > 0 ? bb / d : 0.0);
    if (d == 0.0) d = -1e-300;
    if (d < 0) cnt++;
  }
  return cnt;
}

static double bisect_eig(int k, const double *a, const double *b, int which,
                         double lo, double hi) {
  /* which-th smallest eigenvalue (0-based) */
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid == lo || mid == hi) break;
    if (sturm_count(k, a, b, mid) > which) hi = mid;
    else lo = mid;
  }
  return 0.5 * (lo + hi);
}

void orc_tridiag_extremes(int k, const double *a, const double *b, double *lmin,
                          double *lmax) {
  double lo = a[0], hi = a[0];
  for (int i = 0; i < k; ++i) {
    const double r = (i > 0 ? fabs(b[i - 1]) : 0.) + (i < k - 1 ? fabs(b[i]) : 0.);
    if (a[i] - r < lo) lo = a[i] - r;
    if (a[i] + r > hi) hi = a[i] + r;
  }
  const double pad = 1e-12 * (fabs(lo) + fabs(hi)) + 1e-300;
  *lmin = bisect_eig(k, a, b, 0, lo - pad, hi + pad);
  *lmax = bisect_eig(k, a, b, k - 1, lo - pad, hi + pad);
}

int orc_lanczos(orc_op_fn op, void *ctx, int64_t dim, int k, const double *v0,
                double *lmin, double *lmax, double *alpha_out, double *beta_out) {
  double *Q = (double *)malloc(sizeof(double) * (size_t)dim * (size_t)(k + 1));
  double *w = (double *)malloc(sizeof(double) * (size_t)dim);
  double *a = (double *)calloc((size_t)k, sizeof(double));
  double *bt = (double *)calloc((size_t)k, sizeof(double));
  if (!Q || !w || !a || !bt) return -1;
  const double nv = vnorm(dim, v0);
  for (int64_t i = 0; i < dim; ++i) Q[i] = v0[i] / nv;
  int m = k;
  for (int j = 0; j < k; ++j) {
    double *q = Q + (size_t)j * dim;
    op(ctx, q, w);
    a[j] = vdot(dim, q, w);
    /* full reorthogonalisation, twice (classical Gram-Schmidt x2) */
    for (int pass = 0; pass < 2; ++pass)
      for (int i = 0; i <= j; ++i) {
        const double *qi = Q + (size_t)i * dim;
        const double h = vdot(dim, qi, w);
        for (int64_t t = 0; t < dim; ++t) w[t] -= h * qi[t];
      }
    const double beta = vnorm(dim, w);
    bt[j] = beta;
    if (j == k - 1) break;
    if (beta < 1e-14 * fabs(a[j]) + 1e-300) {
      m = j + 1;
      break;
    }
    double *qn = Q + (size_t)(j + 1) * dim;
    for (int64_t t = 0; t < dim; ++t) qn[t] = w[t] / beta;
  }
  orc_tridiag_extremes(m, a, bt, lmin, lmax);
  if (alpha_out) memcpy(alpha_out, a, sizeof(double) * (size_t)m);
  if (beta_out) memcpy(beta_out, bt, sizeof(double) * (size_t)m);
  free(Q);
  free(w);
  free(a);
  free(bt);
  return m;
}

/* power_iteration, brownian_system.C:846-920 */
int orc_power_iteration(orc_op_fn op, void *ctx, int64_t dim, double tol,
                        int maxits, double *eig) {
  double *v0 = (double *)malloc(sizeof(double) * (size_t)dim);
  double *v1 = (double *)malloc(sizeof(double) * (size_t)dim);
  double *w0 = (double *)malloc(sizeof(double) * (size_t)dim);
  for (int64_t i = 0; i < dim; ++i) v0[i] = 1.0;
  double norm = vnorm(dim, v0);
  for (int64_t i = 0; i < dim; ++i) v0[i] *= 1.0 / norm;
  int found = -1;
  *eig = NAN;
  for (int it = 0; it < maxits; ++it) {
    op(ctx, v0, w0);
    norm = vnorm(dim, w0);
    for (int64_t i = 0; i < dim; ++i) w0[i] *= 1.0 / norm;
    memcpy(v1, w0, sizeof(double) * (size_t)dim);
    for (int64_t i = 0; i < dim; ++i) w0[i] += -1.0 * v0[i];
    norm = vnorm(dim, w0);
    memcpy(v0, v1, sizeof(double) * (size_t)dim);
    if (norm < tol) {
      op(ctx, v0, w0);
      *eig = vdot(dim, v0, w0);
      found = it;
      break;
    }
  }
  free(v0);
  free(v1);
  free(w0);
  return found;
}

void orc_matvec_op(void *ctx, const double *f, double *u) {
  const orc_matvec_ctx *m = (const orc_matvec_ctx *)ctx;
  orc_local_matvec(m->c, m->b, m->n, m->xyz, m->nb, 1, f, u, m->self_mode,
                   m->nthreads);
}

void orc_diag_test_op(void *ctx, const double *f, double *u) {
  const int64_t dim = *(const int64_t *)ctx;
  for (int64_t i = 0; i < dim; ++i) u[i] = f[i] * (double)(i + 1);
}

/* ----------------------------------------------------------------------
 * Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
 * "Parallel random numbers: as easy as 1, 2, 3", SC'11), followed by the
 * Box-Muller transform.  Element 2p and 2p+1 come from counter
 * (p_lo, p_hi, stream_lo, stream_hi) with key (seed_lo, seed_hi).
 * -------------------------------------------------------------------- */
static void philox_round(uint32_t c[4], const uint32_t k[2]) {
  const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
  const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
  const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
  const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
  const uint32_t n0 = hi1 ^ c[1] ^ k[0];
  const uint32_t n2 = hi0 ^ c[3] ^ k[1];
  c[0] = n0;
  c[1] = lo1;
  c[2] = n2;
  c[3] = lo0;
}

static void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  uint32_t k[2] = {k0, k1};
  for (int r = 0; r < 10; ++r) {
    philox_round(c, k);
    k[0] += 0x9E3779B9u;
    k[1] += 0xBB67AE85u;
  }
}

/* counter (p, stream) -> elements 4p .. 4p+3; the uniforms are formed in
 * FP32 exactly as on the device (u1 rounded once, u2 exact), the transform
 * runs in FP64 here: the device's FP32 transform agrees to a few FP32 ulps */
void orc_philox_normals(uint64_t seed, uint64_t stream, int64_t n, double *out) {
  const double two_pi = 2.0 * ORC_PI;
  for (int64_t p = 0; 4 * p < n; ++p) {
    uint32_t c[4] = {(uint32_t)p, (uint32_t)((uint64_t)p >> 32), (uint32_t)stream,
                     (uint32_t)(stream >> 32)};
    philox10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    for (int h = 0; h < 2; ++h) {
      /* (float)c0 * 2^-32 is exact, so the sum is the device's single fmaf rounding */
      const float u1 = (float)c[2 * h] * 0x1p-32f + 0x1p-33f;
      const float u2 = (float)(c[2 * h + 1] >> 9) * 0x1p-23f + 0x1p-24f;
      const double r = sqrt(-2.0 * log((double)u1));
      const int64_t k = 4 * p + 2 * h;
      if (k < n) out[k] = r * cos(two_pi * (double)u2);
      if (k + 1 < n) out[k + 1] = r * sin(two_pi * (double)u2);
    }
  }
}


/* ---- force fixes ------------------------------------------------------- */

/* fix/fix_base.C:150-162: -c1 c2 exp(-c2 |r|^2) r, |r| from its norm */
void orc_ev_gaussian(const orc_box *b, int64_t n, const double *xyz, const orc_nblist *nb,
                     double c1, double c2, double *f) {
  for (int64_t i = 0; i < n; ++i) {
    double acc[3] = {0.0, 0.0, 0.0};
    for (int64_t k = nb->offsets[i]; k < nb->offsets[i + 1]; ++k) {
      const int64_t j = nb->ids[k];
      double r[3];
      orc_point_vector(b, xyz + 3 * i, xyz + 3 * j, r);
      const double len = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
      const double w = -c1 * c2 * exp(-c2 * len * len);
      for (int d = 0; d < 3; ++d) acc[d] += w * r[d];
    }
    for (int d = 0; d < 3; ++d) f[3 * i + d] += acc[d];
  }
}

/* fix/fix_base.C:55-148, tol = 1e-3 (fix/fix_base.h:50) */
void orc_spring_force(int kind, const double R_ij[3], double c1, double Ls, double F[3]) {
  const double tol = 1e-3;
  const double R = sqrt(R_ij[0] * R_ij[0] + R_ij[1] * R_ij[1] + R_ij[2] * R_ij[2]);
  double scale;
  if (kind == 0) {         /* worm-like spring, :55-74 */
    const double ratio = R / Ls;
    double v0 = 1.0 - ratio;
    if (fabs(v0) < tol) v0 = v0 / fabs(v0) * tol;
    scale = c1 * (1.0 / (v0 * v0) - 1.0 + 4.0 * ratio) / R;
  } else if (kind == 1) {  /* FENE, :77-96 */
    const double ratio = R / Ls;
    double v0 = 1.0 - ratio * ratio;
    if (fabs(v0) < tol) v0 = v0 / fabs(v0) * tol * tol;
    scale = c1 * ratio / v0 / R;
  } else if (kind == 2) {  /* Underhill-Doyle, :99-124 */
    const double ratio = R / Ls, r2 = ratio * ratio, cc = c1 * c1;
    const double a1 = 1.0, a2 = -7.0 * c1, a3 = 3.0 / 32.0 - 0.75 * c1 - 6.0 * cc;
    const double a4 = (13.0 / 32.0 + 0.8172 * c1 - 14.79 * cc) / (1.0 - 4.225 * c1 + 4.87 * cc);
    const double T4 = 1.0 - r2, T2 = 1.0 / T4, T1 = T2 / T4;
    scale = (a1 * T1 + a2 * T2 + a3 + a4 * T4) / R;
  } else {                 /* linear Hookean spring, :127-148 */
    scale = Ls * (R - c1) / R;
  }
  for (int d = 0; d < 3; ++d) F[d] = scale * R_ij[d];
}

/* fix/fix_point_wls.C:66-92 */
void orc_spring_forces(const orc_box *b, int64_t n, const double *xyz, int64_t m,
                       const int64_t *bonds, int kind, double c1, double Ls, double *f) {
  (void)n;
  for (int64_t k = 0; k < m; ++k) {
    const int64_t i = bonds[2 * k], j = bonds[2 * k + 1];
    double R[3], F[3];
    orc_point_vector(b, xyz + 3 * i, xyz + 3 * j, R);
    orc_spring_force(kind, R, c1, Ls, F);
    for (int d = 0; d < 3; ++d) {
      f[3 * i + d] += F[d];
      f[3 * j + d] -= F[d];
    }
  }
}


/* ---- FEM velocity at points -------------------------------------------- */

/* libMesh Hex20 nodes on [-1, 1]^3: corners 0-7, then the edge midpoints of
 * edges 0-1, 1-2, 2-3, 3-0, 0-4, 1-5, 2-6, 3-7, 4-5, 5-6, 6-7, 7-4 */
static const int HEX20_X[20] = {-1, 1, 1, -1, -1, 1, 1, -1, 0, 1, 0, -1, -1, 1, 1, -1, 0, 1, 0, -1};
static const int HEX20_Y[20] = {-1, -1, 1, 1, -1, -1, 1, 1, -1, 0, 1, 0, -1, -1, 1, 1, -1, 0, 1, 0};
static const int HEX20_Z[20] = {-1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0, 1, 1, 1, 1};

void orc_hex20_shape(double x, double y, double z, double n[20]) {
  for (int k = 0; k < 20; ++k) {
    const double a = HEX20_X[k], b = HEX20_Y[k], c = HEX20_Z[k];
    if (k < 8)
      n[k] = (1.0 + a * x) * (1.0 + b * y) * (1.0 + c * z) * (a * x + b * y + c * z - 2.0) / 8.0;
    else if (a == 0.0)
      n[k] = (1.0 - x * x) * (1.0 + b * y) * (1.0 + c * z) / 4.0;
    else if (b == 0.0)
      n[k] = (1.0 + a * x) * (1.0 - y * y) * (1.0 + c * z) / 4.0;
    else
      n[k] = (1.0 + a * x) * (1.0 + b * y) * (1.0 - z * z) / 4.0;
  }
}

/* element containing x on the uniform mesh (floor((x - lo) / h), periodic
 * axes wrapped first, clamped to the mesh) and the reference coordinate */
int64_t orc_fem_point_values(int64_t n, const double *xyz, const int ne[3], const double lo[3],
                             const double hi[3], const int periodic[3],
                             const int64_t *elem_dofs, const double *sol, double *u) {
  int64_t outside = 0;
  for (int64_t i = 0; i < n; ++i) {
    int e[3];
    double xi[3];
    for (int d = 0; d < 3; ++d) {
      const double L = hi[d] - lo[d], h = L / ne[d];
      double t = xyz[3 * i + d] - lo[d];
      if (periodic[d]) {
        t = fmod(t, L);
        if (t < 0) t += L;
        if (t >= L) t = 0.0;
      } else if (!(t >= 0.0 && t <= L)) {
        ++outside;
      }
      int k = (int)floor(t / h);
      k = k < 0 ? 0 : (k >= ne[d] ? ne[d] - 1 : k);
      e[d] = k;
      xi[d] = 2.0 * (t - k * h) / h - 1.0;
    }
    double nf[20];
    orc_hex20_shape(xi[0], xi[1], xi[2], nf);
    const int64_t elem = e[0] + (int64_t)ne[0] * (e[1] + (int64_t)ne[1] * e[2]);
    for (int v = 0; v < 3; ++v) {
      double s = 0.0;
      for (int k = 0; k < 20; ++k) s += nf[k] * sol[elem_dofs[elem * 60 + 20 * v + k]];
      u[3 * i + v] = s;
    }
  }
  return outside;
}
