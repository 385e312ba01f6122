/*
 * oracle_mg.cpp -- CPU FP64 restatement of afivo's ghost-cell fill and FAS
 * multigrid (TEST INFRASTRUCTURE ONLY: the checker for the GPU path; see
 * oracle_common.h).
 *
 * Each routine cites the reference lines it restates.  Loops over boxes are
 * OpenMP-parallel exactly where the reference's are (!$omp do over
 * tree%lvls(lvl)%ids), so the same code serves as the timed CPU baseline.
 *
 * One substitution: the coarse-grid solve.  The reference calls hypre 2.31.0
 * Struct PFMG (m_coarse_solver.f90:393-439, tol 1e-6, <=50 iterations),
 * which is not vendored.  The oracle solves the same matrix (built as
 * hypre_set_matrix + stencil_handle_boundaries do, m_coarse_solver.f90:104-194,
 * 442-491) exactly, with an FP64 inverse applied in a fixed summation order
 * shared with the GPU.
 */
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <omp.h>

#include "oracle_common.h"

namespace orc {

static const int EDGE_DIM[12] = {0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2};
static const int EDGE_DIR[12][3] = {{0, -1, -1}, {0, 1, -1}, {0, -1, 1}, {0, 1, 1},
                                    {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1}, {1, 0, 1},
                                    {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 1, 0}};

/* index of a cell given the normal dimension d, the normal index x and the
 * tangential indices p (lower dim) and q (higher dim) */
static inline int face_at(const Tree& t, int d, int x, int p, int q) {
  if (t.D == 2) return d == 0 ? t.at(x, p) : t.at(p, x);
  if (d == 0) return t.at(x, p, q);
  if (d == 1) return t.at(p, x, q);
  return t.at(p, q, x);
}

/* bc_to_gc, m_af_ghostcell.f90:173-279 */
static void bc_to_gc(const Tree& t, double* a, int id, int nb, int bc_type, double b) {
  const int nc = t.nc, d = nb / 2;
  const bool low = (nb % 2) == 0;
  double c0, c1, c2;
  switch (bc_type) {
    case AFG_BC_DIRICHLET: c0 = 2; c1 = -1; c2 = 0; break;
    case AFG_BC_NEUMANN: c0 = t.dr_of(id, d) * (low ? -1 : 1); c1 = 1; c2 = 0; break;
    case AFG_BC_CONTINUOUS: c0 = 0; c1 = 2; c2 = -1; break;
    default: c0 = 1; c1 = 0; c2 = 0; break;  // AFG_BC_DIRICHLET_COPY
  }
  const int gi = low ? 0 : nc + 1, i1 = low ? 1 : nc, i2 = low ? 2 : nc - 1;
  const int qn = t.D == 3 ? nc : 1;
  for (int q = 1; q <= qn; q++)
    for (int p = 1; p <= nc; p++)
      a[face_at(t, d, gi, p, q)] = c0 * b + c1 * a[face_at(t, d, i1, p, q)] +
                                   c2 * a[face_at(t, d, i2, p, q)];
}

/* mg_sides_rb, m_af_multigrid.f90:294-461 */
static void sides_rb(const Tree& t, double* cc, int id, int nb, int iv) {
  const int nc = t.nc, hnc = nc / 2, d = nb / 2;
  const bool low = (nb % 2) == 0;
  const int p_id = t.parent[id - 1];
  const int p_nb = t.nb_of(p_id, nb);
  const double* c = t.var(cc, p_nb, iv);
  double* a = t.var(cc, id, iv);
  int co[3];
  for (int k = 0; k < t.D; k++) co[k] = t.child_offset(id, k);
  // tangential dims
  int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
  const int xc = low ? nc : 1;
  const int ix = low ? 1 : nc, dix = low ? 1 : -1;
  if (t.D == 2) {
    double tmp[64 + 2], gc[64 + 1];
    for (int a_ = 0; a_ <= hnc + 1; a_++) tmp[a_] = c[face_at(t, d, xc, co[t1] + a_, 0)];
    for (int i = 1; i <= hnc; i++) {
      double grad = 0.125 * (tmp[i + 1] - tmp[i - 1]);
      gc[2 * i - 1] = tmp[i] - grad;
      gc[2 * i] = tmp[i] + grad;
    }
    for (int p = 1; p <= nc; p++)
      a[face_at(t, d, ix - dix, p, 0)] = 0.5 * gc[p] + 0.75 * a[face_at(t, d, ix, p, 0)] -
                                         0.25 * a[face_at(t, d, ix + dix, p, 0)];
  } else {
    const int m = hnc + 2;
    std::vector<double> tmp((size_t)m * m), gc((size_t)(nc + 1) * (nc + 1));
    for (int b_ = 0; b_ <= hnc + 1; b_++)
      for (int a_ = 0; a_ <= hnc + 1; a_++)
        tmp[a_ + m * b_] = c[face_at(t, d, xc, co[t1] + a_, co[t2] + b_)];
    auto T = [&](int i, int j) { return tmp[i + m * j]; };
    auto G = [&](int i, int j) -> double& { return gc[i + (nc + 1) * j]; };
    for (int j = 1; j <= hnc; j++)
      for (int i = 1; i <= hnc; i++) {
        double g1 = 0.125 * (T(i + 1, j) - T(i - 1, j));
        double g2 = 0.125 * (T(i, j + 1) - T(i, j - 1));
        G(2 * i - 1, 2 * j - 1) = T(i, j) - g1 - g2;
        G(2 * i, 2 * j - 1) = T(i, j) + g1 - g2;
        G(2 * i - 1, 2 * j) = T(i, j) - g1 + g2;
        G(2 * i, 2 * j) = T(i, j) + g1 + g2;
      }
    for (int q = 1; q <= nc; q++)
      for (int p = 1; p <= nc; p++)
        a[face_at(t, d, ix - dix, p, q)] = 0.5 * G(p, q) + 0.75 * a[face_at(t, d, ix, p, q)] -
                                           0.25 * a[face_at(t, d, ix + dix, p, q)];
  }
}

/* af_gc_interp (m_af_ghostcell.f90:394-498) and af_gc_interp_lim (503-612) */
static void interp_rb(const Tree& t, double* cc, int id, int nb, int iv, bool lim) {
  const int nc = t.nc, d = nb / 2;
  const bool low = (nb % 2) == 0;
  const int p_id = t.parent[id - 1];
  const int p_nb = t.nb_of(p_id, nb);
  const double* C = t.var(cc, p_nb, iv);
  double* a = t.var(cc, id, iv);
  const double third = 1 / 3.0, sixth = 1 / 6.0;
  int off[3];
  for (int k = 0; k < t.D; k++) off[k] = t.child_offset(id, k);
  const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
  const int gx = low ? 0 : nc + 1, fx = low ? 1 : nc, cx = low ? nc : 1;
  const int qn = t.D == 3 ? nc : 1;
  for (int q = 1; q <= qn; q++) {
    int q1 = 0, q2 = 0;
    if (t.D == 3) {
      q1 = off[t2] + ((q + 1) >> 1);
      q2 = q1 + 1 - 2 * (q & 1);
    }
    for (int p = 1; p <= nc; p++) {
      int p1 = off[t1] + ((p + 1) >> 1);
      int p2 = p1 + 1 - 2 * (p & 1);
      double f = a[face_at(t, d, fx, p, q)];
      double v;
      if (t.D == 2) {
        double c1 = C[face_at(t, d, cx, p1, 0)], c2 = C[face_at(t, d, cx, p2, 0)];
        v = 0.5 * c1 + sixth * c2 + third * f;
        if (lim && v > 2 * c1) v = 2 * c1;
      } else {
        double c1 = C[face_at(t, d, cx, p1, q1)];
        double c2, c3;
        if (d < 2) {
          c2 = C[face_at(t, d, cx, p2, q1)];
          c3 = C[face_at(t, d, cx, p1, q2)];
        } else {  // z-face: the reference lists (i_c1, j_c2) before (i_c2, j_c1)
          c2 = C[face_at(t, d, cx, p1, q2)];
          c3 = C[face_at(t, d, cx, p2, q1)];
        }
        v = third * c1 + sixth * c2 + sixth * c3 + third * f;
        if (lim && v > 2 * c1) v = 2 * c1;
      }
      a[face_at(t, d, gx, p, q)] = v;
    }
  }
}

/* af_gc_box_corner (m_af_ghostcell.f90:125-170) with af_corner_gc_extrap
 * (860-879) and af_edge_gc_extrap (885-924) */
static void gc_corners(const Tree& t, double* cc, int id, int iv) {
  const int nc = t.nc;
  double* a = t.var(cc, id, iv);
  if (t.D == 3) {
    for (int n = 0; n < 12; n++) {
      const int dim = EDGE_DIM[n];
      const int* dir = EDGE_DIR[n];
      const int nb_id = t.mat_of(id, dir[0], dir[1], dir[2]);
      int lo[3];
      for (int k = 0; k < 3; k++) lo[k] = (dir[k] == 1 ? 1 : 0) * (nc + 1);
      lo[dim] = 1;
      if (nb_id > 0) {
        const double* b = t.var(cc, nb_id, iv);
        for (int p = 1; p <= nc; p++) {
          int x[3] = {lo[0], lo[1], lo[2]};
          x[dim] = p;
          a[t.at(x[0], x[1], x[2])] =
              b[t.at(x[0] - dir[0] * nc, x[1] - dir[1] * nc, x[2] - dir[2] * nc)];
        }
      } else {
        int o1 = (dim + 1) % 3, o2 = (dim + 2) % 3;
        int di[3];
        for (int k = 0; k < 3; k++) di[k] = 1 - 2 * (lo[k] & 1);
        di[dim] = 0;
        for (int p = 1; p <= nc; p++) {
          int x[3] = {lo[0], lo[1], lo[2]};
          x[dim] = p;
          int ia[3] = {x[0], x[1], x[2]}, ib[3] = {x[0], x[1], x[2]};
          ia[o1] += di[o1];
          ib[o2] += di[o2];
          a[t.at(x[0], x[1], x[2])] = a[t.at(ia[0], ia[1], ia[2])] + a[t.at(ib[0], ib[1], ib[2])] -
                                      a[t.at(x[0] + di[0], x[1] + di[1], x[2] + di[2])];
        }
      }
    }
  }
  for (int n = 0; n < t.nchild(); n++) {
    int cd[3] = {n & 1, (n >> 1) & 1, (n >> 2) & 1};
    int dnb[3] = {2 * cd[0] - 1, 2 * cd[1] - 1, t.D == 3 ? 2 * cd[2] - 1 : 0};
    const int nb_id = t.mat_of(id, dnb[0], dnb[1], dnb[2]);
    int lo[3] = {cd[0] * (nc + 1), cd[1] * (nc + 1), t.D == 3 ? cd[2] * (nc + 1) : 0};
    if (nb_id > 0) {
      const double* b = t.var(cc, nb_id, iv);
      a[t.at(lo[0], lo[1], lo[2])] =
          b[t.at(lo[0] - dnb[0] * nc, lo[1] - dnb[1] * nc, lo[2] - dnb[2] * nc)];
    } else {
      int di[3];
      for (int k = 0; k < 3; k++) di[k] = 1 - 2 * (lo[k] & 1);
      const int x = lo[0], y = lo[1], z = lo[2];
      if (t.D == 2) {
        a[t.at(x, y)] = a[t.at(x + di[0], y)] + a[t.at(x, y + di[1])] - a[t.at(x + di[0], y + di[1])];
      } else {
        a[t.at(x, y, z)] = a[t.at(x, y + di[1], z + di[2])] + a[t.at(x + di[0], y, z + di[2])] +
                           a[t.at(x + di[0], y + di[1], z)] -
                           2 * a[t.at(x + di[0], y + di[1], z + di[2])];
      }
    }
  }
}

/* af_gc_box, m_af_ghostcell.f90:64-120 (copy_from_nb 654-669) */
void gc_box(const Tree& t, double* cc, int id, int iv, const GcSpec& g, bool corners) {
  const int nc = t.nc;
  double* a = t.var(cc, id, iv);
  for (int nb = 0; nb < t.nnb(); nb++) {
    const int nb_id = t.nb_of(id, nb);
    const int d = nb / 2;
    const bool low = (nb % 2) == 0;
    if (nb_id > 0) {
      const double* b = t.var(cc, nb_id, iv);
      const int gi = low ? 0 : nc + 1, si = low ? nc : 1;
      const int qn = t.D == 3 ? nc : 1;
      for (int q = 1; q <= qn; q++)
        for (int p = 1; p <= nc; p++) a[face_at(t, d, gi, p, q)] = b[face_at(t, d, si, p, q)];
    } else if (nb_id == 0) {
      if (g.rb == AFG_RB_MG_SIDES)
        sides_rb(t, cc, id, nb, iv);
      else
        interp_rb(t, cc, id, nb, iv, g.rb == AFG_RB_INTERP_LIM);
    } else {
      bc_to_gc(t, a, id, nb, g.bc_type[nb], g.bc_val[nb]);
    }
  }
  if (corners) gc_corners(t, cc, id, iv);
}

/* af_gc_lvl, m_af_ghostcell.f90:49-61 */
void gc_lvl(const Tree& t, double* cc, int lvl, int iv, const GcSpec& g, bool corners) {
  const std::vector<int>& ids = t.ids[lvl - 1];
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < ids.size(); i++) gc_box(t, cc, ids[i], iv, g, corners);
}

/* ---------------------------------------------------------------------- */
/* Operator coefficients: mg_box_lpl_stencil (m_af_multigrid.f90:1246-1264)
 * and the cylindrical correction of stencil_apply_357 / stencil_gsrb_357
 * (m_af_stencil.f90:400-420, 884-906) with af_cyl_flux_factors
 * (m_af_types.f90:1199-1211). */
struct Stencil {
  double c[7];
  bool cyl = false;
  double cyl1[64 + 1], cyl2[64 + 1], cyl3[64 + 1], inv1[64 + 1];
  double inv_c1;
};

static void make_stencil(const Tree& t, const afg_mg_desc& m, int id, Stencil& s) {
  const int D = t.D;
  double inv_dr2[3];
  for (int d = 0; d < D; d++) {
    double h = t.dr_of(id, d);
    inv_dr2[d] = 1 / (h * h);
  }
  for (int d = 0; d < D; d++) s.c[1 + 2 * d] = s.c[2 + 2 * d] = inv_dr2[d];
  double sum = 0;
  for (int k = 1; k <= 2 * D; k++) sum += s.c[k];
  s.c[0] = -sum - m.helmholtz_lambda;
  s.inv_c1 = 1 / s.c[0];
  s.cyl = (t.coord == AFG_CYL && D == 2);
  if (s.cyl) {
    const double rmin = t.rmin_of(id, 0), h = t.dr_of(id, 0);
    for (int i = 1; i <= t.nc; i++) {
      double r = rmin + (i - 0.5) * h;
      double inv_r = 1 / r;
      double f1 = (r - 0.5 * h) * inv_r, f2 = (r + 0.5 * h) * inv_r;
      s.cyl2[i] = f1 * s.c[1];
      s.cyl3[i] = f2 * s.c[2];
      s.cyl1[i] = s.c[0] - (s.cyl2[i] - s.c[1]) - (s.cyl3[i] - s.c[2]);
      s.inv1[i] = 1 / s.cyl1[i];
    }
  }
}

/* stencil_gsrb_357 with a variable stencil and bc_correction
 * (m_af_stencil.f90:838-998): rhs += bcc on the interior, the half sweep
 * dividing by v(1), rhs -= bcc; stored ghost cells */
static void gsrb_box_lsf(const Tree& t, double* cc, const afg_mg_desc& m, const Lsf& L, int id, int redblack) {
  const int q = L.of(id), SI = L.SI, nc = t.nc, D = t.D;
  double* p = t.var(cc, id, m.i_phi);
  double* f = t.var(cc, id, m.i_rhs);
  const double* v = L.v.data() + (size_t)q * (2 * D + 1) * SI;
  const double* bcc = L.bcc.data() + (size_t)q * SI;
  const int kn = D == 3 ? nc : 1, sj = t.n2, sk = t.n2 * t.n2;
  int c = 0;
  for (int k = 1; k <= kn; k++)
    for (int j = 1; j <= nc; j++)
      for (int i = 1; i <= nc; i++, c++) {
        const int x = t.at(i, j, D == 3 ? k : 0);
        f[x] = f[x] + bcc[c];
      }
  c = 0;
  for (int k = 1; k <= kn; k++)
    for (int j = 1; j <= nc; j++)
      for (int i = 1; i <= nc; i++, c++) {
        if (((i + j + (D == 3 ? k : 0) + redblack) & 1) != 0) continue;
        const int x = t.at(i, j, D == 3 ? k : 0);
        double val = f[x] - v[(size_t)1 * SI + c] * p[x - 1] - v[(size_t)2 * SI + c] * p[x + 1] -
                     v[(size_t)3 * SI + c] * p[x - sj] - v[(size_t)4 * SI + c] * p[x + sj];
        if (D == 3) val = val - v[(size_t)5 * SI + c] * p[x - sk] - v[(size_t)6 * SI + c] * p[x + sk];
        p[x] = val / v[c];
      }
  c = 0;
  for (int k = 1; k <= kn; k++)
    for (int j = 1; j <= nc; j++)
      for (int i = 1; i <= nc; i++, c++) {
        const int x = t.at(i, j, D == 3 ? k : 0);
        f[x] = f[x] - bcc[c];
      }
}

/* stencil_apply_357 with a variable stencil, then - bc_correction
 * (m_af_stencil.f90:367-496) into out[c] (interior cells, i fastest) */
static void apply_lsf(const Tree& t, const double* cc, const afg_mg_desc& m, const Lsf& L, int id, double* out) {
  const int q = L.of(id), SI = L.SI, nc = t.nc, D = t.D;
  const double* p = t.var(const_cast<double*>(cc), id, m.i_phi);
  const double* v = L.v.data() + (size_t)q * (2 * D + 1) * SI;
  const double* bcc = L.bcc.data() + (size_t)q * SI;
  const int kn = D == 3 ? nc : 1, sj = t.n2, sk = t.n2 * t.n2;
  int c = 0;
  for (int k = 1; k <= kn; k++)
    for (int j = 1; j <= nc; j++)
      for (int i = 1; i <= nc; i++, c++) {
        const int x = t.at(i, j, D == 3 ? k : 0);
        double lp = v[c] * p[x] + v[(size_t)1 * SI + c] * p[x - 1] + v[(size_t)2 * SI + c] * p[x + 1] +
                    v[(size_t)3 * SI + c] * p[x - sj] + v[(size_t)4 * SI + c] * p[x + sj];
        if (D == 3) lp = lp + v[(size_t)5 * SI + c] * p[x - sk] + v[(size_t)6 * SI + c] * p[x + sk];
        out[c] = lp - bcc[c];
      }
}

/* stencil_gsrb_357, m_af_stencil.f90:838-998 */
static void gsrb_box(const Tree& t, double* cc, const Mg& mg, int id, int redblack) {
  if (mg.lsf && mg.lsf->of(id) >= 0) return gsrb_box_lsf(t, cc, mg.d, *mg.lsf, id, redblack);
  const afg_mg_desc& m = mg.d;
  Stencil s;
  make_stencil(t, m, id, s);
  double* p = t.var(cc, id, m.i_phi);
  const double* f = t.var(cc, id, m.i_rhs);
  const int nc = t.nc;
  if (t.D == 2) {
    for (int j = 1; j <= nc; j++) {
      int i0 = 2 - ((redblack ^ j) & 1);
      for (int i = i0; i <= nc; i += 2) {
        int x = t.at(i, j);
        if (s.cyl) {
          p[x] = (f[x] - s.cyl2[i] * p[x - 1] - s.cyl3[i] * p[x + 1] - s.c[3] * p[x - t.n2] -
                  s.c[4] * p[x + t.n2]) *
                 s.inv1[i];
        } else {
          p[x] = (f[x] - s.c[1] * p[x - 1] - s.c[2] * p[x + 1] - s.c[3] * p[x - t.n2] -
                  s.c[4] * p[x + t.n2]) *
                 s.inv_c1;
        }
      }
    }
  } else {
    const int sj = t.n2, sk = t.n2 * t.n2;
    for (int k = 1; k <= nc; k++)
      for (int j = 1; j <= nc; j++) {
        int i0 = 2 - ((redblack ^ (k + j)) & 1);
        for (int i = i0; i <= nc; i += 2) {
          int x = t.at(i, j, k);
          p[x] = (f[x] - s.c[1] * p[x - 1] - s.c[2] * p[x + 1] - s.c[3] * p[x - sj] -
                  s.c[4] * p[x + sj] - s.c[5] * p[x - sk] - s.c[6] * p[x + sk]) *
                 s.inv_c1;
        }
      }
  }
}

/* stencil_apply_357 (m_af_stencil.f90:367-496) then residual_box
 * (m_af_multigrid.f90:801-810): out = rhs - L phi on interior cells */
static void residual_into(const Tree& t, const double* cc, const Mg& mg, int id,
                          double* out /* nc^D, i fastest */) {
  const afg_mg_desc& m = mg.d;
  if (mg.lsf && mg.lsf->of(id) >= 0) {
    apply_lsf(t, cc, m, *mg.lsf, id, out);
    const double* f = t.var(const_cast<double*>(cc), id, m.i_rhs);
    int c = 0;
    for (int k = (t.D == 3 ? 1 : 0); k <= (t.D == 3 ? t.nc : 0); k++)
      for (int j = 1; j <= t.nc; j++)
        for (int i = 1; i <= t.nc; i++, c++) out[c] = f[t.at(i, j, k)] - out[c];
    return;
  }
  Stencil s;
  make_stencil(t, m, id, s);
  const double* p = t.var(const_cast<double*>(cc), id, m.i_phi);
  const double* f = t.var(const_cast<double*>(cc), id, m.i_rhs);
  const int nc = t.nc;
  int n = 0;
  if (t.D == 2) {
    for (int j = 1; j <= nc; j++)
      for (int i = 1; i <= nc; i++) {
        int x = t.at(i, j);
        double lp;
        if (s.cyl)
          lp = s.cyl1[i] * p[x] + s.cyl2[i] * p[x - 1] + s.cyl3[i] * p[x + 1] + s.c[3] * p[x - t.n2] +
               s.c[4] * p[x + t.n2];
        else
          lp = s.c[0] * p[x] + s.c[1] * p[x - 1] + s.c[2] * p[x + 1] + s.c[3] * p[x - t.n2] +
               s.c[4] * p[x + t.n2];
        out[n++] = f[x] - lp;
      }
  } else {
    const int sj = t.n2, sk = t.n2 * t.n2;
    for (int k = 1; k <= nc; k++)
      for (int j = 1; j <= nc; j++)
        for (int i = 1; i <= nc; i++) {
          int x = t.at(i, j, k);
          double lp = s.c[0] * p[x] + s.c[1] * p[x - 1] + s.c[2] * p[x + 1] + s.c[3] * p[x - sj] +
                      s.c[4] * p[x + sj] + s.c[5] * p[x - sk] + s.c[6] * p[x + sk];
          out[n++] = f[x] - lp;
        }
  }
}

/* stencil_apply_357 alone into variable iv_out (interior) */
static void apply_into(const Tree& t, double* cc, const Mg& mg, int id, int iv_out) {
  const afg_mg_desc& m = mg.d;
  if (mg.lsf && mg.lsf->of(id) >= 0) {
    std::vector<double> out(mg.lsf->SI);
    apply_lsf(t, cc, m, *mg.lsf, id, out.data());
    double* o = t.var(cc, id, iv_out);
    int c = 0;
    for (int k = (t.D == 3 ? 1 : 0); k <= (t.D == 3 ? t.nc : 0); k++)
      for (int j = 1; j <= t.nc; j++)
        for (int i = 1; i <= t.nc; i++, c++) o[t.at(i, j, k)] = out[c];
    return;
  }
  Stencil s;
  make_stencil(t, m, id, s);
  const double* p = t.var(cc, id, m.i_phi);
  double* o = t.var(cc, id, iv_out);
  const int nc = t.nc;
  if (t.D == 2) {
    for (int j = 1; j <= nc; j++)
      for (int i = 1; i <= nc; i++) {
        int x = t.at(i, j);
        if (s.cyl)
          o[x] = s.cyl1[i] * p[x] + s.cyl2[i] * p[x - 1] + s.cyl3[i] * p[x + 1] + s.c[3] * p[x - t.n2] +
                 s.c[4] * p[x + t.n2];
        else
          o[x] = s.c[0] * p[x] + s.c[1] * p[x - 1] + s.c[2] * p[x + 1] + s.c[3] * p[x - t.n2] +
                 s.c[4] * p[x + t.n2];
      }
  } else {
    const int sj = t.n2, sk = t.n2 * t.n2;
    for (int k = 1; k <= nc; k++)
      for (int j = 1; j <= nc; j++)
        for (int i = 1; i <= nc; i++) {
          int x = t.at(i, j, k);
          o[x] = s.c[0] * p[x] + s.c[1] * p[x - 1] + s.c[2] * p[x + 1] + s.c[3] * p[x - sj] +
                 s.c[4] * p[x + sj] + s.c[5] * p[x - sk] + s.c[6] * p[x + sk];
        }
  }
}

/* af_restrict_box, m_af_restrict.f90:62-136: child data src (nc^D dense,
 * i fastest, or a full box array when full=true) averaged into the parent's
 * variable iv at the child's offset */
static void restrict_to_parent(const Tree& t, double* cc, int id, const double* src, bool src_full,
                               int iv, bool use_geom) {
  const int nc = t.nc, hnc = nc / 2;
  const int p_id = t.parent[id - 1];
  double* pp = t.var(cc, p_id, iv);
  int off[3] = {0, 0, 0};
  for (int d = 0; d < t.D; d++) off[d] = t.child_offset(id, d);
  auto F = [&](int i, int j, int k) -> double {
    if (src_full) return src[t.at(i, j, k)];
    return src[(i - 1) + nc * ((j - 1) + nc * (k > 0 ? k - 1 : 0))];
  };
  if (t.D == 2) {
    const bool cyl = (t.coord == AFG_CYL) && use_geom;
    for (int j = 1; j <= hnc; j++) {
      int jc = off[1] + j, jf = 2 * j - 1;
      for (int i = 1; i <= hnc; i++) {
        int ic = off[0] + i, if_ = 2 * i - 1;
        double v;
        if (cyl) {
          double r = t.rmin_of(p_id, 0) + (ic - 0.5) * t.dr_of(p_id, 0);
          double tmp = 0.25 * t.dr_of(p_id, 0) / r;
          double w1 = 1 - tmp, w2 = 1 + tmp;
          double s1 = 0, s2 = 0;
          s1 += F(if_, jf, 0); s1 += F(if_, jf + 1, 0);
          s2 += F(if_ + 1, jf, 0); s2 += F(if_ + 1, jf + 1, 0);
          v = 0.25 * (w1 * s1 + w2 * s2);
        } else {
          double s = 0;
          s += F(if_, jf, 0); s += F(if_ + 1, jf, 0);
          s += F(if_, jf + 1, 0); s += F(if_ + 1, jf + 1, 0);
          v = 0.25 * s;
        }
        pp[t.at(ic, jc)] = v;
      }
    }
  } else {
    for (int k = 1; k <= hnc; k++) {
      int kc = off[2] + k, kf = 2 * k - 1;
      for (int j = 1; j <= hnc; j++) {
        int jc = off[1] + j, jf = 2 * j - 1;
        for (int i = 1; i <= hnc; i++) {
          int ic = off[0] + i, if_ = 2 * i - 1;
          double s = 0;
          for (int dk = 0; dk < 2; dk++)
            for (int dj = 0; dj < 2; dj++)
              for (int di = 0; di < 2; di++) s += F(if_ + di, jf + dj, kf + dk);
          pp[t.at(ic, jc, kc)] = 0.125 * s;
        }
      }
    }
  }
}

/* stencil_prolong_248 with add=.true., m_af_stencil.f90:695-815 (coefficients
 * mg_box_prolong_linear_stencil, m_af_multigrid.f90:1267-1284) */
static void prolong_add(const Tree& t, double* cc, int p_id, int c_id, int iv_from, int iv_to) {
  const int nc = t.nc;
  const double* P = t.var(cc, p_id, iv_from);
  double* C = t.var(cc, c_id, iv_to);
  int off[3] = {0, 0, 0};
  for (int d = 0; d < t.D; d++) off[d] = t.child_offset(c_id, d);
  if (t.D == 2) {
    const double c1 = 9 / 16.0, c2 = 3 / 16.0, c3 = 3 / 16.0, c4 = 1 / 16.0;
    for (int j = 1; j <= nc; j++) {
      int j1 = off[1] + ((j + 1) >> 1), j2 = j1 + 1 - 2 * (j & 1);
      for (int i = 1; i <= nc; i++) {
        int i1 = off[0] + ((i + 1) >> 1), i2 = i1 + 1 - 2 * (i & 1);
        int x = t.at(i, j);
        C[x] = C[x] + c1 * P[t.at(i1, j1)] + c2 * P[t.at(i2, j1)] + c3 * P[t.at(i1, j2)] +
               c4 * P[t.at(i2, j2)];
      }
    }
  } else {
    const double w[8] = {27 / 64.0, 9 / 64.0, 9 / 64.0, 3 / 64.0, 9 / 64.0, 3 / 64.0, 3 / 64.0, 1 / 64.0};
    for (int k = 1; k <= nc; k++) {
      int k1 = off[2] + ((k + 1) >> 1), k2 = k1 + 1 - 2 * (k & 1);
      for (int j = 1; j <= nc; j++) {
        int j1 = off[1] + ((j + 1) >> 1), j2 = j1 + 1 - 2 * (j & 1);
        for (int i = 1; i <= nc; i++) {
          int i1 = off[0] + ((i + 1) >> 1), i2 = i1 + 1 - 2 * (i & 1);
          int x = t.at(i, j, k);
          C[x] = C[x] + w[0] * P[t.at(i1, j1, k1)] + w[1] * P[t.at(i2, j1, k1)] +
                 w[2] * P[t.at(i1, j2, k1)] + w[3] * P[t.at(i2, j2, k1)] + w[4] * P[t.at(i1, j1, k2)] +
                 w[5] * P[t.at(i2, j1, k2)] + w[6] * P[t.at(i1, j2, k2)] + w[7] * P[t.at(i2, j2, k2)];
        }
      }
    }
  }
}

/* ---------------------------------------------------------------------- */
/* gsrb_boxes, m_af_multigrid.f90:648-687 */
static void gsrb_boxes(Oracle& o, double* cc, const Mg& m, int lvl, int type) {
  const Tree& t = o.t;
  const int n_cycle = type == AFG_CYCLE_DOWN ? m.d.n_cycle_down : m.d.n_cycle_up;
  const std::vector<int>& ids = t.ids[lvl - 1];
  const GcSpec g = m.gc();
  for (int n = 1; n <= 2 * n_cycle; n++) {
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < ids.size(); i++) gsrb_box(t, cc, m, ids[i], n);
    const bool use_corners = (type != AFG_CYCLE_DOWN && n == 2 * n_cycle);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < ids.size(); i++) gc_box(t, cc, ids[i], m.d.i_phi, g, use_corners);
  }
}

/* update_coarse, m_af_multigrid.f90:691-738 (the residual is restricted
 * straight from a temporary; the reference stores it in i_tmp and restores
 * i_tmp afterwards, which leaves the same state) */
static void update_coarse(Oracle& o, double* cc, const Mg& m, int lvl) {
  const Tree& t = o.t;
  const std::vector<int>& ids = t.ids[lvl - 1];
  const int ncd = (int)std::pow((double)t.nc, (double)t.D);
#pragma omp parallel
  {
    std::vector<double> r(ncd);
#pragma omp for schedule(static)
    for (size_t i = 0; i < ids.size(); i++) {
      int id = ids[i];
      residual_into(t, cc, m, id, r.data());
      restrict_to_parent(t, cc, id, r.data(), false, m.d.i_tmp, true);
      restrict_to_parent(t, cc, id, t.var(cc, id, m.d.i_phi), true, m.d.i_phi, false);
    }
  }
  gc_lvl(t, cc, lvl - 1, m.d.i_phi, m.gc(), true);
  const std::vector<int>& par = t.parents[lvl - 2];
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < par.size(); i++) {
    int id = par[i];
    apply_into(t, cc, m, id, m.d.i_rhs);
    double* f = t.var(cc, id, m.d.i_rhs);
    double* tm = t.var(cc, id, m.d.i_tmp);
    const double* p = t.var(cc, id, m.d.i_phi);
    for (int x = 0; x < t.S; x++) f[x] = f[x] + tm[x];  // af_box_add_cc (whole array)
    for (int x = 0; x < t.S; x++) tm[x] = p[x];         // af_box_copy_cc (whole array)
  }
}

/* set_coarse_phi_rhs, m_af_multigrid.f90:742-776 */
static void set_coarse_phi_rhs(Oracle& o, double* cc, const Mg& m, int lvl) {
  const Tree& t = o.t;
  if (lvl == t.highest_lvl) gc_lvl(t, cc, lvl, m.d.i_phi, m.gc(), true);
  const std::vector<int>& ids = t.ids[lvl - 1];
  const int ncd = (int)std::pow((double)t.nc, (double)t.D);
#pragma omp parallel
  {
    std::vector<double> r(ncd);
#pragma omp for schedule(static)
    for (size_t i = 0; i < ids.size(); i++) {
      int id = ids[i];
      residual_into(t, cc, m, id, r.data());
      double* tm = t.var(cc, id, m.d.i_tmp);
      int n = 0;
      for (int k = (t.D == 3 ? 1 : 0); k <= (t.D == 3 ? t.nc : 0); k++)
        for (int j = 1; j <= t.nc; j++)
          for (int ii = 1; ii <= t.nc; ii++) tm[t.at(ii, j, k)] = r[n++];
      restrict_to_parent(t, cc, id, r.data(), false, m.d.i_tmp, true);
      restrict_to_parent(t, cc, id, t.var(cc, id, m.d.i_phi), true, m.d.i_phi, false);
    }
  }
  gc_lvl(t, cc, lvl - 1, m.d.i_phi, m.gc(), true);
  const std::vector<int>& par = t.parents[lvl - 2];
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < par.size(); i++) {
    int id = par[i];
    apply_into(t, cc, m, id, m.d.i_rhs);
    double* f = t.var(cc, id, m.d.i_rhs);
    double* tm = t.var(cc, id, m.d.i_tmp);
    for (int x = 0; x < t.S; x++) f[x] = f[x] + tm[x];
  }
}

/* init_phi_rhs, m_af_multigrid.f90:779-799 */
static void init_phi_rhs(Oracle& o, double* cc, const Mg& m) {
  const Tree& t = o.t;
  for (int lvl = t.highest_lvl; lvl >= 2; lvl--) {
    const std::vector<int>& ids = t.ids[lvl - 1];
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < ids.size(); i++) {
      int id = ids[i];
      double* p = t.var(cc, id, m.d.i_phi);
      for (int x = 0; x < t.S; x++) p[x] = 0;
      restrict_to_parent(t, cc, id, t.var(cc, id, m.d.i_rhs), true, m.d.i_rhs, true);
    }
  }
}

/* correct_children, m_af_multigrid.f90:624-646 */
static void correct_children(Oracle& o, double* cc, const Mg& m, int lvl_parent) {
  const Tree& t = o.t;
  const std::vector<int>& par = t.parents[lvl_parent - 1];
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < par.size(); i++) {
    int id = par[i];
    double* tm = t.var(cc, id, m.d.i_tmp);
    const double* p = t.var(cc, id, m.d.i_phi);
    for (int x = 0; x < t.S; x++) tm[x] = p[x] - tm[x];
    for (int c = 0; c < t.nchild(); c++) {
      int c_id = t.child_of(id, c);
      if (c_id == 0) continue;  // af_no_box
      prolong_add(t, cc, id, c_id, m.d.i_tmp, m.d.i_phi);
    }
  }
}

/* Coarse matrix, hypre_set_matrix + stencil_handle_boundaries
 * (m_coarse_solver.f90:104-194, 442-491).  Unknown g = I + gx*(J + gy*K)
 * with global 0-based cell indices on level 1. */
static int build_coarse(Oracle& o, Mg& m) {
  const Tree& t = o.t;
  const int D = t.D, nc = t.nc;
  for (int d = 0; d < 3; d++) m.gx[d] = d < D ? t.cgs[d] : 1;
  const long n = (long)m.gx[0] * m.gx[1] * m.gx[2];
  if (n > 4096) return AFG_ERR_UNSUPPORTED;
  m.n_coarse = (int)n;
  std::vector<double> A((size_t)n * n, 0.0);
  const std::vector<int>& ids = t.ids[0];
  m.bc_to_rhs.assign(ids.size() * t.nnb() * (D == 3 ? nc * nc : nc), 0.0);
  for (size_t bi = 0; bi < ids.size(); bi++) {
    const int id = ids[bi];
    Stencil s;
    make_stencil(t, m.d, id, s);
    const int kn = D == 3 ? nc : 1;
    // an electrode box: its variable stencil (stencil_get_357 of a
    // variable stencil without cylindrical factors)
    const double* vq = nullptr;
    if (m.lsf && m.lsf->of(id) >= 0) vq = m.lsf->v.data() + (size_t)m.lsf->of(id) * (2 * D + 1) * m.lsf->SI;
    for (int k = 1; k <= kn; k++)
      for (int j = 1; j <= nc; j++)
        for (int i = 1; i <= nc; i++) {
          double st[7];
          for (int q = 0; q < 7; q++) st[q] = s.c[q];
          if (vq) {
            const int c = (i - 1) + nc * ((j - 1) + nc * (k - 1));
            for (int q = 0; q < 7; q++) st[q] = q <= 2 * D ? vq[(size_t)q * m.lsf->SI + c] : 0.0;
          } else if (s.cyl) {  // stencil_get_357, m_af_stencil.f90:1073-1084
            st[1] = s.cyl2[i];
            st[2] = s.cyl3[i];
            st[0] = s.cyl1[i];
          }
          int cidx[3] = {i, j, k};
          for (int nb = 0; nb < 2 * D; nb++) {
            if (t.nb_of(id, nb) >= 0) continue;
            const int d = nb / 2;
            const bool low = (nb % 2) == 0;
            if (cidx[d] != (low ? 1 : nc)) continue;
            int p = d == 0 ? (D == 3 ? j + nc * (k - 1) : j) : (d == 1 ? (D == 3 ? i + nc * (k - 1) : i) : i + nc * (j - 1));
            double& b2r = m.bc_to_rhs[(bi * t.nnb() + nb) * (D == 3 ? nc * nc : nc) + (p - 1)];
            if (m.d.bc_type[nb] == AFG_BC_DIRICHLET) {
              st[0] = st[0] - st[nb + 1];
              b2r = -2 * st[nb + 1];
              st[nb + 1] = 0.0;
            } else if (m.d.bc_type[nb] == AFG_BC_NEUMANN) {
              st[0] = st[0] + st[nb + 1];
              b2r = -(st[nb + 1] * t.dr_of(id, d)) * (low ? -1 : 1);
              st[nb + 1] = 0.0;
            } else {
              return AFG_ERR_UNSUPPORTED;
            }
          }
          long I = (long)(t.ix_of(id, 0) - 1) * nc + (i - 1);
          long J = (long)(t.ix_of(id, 1) - 1) * nc + (j - 1);
          long K = D == 3 ? (long)(t.ix_of(id, 2) - 1) * nc + (k - 1) : 0;
          long g = I + m.gx[0] * (J + (long)m.gx[1] * K);
          A[(size_t)g * n + g] += st[0];
          long G[3] = {I, J, K};
          for (int nb = 0; nb < 2 * D; nb++) {
            if (st[nb + 1] == 0.0) continue;
            long H[3] = {G[0], G[1], G[2]};
            H[nb / 2] += (nb % 2) ? 1 : -1;
            if (H[nb / 2] < 0 || H[nb / 2] >= m.gx[nb / 2]) return AFG_ERR_ARG;
            long h = H[0] + m.gx[0] * (H[1] + (long)m.gx[1] * H[2]);
            A[(size_t)g * n + h] += st[nb + 1];
          }
        }
  }
  m.amat = A;
  // Gauss-Jordan elimination with partial pivoting: ainv = A^-1
  std::vector<double> I((size_t)n * n, 0.0);
  for (long r = 0; r < n; r++) I[(size_t)r * n + r] = 1.0;
  for (long c = 0; c < n; c++) {
    long piv = c;
    double best = std::fabs(A[(size_t)c * n + c]);
    for (long r = c + 1; r < n; r++) {
      double v = std::fabs(A[(size_t)r * n + c]);
      if (v > best) { best = v; piv = r; }
    }
    if (best == 0.0) return AFG_ERR_ARG;
    if (piv != c) {
      for (long q = 0; q < n; q++) {
        std::swap(A[(size_t)c * n + q], A[(size_t)piv * n + q]);
        std::swap(I[(size_t)c * n + q], I[(size_t)piv * n + q]);
      }
    }
    const double inv = 1.0 / A[(size_t)c * n + c];
    for (long q = 0; q < n; q++) {
      A[(size_t)c * n + q] *= inv;
      I[(size_t)c * n + q] *= inv;
    }
#pragma omp parallel for schedule(static)
    for (long r = 0; r < n; r++) {
      if (r == c) continue;
      const double f = A[(size_t)r * n + c];
      if (f == 0.0) continue;
      for (long q = 0; q < n; q++) {
        A[(size_t)r * n + q] -= f * A[(size_t)c * n + q];
        I[(size_t)r * n + q] -= f * I[(size_t)c * n + q];
      }
    }
  }
  m.ainv.swap(I);
  return AFG_OK;
}

/* Fixed-order dense mat-vec: 32 strided partial sums per row, then an xor
 * butterfly (the order of the GPU warp reduction). */
static void coarse_matvec(const Mg& m, const double* b, double* x) {
  const int n = m.n_coarse;
#pragma omp parallel for schedule(static)
  for (int r = 0; r < n; r++) {
    double p[32];
    const double* row = m.ainv.data() + (size_t)r * n;
    for (int l = 0; l < 32; l++) {
      double s = 0.0;
      for (int c = l; c < n; c += 32) s = s + row[c] * b[c];
      p[l] = s;
    }
    for (int off = 16; off >= 1; off >>= 1) {
      double q[32];
      for (int l = 0; l < 32; l++) q[l] = p[l] + p[l ^ off];
      for (int l = 0; l < 32; l++) p[l] = q[l];
    }
    x[r] = p[0];
  }
}

/* solve_coarse_grid, m_af_multigrid.f90:266-291, with
 * coarse_solver_set_rhs_phi / coarse_solver_get_phi
 * (m_coarse_solver.f90:286-358) */
static void coarse_solve(Oracle& o, double* cc, const Mg& m) {
  const Tree& t = o.t;
  const int D = t.D, nc = t.nc, n = m.n_coarse;
  const int fn = D == 3 ? nc * nc : nc;
  std::vector<double> b(n), x(n);
  const std::vector<int>& ids = t.ids[0];
  for (size_t bi = 0; bi < ids.size(); bi++) {
    const int id = ids[bi];
    const double* f = t.var(cc, id, m.d.i_rhs);
    const int kn = D == 3 ? nc : 1;
    for (int k = 1; k <= kn; k++)
      for (int j = 1; j <= nc; j++)
        for (int i = 1; i <= nc; i++) {
          double v = f[t.at(i, j, D == 3 ? k : 0)];
          int cidx[3] = {i, j, k};
          for (int nb = 0; nb < 2 * D; nb++) {
            if (t.nb_of(id, nb) >= 0) continue;
            const int d = nb / 2;
            if (cidx[d] != ((nb % 2) == 0 ? 1 : nc)) continue;
            int p = d == 0 ? (D == 3 ? j + nc * (k - 1) : j) : (d == 1 ? (D == 3 ? i + nc * (k - 1) : i) : i + nc * (j - 1));
            v = v + m.bc_to_rhs[(bi * t.nnb() + nb) * fn + (p - 1)] * m.d.bc_val[nb];
          }
          // the level-set term lsf_fac * boundary value (m_coarse_solver.f90:323-327)
          if (m.lsf && m.lsf->of(id) >= 0) {
            const int c = (i - 1) + nc * ((j - 1) + nc * (k - 1));
            v = v + m.lsf->bcc[(size_t)m.lsf->of(id) * m.lsf->SI + c];
          }
          long I = (long)(t.ix_of(id, 0) - 1) * nc + (i - 1);
          long J = (long)(t.ix_of(id, 1) - 1) * nc + (j - 1);
          long K = D == 3 ? (long)(t.ix_of(id, 2) - 1) * nc + (k - 1) : 0;
          b[I + m.gx[0] * (J + (long)m.gx[1] * K)] = v;
        }
  }
  coarse_matvec(m, b.data(), x.data());
  // Sensitivity experiment (environment ORC_COARSE_RELTOL = tol): the
  // reference solves the coarse grid iteratively (hypre PFMG, stopped at a
  // relative residual of 1e-6, m_coarse_solver.f90:421-439) from the current
  // phi; model its answer as the current phi moved towards the exact
  // solution just far enough that ||b - A x|| / ||b|| = tol.  Off by default.
  static const double reltol = [] {
    const char* e = std::getenv("ORC_COARSE_RELTOL");
    return e ? std::atof(e) : 0.0;
  }();
  if (reltol > 0) {
    std::vector<double> x0(n, 0.0);
    for (size_t bi = 0; bi < ids.size(); bi++) {
      const int id = ids[bi];
      const double* p = t.var(cc, id, m.d.i_phi);
      const int kn = D == 3 ? nc : 1;
      for (int k = 1; k <= kn; k++)
        for (int j = 1; j <= nc; j++)
          for (int i = 1; i <= nc; i++) {
            long I = (long)(t.ix_of(id, 0) - 1) * nc + (i - 1);
            long J = (long)(t.ix_of(id, 1) - 1) * nc + (j - 1);
            long K = D == 3 ? (long)(t.ix_of(id, 2) - 1) * nc + (k - 1) : 0;
            x0[I + m.gx[0] * (J + (long)m.gx[1] * K)] = p[t.at(i, j, D == 3 ? k : 0)];
          }
    }
    double rn = 0, bn = 0;
    for (int r = 0; r < n; r++) {
      double ax = 0;
      for (int c = 0; c < n; c++) ax += m.amat[(size_t)r * n + c] * x0[c];
      rn += (b[r] - ax) * (b[r] - ax);
      bn += b[r] * b[r];
    }
    rn = std::sqrt(rn);
    bn = std::sqrt(bn);
    const double eps = rn > 0 ? std::min(1.0, reltol * bn / rn) : 0.0;
    for (int r = 0; r < n; r++) x[r] = x[r] + eps * (x0[r] - x[r]);
  }
  for (size_t bi = 0; bi < ids.size(); bi++) {
    const int id = ids[bi];
    double* p = t.var(cc, id, m.d.i_phi);
    const int kn = D == 3 ? nc : 1;
    for (int k = 1; k <= kn; k++)
      for (int j = 1; j <= nc; j++)
        for (int i = 1; i <= nc; i++) {
          long I = (long)(t.ix_of(id, 0) - 1) * nc + (i - 1);
          long J = (long)(t.ix_of(id, 1) - 1) * nc + (j - 1);
          long K = D == 3 ? (long)(t.ix_of(id, 2) - 1) * nc + (k - 1) : 0;
          p[t.at(i, j, D == 3 ? k : 0)] = x[I + m.gx[0] * (J + (long)m.gx[1] * K)];
        }
  }
  gc_lvl(t, cc, 1, m.d.i_phi, m.gc(), true);
}

static void residual_lvls(Oracle& o, double* cc, const Mg& m, int max_lvl) {
  const Tree& t = o.t;
  const int ncd = (int)std::pow((double)t.nc, (double)t.D);
  for (int lvl = 1; lvl <= max_lvl; lvl++) {
    const std::vector<int>& ids = t.ids[lvl - 1];
#pragma omp parallel
    {
      std::vector<double> r(ncd);
#pragma omp for schedule(static)
      for (size_t i = 0; i < ids.size(); i++) {
        int id = ids[i];
        residual_into(t, cc, m, id, r.data());
        double* tm = t.var(cc, id, m.d.i_tmp);
        int n = 0;
        for (int k = (t.D == 3 ? 1 : 0); k <= (t.D == 3 ? t.nc : 0); k++)
          for (int j = 1; j <= t.nc; j++)
            for (int ii = 1; ii <= t.nc; ii++) tm[t.at(ii, j, k)] = r[n++];
      }
    }
  }
}

double maxabs(const Tree& t, const double* cc, int iv, bool leaves_only) {
  double res = 0.0;
  for (int lvl = 1; lvl <= t.highest_lvl; lvl++) {
    const std::vector<int>& ids = leaves_only ? t.leaves[lvl - 1] : t.ids[lvl - 1];
#pragma omp parallel for reduction(max : res) schedule(static)
    for (size_t i = 0; i < ids.size(); i++) {
      const double* a = t.var(const_cast<double*>(cc), ids[i], iv);
      for (int k = (t.D == 3 ? 1 : 0); k <= (t.D == 3 ? t.nc : 0); k++)
        for (int j = 1; j <= t.nc; j++)
          for (int ii = 1; ii <= t.nc; ii++) res = std::max(res, std::fabs(a[t.at(ii, j, k)]));
    }
  }
  return res;
}

/* mg_fas_vcycle, m_af_multigrid.f90:185-264 */
static void vcycle(Oracle& o, double* cc, const Mg& m, bool set_residual, int max_lvl) {
  for (int lvl = max_lvl; lvl >= 2; lvl--) {
    gsrb_boxes(o, cc, m, lvl, AFG_CYCLE_DOWN);
    update_coarse(o, cc, m, lvl);
  }
  coarse_solve(o, cc, m);
  for (int lvl = 2; lvl <= max_lvl; lvl++) {
    correct_children(o, cc, m, lvl - 1);
    gc_lvl(o.t, cc, lvl, m.d.i_phi, m.gc(), true);
    gsrb_boxes(o, cc, m, lvl, AFG_CYCLE_UP);
  }
  if (set_residual) residual_lvls(o, cc, m, max_lvl);
}

static void copy_lvl(const Tree& t, double* cc, int lvl, int from, int to) {
  const std::vector<int>& ids = t.ids[lvl - 1];
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < ids.size(); i++) {
    const double* a = t.var(cc, ids[i], from);
    double* b = t.var(cc, ids[i], to);
    std::memcpy(b, a, sizeof(double) * t.S);
  }
}

/* mg_fas_fmg, m_af_multigrid.f90:137-180 */
static void fmg(Oracle& o, double* cc, const Mg& m, bool set_residual, bool have_guess) {
  const Tree& t = o.t;
  if (have_guess) {
    for (int lvl = t.highest_lvl; lvl >= 2; lvl--) set_coarse_phi_rhs(o, cc, m, lvl);
  } else {
    init_phi_rhs(o, cc, m);
  }
  copy_lvl(t, cc, 1, m.d.i_phi, m.d.i_tmp);
  vcycle(o, cc, m, set_residual && t.highest_lvl == 1, 1);
  for (int lvl = 2; lvl <= t.highest_lvl; lvl++) {
    copy_lvl(t, cc, lvl, m.d.i_phi, m.d.i_tmp);
    correct_children(o, cc, m, lvl - 1);
    gc_lvl(t, cc, lvl, m.d.i_phi, m.gc(), true);
    vcycle(o, cc, m, set_residual && lvl == t.highest_lvl, lvl);
  }
}

}  // namespace orc

/* ========================================================================= */
using namespace orc;

extern "C" {

int orc_transport_set_electrode(void*, int i_lsf);

void* orc_create(const afg_tree_desc* d, int n_var, int n_var_face) {
  // the transport state is process-wide: a new instance starts without the
  // electrode mask of an earlier one
  orc_transport_set_electrode(nullptr, 0);
  Oracle* o = new Oracle();
  Tree& t = o->t;
  t.D = d->ndim;
  t.nc = d->n_cell;
  t.coord = d->coord;
  t.n_boxes = d->n_boxes;
  t.highest_lvl = d->highest_lvl;
  t.n2 = t.nc + 2;
  t.S = t.D == 3 ? t.n2 * t.n2 * t.n2 : t.n2 * t.n2;
  t.NF = t.D == 3 ? (t.nc + 1) * (t.nc + 1) * (t.nc + 1) : (t.nc + 1) * (t.nc + 1);
  t.n_var = n_var;
  t.n_var_face = n_var_face;
  for (int k = 0; k < 3; k++) t.cgs[k] = d->coarse_grid_size[k];
  const size_t nb = d->n_boxes;
  t.lvl.assign(d->lvl, d->lvl + nb);
  t.ix.assign(d->ix, d->ix + nb * t.D);
  t.parent.assign(d->parent, d->parent + nb);
  t.children.assign(d->children, d->children + nb * t.nchild());
  t.neighbors.assign(d->neighbors, d->neighbors + nb * t.nnb());
  t.nbmat.assign(d->neighbor_mat, d->neighbor_mat + nb * t.nmat());
  t.r_min.assign(d->r_min, d->r_min + nb * t.D);
  t.dr.assign(d->dr, d->dr + nb * t.D);
  for (int l = 0; l < t.highest_lvl; l++) {
    t.ids.emplace_back(d->ids + d->ids_off[l], d->ids + d->ids_off[l + 1]);
    t.leaves.emplace_back(d->leaves + d->leaves_off[l], d->leaves + d->leaves_off[l + 1]);
    t.parents.emplace_back(d->parents + d->parents_off[l], d->parents + d->parents_off[l + 1]);
  }
  return o;
}

void orc_destroy(void* p) { delete static_cast<Oracle*>(p); }

int orc_set_num_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
}

int orc_set_cc_methods(void* p, int iv, const afg_gc_desc* g) {
  Oracle* o = static_cast<Oracle*>(p);
  GcSpec s;
  for (int n = 0; n < 6; n++) { s.bc_type[n] = g->bc_type[n]; s.bc_val[n] = g->bc_val[n]; }
  s.rb = g->rb;
  o->methods[iv] = s;
  return AFG_OK;
}

int orc_gc(void* p, double* cc, int iv, int lvl, int corners) {
  Oracle* o = static_cast<Oracle*>(p);
  auto it = o->methods.find(iv);
  if (it == o->methods.end()) return AFG_ERR_STATE;
  if (lvl <= 0) {
    for (int l = 1; l <= o->t.highest_lvl; l++) gc_lvl(o->t, cc, l, iv, it->second, corners != 0);
  } else {
    gc_lvl(o->t, cc, lvl, iv, it->second, corners != 0);
  }
  return AFG_OK;
}

int orc_mg_setup(void* p, int mg_id, const afg_mg_desc* d) {
  Oracle* o = static_cast<Oracle*>(p);
  Mg m;
  m.d = *d;
  int rc = build_coarse(*o, m);
  if (rc) return rc;
  o->mg[mg_id] = m;
  auto& g = o->methods[d->i_phi];
  g = m.gc();
  return AFG_OK;
}

int orc_mg_set_bc_values(void* p, int mg_id, const double* v) {
  Oracle* o = static_cast<Oracle*>(p);
  auto it = o->mg.find(mg_id);
  if (it == o->mg.end()) return AFG_ERR_STATE;
  for (int n = 0; n < 6; n++) it->second.d.bc_val[n] = v[n];
  o->methods[it->second.d.i_phi] = it->second.gc();
  return AFG_OK;
}

int orc_mg_coarse_inverse(void* p, int mg_id, double* out, int n_max) {
  Oracle* o = static_cast<Oracle*>(p);
  auto it = o->mg.find(mg_id);
  if (it == o->mg.end()) return AFG_ERR_STATE;
  const int n = it->second.n_coarse;
  if (out && (long)n * n <= (long)n_max) std::memcpy(out, it->second.ainv.data(), sizeof(double) * n * n);
  return n;
}

#define GET_MG                                   \
  Oracle* o = static_cast<Oracle*>(p);           \
  auto it = o->mg.find(mg_id);                   \
  if (it == o->mg.end()) return AFG_ERR_STATE;   \
  const Mg& m = it->second;

int orc_mg_gsrb_lvl(void* p, double* cc, int mg_id, int lvl, int type) {
  GET_MG
  gsrb_boxes(*o, cc, m, lvl, type);
  return AFG_OK;
}

int orc_mg_update_coarse(void* p, double* cc, int mg_id, int lvl) {
  GET_MG
  update_coarse(*o, cc, m, lvl);
  return AFG_OK;
}

int orc_mg_correct_lvl(void* p, double* cc, int mg_id, int lvl) {
  GET_MG
  correct_children(*o, cc, m, lvl - 1);
  gc_lvl(o->t, cc, lvl, m.d.i_phi, m.gc(), true);
  return AFG_OK;
}

int orc_mg_coarse_solve(void* p, double* cc, int mg_id) {
  GET_MG
  coarse_solve(*o, cc, m);
  return AFG_OK;
}

int orc_mg_residual(void* p, double* cc, int mg_id, int max_lvl) {
  GET_MG
  residual_lvls(*o, cc, m, max_lvl <= 0 ? o->t.highest_lvl : max_lvl);
  return AFG_OK;
}

int orc_mg_vcycle(void* p, double* cc, int mg_id, int set_residual, int max_lvl, double* max_res) {
  GET_MG
  vcycle(*o, cc, m, set_residual != 0, max_lvl <= 0 ? o->t.highest_lvl : max_lvl);
  if (set_residual && max_res) *max_res = maxabs(o->t, cc, m.d.i_tmp, true);
  return AFG_OK;
}

int orc_mg_fmg(void* p, double* cc, int mg_id, int set_residual, int have_guess, double* max_res) {
  GET_MG
  fmg(*o, cc, m, set_residual != 0, have_guess != 0);
  if (set_residual && max_res) *max_res = maxabs(o->t, cc, m.d.i_tmp, true);
  return AFG_OK;
}

int orc_mg_solve(void* p, double* cc, int mg_id, double threshold, int max_cycles, int* n_done,
                 double* residuals) {
  GET_MG
  int n = 0;
  for (n = 0; n < max_cycles; n++) {
    vcycle(*o, cc, m, true, o->t.highest_lvl);
    double r = maxabs(o->t, cc, m.d.i_tmp, true);
    if (residuals) residuals[n] = r;
    if (r < threshold) { n++; break; }
  }
  if (n_done) *n_done = n;
  return AFG_OK;
}

double orc_maxabs(void* p, const double* cc, int iv, int leaves_only) {
  Oracle* o = static_cast<Oracle*>(p);
  return maxabs(o->t, cc, iv, leaves_only != 0);
}

}  // extern "C"

/* ---- electrode (level set) -------------------------------------------- */
namespace orc {

/* get_conical_rod_properties (src/m_field.f90:406-428); the cone length
 * uses electrode 1's cone_length_frac for either electrode, as there */
static void conical_props(const double* r0, const double* r1, int D, double radius, double tip_radius,
                          double cone_frac, double* center, double& r_curv) {
  double h[3];
  for (int d = 0; d < D; d++) h[d] = r1[d] - r0[d];
  const double len = afg_lsf::norm2(h, D);
  const double angle = std::atan((radius - tip_radius) / (cone_frac * len));
  r_curv = tip_radius / std::cos(angle);
  for (int d = 0; d < D; d++) center[d] = r1[d] - std::sin(angle) * r_curv * (r1[d] - r0[d]) / len;
}

/* mg_lsf_boundary_value (m_coarse_solver.f90:494-511) per electrode cell
 * and bc_correction = f * value (mg_set_operators_lvl,
 * m_af_multigrid.f90:1169-1174) */
static void lsf_voltage(const Tree& t, Lsf& L, double voltage) {
  const int SI = L.SI, nc = t.nc, D = t.D;
  for (size_t q = 0; q < L.ids.size(); q++) {
    const int id = L.ids[q];
    for (int c = 0; c < SI; c++) {
      const int ix[3] = {c % nc + 1, (c / nc) % nc + 1, D == 3 ? c / (nc * nc) + 1 : 0};
      double r[3];
      for (int d = 0; d < D; d++) r[d] = t.rmin_of(id, d) + (ix[d] - 0.5) * t.dr_of(id, d);
      const double b = afg_lsf::boundary_value(L.e, r, voltage);
      L.bv[q * SI + c] = b;
      L.bcc[q * SI + c] = L.f[q * SI + c] * b;
    }
  }
}

}  // namespace orc

extern "C" {

/* tree%mg_i_lsf / mg%lsf for problem mg_id: set_lsf_box on every box
 * (src/m_field.f90:673-683), mg_set_box_tag + store_lsf_distance_matrix
 * (m_af_multigrid.f90:977-1145) and mg_box_lsf_stencil (1779-1853) for the
 * boxes with a boundary, the coarse matrix with their stencils
 * (coarse_solver_initialize); boundary value 0 */
int orc_mg_set_lsf(void* p, double* cc, int mg_id, const afg_lsf_desc* d) {
  Oracle* o = static_cast<Oracle*>(p);
  auto it = o->mg.find(mg_id);
  if (it == o->mg.end()) return AFG_ERR_STATE;
  Mg& m = it->second;
  const Tree& t = o->t;
  const int D = t.D, nc = t.nc;
  auto L = std::make_shared<Lsf>();
  afg_lsf::Electrode& e = L->e;
  e.shape = d->shape;
  e.D = D;
  e.cyl = t.coord == AFG_CYL;
  for (int k = 0; k < 3; k++) {
    e.r0[k] = d->r0[k], e.r1[k] = d->r1[k], e.q0[k] = d->r2_0[k], e.q1[k] = d->r2_1[k];
    e.center[k] = d->center[k];
  }
  e.radius = d->radius;
  e.radius2 = d->radius2;
  e.tip_radius = d->cone_tip_radius;
  e.cone_frac = d->cone_length_frac;
  e.tip_radius2 = d->cone2_tip_radius;
  e.cone_frac2 = d->cone2_length_frac;
  e.grounded = d->grounded;
  e.grounded2 = d->grounded2;
  e.length_scale = d->length_scale;
  e.safety = d->gradient_safety_factor;
  e.tol = d->tol;
  e.min_rel = d->min_rel_distance;
  if (e.shape == AFG_LSF_ROD_CONE_TOP || e.shape == AFG_LSF_TWO_ROD_CONE)
    conical_props(e.r0, e.r1, D, e.radius, e.tip_radius, e.cone_frac, e.tip_center, e.r_curv);
  if (e.shape == AFG_LSF_TWO_ROD_CONE)
    conical_props(e.q0, e.q1, D, e.radius2, e.tip_radius2, e.cone_frac, e.tip_center2, e.r_curv2);
  L->i_lsf = d->i_lsf;
  L->SI = D == 2 ? nc * nc : nc * nc * nc;
  const int SI = L->SI;
  L->q.assign(t.n_boxes, -1);
  for (int lvl = 1; lvl <= t.highest_lvl; lvl++) {
    for (int id : t.ids[lvl - 1]) {
      // set_lsf_box: all cells, ghost cells included
      double* a = t.var(cc, id, d->i_lsf);
      for (int x = 0; x < t.S; x++) {
        const int ix[3] = {x % t.n2, (x / t.n2) % t.n2, D == 3 ? x / (t.n2 * t.n2) : 0};
        double r[3];
        for (int dd = 0; dd < D; dd++) r[dd] = t.rmin_of(id, dd) + (ix[dd] - 0.5) * t.dr_of(id, dd);
        a[x] = afg_lsf::eval(e, r);
      }
      // distances of every interior cell; a box with one below 1 is an
      // electrode box
      double rm[3], h[3];
      for (int dd = 0; dd < D; dd++) rm[dd] = t.rmin_of(id, dd), h[dd] = t.dr_of(id, dd);
      std::vector<double> dist((size_t)2 * D * SI);
      bool any = false;
      for (int c = 0; c < SI; c++) {
        const int ix[3] = {c % nc + 1, (c / nc) % nc + 1, D == 3 ? c / (nc * nc) + 1 : 0};
        double dv[6];
        afg_lsf::cell_distances(e, rm, h, ix, dv);
        for (int n = 0; n < 2 * D; n++) {
          dist[(size_t)n * SI + c] = dv[n];
          any = any || dv[n] < 1.0;
        }
      }
      if (!any) continue;
      const int q = (int)L->ids.size();
      L->q[id - 1] = q;
      L->ids.push_back(id);
      L->dd.insert(L->dd.end(), dist.begin(), dist.end());
      std::vector<double> v((size_t)(2 * D + 1) * SI), f(SI);
      for (int c = 0; c < SI; c++) {
        double dv[6], w[7], fv;
        for (int n = 0; n < 2 * D; n++) dv[n] = dist[(size_t)n * SI + c];
        afg_lsf::cell_stencil(D, e.cyl != 0, rm, h, c % nc + 1, dv, w, fv);
        for (int n = 0; n <= 2 * D; n++) v[(size_t)n * SI + c] = w[n];
        f[c] = fv;
      }
      L->v.insert(L->v.end(), v.begin(), v.end());
      L->f.insert(L->f.end(), f.begin(), f.end());
    }
  }
  bool coarse_root = false;
  for (int id : t.ids[0]) coarse_root = coarse_root || L->q[id - 1] >= 0;
  if (!coarse_root) return AFG_ERR_ARG;  // check_coarse_representation_lsf
  L->bv.assign(L->ids.size() * SI, 0.0);
  L->bcc.assign(L->ids.size() * SI, 0.0);
  lsf_voltage(t, *L, 0.0);
  m.lsf = L;
  return build_coarse(*o, m);
}

int orc_mg_set_lsf_voltage(void* p, int mg_id, double voltage) {
  Oracle* o = static_cast<Oracle*>(p);
  auto it = o->mg.find(mg_id);
  if (it == o->mg.end() || !it->second.lsf) return AFG_ERR_STATE;
  lsf_voltage(o->t, *it->second.lsf, voltage);
  return AFG_OK;
}

int orc_mg_lsf_info(void* p, int mg_id, int* n_boxes, int* ids, double* v, double* f, double* bcc, double* dd) {
  Oracle* o = static_cast<Oracle*>(p);
  auto it = o->mg.find(mg_id);
  if (it == o->mg.end() || !it->second.lsf) return AFG_ERR_STATE;
  const Lsf& L = *it->second.lsf;
  const int n = (int)L.ids.size();
  if (n_boxes) *n_boxes = n;
  if (ids) std::memcpy(ids, L.ids.data(), sizeof(int) * n);
  if (v) std::memcpy(v, L.v.data(), sizeof(double) * L.v.size());
  if (f) std::memcpy(f, L.f.data(), sizeof(double) * L.f.size());
  if (bcc) std::memcpy(bcc, L.bcc.data(), sizeof(double) * L.bcc.size());
  if (dd) std::memcpy(dd, L.dd.data(), sizeof(double) * L.dd.size());
  return AFG_OK;
}

}  // extern "C"
