/*
 * oracle_transport.cpp -- CPU FP64 restatement of the drift-diffusion
 * transport step, the field computation and the photoionization source
 * (TEST INFRASTRUCTURE ONLY: the checker for the GPU path; see
 * oracle_common.h).
 *
 * Restated routines (reference file:line):
 *   af_restrict_ref_boundary   afivo/src/m_af_restrict.f90:140-161
 *   af_gc2_box, bc_to_gc2,     afivo/src/m_af_ghostcell.f90:672-744, 282-375,
 *   gc2_prolong_rb                                          753-856
 *   limiters                   afivo/src/m_af_limiters.f90:41-149
 *   flux_upwind_tree/_box      afivo/src/m_af_flux_schemes.f90:666-848
 *   reconstruct_upwind_1d      afivo/src/m_af_flux_schemes.f90:282-303
 *   flux_upwind, flux_direction src/m_fluid.f90:102-227
 *   af_consistent_fluxes       afivo/src/m_af_core.f90:1257-1402
 *   flux_update_densities      afivo/src/m_af_flux_schemes.f90:320-436
 *   add_source_terms           src/m_fluid.f90:298-466
 *   get_rates, get_derivatives src/m_chemistry.f90:672-804
 *   LT_get_loc / _col_at_loc   src/lookup_table_fortran/m_lookup_table.f90:330-406
 *   field_set_rhs              src/m_field.f90:406-444
 *   mg_box_lpl_gradient, mg_box_field_norm  afivo/src/m_af_multigrid.f90:1902-2045
 *   photoionization_rate_from_alpha  src/m_photoi.f90:259-291
 *   photoi_helmh_compute       src/m_photoi_helmh.f90:162-204
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <omp.h>

#include "oracle_common.h"
// exp and pow of the analytic rate forms: the project's own functions, so
// that the restatement and the GPU path evaluate them bit for bit alike (the
// reference calls its compiler's libm; the project's are within a few ulp)
#include "../afivo-streamer_gb300/csrc/afg_math.h"

namespace orc {

static const double SI_TO_TD = 1e21;
static const double EPS0 = 8.8541878128e-12;
static const double ELEM = 1.602176634e-19;

struct Transport {
  afg_transport_desc d;
  std::vector<double> lt;  // [n_cols][n_points]
};

static Transport g_tr;  // one transport model per process (test harness)

/* LT_get_loc + LT_get_col_at_loc (linear spacing) */
static inline void lt_loc(const afg_transport_desc& d, double x, int& ix, double& w) {
  const double frac = (x - d.lt_x_min) * d.lt_inv_fac;
  if (frac <= 0) {
    ix = 1;
    w = 1;
  } else if (frac >= d.lt_n_points - 1) {
    ix = d.lt_n_points - 1;
    w = 0;
  } else {
    ix = (int)std::ceil(frac);
    w = ix - frac;
  }
}
static inline double lt_col(const Transport& T, int col, int ix, double w) {
  const double* y = T.lt.data() + (size_t)col * T.d.lt_n_points;
  return w * y[ix - 1] + (1 - w) * y[ix];
}

/* af_limiter_koren (m_af_limiters.f90:72-95) */
static inline double koren(double a, double b) {
  const double third = 1 / 3.0;
  const double aa = a * a, ab = a * b;
  if (ab <= 0) return 0;
  if (aa <= 0.25 * ab) return 2 * a;
  if (aa <= 2.5 * ab) return third * (b + 2 * a);
  return 2 * b;
}

/* af_limiter_gminmod (m_af_limiters.f90:133-149) */
static inline double gminmod(double a, double b, double theta) {
  if (a * b > 0) {
    double m = std::fabs(theta * a);
    m = std::min(m, std::fabs(theta * b));
    m = std::min(m, std::fabs(0.5 * (a + b)));
    return std::copysign(m, a);
  }
  return 0.0;
}

static inline double limiter_apply(double a, double b, int lim) {
  switch (lim) {
    case AFG_LIMITER_KOREN: return koren(a, b);
    case AFG_LIMITER_MINMOD: return gminmod(a, b, 1.0);
    case AFG_LIMITER_MC: return gminmod(a, b, 2.0);
    case AFG_LIMITER_GMINMOD43: return gminmod(a, b, 4 / 3.0);
    default: {  // van Leer
      const double ab = a * b;
      return ab > 0 ? 2 * ab / (a + b) : 0;
    }
  }
}

/* enlarged box array with two ghost layers: index (i,j[,k]) in -1..nc+2 */
struct Big {
  int D, nc, m;  // m = nc+4
  std::vector<double> v;
  Big(int D_, int nc_) : D(D_), nc(nc_), m(nc_ + 4), v((size_t)std::pow(nc_ + 4.0, D_), 0.0) {}
  double& at(int i, int j, int k = 0) {
    return v[(i + 1) + m * ((j + 1) + (D == 3 ? m * (k + 1) : 0))];
  }
};

static inline int fc_at(const Tree& t, int i, int j, int k) {
  // 1-based face index in (nc+1)^D array
  const int m = t.nc + 1;
  return (i - 1) + m * ((j - 1) + (t.D == 3 ? m * (k - 1) : 0));
}
static inline double* fc_var(const Tree& t, double* fc, int id, int ivf, int dim) {
  return fc + (((size_t)(id - 1) * t.n_var_face + (ivf - 1)) * t.D + dim) * t.NF;
}

/* af_gc2_box for variable iv into Big b, then the first ghost layer copied
 * back to the box (m_af_ghostcell.f90:672-744) */
static void gc2_box(const Tree& t, double* cc, int id, int iv, const GcSpec& g, int limiter, Big& b) {
  const int nc = t.nc, D = t.D;
  double* a = t.var(cc, id, iv);
  const int kn = D == 3 ? nc + 1 : 0, k0 = D == 3 ? 0 : 0;
  for (int k = k0; k <= kn; k++)
    for (int j = 0; j <= nc + 1; j++)
      for (int i = 0; i <= nc + 1; i++) b.at(i, j, k) = a[t.at(i, j, k)];
  auto setf = [&](int d, int x, int p, int q, double v) {
    if (D == 2) {
      if (d == 0) b.at(x, p) = v; else b.at(p, x) = v;
    } else {
      if (d == 0) b.at(x, p, q) = v; else if (d == 1) b.at(p, x, q) = v; else b.at(p, q, x) = v;
    }
  };
  auto getb = [&](const double* src, int d, int x, int p, int q) {
    if (D == 2) return d == 0 ? src[t.at(x, p)] : src[t.at(p, x)];
    if (d == 0) return src[t.at(x, p, q)];
    if (d == 1) return src[t.at(p, x, q)];
    return src[t.at(p, q, x)];
  };
  const int qn = D == 3 ? nc : 1;
  for (int nb = 0; nb < 2 * D; nb++) {
    const int nb_id = t.nb_of(id, nb), d = nb / 2;
    const bool low = (nb % 2) == 0;
    if (nb_id > 0) {
      const double* s = t.var(cc, nb_id, iv);
      for (int q = 1; q <= qn; q++)
        for (int p = 1; p <= nc; p++) {
          if (low) {
            setf(d, -1, p, q, getb(s, d, nc - 1, p, q));
            setf(d, 0, p, q, getb(s, d, nc, p, q));
          } else {
            setf(d, nc + 1, p, q, getb(s, d, 1, p, q));
            setf(d, nc + 2, p, q, getb(s, d, 2, p, q));
          }
        }
    } else if (nb_id == 0) {
      /* gc2_prolong_rb (753-856) */
      const int p_id = t.parent[id - 1];
      const int p_nb = t.nb_of(p_id, nb);
      const double* C = t.var(cc, p_nb, iv);
      int off[3] = {0, 0, 0};
      for (int q = 0; q < D; q++) off[q] = t.child_offset(id, q);
      int lo[3], hi[3];
      for (int q = 0; q < D; q++) { lo[q] = 1; hi[q] = nc; }
      lo[d] = low ? -1 : nc + 1;
      hi[d] = low ? 0 : nc + 2;
      int lo_c[3], hi_c[3];
      for (int q = 0; q < D; q++) {
        lo_c[q] = off[q] + (lo[q] + 1) / 2;  // Fortran integer division truncates
        hi_c[q] = off[q] + (hi[q] + 1) / 2;
      }
      lo_c[d] -= (low ? -1 : 1) * nc;
      hi_c[d] -= (low ? -1 : 1) * nc;
      if (D == 2) {
        for (int j = lo_c[1]; j <= hi_c[1]; j++) {
          const int jf = lo[1] + 2 * (j - lo_c[1]);
          for (int i = lo_c[0]; i <= hi_c[0]; i++) {
            const int if_ = lo[0] + 2 * (i - lo_c[0]);
            const double f0 = C[t.at(i, j)];
            const double sa1 = C[t.at(i, j)] - C[t.at(i - 1, j)], sa2 = C[t.at(i, j)] - C[t.at(i, j - 1)];
            const double sb1 = C[t.at(i + 1, j)] - C[t.at(i, j)], sb2 = C[t.at(i, j + 1)] - C[t.at(i, j)];
            const double f1 = 0.25 * limiter_apply(sa1, sb1, limiter);
            const double f2 = 0.25 * limiter_apply(sa2, sb2, limiter);
            b.at(if_, jf) = f0 - f1 - f2;
            b.at(if_, jf + 1) = f0 - f1 + f2;
            b.at(if_ + 1, jf) = f0 + f1 - f2;
            b.at(if_ + 1, jf + 1) = f0 + f1 + f2;
          }
        }
      } else {
        for (int k = lo_c[2]; k <= hi_c[2]; k++) {
          const int kf = lo[2] + 2 * (k - lo_c[2]);
          for (int j = lo_c[1]; j <= hi_c[1]; j++) {
            const int jf = lo[1] + 2 * (j - lo_c[1]);
            for (int i = lo_c[0]; i <= hi_c[0]; i++) {
              const int if_ = lo[0] + 2 * (i - lo_c[0]);
              const double c0 = C[t.at(i, j, k)];
              const double f1 = 0.25 * limiter_apply(c0 - C[t.at(i - 1, j, k)], C[t.at(i + 1, j, k)] - c0, limiter);
              const double f2 = 0.25 * limiter_apply(c0 - C[t.at(i, j - 1, k)], C[t.at(i, j + 1, k)] - c0, limiter);
              const double f3 = 0.25 * limiter_apply(c0 - C[t.at(i, j, k - 1)], C[t.at(i, j, k + 1)] - c0, limiter);
              b.at(if_, jf, kf) = c0 - f1 - f2 - f3;
              b.at(if_, jf, kf + 1) = c0 - f1 - f2 + f3;
              b.at(if_, jf + 1, kf) = c0 - f1 + f2 - f3;
              b.at(if_, jf + 1, kf + 1) = c0 - f1 + f2 + f3;
              b.at(if_ + 1, jf, kf) = c0 + f1 - f2 - f3;
              b.at(if_ + 1, jf, kf + 1) = c0 + f1 - f2 + f3;
              b.at(if_ + 1, jf + 1, kf) = c0 + f1 + f2 - f3;
              b.at(if_ + 1, jf + 1, kf + 1) = c0 + f1 + f2 + f3;
            }
          }
        }
      }
    } else {
      /* bc_to_gc2 (282-375); the reference's 3D high-y second layer uses c0 */
      double c0, c1, c2;
      const double bv = g.bc_val[nb];
      switch (g.bc_type[nb]) {
        case AFG_BC_DIRICHLET: c0 = 2; c1 = -1; c2 = c0; break;
        case AFG_BC_NEUMANN: c0 = t.dr_of(id, d) * (low ? -1 : 1); c1 = 1; c2 = 3 * c0; break;
        default: c0 = 1; c1 = 0; c2 = c0; break;
      }
      if (D == 3 && nb == 3) c2 = c0;
      for (int q = 1; q <= qn; q++)
        for (int p = 1; p <= nc; p++) {
          if (low) {
            setf(d, 0, p, q, c0 * bv + c1 * getb(a, d, 1, p, q));
            setf(d, -1, p, q, c2 * bv + c1 * getb(a, d, 2, p, q));
          } else {
            setf(d, nc + 1, p, q, c0 * bv + c1 * getb(a, d, nc, p, q));
            setf(d, nc + 2, p, q, c2 * bv + c1 * getb(a, d, nc - 1, p, q));
          }
        }
    }
  }
  for (int k = k0; k <= kn; k++)
    for (int j = 0; j <= nc + 1; j++)
      for (int i = 0; i <= nc + 1; i++) a[t.at(i, j, k)] = b.at(i, j, k);
}

/* restriction with geometry (af_restrict_box default) of one variable */
static void restrict_box_geom(const Tree& t, double* cc, int id, int iv) {
  const int nc = t.nc, hnc = nc / 2;
  const int p_id = t.parent[id - 1];
  const double* c = t.var(cc, id, iv);
  double* pp = t.var(cc, p_id, iv);
  int off[3] = {0, 0, 0};
  for (int d = 0; d < t.D; d++) off[d] = t.child_offset(id, d);
  if (t.D == 2) {
    const bool cyl = t.coord == AFG_CYL;
    for (int j = 1; j <= hnc; j++)
      for (int i = 1; i <= hnc; i++) {
        const int ic = off[0] + i, jc = off[1] + j, if_ = 2 * i - 1, jf = 2 * j - 1;
        if (cyl) {
          const double r = t.rmin_of(p_id, 0) + (ic - 0.5) * t.dr_of(p_id, 0);
          const double tmp = 0.25 * t.dr_of(p_id, 0) / r;
          const double w1 = 1 - tmp, w2 = 1 + tmp;
          double s1 = 0, s2 = 0;
          s1 += c[t.at(if_, jf)]; s1 += c[t.at(if_, jf + 1)];
          s2 += c[t.at(if_ + 1, jf)]; s2 += c[t.at(if_ + 1, jf + 1)];
          pp[t.at(ic, jc)] = 0.25 * (w1 * s1 + w2 * s2);
        } else {
          double s = 0;
          s += c[t.at(if_, jf)]; s += c[t.at(if_ + 1, jf)];
          s += c[t.at(if_, jf + 1)]; s += c[t.at(if_ + 1, jf + 1)];
          pp[t.at(ic, jc)] = 0.25 * s;
        }
      }
  } else {
    for (int k = 1; k <= hnc; k++)
      for (int j = 1; j <= hnc; j++)
        for (int i = 1; i <= hnc; i++) {
          double s = 0;
          for (int dk = 0; dk < 2; dk++)
            for (int dj = 0; dj < 2; dj++)
              for (int di = 0; di < 2; di++) s += c[t.at(2 * i - 1 + di, 2 * j - 1 + dj, 2 * k - 1 + dk)];
          pp[t.at(off[0] + i, off[1] + j, off[2] + k)] = 0.125 * s;
        }
  }
}

/* flux_upwind_box (m_af_flux_schemes.f90:715-848) with flux_upwind
 * (m_fluid.f90:102-209); returns max cfl_sum and max sigma of the box */
static void flux_box(const Tree& t, double* cc, double* fc, const Transport& T, int id, int s_deriv,
                     double& max_cfl, double& max_sigma) {
  const afg_transport_desc& d = T.d;
  const int nc = t.nc, D = t.D, nf = d.n_flux;
  std::vector<Big> big;
  GcSpec g;
  for (int n = 0; n < 6; n++) { g.bc_type[n] = d.species_gc.bc_type[n]; g.bc_val[n] = d.species_gc.bc_val[n]; }
  g.rb = d.species_gc.rb;
  for (int f = 0; f < nf; f++) {
    big.emplace_back(D, nc);
    gc2_box(t, cc, id, d.species_iv[d.flux_species[f]] + s_deriv, g, d.prolong_limiter, big.back());
  }
  const int ncd = D == 3 ? nc * nc * nc : nc * nc;
  std::vector<double> cfl_sum(ncd, 0.0);
  const double N_inv = 1 / d.gas_number_density;
  const double* E = t.var(cc, id, d.i_electric_fld);
  const double* ne = t.var(cc, id, d.species_iv[d.flux_species[0]] + s_deriv);
  const int jn = nc, kn = D == 3 ? nc : 1;
  std::vector<double> u(nc + 2), v(nc + 2), dcf(nc + 2), Ex(nc + 2), mu(nc + 2), sigma(nc + 2), flux(nc + 2);
  std::vector<double> line(nc + 4), Ec(nc + 2), nel(nc + 2);
  for (int dim = 0; dim < D; dim++) {
    const double inv_dx = 1 / t.dr_of(id, dim);
    for (int kk = 1; kk <= kn; kk++)
      for (int jj = 1; jj <= jn; jj++) {
        // line through (jj, kk) in the other dimensions
        auto cell = [&](int x) -> int {
          if (D == 2) return dim == 0 ? t.at(x, jj) : t.at(jj, x);
          if (dim == 0) return t.at(x, jj, kk);
          if (dim == 1) return t.at(jj, x, kk);
          return t.at(jj, kk, x);
        };
        auto face = [&](int f) -> int {
          if (D == 2) return dim == 0 ? fc_at(t, f, jj, 1) : fc_at(t, jj, f, 1);
          if (dim == 0) return fc_at(t, f, jj, kk);
          if (dim == 1) return fc_at(t, jj, f, kk);
          return fc_at(t, jj, kk, f);
        };
        const double* efc = fc_var(t, fc, id, d.i_efield_fc, dim);
        for (int f = 1; f <= nc + 1; f++) Ex[f] = efc[face(f)];
        for (int x = 0; x <= nc + 1; x++) {
          Ec[x] = E[cell(x)];
          nel[x] = ne[cell(x)];
        }
        // transport coefficients at faces
        for (int f = 1; f <= nc + 1; f++) {
          const double td = 0.5 * (Ec[f - 1] + Ec[f]) * SI_TO_TD * N_inv;
          int ix; double w;
          lt_loc(d, td, ix, w);
          mu[f] = lt_col(T, d.lt_col_mobility, ix, w) * N_inv;
          dcf[f] = lt_col(T, d.lt_col_diffusion, ix, w) * N_inv;
          v[f] = -mu[f] * Ex[f];
        }
        for (int s = 0; s < nf; s++) {
          Big& b = big[s];
          for (int x = -1; x <= nc + 2; x++) {
            if (D == 2) line[x + 1] = dim == 0 ? b.at(x, jj) : b.at(jj, x);
            else if (dim == 0) line[x + 1] = b.at(x, jj, kk);
            else if (dim == 1) line[x + 1] = b.at(jj, x, kk);
            else line[x + 1] = b.at(jj, kk, x);
          }
          auto L = [&](int x) { return line[x + 1]; };
          for (int f = 1; f <= nc + 1; f++) {
            const bool pos = d.flux_charge_sign[s] * Ex[f] > 0;
            if (pos)
              u[f] = L(f - 1) + 0.5 * koren(L(f) - L(f - 1), L(f - 1) - L(f - 2));
            else
              u[f] = L(f) - 0.5 * koren(L(f) - L(f - 1), L(f + 1) - L(f));
          }
          if (s == 0) {
            for (int f = 1; f <= nc + 1; f++) {
              flux[f] = v[f] * u[f] - dcf[f] * inv_dx * (nel[f] - nel[f - 1]);
              sigma[f] = mu[f] * u[f];
            }
            for (int c = 1; c <= nc; c++) {
              const double cs = 1.0 * std::max(std::fabs(v[c + 1]), std::fabs(v[c])) * inv_dx +
                                2 * std::max(dcf[c + 1], dcf[c]) * (inv_dx * inv_dx);
              int lin;
              if (D == 2) lin = dim == 0 ? (c - 1) + nc * (jj - 1) : (jj - 1) + nc * (c - 1);
              else if (dim == 0) lin = (c - 1) + nc * ((jj - 1) + nc * (kk - 1));
              else if (dim == 1) lin = (jj - 1) + nc * ((c - 1) + nc * (kk - 1));
              else lin = (jj - 1) + nc * ((kk - 1) + nc * (c - 1));
              cfl_sum[lin] = cfl_sum[lin] + cs;
            }
          } else {
            const double mui = d.ion_mobility_N[s] * N_inv;
            for (int f = 1; f <= nc + 1; f++) {
              const double vi = d.flux_charge_sign[s] * mui * Ex[f];
              flux[f] = vi * u[f];
              sigma[f] = sigma[f] + mui * u[f];
            }
          }
          double* out = fc_var(t, fc, id, d.flux_fc[s], dim);
          for (int f = 1; f <= nc + 1; f++) out[face(f)] = flux[f];
        }
        for (int f = 1; f <= nc + 1; f++) max_sigma = std::max(max_sigma, sigma[f]);
      }
  }
  for (double c : cfl_sum) max_cfl = std::max(max_cfl, c);
}

/* flux_from_children (m_af_core.f90:1286-1402) */
static void flux_from_children(const Tree& t, double* fc, int id, int nb, int ivf) {
  const int nc = t.nc, nch = nc / 2, D = t.D, d = nb / 2;
  const bool low = (nb % 2) == 0;
  const int nb_id = t.nb_of(id, nb);
  const int i = low ? 1 : nc + 1, i_nb = low ? nc + 1 : 1;
  for (int c = 0; c < t.nchild(); c++) {
    // children adjacent to the face: child index bit d equals high side
    if (((c >> d) & 1) != (low ? 0 : 1)) continue;
    const int c_id = t.child_of(id, c);
    int ioff[3] = {nch * (c & 1), nch * ((c >> 1) & 1), nch * ((c >> 2) & 1)};
    const double* F = fc_var(t, fc, c_id, ivf, d);
    double* G = fc_var(t, fc, nb_id, ivf, d);
    if (D == 2) {
      const int o = d == 0 ? ioff[1] : ioff[0];
      for (int n = 1; n <= nch; n++) {
        double val;
        if (d == 0) {
          val = 0.5 * (F[fc_at(t, i, 2 * n - 1, 1)] + F[fc_at(t, i, 2 * n, 1)]);
          G[fc_at(t, i_nb, o + n, 1)] = val;
        } else if (t.coord == AFG_CYL) {
          const double r = t.rmin_of(nb_id, 0) + ((o + n) - 0.5) * t.dr_of(nb_id, 0);
          const double tmp = 0.25 * t.dr_of(nb_id, 0) / r;
          const double w1 = 1 - tmp, w2 = 1 + tmp;
          val = 0.5 * (w1 * F[fc_at(t, 2 * n - 1, i, 1)] + w2 * F[fc_at(t, 2 * n, i, 1)]);
          G[fc_at(t, o + n, i_nb, 1)] = val;
        } else {
          val = 0.5 * (F[fc_at(t, 2 * n - 1, i, 1)] + F[fc_at(t, 2 * n, i, 1)]);
          G[fc_at(t, o + n, i_nb, 1)] = val;
        }
      }
    } else {
      const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
      for (int q = 1; q <= nch; q++)
        for (int p = 1; p <= nch; p++) {
          auto FA = [&](int x, int pp, int qq) {
            if (d == 0) return fc_at(t, x, pp, qq);
            if (d == 1) return fc_at(t, pp, x, qq);
            return fc_at(t, pp, qq, x);
          };
          const double val = 0.25 * (F[FA(i, 2 * p - 1, 2 * q - 1)] + F[FA(i, 2 * p, 2 * q - 1)] +
                                     F[FA(i, 2 * p - 1, 2 * q)] + F[FA(i, 2 * p, 2 * q)]);
          G[FA(i_nb, ioff[t1] + p, ioff[t2] + q)] = val;
        }
    }
  }
}

/* get_rates for one cell (src/m_chemistry.f90:672-769) */
static double rate_of(const Transport& T, const afg_reaction& r, double td, int ix, double w) {
  const double c0 = r.rate_factor;
  const double* c = r.c;
  switch (r.rate_type) {
    case AFG_RATE_TABULATED_FIELD: return c0 * lt_col(T, r.lt_col, ix, w);
    case AFG_RATE_CONSTANT: return c0 * c[0];
    case AFG_RATE_LINEAR: return c0 * c[0] * (td - c[1]);
    case AFG_RATE_EXP_V1: { double q = c[1] / (c[2] + td); return c0 * c[0] * afg_math::exp(-(q * q)); }
    case AFG_RATE_EXP_V2: { double q = td / c[1]; return c0 * c[0] * afg_math::exp(-(q * q)); }
    case AFG_RATE_K13: return c0 * c[0] * afg_math::exp(-afg_math::pow(c[1] / (c[2] + td), c[3]));
    case AFG_RATE_K14: return c0 * c[0] * afg_math::exp(-afg_math::pow(td / c[1], c[2]));
    case AFG_RATE_K1: {
      /* rate_analytic_k1: Te = electron_eV_to_K * LT(td_energy_eV, Td) */
      const double Te = (2 * ELEM / (3 * 1.380649e-23)) * lt_col(T, r.lt_col, ix, w);
      return c0 * c[0] * afg_math::pow(300 / Te, c[1]);
    }
  }
  return 0;
}

}  // namespace orc

using namespace orc;

extern "C" {

int orc_transport_setup(void* p, const afg_transport_desc* d) {
  (void)p;
  g_tr.d = *d;
  g_tr.lt.assign(d->lt_data, d->lt_data + (size_t)d->lt_n_cols * d->lt_n_points);
  g_tr.d.lt_data = nullptr;
  return AFG_OK;
}

/* flux_upwind_tree (m_af_flux_schemes.f90:666-712) */
int orc_flux_upwind(void* p, double* cc, double* fc, int s_deriv, double* dt_lim) {
  Oracle* o = static_cast<Oracle*>(p);
  const Tree& t = o->t;
  const afg_transport_desc& d = g_tr.d;
  // af_restrict_ref_boundary on the flux variables of state s_deriv
  for (int lvl = 1; lvl <= t.highest_lvl; lvl++) {
    const std::vector<int>& lv = t.leaves[lvl - 1];
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < lv.size(); i++) {
      const int id = lv[i];
      if (t.parent[id - 1] <= 0) continue;
      bool rb = false;
      for (int nb = 0; nb < t.nnb(); nb++) rb = rb || t.nb_of(id, nb) == 0;
      if (!rb) continue;
      for (int f = 0; f < d.n_flux; f++) restrict_box_geom(t, cc, id, d.species_iv[d.flux_species[f]] + s_deriv);
    }
  }
  double max_cfl = 0, max_sigma = 0;
  for (int lvl = 1; lvl <= t.highest_lvl; lvl++) {
    const std::vector<int>& lv = t.leaves[lvl - 1];
#pragma omp parallel for schedule(static) reduction(max : max_cfl, max_sigma)
    for (size_t i = 0; i < lv.size(); i++) flux_box(t, cc, fc, g_tr, lv[i], s_deriv, max_cfl, max_sigma);
  }
  // af_consistent_fluxes
  for (int lvl = 1; lvl <= t.highest_lvl - 1; lvl++) {
    const std::vector<int>& par = t.parents[lvl - 1];
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < par.size(); i++) {
      const int id = par[i];
      for (int nb = 0; nb < t.nnb(); nb++) {
        const int nb_id = t.nb_of(id, nb);
        if (nb_id <= 0) continue;
        bool has_children = false;
        for (int c = 0; c < t.nchild(); c++) has_children = has_children || t.child_of(nb_id, c) > 0;
        if (has_children) continue;
        for (int f = 0; f < d.n_flux; f++) flux_from_children(t, fc, id, nb, d.flux_fc[f]);
      }
    }
  }
  dt_lim[0] = 1 / max_cfl;
  dt_lim[1] = EPS0 / (ELEM * std::max(max_sigma, 1e-100));
  return AFG_OK;
}

/* flux_update_densities + add_source_terms */
/* the electrode's level-set variable for set_box_mask (0: none) */
static int g_mask_iv = 0;

int orc_transport_set_electrode(void*, int i_lsf) {
  g_mask_iv = i_lsf;
  return AFG_OK;
}

int orc_update_densities(void* p, double* cc, double* fc, double dt, int s_deriv, int n_prev, const int* s_prev,
                         const double* w_prev, int s_out, int last_step, double* dt_chem) {
  Oracle* o = static_cast<Oracle*>(p);
  const Tree& t = o->t;
  const afg_transport_desc& d = g_tr.d;
  const int nc = t.nc, D = t.D, ns = d.n_species;
  double chem = 1e100;
  for (int lvl = 1; lvl <= t.highest_lvl; lvl++) {
    const std::vector<int>& lv = t.leaves[lvl - 1];
#pragma omp parallel for schedule(static) reduction(min : chem)
    for (size_t bi = 0; bi < lv.size(); bi++) {
      const int id = lv[bi];
      /* set_box_mask (src/m_fluid.f90:469-515): gas cells have lsf > 0;
       * add_source_terms returns at once for a box without any (332) */
      const double* lsf = g_mask_iv > 0 ? t.var(cc, id, g_mask_iv) : nullptr;
      auto gas = [&](int x) { return lsf == nullptr || lsf[x] > 0.0; };
      bool any_gas = false;
      for (int k = (D == 3 ? 1 : 0); k <= (D == 3 ? nc : 0); k++)
        for (int j = 1; j <= nc; j++)
          for (int i = 1; i <= nc; i++) any_gas = any_gas || gas(t.at(i, j, k));
      double dt_dr[3];
      for (int q = 0; q < D; q++) dt_dr[q] = dt / t.dr_of(id, q);
      // weighted sum of previous states
      for (int s = 0; s < ns; s++) {
        const int iv = d.species_iv[s];
        double* out = t.var(cc, id, iv + s_out);
        for (int k = (D == 3 ? 1 : 0); k <= (D == 3 ? nc : 0); k++)
          for (int j = 1; j <= nc; j++)
            for (int i = 1; i <= nc; i++) {
              const int x = t.at(i, j, k);
              double tmp = 0.0;
              for (int m = 0; m < n_prev; m++) tmp = tmp + w_prev[m] * t.var(cc, id, iv + s_prev[m])[x];
              out[x] = tmp;
            }
      }
      // sources
      const double Ninv = 1 / d.gas_number_density;
      const double* E = t.var(cc, id, d.i_electric_fld);
      const double* ph = d.i_photo > 0 ? t.var(cc, id, d.i_photo) : nullptr;
      double my_chem = 1e100;
      for (int k = (D == 3 ? 1 : 0); k <= (D == 3 ? nc : 0); k++)
        for (int j = 1; j <= nc; j++)
          for (int i = 1; i <= nc; i++) {
            const int x = t.at(i, j, k);
            const double td = SI_TO_TD * Ninv * E[x];
            double dens[AFG_MAX_SPECIES], der[AFG_MAX_SPECIES];
            for (int s = 0; s < ns; s++) {
              dens[s] = std::max(t.var(cc, id, d.species_iv[s] + s_deriv)[x], 0.0);
              der[s] = 0.0;
            }
            int ix; double w;
            lt_loc(d, td, ix, w);
            for (int n = 0; n < d.n_reactions; n++) {
              const afg_reaction& r = d.reactions[n];
              double rate = rate_of(g_tr, r, td, ix, w);
              double prod = 1.0;
              for (int q = 0; q < r.n_in; q++) prod = prod * dens[r.ix_in[q]];
              rate = rate * prod;
              for (int q = 0; q < r.n_in; q++) der[r.ix_in[q]] = der[r.ix_in[q]] - rate;
              for (int q = 0; q < r.n_out; q++) der[r.ix_out[q]] = der[r.ix_out[q]] + rate * r.mult_out[q];
            }
            if (!any_gas) continue;
            if (last_step) {
              const double eps = 1e-100;
              double tmp = 1e100;
              if (d.dt_chemistry_nmin > 0) {
                for (int s = 0; s < ns; s++)
                  tmp = std::min(tmp, (dens[s] + d.dt_chemistry_nmin) / std::max(std::fabs(der[s]), eps));
              } else if (d.dt_chemistry_limit_loss) {
                for (int s = 0; s < ns; s++) tmp = std::min(tmp, std::max(dens[s], eps) / std::max(-der[s], eps));
              }
              my_chem = std::min(my_chem, tmp);
            }
            if (ph) {
              der[d.flux_species[0]] = der[d.flux_species[0]] + ph[x];
              der[d.photoi_species] = der[d.photoi_species] + ph[x];
            }
            if (!gas(x)) continue;
            for (int s = 0; s < ns; s++) {
              double* out = t.var(cc, id, d.species_iv[s] + s_out);
              out[x] = out[x] + dt * der[s];
            }
          }
      chem = std::min(chem, my_chem);
      // flux divergence
      for (int f = 0; f < d.n_flux; f++) {
        double* out = t.var(cc, id, d.species_iv[d.flux_species[f]] + s_out);
        const double* F0 = fc_var(t, fc, id, d.flux_fc[f], 0);
        const double* F1 = fc_var(t, fc, id, d.flux_fc[f], 1);
        const double* F2 = D == 3 ? fc_var(t, fc, id, d.flux_fc[f], 2) : nullptr;
        for (int k = (D == 3 ? 1 : 0); k <= (D == 3 ? nc : 0); k++)
          for (int j = 1; j <= nc; j++)
            for (int i = 1; i <= nc; i++) {
              const int x = t.at(i, j, k);
              const int kk = D == 3 ? k : 1;
              if (!gas(x)) continue;
              if (D == 2 && t.coord == AFG_CYL) {
                const double r = t.rmin_of(id, 0) + (i - 0.5) * t.dr_of(id, 0);
                const double inv_r = 1 / r;
                const double f1 = (r - 0.5 * t.dr_of(id, 0)) * inv_r, f2 = (r + 0.5 * t.dr_of(id, 0)) * inv_r;
                out[x] = out[x] + dt_dr[0] * (f1 * F0[fc_at(t, i, j, 1)] - f2 * F0[fc_at(t, i + 1, j, 1)]) +
                         dt_dr[1] * (F1[fc_at(t, i, j, 1)] - F1[fc_at(t, i, j + 1, 1)]);
              } else if (D == 2) {
                out[x] = out[x] + dt_dr[0] * (F0[fc_at(t, i, j, 1)] - F0[fc_at(t, i + 1, j, 1)]) +
                         dt_dr[1] * (F1[fc_at(t, i, j, 1)] - F1[fc_at(t, i, j + 1, 1)]);
              } else {
                out[x] = out[x] + dt_dr[0] * (F0[fc_at(t, i, j, kk)] - F0[fc_at(t, i + 1, j, kk)]) +
                         dt_dr[1] * (F1[fc_at(t, i, j, kk)] - F1[fc_at(t, i, j + 1, kk)]) +
                         dt_dr[2] * (F2[fc_at(t, i, j, kk)] - F2[fc_at(t, i, j, kk + 1)]);
              }
            }
      }
    }
  }
  if (dt_chem) *dt_chem = chem;
  return AFG_OK;
}

/* field_set_rhs (src/m_field.f90:406-444) */
int orc_field_set_rhs(void* p, double* cc, int i_rhs, int s_in) {
  Oracle* o = static_cast<Oracle*>(p);
  const Tree& t = o->t;
  const afg_transport_desc& d = g_tr.d;
  const double fac = -ELEM / EPS0;
  for (int lvl = 1; lvl <= t.highest_lvl; lvl++) {
    const std::vector<int>& lv = t.leaves[lvl - 1];
#pragma omp parallel for schedule(static)
    for (size_t bi = 0; bi < lv.size(); bi++) {
      const int id = lv[bi];
      double* f = t.var(cc, id, i_rhs);
      for (int x = 0; x < t.S; x++) f[x] = 0.0;
      for (int s = 0; s < d.n_species; s++) {
        if (d.species_charge[s] == 0) continue;
        const double q = d.species_charge[s] * fac;
        const double* n = t.var(cc, id, d.species_iv[s] + s_in);
        for (int x = 0; x < t.S; x++) f[x] = f[x] + q * n[x];
      }
    }
  }
  return AFG_OK;
}

/* mg_compute_phi_gradient(fac=-1) + mg_box_field_norm on all boxes, then
 * af_gc_tree of |E| (field_from_potential, src/m_field.f90:531-548) */
int orc_field_from_potential(void* p, double* cc, double* fc, int i_phi) {
  Oracle* o = static_cast<Oracle*>(p);
  const Tree& t = o->t;
  const afg_transport_desc& d = g_tr.d;
  const int nc = t.nc, D = t.D;
  // the electrode of the field whose potential this is
  const Lsf* L = nullptr;
  for (const auto& kv : o->mg)
    if (kv.second.lsf && kv.second.d.i_phi == i_phi) L = kv.second.lsf.get();
  for (int lvl = 1; lvl <= t.highest_lvl; lvl++) {
    const std::vector<int>& ids = t.ids[lvl - 1];
#pragma omp parallel for schedule(static)
    for (size_t bi = 0; bi < ids.size(); bi++) {
      const int id = ids[bi];
      const double* ph = t.var(cc, id, i_phi);
      double inv_dr[3];
      for (int q = 0; q < D; q++) inv_dr[q] = -1.0 / t.dr_of(id, q);
      double* F[3];
      for (int q = 0; q < D; q++) F[q] = fc_var(t, fc, id, d.i_efield_fc, q);
      const int kn = D == 3 ? nc : 1;
      for (int k = 1; k <= kn; k++)
        for (int j = 1; j <= nc; j++)
          for (int i = 1; i <= nc + 1; i++) {
            const int kc = D == 3 ? k : 0;
            F[0][fc_at(t, i, j, k)] = inv_dr[0] * (ph[t.at(i, j, kc)] - ph[t.at(i - 1, j, kc)]);
            F[1][fc_at(t, j, i, k)] = inv_dr[1] * (ph[t.at(j, i, kc)] - ph[t.at(j, i - 1, kc)]);
            if (D == 3) F[2][fc_at(t, j, k, i)] = inv_dr[2] * (ph[t.at(j, k, i)] - ph[t.at(j, k, i - 1)]);
          }
      // mg_box_lpllsf_gradient (m_af_multigrid.f90:2049-2141) on electrode
      // boxes without children: faces next to a boundary point from cells
      // with lsf >= 0, in the order of the stored cells
      bool has_children = false;
      for (int c = 0; c < t.nchild(); c++) has_children = has_children || t.child_of(id, c) > 0;
      if (L && L->of(id) >= 0 && !has_children) {
        const int q = L->of(id), SI = L->SI;
        const double* dd = L->dd.data() + (size_t)q * 2 * D * SI;
        const double* bv = L->bv.data() + (size_t)q * SI;
        const double* ls = t.var(cc, id, L->i_lsf);
        for (int c = 0; c < SI; c++) {
          bool any = false;
          for (int n = 0; n < 2 * D; n++) any = any || dd[(size_t)n * SI + c] < 1.0;
          if (!any) continue;
          const int i = c % nc + 1, j = (c / nc) % nc + 1, k = D == 3 ? c / (nc * nc) + 1 : 0;
          const int kk = D == 3 ? k : 1;
          const int x = t.at(i, j, k);
          for (int n = 0; n < 2 * D; n++) {
            const double dn = dd[(size_t)n * SI + c];
            if (!(dn < 1 && ls[x] >= 0)) continue;
            const int dim = n / 2;
            const bool hi = n % 2;
            int fi = i, fj = j, fk = kk;
            if (hi) (dim == 0 ? fi : dim == 1 ? fj : fk) += 1;
            F[dim][fc_at(t, fi, fj, fk)] = hi ? inv_dr[dim] * (bv[c] - ph[x]) / dn : inv_dr[dim] * (ph[x] - bv[c]) / dn;
          }
        }
      }
      double* en = t.var(cc, id, d.i_electric_fld);
      for (int k = 1; k <= kn; k++)
        for (int j = 1; j <= nc; j++)
          for (int i = 1; i <= nc; i++) {
            const int kk = D == 3 ? k : 1;
            const double a = F[0][fc_at(t, i, j, kk)] + F[0][fc_at(t, i + 1, j, kk)];
            const double b = F[1][fc_at(t, i, j, kk)] + F[1][fc_at(t, i, j + 1, kk)];
            double s = a * a + b * b;
            if (D == 3) {
              const double c = F[2][fc_at(t, i, j, kk)] + F[2][fc_at(t, i, j, kk + 1)];
              s = s + c * c;
            }
            en[t.at(i, j, D == 3 ? k : 0)] = 0.5 * std::sqrt(s);
          }
    }
  }
  auto it = o->methods.find(d.i_electric_fld);
  if (it == o->methods.end()) return AFG_ERR_STATE;
  for (int l = 1; l <= t.highest_lvl; l++) gc_lvl(t, cc, l, d.i_electric_fld, it->second, true);
  return AFG_OK;
}

/* photoionization_rate_from_alpha (src/m_photoi.f90:259-291) */
int orc_photoi_source(void* p, double* cc, double coeff, int i_rhs) {
  Oracle* o = static_cast<Oracle*>(p);
  const Tree& t = o->t;
  const afg_transport_desc& d = g_tr.d;
  const int nc = t.nc, D = t.D;
  for (int lvl = 1; lvl <= t.highest_lvl; lvl++) {
    const std::vector<int>& lv = t.leaves[lvl - 1];
#pragma omp parallel for schedule(static)
    for (size_t bi = 0; bi < lv.size(); bi++) {
      const int id = lv[bi];
      const double* E = t.var(cc, id, d.i_electric_fld);
      const double* ne = t.var(cc, id, d.species_iv[d.flux_species[0]]);
      double* f = t.var(cc, id, i_rhs);
      for (int k = (D == 3 ? 1 : 0); k <= (D == 3 ? nc : 0); k++)
        for (int j = 1; j <= nc; j++)
          for (int i = 1; i <= nc; i++) {
            const int x = t.at(i, j, k);
            const double fld = E[x];
            const double td = fld * SI_TO_TD / d.gas_number_density;
            int ix; double w;
            lt_loc(d, td, ix, w);
            const double alpha = lt_col(g_tr, d.lt_col_alpha, ix, w);
            const double mob = lt_col(g_tr, d.lt_col_mobility, ix, w);
            double tmp = fld * mob * alpha * ne[x] * coeff;
            if (tmp < 0) tmp = 0;
            f[x] = tmp;
          }
    }
  }
  return AFG_OK;
}


/* default_refinement (src/m_refine.f90:197-298) for one box: cell flags,
 * i fastest; constant gas density, no electrode boxes. */
static void default_refinement(const Tree& t, const double* cc, int id, const afg_refine_desc& a,
                               std::vector<int>& cf, const Lsf* L = nullptr) {
  const int nc = t.nc, D = t.D;
  const double* E = t.var(const_cast<double*>(cc), id, a.i_electric_fld);
  const double* ne = t.var(const_cast<double*>(cc), id, a.i_electron);
  double max_dx = t.dr_of(id, 0), min_dx = t.dr_of(id, 0);
  for (int d = 1; d < D; d++) {
    max_dx = std::max(max_dx, t.dr_of(id, d));
    min_dx = std::min(min_dx, t.dr_of(id, d));
  }
  const int kn = D == 3 ? nc : 1;
  cf.assign((size_t)nc * nc * kn, AFG_REF_KEEP);
  for (int k = 1; k <= kn; k++)
    for (int j = 1; j <= nc; j++)
      for (int i = 1; i <= nc; i++) {
        const int x = D == 3 ? t.at(i, j, k) : t.at(i, j);
        const double gas_dens = a.gas_number_density;
        const double fld = E[x] * SI_TO_TD / gas_dens;
        int ix;
        double w;
        lt_loc(g_tr.d, a.adx_fac * fld, ix, w);
        double alpha;
        if (a.use_alpha_effective) {
          alpha = (lt_col(g_tr, a.lt_col_alpha, ix, w) - lt_col(g_tr, a.lt_col_eta, ix, w)) * gas_dens / a.adx_fac;
          alpha = std::max(0.0, alpha);
        } else {
          alpha = lt_col(g_tr, a.lt_col_alpha, ix, w) * gas_dens / a.adx_fac;
        }
        const double adx = max_dx * alpha;
        int f;
        if (adx > a.adx && ne[x] > a.min_dens)
          f = AFG_REF_DO;
        else if (adx < 0.125 * a.adx && max_dx < a.derefine_dx)
          f = AFG_REF_RM;
        else
          f = AFG_REF_KEEP;
        /* GM_dist_line (src/m_geometry.f90:23-51) from the cell centre */
        const int cix[3] = {i, j, k};
        double rc[3];
        for (int d = 0; d < D; d++) rc[d] = t.rmin_of(id, d) + (cix[d] - 0.5) * t.dr_of(id, d);
        for (int n = 0; n < a.n_seeds; n++) {
          double len2 = 0, frac = 0;
          for (int d = 0; d < D; d++) {
            len2 = len2 + (a.seed_r1[n][d] - a.seed_r0[n][d]) * (a.seed_r1[n][d] - a.seed_r0[n][d]);
            frac = frac + (rc[d] - a.seed_r0[n][d]) * (a.seed_r1[n][d] - a.seed_r0[n][d]);
          }
          double s2 = 0;
          for (int d = 0; d < D; d++) {
            double dv;
            if (frac <= 0)
              dv = rc[d] - a.seed_r0[n][d];
            else if (frac >= len2)
              dv = rc[d] - a.seed_r1[n][d];
            else
              dv = rc[d] - (a.seed_r0[n][d] + frac / len2 * (a.seed_r1[n][d] - a.seed_r0[n][d]));
            s2 = s2 + dv * dv;
          }
          const double dist = std::sqrt(s2);
          if (dist - a.seed_width[n] < 2 * max_dx && max_dx > a.init_fac * a.seed_width[n]) f = AFG_REF_DO;
        }
        /* refine around the electrode (src/m_refine.f90:261-265): boxes with
         * the mg_lsf_box tag of the field */
        if (L && L->of(id) >= 0 && a.electrode_dx > 0 && max_dx > a.electrode_dx) f = AFG_REF_DO;
        cf[(size_t)(i - 1) + nc * ((j - 1) + (size_t)nc * (k - 1))] = f;
      }
  double rmin[3], rmax[3];
  for (int d = 0; d < D; d++) {
    rmin[d] = t.rmin_of(id, d);
    rmax[d] = t.rmin_of(id, d) + t.dr_of(id, d) * nc;
  }
  const int hc = nc / 2;
  const size_t centre = (size_t)(hc - 1) + nc * ((hc - 1) + (size_t)nc * (D == 3 ? hc - 1 : 0));
  for (int n = 0; n < a.n_regions; n++) {
    bool all = max_dx > a.region_dr[n];
    for (int d = 0; d < D; d++) all = all && rmax[d] >= a.region_rmin[n][d] && rmin[d] <= a.region_rmax[n][d];
    if (all) cf[centre] = AFG_REF_DO;
  }
  for (int n = 0; n < a.n_limits; n++) {
    bool all = max_dx < 2 * a.limit_dr[n];
    for (int d = 0; d < D; d++) all = all && rmin[d] >= a.limit_rmin[n][d] && rmax[d] <= a.limit_rmax[n][d];
    if (all)
      for (auto& f : cf)
        if (f == AFG_REF_DO) f = AFG_REF_KEEP;
  }
  if (max_dx > a.max_dx) {
    for (auto& f : cf) f = AFG_REF_DO;
  } else if (min_dx < 2 * a.min_dx) {
    for (auto& f : cf)
      if (f == AFG_REF_DO) f = AFG_REF_KEEP;
  }
}

/* cell_to_ref_flags (afivo/src/m_af_core.f90:1095-1149) */
static void cell_to_ref_flags(const Tree& t, const std::vector<int>& cf, int id, int buf, std::vector<int>& rf) {
  const int nc = t.nc, D = t.D, kn = D == 3 ? nc : 1;
  bool any_do = false, any_keep = false;
  for (int f : cf) {
    any_do = any_do || f == AFG_REF_DO;
    any_keep = any_keep || f == AFG_REF_KEEP;
  }
  if (any_do)
    rf[id - 1] = AFG_REF_DO;
  else if (any_keep)
    rf[id - 1] = std::max(rf[id - 1], (int)AFG_REF_KEEP);
  else
    rf[id - 1] = std::max(rf[id - 1], (int)AFG_REF_RM);
  if (buf <= 0) return;
  for (int dz = (D == 3 ? -1 : 0); dz <= (D == 3 ? 1 : 0); dz++)
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) {
        if (dx == 0 && dy == 0 && dz == 0) continue;
        const int nb_id = t.mat_of(id, dx, dy, dz);
        if (nb_id <= 0) continue;
        const int dir[3] = {dx, dy, dz};
        int lo[3] = {1, 1, 1}, hi[3] = {nc, nc, kn};
        for (int d = 0; d < D; d++) {
          if (dir[d] == 1) lo[d] = nc - buf + 1;
          if (dir[d] == -1) hi[d] = buf;
        }
        bool found = false;
        for (int k = lo[2]; k <= hi[2] && !found; k++)
          for (int j = lo[1]; j <= hi[1] && !found; j++)
            for (int i = lo[0]; i <= hi[0]; i++)
              if (cf[(size_t)(i - 1) + nc * ((j - 1) + (size_t)nc * (k - 1))] == AFG_REF_DO) {
                found = true;
                break;
              }
        if (found) rf[nb_id - 1] = AFG_REF_DO;
      }
}

/* The flag pass of consistent_ref_flags (afivo/src/m_af_core.f90:929-991):
 * leaves, and for the first child of a parent that is itself not refined,
 * the parent; one sequential pass (the reference's per-thread copies are
 * combined with max, which the order does not change). */
int orc_refine_flags(void* p, const double* cc, const afg_refine_desc* a, int* flags) {
  Oracle* o = static_cast<Oracle*>(p);
  const Tree& t = o->t;
  const int unset = -2147483647 - 1;
  std::vector<int> rf(t.n_boxes, unset), cf;
  const Lsf* L = nullptr;
  auto mit = o->mg.find(a->electrode_mg);
  if (mit != o->mg.end() && mit->second.lsf) L = mit->second.lsf.get();
  for (int lvl = 1; lvl <= t.highest_lvl; lvl++)
    for (int id : t.leaves[lvl - 1]) {
      default_refinement(t, cc, id, *a, cf, L);
      cell_to_ref_flags(t, cf, id, a->ref_buffer, rf);
      if (lvl > 1) {
        const int p_id = t.parent[id - 1];
        /* af_ix_to_ichild: child number from the parity of ix */
        int ich = 1;
        for (int d = 0; d < t.D; d++) ich += ((t.ix_of(id, d) - 1) & 1) << d;
        int i_ch;
        for (i_ch = 1; i_ch < ich; i_ch++) {
          const int ch_id = t.child_of(p_id, i_ch - 1);
          if (t.child_of(ch_id, 0) <= 0) break;
        }
        if (i_ch == ich) {
          default_refinement(t, cc, p_id, *a, cf, L);
          cell_to_ref_flags(t, cf, p_id, a->ref_buffer, rf);
        }
      }
    }
  for (int b = 0; b < t.n_boxes; b++) flags[b] = rf[b] == unset ? AFG_REF_KEEP : rf[b];
  return AFG_OK;
}

/* af_prolong_limit (afivo/src/m_af_prolong.f90:311-420) into boxes ids[] */
int orc_prolong_limit(void* p, double* cc, int iv, int n, const int* ids, int limiter) {
  Oracle* o = static_cast<Oracle*>(p);
  const Tree& t = o->t;
  const int nc = t.nc, hnc = nc / 2, D = t.D;
  for (int q = 0; q < n; q++) {
    const int id = ids[q], p_id = t.parent[id - 1];
    const double* P = t.var(cc, p_id, iv);
    double* C = t.var(cc, id, iv);
    const int o0 = t.child_offset(id, 0), o1 = t.child_offset(id, 1), o2 = D == 3 ? t.child_offset(id, 2) : 0;
    for (int k = 1; k <= (D == 3 ? nc : 1); k++)
      for (int j = 1; j <= nc; j++)
        for (int i = 1; i <= nc; i++) C[D == 3 ? t.at(i, j, k) : t.at(i, j)] = 0;
    for (int k = 1; k <= (D == 3 ? hnc : 1); k++)
      for (int j = 1; j <= hnc; j++)
        for (int i = 1; i <= hnc; i++) {
          const int ic = i + o0, jc = j + o1, kc = k + o2;
          const int fi = 2 * i - 1, fj = 2 * j - 1, fk = 2 * k - 1;
          if (D == 2) {
            const double f0 = P[t.at(ic, jc)];
            const double f1 = 0.25 * limiter_apply(P[t.at(ic, jc)] - P[t.at(ic - 1, jc)],
                                                   P[t.at(ic + 1, jc)] - P[t.at(ic, jc)], limiter);
            const double f2 = 0.25 * limiter_apply(P[t.at(ic, jc)] - P[t.at(ic, jc - 1)],
                                                   P[t.at(ic, jc + 1)] - P[t.at(ic, jc)], limiter);
            C[t.at(fi, fj)] = f0 - f1 - f2 + C[t.at(fi, fj)];
            C[t.at(fi + 1, fj)] = f0 + f1 - f2 + C[t.at(fi + 1, fj)];
            C[t.at(fi, fj + 1)] = f0 - f1 + f2 + C[t.at(fi, fj + 1)];
            C[t.at(fi + 1, fj + 1)] = f0 + f1 + f2 + C[t.at(fi + 1, fj + 1)];
          } else {
            const double c0 = P[t.at(ic, jc, kc)];
            const double f1 = 0.25 * limiter_apply(c0 - P[t.at(ic - 1, jc, kc)], P[t.at(ic + 1, jc, kc)] - c0, limiter);
            const double f2 = 0.25 * limiter_apply(c0 - P[t.at(ic, jc - 1, kc)], P[t.at(ic, jc + 1, kc)] - c0, limiter);
            const double f3 = 0.25 * limiter_apply(c0 - P[t.at(ic, jc, kc - 1)], P[t.at(ic, jc, kc + 1)] - c0, limiter);
            for (int dk = 0; dk < 2; dk++)
              for (int dj = 0; dj < 2; dj++)
                for (int di = 0; di < 2; di++) {
                  const int x = t.at(fi + di, fj + dj, fk + dk);
                  const double s1 = di ? f1 : -f1, s2 = dj ? f2 : -f2, s3 = dk ? f3 : -f3;
                  C[x] = c0 + s1 + s2 + s3 + C[x];
                }
          }
        }
  }
  return AFG_OK;
}

/* af_prolong_linear with add = .false. (afivo/src/m_af_prolong.f90:531-679)
 * into boxes ids[]: per fine cell the parent value (weight 9/16, 27/64 in
 * 3D), its face neighbours (3/16; 9/64), and in 3D edge (3/64) and corner
 * (1/64) neighbours, 2D corner (1/16), summed in the reference's order and
 * added to the zeroed child cell. */
int orc_prolong_linear(void* p, double* cc, int iv, int n, const int* ids) {
  Oracle* o = static_cast<Oracle*>(p);
  const Tree& t = o->t;
  const int nc = t.nc, hnc = nc / 2, D = t.D;
  for (int q = 0; q < n; q++) {
    const int id = ids[q], p_id = t.parent[id - 1];
    if (p_id <= 0) return AFG_ERR_ARG;
    const double* P = t.var(cc, p_id, iv);
    double* C = t.var(cc, id, iv);
    const int o0 = t.child_offset(id, 0), o1 = t.child_offset(id, 1), o2 = D == 3 ? t.child_offset(id, 2) : 0;
    for (int k = 1; k <= (D == 3 ? nc : 1); k++)
      for (int j = 1; j <= nc; j++)
        for (int i = 1; i <= nc; i++) C[D == 3 ? t.at(i, j, k) : t.at(i, j)] = 0;
    if (D == 2) {
      const double f1 = 1 / 16.0, f3 = 3 / 16.0, f9 = 9 / 16.0;
      for (int j = 1; j <= hnc; j++)
        for (int i = 1; i <= hnc; i++) {
          const int ic = i + o0, jc = j + o1, fi = 2 * i - 1, fj = 2 * j - 1;
          const double f0 = f9 * P[t.at(ic, jc)];
          const double flx = f3 * P[t.at(ic - 1, jc)], fhx = f3 * P[t.at(ic + 1, jc)];
          const double fly = f3 * P[t.at(ic, jc - 1)], fhy = f3 * P[t.at(ic, jc + 1)];
          const double fll = f1 * P[t.at(ic - 1, jc - 1)], fhl = f1 * P[t.at(ic + 1, jc - 1)];
          const double flh = f1 * P[t.at(ic - 1, jc + 1)], fhh = f1 * P[t.at(ic + 1, jc + 1)];
          C[t.at(fi, fj)] = f0 + flx + fly + fll + C[t.at(fi, fj)];
          C[t.at(fi + 1, fj)] = f0 + fhx + fly + fhl + C[t.at(fi + 1, fj)];
          C[t.at(fi, fj + 1)] = f0 + flx + fhy + flh + C[t.at(fi, fj + 1)];
          C[t.at(fi + 1, fj + 1)] = f0 + fhx + fhy + fhh + C[t.at(fi + 1, fj + 1)];
        }
    } else {
      const double w[4] = {27 / 64.0, 9 / 64.0, 3 / 64.0, 1 / 64.0};  // by number of offsets
      for (int k = 1; k <= hnc; k++)
        for (int j = 1; j <= hnc; j++)
          for (int i = 1; i <= hnc; i++) {
            const int ic = i + o0, jc = j + o1, kc = k + o2;
            const int fi = 2 * i - 1, fj = 2 * j - 1, fk = 2 * k - 1;
            for (int dk = 0; dk < 2; dk++)
              for (int dj = 0; dj < 2; dj++)
                for (int di = 0; di < 2; di++) {
                  const int sx = di ? 1 : -1, sy = dj ? 1 : -1, sz = dk ? 1 : -1;
                  /* terms in the reference's order: 000, x00, 0y0, 00z, xy0, x0z, 0yz, xyz */
                  const int ox[8] = {0, sx, 0, 0, sx, sx, 0, sx};
                  const int oy[8] = {0, 0, sy, 0, sy, 0, sy, sy};
                  const int oz[8] = {0, 0, 0, sz, 0, sz, sz, sz};
                  const int x = t.at(fi + di, fj + dj, fk + dk);
                  double s = w[0] * P[t.at(ic, jc, kc)];
                  for (int m = 1; m < 8; m++) {
                    const int nof = (ox[m] != 0) + (oy[m] != 0) + (oz[m] != 0);
                    s = s + w[nof] * P[t.at(ic + ox[m], jc + oy[m], kc + oz[m])];
                  }
                  C[x] = s + C[x];
                }
          }
    }
  }
  return AFG_OK;
}

/* af_restrict_tree (afivo/src/m_af_restrict.f90:50-59) of one variable:
 * from the highest level's parents down to level 1, each child restricted
 * into its parent by af_restrict_box with geometry */
int orc_restrict_tree(void* p, double* cc, int iv) {
  Oracle* o = static_cast<Oracle*>(p);
  const Tree& t = o->t;
  for (int lvl = t.highest_lvl - 1; lvl >= 1; lvl--) {
    const std::vector<int>& par = t.parents[lvl - 1];
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < par.size(); q++)
      for (int c = 0; c < t.nchild(); c++) {
        const int ch = t.child_of(par[q], c);
        if (ch > 0) restrict_box_geom(t, cc, ch, iv);
      }
  }
  return AFG_OK;
}

/* The project's exp (which 0), log (1) and pow (2) on n arguments, for the
 * accuracy test of afg_math.h against high-precision values. */
int orc_math_eval(int which, int n, const double* x, const double* y, double* out) {
  for (int q = 0; q < n; q++)
    out[q] = which == 0 ? afg_math::exp(x[q]) : which == 1 ? afg_math::log(x[q]) : afg_math::pow(x[q], y[q]);
  return AFG_OK;
}

}  // extern "C"

extern "C" {

/* init_cond_set_box's electrode rule (src/m_init_cond.f90:284-288) on
 * boxes ids[], every cell */
int orc_electrode_init_densities(void* p, double* cc, int mg_id, int n, const int* ids) {
  Oracle* o = static_cast<Oracle*>(p);
  const Tree& t = o->t;
  auto it = o->mg.find(mg_id);
  if (it == o->mg.end() || !it->second.lsf) return AFG_ERR_STATE;
  const int iv = it->second.lsf->i_lsf;
  const afg_transport_desc& d = g_tr.d;
  for (int q = 0; q < n; q++) {
    const double* lsf = t.var(cc, ids[q], iv);
    for (int x = 0; x < t.S; x++)
      if (lsf[x] <= 0)
        for (int s = 0; s < d.n_species; s++) t.var(cc, ids[q], d.species_iv[s])[x] = 0.0;
  }
  return AFG_OK;
}

/* set_electrode_densities: electrode_species_bc (src/streamer.f90:598-656)
 * on the boxes with the mg_lsf_box tag, all levels */
int orc_electrode_species_bc(void* p, double* cc, int mg_id, int electron, int ion, int neumann) {
  Oracle* o = static_cast<Oracle*>(p);
  const Tree& t = o->t;
  auto it = o->mg.find(mg_id);
  if (it == o->mg.end() || !it->second.lsf) return AFG_ERR_STATE;
  const Lsf& L = *it->second.lsf;
  const afg_transport_desc& d = g_tr.d;
  const int nc = t.nc, D = t.D;
  const int st[3] = {1, t.n2, t.n2 * t.n2};
  for (int id : L.ids) {
    const double* lsf = t.var(cc, id, L.i_lsf);
    double* ne = t.var(cc, id, d.species_iv[electron]);
    double* ni = t.var(cc, id, d.species_iv[ion]);
    for (int k = (D == 3 ? 1 : 0); k <= (D == 3 ? nc : 0); k++)
      for (int j = 1; j <= nc; j++)
        for (int i = 1; i <= nc; i++) {
          const int x = t.at(i, j, k);
          if (!(lsf[x] < 0)) continue;
          for (int s = 0; s < d.n_species; s++) t.var(cc, id, d.species_iv[s])[x] = 0.0;
          bool any = false;
          for (int nb = 0; nb < 2 * D; nb++) any = any || lsf[x + ((nb & 1) ? 1 : -1) * st[nb >> 1]] > 0;
          if (!(any && neumann)) continue;
          double sum = 0.0;
          int cnt = 0;
          for (int nb = 0; nb < 2 * D; nb++) {
            const int y = x + ((nb & 1) ? 1 : -1) * st[nb >> 1];
            if (lsf[y] > 0) {
              sum = sum + ne[y];
              cnt++;
            }
          }
          ne[x] = sum / (double)cnt;
          ni[x] = ne[x];
        }
  }
  return AFG_OK;
}

}  // extern "C"
