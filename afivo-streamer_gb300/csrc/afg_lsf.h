// afg_lsf.h -- electrode level-set geometry for the multigrid solver with
// internal Dirichlet boundaries: the electrode shapes of src/m_field.f90
// (sphere, rod, rod with a conical top, two rods, sphere and rod, two conical
// rods, coaxial), the boundary-distance search of afivo's
// m_af_multigrid.f90 (numerical_gradient, golden-section search, bisection,
// mg_lsf_dist_gss), the per-cell distance matrix (store_lsf_distance_matrix)
// and the per-cell stencil (mg_box_lsf_stencil).  One source for device code
// (nvcc) and host code (g++): the device setup kernels and the CPU
// restatement evaluate the same expressions, built without contractions, and
// therefore agree to the bit.  log is afg_math::log, the other operations
// are IEEE-754 correctly rounded (+ - * / sqrt).
#pragma once
#include <math.h>

#include "afg_math.h"

// The search routines are large and called from several set-up kernels:
// out of line on the device (inlining them everywhere multiplies the code
// the device compiler has to schedule), inline on the host.
#if defined(__CUDACC__)
#define AFG_LSF_HD __host__ __device__ __noinline__
#else
#define AFG_LSF_HD inline
#endif

namespace afg_lsf {

enum Shape {
  kSphere = 1,
  kRod = 2,
  kRodConeTop = 3,
  kRodRod = 4,
  kSphereRod = 5,
  kTwoRodCone = 6,
  kCoaxial = 7
};

// Electrode description with every derived quantity precomputed on the host
// (the conical-tip centre and curvature use the C library's atan/cos/sin, as
// get_conical_rod_properties, m_field.f90:406-428, does once at start-up).
struct Electrode {
  int shape, D;
  int cyl;                      // axisymmetric coordinates (coaxial centre on the axis)
  double r0[3], r1[3], radius;  // electrode 1 (sphere: centre r0)
  double q0[3], q1[3], radius2; // electrode 2
  double tip_radius, cone_frac, tip_center[3], r_curv;     // conical top of electrode 1
  double tip_radius2, cone_frac2, tip_center2[3], r_curv2; // of electrode 2
  double center[3];             // coaxial: the axis (first two coordinates)
  int grounded, grounded2;      // field_electrode_grounded, field_electrode2_grounded
  double length_scale;          // mg%lsf_length_scale
  double safety;                // mg%lsf_gradient_safety_factor
  double tol;                   // mg%lsf_tol
  double min_rel;               // mg%lsf_min_rel_distance
};

// NORM2 as gfortran expands it: a scaled sum of squares (scale = the largest
// magnitude so far), sqrt(sum) * scale at the end
AFG_MATH_HD double norm2(const double* x, int n) {
  double scale = 0.0, ssq = 1.0;
  for (int i = 0; i < n; i++) {
    if (x[i] != 0.0) {
      const double a = x[i] < 0 ? -x[i] : x[i];
      if (scale < a) {
        const double v = scale / a;
        ssq = 1.0 + ssq * v * v;
        scale = a;
      } else {
        const double v = a / scale;
        ssq = ssq + v * v;
      }
    }
  }
  return sqrt(ssq) * scale;
}

// GM_dist_vec_line (src/m_geometry.f90:23-43)
AFG_MATH_HD void dist_vec_line(const double* r, const double* r0, const double* r1, int D, double* dv, double& frac) {
  double len2 = 0.0, f = 0.0;
  for (int d = 0; d < D; d++) len2 = len2 + (r1[d] - r0[d]) * (r1[d] - r0[d]);
  for (int d = 0; d < D; d++) f = f + (r[d] - r0[d]) * (r1[d] - r0[d]);
  if (f <= 0.0) {
    frac = 0.0;
    for (int d = 0; d < D; d++) dv[d] = r[d] - r0[d];
  } else if (f >= len2) {
    frac = 1.0;
    for (int d = 0; d < D; d++) dv[d] = r[d] - r1[d];
  } else {
    for (int d = 0; d < D; d++) dv[d] = r[d] - (r0[d] + f / len2 * (r1[d] - r0[d]));
    frac = f / len2;
  }
}

AFG_MATH_HD double dist_line(const double* r, const double* r0, const double* r1, int D) {
  double dv[3], frac;
  dist_vec_line(r, r0, r1, D, dv, frac);
  return norm2(dv, D);
}

// conical_rod_lsf_arg (m_field.f90:432-456)
AFG_LSF_HD double conical_rod(const double* r, const double* r0, const double* r1, const double* tip_center,
                               double radius, double tip_radius, double cone_frac, double r_curv, int D) {
  double dv[3], frac;
  dist_vec_line(r, r0, r1, D, dv, frac);
  if (frac <= 1 - cone_frac) return norm2(dv, D) - radius;
  if (frac < 1.0) {
    const double tmp = (1 - frac) / cone_frac;
    const double rad = tip_radius + tmp * (radius - tip_radius);
    return norm2(dv, D) - rad;
  }
  double x[3];
  for (int d = 0; d < D; d++) x[d] = r[d] - tip_center[d];
  return norm2(x, D) - r_curv;
}

AFG_MATH_HD double sphere(const Electrode& e, const double* r) {
  double x[3];
  for (int d = 0; d < e.D; d++) x[d] = r[d] - e.r0[d];
  return norm2(x, e.D) - e.radius;
}

// coaxial_get_lsf (m_field.f90:846-870): the first two coordinates only
AFG_MATH_HD void coaxial(const Electrode& e, const double* r, double& l1, double& l2) {
  const double x[2] = {r[0] - e.center[0], r[1] - e.center[1]};
  l1 = norm2(x, 2) - e.radius;
  l2 = e.radius2 - norm2(x, 2);
}

// the two electrodes' level-set values (single electrodes: l2 unused)
AFG_LSF_HD void lsf_pair(const Electrode& e, const double* r, double& l1, double& l2) {
  const int D = e.D;
  l2 = 0.0;
  switch (e.shape) {
    case kSphere: l1 = sphere(e, r); break;
    case kRod: l1 = dist_line(r, e.r0, e.r1, D) - e.radius; break;
    case kRodConeTop:
      l1 = conical_rod(r, e.r0, e.r1, e.tip_center, e.radius, e.tip_radius, e.cone_frac, e.r_curv, D);
      break;
    case kRodRod:
      l1 = dist_line(r, e.r0, e.r1, D) - e.radius;
      l2 = dist_line(r, e.q0, e.q1, D) - e.radius2;
      break;
    case kSphereRod:
      l1 = sphere(e, r);
      l2 = dist_line(r, e.q0, e.q1, D) - e.radius2;
      break;
    case kTwoRodCone:
      l1 = conical_rod(r, e.r0, e.r1, e.tip_center, e.radius, e.tip_radius, e.cone_frac, e.r_curv, D);
      l2 = conical_rod(r, e.q0, e.q1, e.tip_center2, e.radius2, e.tip_radius2, e.cone_frac2, e.r_curv2, D);
      break;
    default: coaxial(e, r, l1, l2); break;
  }
}

AFG_MATH_HD bool two_electrodes(const Electrode& e) {
  return e.shape == kRodRod || e.shape == kSphereRod || e.shape == kTwoRodCone || e.shape == kCoaxial;
}

// mg%lsf (sphere_lsf .. coaxial_lsf, m_field.f90:683-878): min of the two
AFG_LSF_HD double eval(const Electrode& e, const double* r) {
  double l1, l2;
  lsf_pair(e, r, l1, l2);
  if (!two_electrodes(e)) return l1;
  return l1 < l2 ? l1 : l2;  // Fortran min: the first argument on ties
}

// Potential of the electrode nearest to r: the lsf_boundary_function of the
// two-electrode shapes (rod_rod_get_potential etc., m_field.f90:505-880);
// single electrodes: mg%lsf_boundary_value = 0 (grounded) or the voltage
// (field_compute, m_field.f90:482-487)
AFG_LSF_HD double boundary_value(const Electrode& e, const double* r, double voltage) {
  if (!two_electrodes(e)) return e.grounded ? 0.0 : voltage;
  double l1, l2;
  lsf_pair(e, r, l1, l2);
  if (e.shape == kCoaxial) return l1 < l2 ? voltage : 0.0;
  if (l1 < l2) return e.grounded ? 0.0 : voltage;
  return e.grounded2 ? 0.0 : voltage;
}

// numerical_gradient (afivo m_af_multigrid.f90:2165-2190): central
// differences with step max(eps, sqrt(eps) |r|)
AFG_LSF_HD void numerical_gradient(const Electrode& e, const double* r, double* grad) {
  const double sqrteps = 1.4901161193847656e-08;  // sqrt(2^-52) = 2^-26
  const double min_step = 2.220446049250313e-16;  // 2^-52
  double re[3];
  for (int d = 0; d < e.D; d++) re[d] = r[d];
  for (int d = 0; d < e.D; d++) {
    const double a = r[d] < 0 ? -r[d] : r[d];
    const double s = sqrteps * a;
    const double step = min_step > s ? min_step : s;
    re[d] = r[d] - step;
    const double flo = eval(e, re);
    re[d] = r[d] + step;
    const double fhi = eval(e, re);
    grad[d] = (fhi - flo) / (2 * step);
    re[d] = r[d];
  }
}

// bisection (m_af_multigrid.f90:1685-1706): the last midpoint
AFG_LSF_HD void bisection(const Electrode& e, const double* in_a, const double* in_b, double* c) {
  const int D = e.D, max_iter = 100;
  double a[3], b[3];
  for (int d = 0; d < D; d++) a[d] = in_a[d], b[d] = in_b[d];
  for (int n = 1; n <= max_iter; n++) {
    for (int d = 0; d < D; d++) c[d] = 0.5 * (a[d] + b[d]);
    const double fc = eval(e, c);
    double h[3];
    for (int d = 0; d < D; d++) h[d] = b[d] - a[d];
    if (0.5 * norm2(h, D) < e.tol || (fc < 0 ? -fc : fc) <= 0) break;
    if (fc * eval(e, a) >= 0) {
      for (int d = 0; d < D; d++) a[d] = c[d];
    } else {
      for (int d = 0; d < D; d++) b[d] = c[d];
    }
  }
}

// gss (m_af_multigrid.f90:1711-1777), find_bracket = .true.: bracket
// [out0, out1] of the extremum of the lsf between in_a and in_b
AFG_LSF_HD void gss(const Electrode& e, const double* in_a, const double* in_b, bool minimization, double* out0,
                     double* out1) {
  const int D = e.D;
  const double sqrt5 = sqrt(5.0);
  const double invphi = (sqrt5 - 1) / 2, invphi2 = (3 - sqrt5) / 2;
  double a[3], b[3], c[3], dd[3], h[3];
  for (int d = 0; d < D; d++) a[d] = in_a[d], b[d] = in_b[d], h[d] = b[d] - a[d];
  const double hn = norm2(h, D);
  if (hn <= e.tol) {
    for (int d = 0; d < D; d++) out0[d] = a[d], out1[d] = b[d];
    return;
  }
  const int n = (int)ceil(afg_math::log(e.tol / hn) / afg_math::log(invphi));
  for (int d = 0; d < D; d++) {
    c[d] = a[d] + invphi2 * h[d];
    dd[d] = a[d] + invphi * h[d];
  }
  const double ya = eval(e, a);
  double yc = eval(e, c), yd = eval(e, dd);
  for (int k = 1; k <= n - 1; k++) {
    if ((yc < yd) == minimization) {
      for (int d = 0; d < D; d++) {
        b[d] = dd[d];
        dd[d] = c[d];
      }
      yd = yc;
      for (int d = 0; d < D; d++) {
        h[d] = invphi * h[d];
        c[d] = a[d] + invphi2 * h[d];
      }
      yc = eval(e, c);
    } else {
      for (int d = 0; d < D; d++) {
        a[d] = c[d];
        c[d] = dd[d];
      }
      yc = yd;
      for (int d = 0; d < D; d++) {
        h[d] = invphi * h[d];
        dd[d] = a[d] + invphi * h[d];
      }
      yd = eval(e, dd);
    }
    if (ya * yc <= 0 && ya * yd <= 0) break;
  }
  if ((yc < yd) == minimization) {
    for (int d = 0; d < D; d++) out0[d] = a[d], out1[d] = dd[d];
  } else {
    for (int d = 0; d < D; d++) out0[d] = c[d], out1[d] = b[d];
  }
}

// mg_lsf_dist_gss (m_af_multigrid.f90:1649-1682): relative distance in
// [min_rel, 1] from a towards b to the boundary, 1 = none
AFG_LSF_HD double dist_gss(const Electrode& e, const double* a, const double* b) {
  const int D = e.D;
  const double la = eval(e, a), lb = eval(e, b);
  double root[3];
  if (la * lb <= 0) {
    bisection(e, a, b, root);
  } else {
    double b0[3], b1[3], bn[3];
    gss(e, a, b, la >= 0, b0, b1);
    if (eval(e, b0) * la <= 0) {
      for (int d = 0; d < D; d++) bn[d] = b0[d];
    } else {
      for (int d = 0; d < D; d++) bn[d] = b1[d];
    }
    if (eval(e, bn) * la > 0) return 1.0;
    bisection(e, a, bn, root);
  }
  double x[3], y[3];
  for (int d = 0; d < D; d++) x[d] = root[d] - a[d], y[d] = b[d] - a[d];
  const double dist = norm2(x, D) / norm2(y, D);
  return dist > e.min_rel ? dist : e.min_rel;
}

// af_r_cc: centre of cell (i, j, k) (1-based, 0 and nc+1 are ghost cells)
AFG_MATH_HD void r_cc(const double* rmin, const double* dr, int D, const int* ix, double* r) {
  for (int d = 0; d < D; d++) r[d] = rmin[d] + (ix[d] - 0.5) * dr[d];
}

// store_lsf_distance_matrix for one interior cell (m_af_multigrid.f90:
// 954-1097): the root mask from the stored level-set value and the
// numerical gradient, the distances to the 2D neighbours, and for thin
// structures (cells larger than the length scale) a search along the
// gradient.  dd[2D] in (0, 1], 1 = no boundary on that side.  Returns
// whether the cell is in the root mask.
AFG_LSF_HD bool cell_distances(const Electrode& e, const double* rmin, const double* dr, const int* ix, double* dd) {
  const int D = e.D;
  for (int n = 0; n < 2 * D; n++) dd[n] = 1.0;
  double a[3], g[3];
  r_cc(rmin, dr, D, ix, a);
  const double lsf_c = eval(e, a);  // set_lsf_box's stored value
  numerical_gradient(e, a, g);
  const double gradnorm = norm2(g, D);
  const double dmax = norm2(dr, D);
  const double alsf = lsf_c < 0 ? -lsf_c : lsf_c;
  if (!(alsf < dmax * gradnorm * e.safety)) return false;
  for (int d = 0; d < D; d++) {
    for (int s = 0; s < 2; s++) {
      int nix[3] = {ix[0], ix[1], D == 3 ? ix[2] : 0};
      nix[d] += s == 0 ? -1 : 1;
      double b[3];
      r_cc(rmin, dr, D, nix, b);
      dd[2 * d + s] = dist_gss(e, a, b);
    }
  }
  double min_dr = dr[0];
  for (int d = 1; d < D; d++) min_dr = dr[d] < min_dr ? dr[d] : min_dr;
  bool all_ge1 = true;
  for (int n = 0; n < 2 * D; n++) all_ge1 = all_ge1 && dd[n] >= 1;
  if (min_dr > e.length_scale && all_ge1) {
    const int n_steps = (int)ceil(min_dr / e.length_scale);
    const double step = copysign(e.length_scale, lsf_c);  // Fortran sign(length_scale, lsf)
    double x[3];
    for (int d = 0; d < D; d++) x[d] = a[d];
    for (int it = 1; it <= n_steps; it++) {
      double gr[3];
      numerical_gradient(e, x, gr);
      const double gn = norm2(gr, D);
      const double den = gn > 1e-50 ? gn : 1e-50;
      for (int d = 0; d < D; d++) gr[d] = gr[d] / den;
      for (int d = 0; d < D; d++) x[d] = x[d] - gr[d] * step;
      if (eval(e, x) * lsf_c <= 0) break;
    }
    double dist = dist_gss(e, a, x);
    if (dist < 1) {
      double dvec[3];
      for (int d = 0; d < D; d++) dvec[d] = x[d] - a[d];
      dist = dist * norm2(dvec, D) / min_dr;
      int dim = 0;
      double best = dvec[0] < 0 ? -dvec[0] : dvec[0];
      for (int d = 1; d < D; d++) {
        const double v = dvec[d] < 0 ? -dvec[d] : dvec[d];
        if (v > best) best = v, dim = d;  // maxloc: the first maximum
      }
      const int nb = 2 * dim + (dvec[dim] > 0 ? 1 : 0);
      dd[nb] = dist;
    }
  }
  return true;
}

// mg_box_lsf_stencil for one cell (m_af_multigrid.f90:1779-1853): the
// generalised Laplacian for neighbours at distance dd dx, the axisymmetric
// 1/r d/dr term, v[0] = -sum(v[1:]), and the couplings to boundary points
// moved into f (the right-hand-side factor of the boundary value).
// v[2D+1] in the order centre, i-1, i+1, j-1, j+1(, k-1, k+1).
AFG_LSF_HD void cell_stencil(int D, bool cyl, const double* rmin, const double* dr, int i, const double* dd,
                              double* v, double& f) {
  for (int d = 0; d < D; d++) {
    const double dr2 = dr[d] * dr[d];
    v[1 + 2 * d] = 1 / (0.5 * dr2 * (dd[2 * d] + dd[2 * d + 1]) * dd[2 * d]);
    v[2 + 2 * d] = 1 / (0.5 * dr2 * (dd[2 * d] + dd[2 * d + 1]) * dd[2 * d + 1]);
  }
  if (cyl) {
    const double rc = rmin[0] + (i - 0.5) * dr[0];  // af_cyl_radius_cc
    const double tmp = 1 / (dr[0] * (dd[0] + dd[1]) * rc);
    v[1] = v[1] - tmp;
    v[2] = v[2] + tmp;
  }
  double s = 0.0;
  for (int n = 1; n <= 2 * D; n++) s = s + v[n];
  v[0] = -s;
  f = 0.0;
  for (int n = 0; n < 2 * D; n++) {
    if (dd[n] < 1.0) {
      f = f - v[n + 1];
      v[n + 1] = 0.0;
    }
  }
}

}  // namespace afg_lsf
