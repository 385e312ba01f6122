// afg_transport.cuh -- drift-diffusion transport, field and photoionization
// kernels of the streamer step (src/m_fluid.f90, src/m_field.f90,
// src/m_photoi.f90; afivo/src/m_af_flux_schemes.f90, m_af_ghostcell.f90,
// m_af_core.f90).  FP64 throughout: the densities span 1e9..1e20 m^-3.
#pragma once
#include "../../include/afivo_gpu.h"
#include "afg_common.cuh"
#include "afg_math.h"

namespace afg {

constexpr double kSiToTd = 1e21;               // SI_to_Townsend (src/m_gas.f90:39)
constexpr double kEps0 = 8.8541878128e-12;     // UC_eps0 (src/m_units_constants.f90:13)
constexpr double kElem = 1.602176634e-19;      // UC_elem_charge (16)

struct Reac32;
struct TransportState {
  bool ready = false;
  afg_transport_desc d{};
  double* d_lt = nullptr;              // [n_cols][n_points]
  afg_reaction* d_reactions = nullptr; // [n_reactions]
  float* d_ltf = nullptr;              // the table in FP32 (mixed precision)
  Reac32* d_reac32 = nullptr;          // reactions in FP32 form
  // task lists (slots): leaves with a refinement boundary and a parent;
  // (coarse box, face) pairs for af_consistent_fluxes
  int* d_rrb = nullptr;
  int n_rrb = 0;
  int* d_cflux = nullptr;              // pairs (slot, nb)
  int n_cflux = 0;
  // electrode: the level-set variable whose cells <= 0 the update leaves out
  int mask_iv = 0;
};

inline void transport_free(TransportState& s) {
  if (s.d_lt) cudaFree(s.d_lt);
  if (s.d_reactions) cudaFree(s.d_reactions);
  if (s.d_ltf) cudaFree(s.d_ltf);
  if (s.d_reac32) cudaFree(s.d_reac32);
  if (s.d_rrb) cudaFree(s.d_rrb);
  if (s.d_cflux) cudaFree(s.d_cflux);
  s = TransportState();
}

// Lookup table LT_get_loc + LT_get_col_at_loc, linear spacing
// (src/lookup_table_fortran/m_lookup_table.f90:330-406)
struct LtDev {
  const double* y;  // [n_cols][n]
  int n;
  double x_min, inv_fac;
};

__device__ __forceinline__ void lt_loc(const LtDev& lt, double x, int& ix, double& w) {
  const double frac = (x - lt.x_min) * lt.inv_fac;
  if (frac <= 0) {
    ix = 1;
    w = 1;
  } else if (frac >= lt.n - 1) {
    ix = lt.n - 1;
    w = 0;
  } else {
    ix = (int)ceil(frac);
    w = ix - frac;
  }
}
__device__ __forceinline__ double lt_col(const LtDev& lt, int col, int ix, double w) {
  const double* y = lt.y + (size_t)col * lt.n;
  return w * y[ix - 1] + (1 - w) * y[ix];
}

// af_limiter_koren (afivo/src/m_af_limiters.f90:72-95)
__device__ __forceinline__ double koren(double a, double b) {
  const double third = 1 / 3.0;
  const double aa = a * a, ab = a * b;
  if (ab <= 0) return 0;
  if (aa <= 0.25 * ab) return 2 * a;
  if (aa <= 2.5 * ab) return third * (b + 2 * a);
  return 2 * b;
}

// af_limiter_gminmod (m_af_limiters.f90:133-149)
__device__ __forceinline__ double gminmod(double a, double b, double theta) {
  if (a * b > 0) {
    double m = fabs(theta * a);
    m = fmin(m, fabs(theta * b));
    m = fmin(m, fabs(0.5 * (a + b)));
    return copysign(m, a);
  }
  return 0.0;
}

__device__ __forceinline__ double limiter_apply(double a, double b, int lim) {
  switch (lim) {
    case AFG_LIMITER_KOREN: return koren(a, b);
    case AFG_LIMITER_MINMOD: return gminmod(a, b, 1.0);
    case AFG_LIMITER_MC: return gminmod(a, b, 2.0);
    case AFG_LIMITER_GMINMOD43: return gminmod(a, b, 4 / 3.0);
    default: {
      const double ab = a * b;
      return ab > 0 ? 2 * ab / (a + b) : 0;
    }
  }
}

__device__ __forceinline__ int fc_at(int nf1, int i, int j, int k) {
  return (i - 1) + nf1 * ((j - 1) + nf1 * (k - 1));
}

struct FluxArgs {
  int nf;
  double* n[AFG_MAX_FLUX];      // densities (state s_deriv); first ghost layer written back
  double* flux[AFG_MAX_FLUX];   // fc pools of the fluxes
  double sign[AFG_MAX_FLUX];
  double mu_ion_N[AFG_MAX_FLUX];
  const double* E;              // cc |E|
  const double* Efc;            // fc E
  GcDev bc;
  int limiter;
  double N_inv;
  LtDev lt;
  int col_mu, col_dc;
  unsigned long long* max_cfl;
  unsigned long long* max_sigma;
};

// af_restrict_box with geometry of one variable (m_af_restrict.f90:62-136)
template <int D, bool CYL, int NC = 0>
__global__ void __launch_bounds__(256) k_restrict_geom(KTree t0, const int* __restrict__ list, ModeArg<double> v_) {
  const KTree t = fix_dims<D, NC>(t0);
  double* __restrict__ v = v_.get();
  const int slot = list[blockIdx.x];
  if (box_frozen(t, slot)) return;
  const int pslot = t.parent[slot];
  const int nc = t.nc, n2 = t.n2, hnc = nc / 2;
  const double* c = v + (size_t)slot * t.S;
  double* pp = v + (size_t)pslot * t.S;
  const int o0 = child_offset(t, slot, 0), o1 = child_offset(t, slot, 1), o2 = D == 3 ? child_offset(t, slot, 2) : 0;
  const int count = D == 2 ? hnc * hnc : hnc * hnc * hnc;
  for (int w = threadIdx.x; w < count; w += blockDim.x) {
    const int i = w % hnc + 1, r = w / hnc;
    const int j = D == 2 ? r + 1 : r % hnc + 1, k = D == 2 ? 0 : r / hnc + 1;
    const int fi = 2 * i - 1, fj = 2 * j - 1;
    if (D == 2) {
      const int ic = o0 + i;
      double val;
      if (CYL) {
        const double* gw = t.geo + ((size_t)pslot * nc + (ic - 1)) * 4;
        const double w1 = gw[2], w2 = gw[3];
        double s1 = 0, s2 = 0;
        s1 = s1 + c[at2(n2, fi, fj)]; s1 = s1 + c[at2(n2, fi, fj + 1)];
        s2 = s2 + c[at2(n2, fi + 1, fj)]; s2 = s2 + c[at2(n2, fi + 1, fj + 1)];
        val = 0.25 * (w1 * s1 + w2 * s2);
      } else {
        double s = 0;
        s = s + c[at2(n2, fi, fj)]; s = s + c[at2(n2, fi + 1, fj)];
        s = s + c[at2(n2, fi, fj + 1)]; s = s + c[at2(n2, fi + 1, fj + 1)];
        val = 0.25 * s;
      }
      pp[at2(n2, ic, o1 + j)] = val;
    } else {
      const int fk = 2 * k - 1;
      double s = 0;
      for (int dk = 0; dk < 2; dk++)
        for (int dj = 0; dj < 2; dj++)
          for (int di = 0; di < 2; di++) s = s + c[at3(n2, fi + di, fj + dj, fk + dk)];
      pp[at3(n2, o0 + i, o1 + j, o2 + k)] = 0.125 * s;
    }
  }
}

// Index into the two-ghost-layer tile: cells -1..nc+2 per dimension.
template <int D>
__device__ __forceinline__ int big_at(int m, int i, int j, int k) {
  return (i + 1) + m * ((j + 1) + (D == 3 ? m * (k + 1) : 0));
}
template <int D>
__device__ __forceinline__ int big_face(int m, int d, int x, int p, int q) {
  if (D == 2) return d == 0 ? big_at<D>(m, x, p, 0) : big_at<D>(m, p, x, 0);
  if (d == 0) return big_at<D>(m, x, p, q);
  if (d == 1) return big_at<D>(m, p, x, q);
  return big_at<D>(m, p, q, x);
}

// Two ghost layers of one face cell (af_gc2_box, m_af_ghostcell.f90:672-744):
// same-level copy, gc2_prolong_rb (753-856) or bc_to_gc2 (282-375).
// layer 0 is adjacent to the box, layer 1 the outer one.
template <int D>
__device__ __forceinline__ double gc2_value(const KTree& t, const double* __restrict__ v, int slot, int nb, int nbs,
                                            int layer, int p, int q, const GcDev& g, int limiter) {
  const int nc = t.nc, n2 = t.n2, d = nb >> 1;
  const bool low = (nb & 1) == 0;
  if (nbs >= 0) {
    const double* b = v + (size_t)nbs * t.S;
    const int x = low ? nc - layer : 1 + layer;
    return b[face_at<D>(n2, d, x, p, q)];
  }
  if (nbs == kNbPhys) {
    const double* a = v + (size_t)slot * t.S;
    double c0, c1, c2;
    switch (gc_type(g, nb)) {
      case AFG_BC_DIRICHLET: c0 = 2; c1 = -1; c2 = c0; break;
      case AFG_BC_NEUMANN: c0 = t.dr[slot * D + d] * (low ? -1 : 1); c1 = 1; c2 = 3 * c0; break;
      default: c0 = 1; c1 = 0; c2 = c0; break;
    }
    if (D == 3 && nb == 3) c2 = c0;  // as in the reference's 3D high-y branch
    const int xi = layer == 0 ? (low ? 1 : nc) : (low ? 2 : nc - 1);
    const double cc0 = layer == 0 ? c0 : c2;
    return cc0 * gc_val(g, nb, t, slot) + c1 * a[face_at<D>(n2, d, xi, p, q)];
  }
  // refinement boundary: limited prolongation from the parent's neighbour
  const int cs = t.pnb[slot * 2 * D + nb];
  const double* C = v + (size_t)cs * t.S;
  int ci[3], sgn[3];
  const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
  ci[d] = low ? nc : 1;
  // fine normal index -1 / nc+1 is the lower fine cell of the coarse cell
  sgn[d] = low ? (layer == 1 ? -1 : 1) : (layer == 0 ? -1 : 1);
  ci[t1] = child_offset(t, slot, t1) + ((p + 1) >> 1);
  sgn[t1] = (p & 1) ? -1 : 1;
  if (D == 3) {
    ci[t2] = child_offset(t, slot, t2) + ((q + 1) >> 1);
    sgn[t2] = (q & 1) ? -1 : 1;
  }
  const int x0 = D == 2 ? at2(n2, ci[0], ci[1]) : at3(n2, ci[0], ci[1], ci[2]);
  const double f0 = C[x0];
  double val = f0;
  int stride = 1;
  for (int dd = 0; dd < D; dd++) {
    const double fd = 0.25 * limiter_apply(C[x0] - C[x0 - stride], C[x0 + stride] - C[x0], limiter);
    val = sgn[dd] < 0 ? val - fd : val + fd;
    stride *= n2;
  }
  return val;
}

// flux_upwind_box (m_af_flux_schemes.f90:715-848) with flux_upwind and
// flux_direction of the fluid model (src/m_fluid.f90:102-227): Koren-limited
// upwind reconstruction, v = -mu(E)*E_x, Gamma = v*u - D/dx*(n_f - n_f-1),
// ions drift only; CFL sum and conductivity maxima reduced to the device.
template <int D, bool CYL, int NC = 0>
__global__ void __launch_bounds__(256) k_flux(KTree t0, const int* __restrict__ list, FluxArgs a) {
  const KTree t = fix_dims<D, NC>(t0);
  extern __shared__ double sm[];
  __shared__ double sred[32];
  const int slot = list[blockIdx.x];
  const int nc = t.nc, n2 = t.n2, m = nc + 4, nf1 = nc + 1;
  const int tile = D == 2 ? m * m : m * m * m;
  const int nfaces = D == 2 ? nc * nf1 : nc * nc * nf1;  // per dimension
  double* big = sm;                             // [nf][tile]
  double* vf = sm + a.nf * tile;                // [D][nfaces] velocity
  double* df = vf + D * nfaces;                 // [D][nfaces] diffusion
  // 1. tiles: box array (one ghost layer), then the two face ghost layers
  for (int s = 0; s < a.nf; s++) {
    const double* src = a.n[s] + (size_t)slot * t.S;
    for (int x = threadIdx.x; x < t.S; x += blockDim.x) {
      const int i = x % n2, r = x / n2;
      const int j = D == 2 ? r : r % n2, k = D == 2 ? 0 : r / n2;
      big[s * tile + big_at<D>(m, i, j, k)] = src[x];
    }
  }
  __syncthreads();
  const int nface = D == 2 ? nc : nc * nc;
  for (int s = 0; s < a.nf; s++) {
    for (int w = threadIdx.x; w < 2 * D * nface * 2; w += blockDim.x) {
      const int layer = w & 1, w2 = w >> 1;
      const int nb = w2 / nface, pq = w2 - nb * nface;
      const int p = pq % nc + 1, q = D == 3 ? pq / nc + 1 : 0;
      const int d = nb >> 1;
      const bool low = (nb & 1) == 0;
      const double val = gc2_value<D>(t, a.n[s], slot, nb, t.nbr[slot * 2 * D + nb], layer, p, q, a.bc, a.limiter);
      const int x = low ? -layer : nc + 1 + layer;
      big[s * tile + big_face<D>(m, d, x, p, q)] = val;
    }
  }
  __syncthreads();
  // write back the first ghost layer (af_gc2_box copies cc(0:nc+1) back)
  for (int s = 0; s < a.nf; s++) {
    double* dst = a.n[s] + (size_t)slot * t.S;
    for (int w = threadIdx.x; w < 2 * D * nface; w += blockDim.x) {
      const int nb = w / nface, pq = w - nb * nface;
      const int p = pq % nc + 1, q = D == 3 ? pq / nc + 1 : 0;
      const int d = nb >> 1;
      const int x = (nb & 1) ? nc + 1 : 0;
      dst[face_at<D>(n2, d, x, p, q)] = big[s * tile + big_face<D>(m, d, x, p, q)];
    }
  }
  // 2. fluxes on all faces
  const double* E = a.E + (size_t)slot * t.S;
  double smax = 0.0;
  for (int w = threadIdx.x; w < D * nfaces; w += blockDim.x) {
    const int dim = w / nfaces, fw = w - dim * nfaces;
    const int f = fw % nf1 + 1, ln = fw / nf1;  // face index along dim, line index
    const int jj = ln % nc + 1, kk = D == 3 ? ln / nc + 1 : 1;
    const double inv_dx = t.idr[slot * D + dim];
    int fidx;
    if (D == 2) fidx = dim == 0 ? fc_at(nf1, f, jj, 1) : fc_at(nf1, jj, f, 1);
    else if (dim == 0) fidx = fc_at(nf1, f, jj, kk);
    else if (dim == 1) fidx = fc_at(nf1, jj, f, kk);
    else fidx = fc_at(nf1, jj, kk, f);
    const double Ex = a.Efc[((size_t)slot * D + dim) * t.NF + fidx];
    auto cidx = [&](int x) -> int {
      if (D == 2) return dim == 0 ? at2(n2, x, jj) : at2(n2, jj, x);
      if (dim == 0) return at3(n2, x, jj, kk);
      if (dim == 1) return at3(n2, jj, x, kk);
      return at3(n2, jj, kk, x);
    };
    auto bidx = [&](int x) -> int {
      if (D == 2) return dim == 0 ? big_at<D>(m, x, jj, 0) : big_at<D>(m, jj, x, 0);
      if (dim == 0) return big_at<D>(m, x, jj, kk);
      if (dim == 1) return big_at<D>(m, jj, x, kk);
      return big_at<D>(m, jj, kk, x);
    };
    const double td = 0.5 * (E[cidx(f - 1)] + E[cidx(f)]) * kSiToTd * a.N_inv;
    int ix;
    double lw;
    lt_loc(a.lt, td, ix, lw);
    const double mu = lt_col(a.lt, a.col_mu, ix, lw) * a.N_inv;
    const double dc = lt_col(a.lt, a.col_dc, ix, lw) * a.N_inv;
    const double v = -mu * Ex;
    double sigma = 0;
    for (int s = 0; s < a.nf; s++) {
      const double* L = big + s * tile;
      const double lm2 = L[bidx(f - 2)], lm1 = L[bidx(f - 1)], l0 = L[bidx(f)], lp1 = L[bidx(f + 1)];
      const bool pos = a.sign[s] * Ex > 0;
      const double u = pos ? lm1 + 0.5 * koren(l0 - lm1, lm1 - lm2) : l0 - 0.5 * koren(l0 - lm1, lp1 - l0);
      double fl;
      if (s == 0) {
        fl = v * u - dc * inv_dx * (l0 - lm1);
        sigma = mu * u;
      } else {
        const double mui = a.mu_ion_N[s] * a.N_inv;
        const double vi = a.sign[s] * mui * Ex;
        fl = vi * u;
        sigma = sigma + mui * u;
      }
      a.flux[s][((size_t)slot * D + dim) * t.NF + fidx] = fl;
    }
    smax = sigma > smax ? sigma : smax;
    vf[w] = v;
    df[w] = dc;
  }
  __syncthreads();
  // 3. CFL sum per cell, summed over dimensions in order
  double cmax = 0.0;
  const int ncell = D == 2 ? nc * nc : nc * nc * nc;
  for (int w = threadIdx.x; w < ncell; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 1 : r / nc + 1;
    double cfl = 0.0;
    for (int dim = 0; dim < D; dim++) {
      const double inv_dx = t.idr[slot * D + dim];
      int c, ln;
      if (D == 2) { c = dim == 0 ? i : j; ln = dim == 0 ? j - 1 : i - 1; }
      else if (dim == 0) { c = i; ln = (j - 1) + nc * (k - 1); }
      else if (dim == 1) { c = j; ln = (i - 1) + nc * (k - 1); }
      else { c = k; ln = (i - 1) + nc * (j - 1); }
      const int base = dim * nfaces + ln * nf1;
      const double vmax = fmax(fabs(vf[base + c]), fabs(vf[base + c - 1]));
      const double dmax = fmax(df[base + c], df[base + c - 1]);
      cfl = cfl + (1.0 * vmax * inv_dx + 2 * dmax * (inv_dx * inv_dx));
    }
    cmax = cfl > cmax ? cfl : cmax;
  }
  cmax = block_max<double>(cmax, sred);
  if (threadIdx.x == 0) atomic_max_nonneg(a.max_cfl, cmax);
  __syncthreads();
  smax = block_max<double>(smax, sred);
  if (threadIdx.x == 0) atomic_max_nonneg(a.max_sigma, smax);
}

// af_consistent_fluxes / flux_from_children (afivo/src/m_af_core.f90:
// 1257-1402): one CTA per (parent box, face) task.
template <int D, bool CYL, int NC = 0>
__global__ void __launch_bounds__(128) k_consistent_flux(KTree t0, const int* __restrict__ tasks, int nf,
                                                         FluxArgs a) {
  const KTree t = fix_dims<D, NC>(t0);
  const int slot = tasks[2 * blockIdx.x], nb = tasks[2 * blockIdx.x + 1];
  const int nc = t.nc, nch = nc / 2, d = nb >> 1, nf1 = nc + 1;
  const bool low = (nb & 1) == 0;
  const int nbs = t.nbr[slot * 2 * D + nb];
  const int i = low ? 1 : nc + 1, i_nb = low ? nc + 1 : 1;
  const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
  const int nchild = 1 << D;
  const int per_child = D == 2 ? nch : nch * nch;
  for (int w = threadIdx.x; w < nchild * per_child * nf; w += blockDim.x) {
    const int s = w / (nchild * per_child), w2 = w - s * nchild * per_child;
    const int c = w2 / per_child, pq = w2 - c * per_child;
    if (((c >> d) & 1) != (low ? 0 : 1)) continue;
    const int cs = t.children[slot * nchild + c];
    const int ioff[3] = {nch * (c & 1), nch * ((c >> 1) & 1), nch * ((c >> 2) & 1)};
    const double* F = a.flux[s] + ((size_t)cs * D + d) * t.NF;
    double* G = a.flux[s] + ((size_t)nbs * D + d) * t.NF;
    if (D == 2) {
      const int n = pq + 1;
      const int o = ioff[t1];
      if (d == 0) {
        G[fc_at(nf1, i_nb, o + n, 1)] = 0.5 * (F[fc_at(nf1, i, 2 * n - 1, 1)] + F[fc_at(nf1, i, 2 * n, 1)]);
      } else if (CYL) {
        const double* gw = t.geo + ((size_t)nbs * nc + (o + n - 1)) * 4;
        const double w1 = gw[2], w2 = gw[3];
        G[fc_at(nf1, o + n, i_nb, 1)] = 0.5 * (w1 * F[fc_at(nf1, 2 * n - 1, i, 1)] + w2 * F[fc_at(nf1, 2 * n, i, 1)]);
      } else {
        G[fc_at(nf1, o + n, i_nb, 1)] = 0.5 * (F[fc_at(nf1, 2 * n - 1, i, 1)] + F[fc_at(nf1, 2 * n, i, 1)]);
      }
    } else {
      const int p = pq % nch + 1, q = pq / nch + 1;
      auto FA = [&](int x, int pp, int qq) {
        if (d == 0) return fc_at(nf1, x, pp, qq);
        if (d == 1) return fc_at(nf1, pp, x, qq);
        return fc_at(nf1, pp, qq, x);
      };
      G[FA(i_nb, ioff[t1] + p, ioff[t2] + q)] =
          0.25 * (F[FA(i, 2 * p - 1, 2 * q - 1)] + F[FA(i, 2 * p, 2 * q - 1)] + F[FA(i, 2 * p - 1, 2 * q)] +
                  F[FA(i, 2 * p, 2 * q)]);
    }
  }
}

struct UpdateArgs {
  int ns, nf;
  double* out[AFG_MAX_SPECIES];               // state s_out
  const double* deriv[AFG_MAX_SPECIES];       // state s_deriv
  const double* prev[4][AFG_MAX_SPECIES];     // states s_prev[m]
  double w_prev[4];
  int n_prev;
  int flux_species[AFG_MAX_FLUX];
  const double* flux[AFG_MAX_FLUX];
  const double* E;
  const double* photo;  // may be null
  int photoi_species;
  double dt, N_inv;
  LtDev lt;
  const afg_reaction* reactions;
  int n_reactions;
  int last_step;
  double nmin;
  int limit_loss;
  unsigned long long* min_chem;  // bits of a non-negative double (atomicMin)
  // electrode: level-set values; cells with lsf <= 0 keep the weighted
  // previous states (set_box_mask, src/m_fluid.f90:469-515); null = none
  const double* mask;
};

// x**c for the exponents of the analytic forms.  FP64: the project's pow
// (afg_math.h), bit-identical to the CPU restatement's; it returns x itself
// for c == 1, as the reference's pow does.
__device__ __forceinline__ double pow_c(double x, double c) { return afg_math::pow(x, c); }
__device__ __forceinline__ float pow_c(float x, float c) { return c == 1.0f ? x : powf(x, c); }

// Rate coefficient of one reaction (get_rates, src/m_chemistry.f90:672-760).
// F32: the argument of the exponential and the exponential in FP32 (the
// mixed-precision transport); the factors c0 * c1 stay FP64.
template <bool F32>
__device__ __forceinline__ double rate_of(const LtDev& lt, const afg_reaction& r, double td, int ix, double w) {
  const double c0 = r.rate_factor;
  switch (r.rate_type) {
    case AFG_RATE_TABULATED_FIELD: return c0 * lt_col(lt, r.lt_col, ix, w);
    case AFG_RATE_CONSTANT: return c0 * r.c[0];
    case AFG_RATE_LINEAR: return c0 * r.c[0] * (td - r.c[1]);
    case AFG_RATE_EXP_V1:
      if (F32) {
        const float q = (float)r.c[1] / ((float)r.c[2] + (float)td);
        return c0 * r.c[0] * (double)expf(-(q * q));
      } else {
        const double q = r.c[1] / (r.c[2] + td);
        return c0 * r.c[0] * afg_math::exp(-(q * q));
      }
    case AFG_RATE_EXP_V2:
      if (F32) {
        const float q = (float)td / (float)r.c[1];
        return c0 * r.c[0] * (double)expf(-(q * q));
      } else {
        const double q = td / r.c[1];
        return c0 * r.c[0] * afg_math::exp(-(q * q));
      }
    case AFG_RATE_K13:
      if (F32)
        return c0 * r.c[0] * (double)expf(-pow_c((float)r.c[1] / ((float)r.c[2] + (float)td), (float)r.c[3]));
      else
        return c0 * r.c[0] * afg_math::exp(-pow_c(r.c[1] / (r.c[2] + td), r.c[3]));
    case AFG_RATE_K14:
      if (F32)
        return c0 * r.c[0] * (double)expf(-pow_c((float)td / (float)r.c[1], (float)r.c[2]));
      else
        return c0 * r.c[0] * afg_math::exp(-pow_c(td / r.c[1], r.c[2]));
    case AFG_RATE_K1: {
      // electron temperature from the tabulated mean energy (eV -> K)
      const double Te = (2 * 1.602176634e-19 / (3 * 1.380649e-23)) * lt_col(lt, r.lt_col, ix, w);
      if (F32) return c0 * r.c[0] * (double)pow_c(300.0f / (float)Te, (float)r.c[1]);
      return c0 * r.c[0] * pow_c(300 / Te, r.c[1]);
    }
  }
  return 0;
}

// Species arrays are indexed through the reaction tables at run time; to
// keep them in registers every access goes through a fully unrolled loop over
// the compile-time bound NSMAX (static indices only).
template <int NSMAX>
__device__ __forceinline__ double pick(const double (&v)[NSMAX], int s) {
  double r = 0.0;
#pragma unroll
  for (int k = 0; k < NSMAX; k++)
    if (k == s) r = v[k];
  return r;
}
template <int NSMAX>
__device__ __forceinline__ void add_to(double (&v)[NSMAX], int s, double x) {
#pragma unroll
  for (int k = 0; k < NSMAX; k++)
    if (k == s) v[k] = v[k] + x;
}

// flux_update_densities + add_source_terms for each leaf cell
template <int D, bool CYL, int NSMAX, int NC = 0>
__global__ void __launch_bounds__(128) k_update(KTree t0, const int* __restrict__ list, UpdateArgs a) {
  const KTree t = fix_dims<D, NC>(t0);
  __shared__ double sred[32];
  const int slot = list[blockIdx.x];
  const int nc = t.nc, n2 = t.n2, nf1 = nc + 1;
  const int ncell = D == 2 ? nc * nc : nc * nc * nc;
  double dt_dr[3];
  for (int q = 0; q < D; q++) dt_dr[q] = a.dt / t.dr[slot * D + q];
  double my_chem = 1e100;
  const size_t base = (size_t)slot * t.S;
  // a box without gas cells adds no source terms and no chemistry limit
  // (add_source_terms returns early, src/m_fluid.f90:332)
  int any_gas = a.mask == nullptr ? 1 : 0;
  if (a.mask != nullptr) {
    for (int w = threadIdx.x; w < ncell; w += blockDim.x) {
      const int i = w % nc + 1, r = w / nc;
      const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 0 : r / nc + 1;
      any_gas |= a.mask[base + (D == 2 ? at2(n2, i, j) : at3(n2, i, j, k))] > 0.0;
    }
    any_gas = __syncthreads_or(any_gas);
  }
  for (int w = threadIdx.x; w < ncell; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 0 : r / nc + 1;
    const int x = D == 2 ? at2(n2, i, j) : at3(n2, i, j, k);
    const bool gas = a.mask == nullptr || a.mask[base + x] > 0.0;
    double outv[NSMAX], dens[NSMAX], der[NSMAX];
#pragma unroll
    for (int s = 0; s < NSMAX; s++) {
      outv[s] = 0.0;
      dens[s] = 0.0;
      der[s] = 0.0;
      if (s < a.ns) {
        double tmp = 0.0;
        for (int mm = 0; mm < a.n_prev; mm++) tmp = tmp + a.w_prev[mm] * a.prev[mm][s][base + x];
        outv[s] = tmp;
        dens[s] = fmax(a.deriv[s][base + x], 0.0);
      }
    }
    const double td = kSiToTd * a.N_inv * a.E[base + x];
    int ix;
    double lw;
    lt_loc(a.lt, td, ix, lw);
    for (int n = 0; n < a.n_reactions; n++) {
      const afg_reaction& rc = a.reactions[n];
      double rate = rate_of<false>(a.lt, rc, td, ix, lw);
      double prod = 1.0;
      for (int q = 0; q < rc.n_in; q++) prod = prod * pick<NSMAX>(dens, rc.ix_in[q]);
      rate = rate * prod;
      for (int q = 0; q < rc.n_in; q++) add_to<NSMAX>(der, rc.ix_in[q], -rate);
      for (int q = 0; q < rc.n_out; q++) add_to<NSMAX>(der, rc.ix_out[q], rate * rc.mult_out[q]);
    }
    if (a.last_step && any_gas) {
      const double eps = 1e-100;
      double tmp = 1e100;
#pragma unroll
      for (int s = 0; s < NSMAX; s++) {
        if (s >= a.ns) continue;
        if (a.nmin > 0)
          tmp = fmin(tmp, (dens[s] + a.nmin) / fmax(fabs(der[s]), eps));
        else if (a.limit_loss)
          tmp = fmin(tmp, fmax(dens[s], eps) / fmax(-der[s], eps));
      }
      my_chem = fmin(my_chem, tmp);
    }
    if (a.photo != nullptr) {
      const double ph = a.photo[base + x];
      add_to<NSMAX>(der, a.flux_species[0], ph);
      add_to<NSMAX>(der, a.photoi_species, ph);
    }
    if (!gas) {
#pragma unroll
      for (int s = 0; s < NSMAX; s++)
        if (s < a.ns) a.out[s][base + x] = outv[s];
      continue;
    }
#pragma unroll
    for (int s = 0; s < NSMAX; s++) outv[s] = outv[s] + a.dt * der[s];
    for (int f = 0; f < a.nf; f++) {
      const int s = a.flux_species[f];
      const double* F0 = a.flux[f] + ((size_t)slot * D + 0) * t.NF;
      const double* F1 = a.flux[f] + ((size_t)slot * D + 1) * t.NF;
      const int kk = D == 3 ? k : 1;
      double div;
      if (D == 2 && CYL) {
        const double* gw = t.geo + ((size_t)slot * nc + (i - 1)) * 4;
        const double f1 = gw[0], f2 = gw[1];
        div = dt_dr[0] * (f1 * F0[fc_at(nf1, i, j, 1)] - f2 * F0[fc_at(nf1, i + 1, j, 1)]);
        div = pick<NSMAX>(outv, s) + div + dt_dr[1] * (F1[fc_at(nf1, i, j, 1)] - F1[fc_at(nf1, i, j + 1, 1)]);
      } else if (D == 2) {
        div = pick<NSMAX>(outv, s) + dt_dr[0] * (F0[fc_at(nf1, i, j, 1)] - F0[fc_at(nf1, i + 1, j, 1)]) +
              dt_dr[1] * (F1[fc_at(nf1, i, j, 1)] - F1[fc_at(nf1, i, j + 1, 1)]);
      } else {
        const double* F2 = a.flux[f] + ((size_t)slot * D + 2) * t.NF;
        div = pick<NSMAX>(outv, s) + dt_dr[0] * (F0[fc_at(nf1, i, j, kk)] - F0[fc_at(nf1, i + 1, j, kk)]) +
              dt_dr[1] * (F1[fc_at(nf1, i, j, kk)] - F1[fc_at(nf1, i, j + 1, kk)]) +
              dt_dr[2] * (F2[fc_at(nf1, i, j, kk)] - F2[fc_at(nf1, i, j, kk + 1)]);
      }
#pragma unroll
      for (int q = 0; q < NSMAX; q++)
        if (q == s) outv[q] = div;
    }
#pragma unroll
    for (int s = 0; s < NSMAX; s++)
      if (s < a.ns) a.out[s][base + x] = outv[s];
  }
  if (a.last_step) {
    for (int o = 16; o > 0; o >>= 1) my_chem = fmin(my_chem, __shfl_xor_sync(0xffffffffu, my_chem, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sred[warp] = my_chem;
    __syncthreads();
    if (threadIdx.x == 0) {
      double v = sred[0];
      for (int q = 1; q < (int)((blockDim.x + 31) >> 5); q++) v = fmin(v, sred[q]);
      atomicMin(a.min_chem, (unsigned long long)__double_as_longlong(v));
    }
  }
}

// field_set_rhs (src/m_field.f90:406-444) on leaves, whole arrays
struct RhsArgs {
  int ns;
  const double* n[AFG_MAX_SPECIES];
  double q[AFG_MAX_SPECIES];  // charge * (-e/eps0), 0 = uncharged (skipped)
  double* rhs;
};
static __global__ void __launch_bounds__(256) k_field_rhs(int S, const int* __restrict__ list, RhsArgs a) {
  const size_t base = (size_t)list[blockIdx.x] * S;
  for (int x = threadIdx.x; x < S; x += blockDim.x) {
    double v = 0.0;
    for (int s = 0; s < a.ns; s++)
      if (a.q[s] != 0.0) v = v + a.q[s] * a.n[s][base + x];
    a.rhs[base + x] = v;
  }
}

// mg_box_lpl_gradient with fac = -1 (m_af_multigrid.f90:1902-1994) and
// mg_box_field_norm (2015-2045) on each box of the list
template <int D, int NC = 0>
__global__ void __launch_bounds__(256) k_field_grad(KTree t0, const int* __restrict__ list, const double* __restrict__ phi,
                                                    double* __restrict__ efc, double* __restrict__ enorm) {
  const KTree t = fix_dims<D, NC>(t0);
  const int slot = list[blockIdx.x];
  const int nc = t.nc, n2 = t.n2, nf1 = nc + 1;
  const double* p = phi + (size_t)slot * t.S;
  const int nfaces = D == 2 ? nc * nf1 : nc * nc * nf1;
  for (int w = threadIdx.x; w < D * nfaces; w += blockDim.x) {
    const int dim = w / nfaces, fw = w - dim * nfaces;
    const int f = fw % nf1 + 1, ln = fw / nf1;
    const int jj = ln % nc + 1, kk = D == 3 ? ln / nc + 1 : 1;
    const double inv_dr = -t.idr[slot * D + dim];
    int fidx, c1, c0;
    if (D == 2) {
      if (dim == 0) { fidx = fc_at(nf1, f, jj, 1); c1 = at2(n2, f, jj); c0 = at2(n2, f - 1, jj); }
      else { fidx = fc_at(nf1, jj, f, 1); c1 = at2(n2, jj, f); c0 = at2(n2, jj, f - 1); }
    } else if (dim == 0) { fidx = fc_at(nf1, f, jj, kk); c1 = at3(n2, f, jj, kk); c0 = at3(n2, f - 1, jj, kk); }
    else if (dim == 1) { fidx = fc_at(nf1, jj, f, kk); c1 = at3(n2, jj, f, kk); c0 = at3(n2, jj, f - 1, kk); }
    else { fidx = fc_at(nf1, jj, kk, f); c1 = at3(n2, jj, kk, f); c0 = at3(n2, jj, kk, f - 1); }
    efc[((size_t)slot * D + dim) * t.NF + fidx] = inv_dr * (p[c1] - p[c0]);
  }
  __syncthreads();
  const int ncell = D == 2 ? nc * nc : nc * nc * nc;
  const double* F0 = efc + ((size_t)slot * D + 0) * t.NF;
  const double* F1 = efc + ((size_t)slot * D + 1) * t.NF;
  for (int w = threadIdx.x; w < ncell; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 1 : r / nc + 1;
    const double a = F0[fc_at(nf1, i, j, k)] + F0[fc_at(nf1, i + 1, j, k)];
    const double b = F1[fc_at(nf1, i, j, k)] + F1[fc_at(nf1, i, j + 1, k)];
    double s = a * a + b * b;
    if (D == 3) {
      const double* F2 = efc + ((size_t)slot * D + 2) * t.NF;
      const double c = F2[fc_at(nf1, i, j, k)] + F2[fc_at(nf1, i, j, k + 1)];
      s = s + c * c;
    }
    enorm[(size_t)slot * t.S + (D == 2 ? at2(n2, i, j) : at3(n2, i, j, k))] = 0.5 * sqrt(s);
  }
}

// photoionization_rate_from_alpha (src/m_photoi.f90:259-291) on leaves
template <int D, int NC = 0>
__global__ void __launch_bounds__(256) k_photo_source(KTree t0, const int* __restrict__ list, const double* __restrict__ E,
                                                      const double* __restrict__ ne, double* __restrict__ rhs, LtDev lt,
                                                      int col_alpha, int col_mu, double N, double coeff) {
  const KTree t = fix_dims<D, NC>(t0);
  const int slot = list[blockIdx.x];
  const int nc = t.nc, n2 = t.n2;
  const int ncell = D == 2 ? nc * nc : nc * nc * nc;
  const size_t base = (size_t)slot * t.S;
  for (int w = threadIdx.x; w < ncell; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 0 : r / nc + 1;
    const int x = D == 2 ? at2(n2, i, j) : at3(n2, i, j, k);
    const double fld = E[base + x];
    const double td = fld * kSiToTd / N;
    int ix;
    double w_;
    lt_loc(lt, td, ix, w_);
    const double alpha = lt_col(lt, col_alpha, ix, w_);
    const double mob = lt_col(lt, col_mu, ix, w_);
    double tmp = fld * mob * alpha * ne[base + x] * coeff;
    if (tmp < 0) tmp = 0;
    rhs[base + x] = tmp;
  }
}

// i_photo = i_photo - coeff * phi_n on whole leaf arrays
static __global__ void __launch_bounds__(256) k_axpy_boxes(int S, const int* __restrict__ list, double* __restrict__ y,
                                                    const double* __restrict__ x, double c) {
  const size_t base = (size_t)list[blockIdx.x] * S;
  for (int q = threadIdx.x; q < S; q += blockDim.x) y[base + q] = y[base + q] - c * x[base + q];
}

}  // namespace afg
