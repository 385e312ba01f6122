// afg_lsf.cuh -- multigrid with an electrode (internal Dirichlet boundary
// given by a level-set function), FP64: the boxes the electrode surface
// crosses carry a per-cell 5/7-point stencil v and boundary-value factor f
// (mg_box_lsf_stencil, afivo/src/m_af_multigrid.f90:1779-1853) and the
// right-hand-side correction bcc = f * boundary value
// (mg_set_operators_lvl, 1169-1174).  The V-cycle kernels of ordinary boxes
// skip these boxes (KTree::lsf) and the kernels here process them with the
// reference's variable-stencil arithmetic:
//   k_lsf_gsrb        stencil_gsrb_357 (m_af_stencil.f90:838-998): rhs += bcc,
//                     the half sweep with division by v(1), rhs -= bcc
//   k_lsf_residual    residual_box (m_af_multigrid.f90:801-810) with
//                     stencil_apply_357 (m_af_stencil.f90:367-496)
//   k_lsf_rrestrict   update_coarse's residual + restriction (691-719)
//   k_lsf_coarse_fas  update_coarse's rhs = L phi + tmp on parents (723-737)
//   k_lsf_coarse_bcc  the level-set term of the coarse right-hand side
//                     (coarse_solver_set_rhs_phi, m_coarse_solver.f90:323-327)
//   k_lsf_grad        mg_box_lpllsf_gradient (m_af_multigrid.f90:2049-2141)
//                     and the field norm on leaf boxes
// and the set-up kernels: level-set values (set_lsf_box, src/m_field.f90:
// 673-683), root mask, distances and stencils (store_lsf_distance_matrix,
// m_af_multigrid.f90:977-1097) and boundary values.
#pragma once
#include "afg_lsf.h"

namespace afg {

struct LsfDev {
  const int* idx;     // [n_boxes] index of a slot's electrode data or -1
  const double* v;    // [n][2D+1][SI] stencil: centre, i-1, i+1, j-1, j+1(, k-1, k+1)
  const double* bcc;  // [n][SI] right-hand-side correction f * boundary value
  const double* bv;   // [n][SI] boundary value at the cell centre
  const double* dd;   // [n][2D][SI] relative boundary distances (1 = none)
  int SI;
};

// interior cell c (i fastest) -> (i, j, k), 1-based
template <int D>
__device__ __forceinline__ void lsf_ijk(int nc, int c, int& i, int& j, int& k) {
  i = c % nc + 1;
  j = (c / nc) % nc + 1;
  k = D == 3 ? c / (nc * nc) + 1 : 0;
}

template <int D>
__device__ __forceinline__ int lsf_at(int n2, int i, int j, int k) {
  return D == 2 ? at2(n2, i, j) : at3(n2, i, j, k);
}

// value of neighbour nb (0: i-1, 1: i+1, 2: j-1, ...) of interior cell
// (i, j, k): a cell of the box, or across a box face the stored ghost cell
// (otf = 0) or the value the ghost-cell rule gives now (otf = 1)
template <int D>
__device__ __forceinline__ double lsf_nbv(const KTree& t, const double* __restrict__ phi, const double* __restrict__ p,
                                          int slot, int i, int j, int k, int nb, const GcDev& g, int otf) {
  const int nc = t.nc, n2 = t.n2;
  const int d = nb >> 1, s = (nb & 1) ? 1 : -1;
  const int ci[3] = {i, j, k};
  const int x = lsf_at<D>(n2, i, j, k);
  const int stride = d == 0 ? 1 : d == 1 ? n2 : n2 * n2;
  const bool face = (s < 0 && ci[d] == 1) || (s > 0 && ci[d] == nc);
  if (face && otf) {
    const int pp = d == 0 ? j : i, qq = d == 2 ? j : (D == 3 ? k : 0);
    return face_ghost<D, double>(t, phi, slot, nb, pp, qq, g);
  }
  return p[x + s * stride];
}

// One half sweep on the electrode boxes of a level.  bcc applied: the
// right-hand side gets +bcc before and -bcc after the sweep in every cell,
// as the reference modifies the stored rhs (rounding included).
template <int D>
__global__ void __launch_bounds__(256) k_lsf_gsrb(KTree t, LsfDev L, const int* __restrict__ list,
                                                  double* __restrict__ phi, double* __restrict__ rhs, int redblack,
                                                  GcDev g, int otf, int use_bcc) {
  const int slot = list[blockIdx.x];
  const int q = L.idx[slot], SI = L.SI, nc = t.nc, n2 = t.n2;
  double* p = phi + (size_t)slot * t.S;
  double* f = rhs + (size_t)slot * t.S;
  const double* bcc = L.bcc + (size_t)q * SI;
  int i, j, k;
  if (use_bcc) {
    for (int c = threadIdx.x; c < SI; c += blockDim.x) {
      lsf_ijk<D>(nc, c, i, j, k);
      const int x = lsf_at<D>(n2, i, j, k);
      f[x] = f[x] + bcc[c];
    }
    __syncthreads();
  }
  const double* v = L.v + (size_t)q * (2 * D + 1) * SI;
  for (int c = threadIdx.x; c < SI; c += blockDim.x) {
    lsf_ijk<D>(nc, c, i, j, k);
    if (((i + j + (D == 3 ? k : 0) + redblack) & 1) != 0) continue;
    const int x = lsf_at<D>(n2, i, j, k);
    double nbv[6];
    for (int nb = 0; nb < 2 * D; nb++) nbv[nb] = lsf_nbv<D>(t, phi, p, slot, i, j, k, nb, g, otf);
    double val = f[x];
    for (int nb = 0; nb < 2 * D; nb++) val = val - v[(size_t)(nb + 1) * SI + c] * nbv[nb];
    p[x] = val / v[c];
  }
  if (use_bcc) {
    __syncthreads();
    for (int c = threadIdx.x; c < SI; c += blockDim.x) {
      lsf_ijk<D>(nc, c, i, j, k);
      const int x = lsf_at<D>(n2, i, j, k);
      f[x] = f[x] - bcc[c];
    }
  }
}

// stencil_apply_357 of a variable stencil, then - bcc
template <int D>
__device__ __forceinline__ double lsf_apply(const KTree& t, const LsfDev& L, int q, int c, const double* __restrict__ phi,
                                            const double* __restrict__ p, int slot, int i, int j, int k,
                                            const GcDev& g, int otf, int use_bcc) {
  const int SI = L.SI;
  const double* v = L.v + (size_t)q * (2 * D + 1) * SI;
  const int x = lsf_at<D>(t.n2, i, j, k);
  double acc = v[c] * p[x];
  for (int nb = 0; nb < 2 * D; nb++) acc = acc + v[(size_t)(nb + 1) * SI + c] * lsf_nbv<D>(t, phi, p, slot, i, j, k, nb, g, otf);
  if (use_bcc) acc = acc - L.bcc[(size_t)q * SI + c];
  return acc;
}

// residual_box on the electrode boxes: tmp = rhs - (L phi - bcc), stored
// ghost cells; |tmp| of leaves folded into *maxbits (may be null)
template <int D>
__global__ void __launch_bounds__(256) k_lsf_residual(KTree t, LsfDev L, const int* __restrict__ list,
                                                      const double* __restrict__ phi, const double* __restrict__ rhs,
                                                      double* __restrict__ tmp, GcDev g,
                                                      const unsigned char* __restrict__ is_leaf,
                                                      unsigned long long* maxbits, int use_bcc) {
  __shared__ double sred[32];
  const int slot = list[blockIdx.x];
  const int q = L.idx[slot], SI = L.SI, nc = t.nc, n2 = t.n2;
  const double* p = phi + (size_t)slot * t.S;
  const double* f = rhs + (size_t)slot * t.S;
  double* o = tmp + (size_t)slot * t.S;
  double mx = 0.0;
  int i, j, k;
  for (int c = threadIdx.x; c < SI; c += blockDim.x) {
    lsf_ijk<D>(nc, c, i, j, k);
    const int x = lsf_at<D>(n2, i, j, k);
    const double r = f[x] - lsf_apply<D>(t, L, q, c, phi, p, slot, i, j, k, g, 0, use_bcc);
    o[x] = r;
    acc_absmax(mx, r);
  }
  if (maxbits != nullptr && is_leaf[slot]) {
    mx = block_max<double>(mx, sred);
    if (threadIdx.x == 0) atomic_max_nonneg(maxbits, mx);
  }
}

// update_coarse / set_coarse_phi_rhs on electrode child boxes: the residual
// with the electrode stencil (optionally stored in the child's tmp), its
// restriction (cylindrical weights in 2D axisymmetric trees) and phi's
// restriction to the parent, in k_residual_restrict's operation order.
// Dynamic shared memory: SI doubles.
template <int D, bool CYL>
__global__ void __launch_bounds__(256) k_lsf_rrestrict(KTree t, LsfDev L, const int* __restrict__ list,
                                                       double* __restrict__ phi, const double* __restrict__ rhs,
                                                       double* __restrict__ tmp, int store_child, GcDev g, int otf,
                                                       int use_bcc) {
  extern __shared__ double sres[];
  const int slot = list[blockIdx.x];
  const int q = L.idx[slot], SI = L.SI, nc = t.nc, n2 = t.n2, hnc = nc / 2;
  const int pslot = t.parent[slot];
  const double* p = phi + (size_t)slot * t.S;
  const double* f = rhs + (size_t)slot * t.S;
  double* ct = tmp + (size_t)slot * t.S;
  int i, j, k;
  for (int c = threadIdx.x; c < SI; c += blockDim.x) {
    lsf_ijk<D>(nc, c, i, j, k);
    const int x = lsf_at<D>(n2, i, j, k);
    const double r = f[x] - lsf_apply<D>(t, L, q, c, phi, p, slot, i, j, k, g, otf, use_bcc);
    sres[c] = r;
    if (store_child) ct[x] = r;
  }
  __syncthreads();
  double* pp = phi + (size_t)pslot * t.S;
  double* pt = tmp + (size_t)pslot * t.S;
  const int o0 = child_offset(t, slot, 0), o1 = child_offset(t, slot, 1);
  const int o2 = D == 3 ? child_offset(t, slot, 2) : 0;
  const int count = D == 2 ? hnc * hnc : hnc * hnc * hnc;
  for (int w = threadIdx.x; w < count; w += blockDim.x) {
    const int a = w % hnc + 1, r = w / hnc;
    const int b = D == 2 ? r + 1 : r % hnc + 1, e = D == 2 ? 0 : r / hnc + 1;
    const int fi = 2 * a - 1, fj = 2 * b - 1, fk = D == 3 ? 2 * e - 1 : 1;
    auto cidx = [&](int ii, int jj, int kk) { return (ii - 1) + nc * ((jj - 1) + nc * (D == 3 ? kk - 1 : 0)); };
    if (D == 2) {
      const double r00 = sres[cidx(fi, fj, 0)], r01 = sres[cidx(fi + 1, fj, 0)];
      const double r10 = sres[cidx(fi, fj + 1, 0)], r11 = sres[cidx(fi + 1, fj + 1, 0)];
      double rv;
      if (CYL) {
        const double* gw = t.geo + ((size_t)pslot * nc + (o0 + a - 1)) * 4;
        double s1 = 0.0, s2 = 0.0;
        s1 = s1 + r00; s1 = s1 + r10;
        s2 = s2 + r01; s2 = s2 + r11;
        rv = 0.25 * (gw[2] * s1 + gw[3] * s2);
      } else {
        double s = 0.0;
        s = s + r00; s = s + r01; s = s + r10; s = s + r11;
        rv = 0.25 * s;
      }
      pt[at2(n2, o0 + a, o1 + b)] = rv;
      double s = 0.0;
      s = s + p[at2(n2, fi, fj)]; s = s + p[at2(n2, fi + 1, fj)];
      s = s + p[at2(n2, fi, fj + 1)]; s = s + p[at2(n2, fi + 1, fj + 1)];
      pp[at2(n2, o0 + a, o1 + b)] = 0.25 * s;
    } else {
      double sr = 0.0, sp = 0.0;
      for (int dk = 0; dk < 2; dk++)
        for (int dj = 0; dj < 2; dj++)
          for (int di = 0; di < 2; di++) {
            sr = sr + sres[cidx(fi + di, fj + dj, fk + dk)];
            sp = sp + p[at3(n2, fi + di, fj + dj, fk + dk)];
          }
      pt[at3(n2, o0 + a, o1 + b, o2 + e)] = 0.125 * sr;
      pp[at3(n2, o0 + a, o1 + b, o2 + e)] = 0.125 * sp;
    }
  }
}

// update_coarse's second half on electrode parents: optional ghost fill of
// phi (faces, then edges and corners), rhs = (L phi - bcc) + tmp on the
// interior, tmp = phi on the whole array when copy_tmp
template <int D>
__global__ void __launch_bounds__(256) k_lsf_coarse_fas(KTree t, LsfDev L, const int* __restrict__ list,
                                                        double* __restrict__ phi, double* __restrict__ rhs,
                                                        double* __restrict__ tmp, int copy_tmp, int fill, GcDev g,
                                                        int use_bcc) {
  const int slot = list[blockIdx.x];
  const int q = L.idx[slot], nc = t.nc, n2 = t.n2;
  if (fill) {
    double* a = phi + (size_t)slot * t.S;
    const int nface = D == 2 ? nc : nc * nc;
    for (int w = threadIdx.x; w < 2 * D * nface; w += blockDim.x) {
      const int nb = w / nface, pq = w - nb * nface;
      const int pi = pq % nc + 1, qi = D == 3 ? pq / nc + 1 : 0;
      const double val = face_ghost<D, double>(t, phi, slot, nb, pi, qi, g);
      a[face_at<D>(n2, nb >> 1, (nb & 1) ? nc + 1 : 0, pi, qi)] = val;
    }
    __syncthreads();
    corner_ghosts<D, double>(t, phi, slot);
    __syncthreads();
  }
  const double* p = phi + (size_t)slot * t.S;
  double* f = rhs + (size_t)slot * t.S;
  double* o = tmp + (size_t)slot * t.S;
  for (int x = threadIdx.x; x < t.S; x += blockDim.x) {
    const int i = x % n2, r = x / n2;
    const int j = D == 2 ? r : r % n2, k = D == 2 ? 0 : r / n2;
    const bool interior = i >= 1 && i <= nc && j >= 1 && j <= nc && (D == 2 || (k >= 1 && k <= nc));
    if (interior) {
      const int c = (i - 1) + nc * ((j - 1) + nc * (D == 3 ? k - 1 : 0));
      const double lp = lsf_apply<D>(t, L, q, c, phi, p, slot, i, j, k, g, 0, use_bcc);
      f[x] = lp + o[x];
    }
  }
  if (copy_tmp) {
    __syncthreads();
    for (int x = threadIdx.x; x < t.S; x += blockDim.x) o[x] = p[x];
  }
}

// b[cg[n]] += bcc_flat[ck[n]]: the boundary-value term of the coarse
// right-hand side for the cells of level-1 electrode boxes
__global__ void k_lsf_coarse_bcc(int n, const int* __restrict__ cg, const int* __restrict__ ck,
                                 const double* __restrict__ bcc, double* __restrict__ b) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w < n) b[cg[w]] = b[cg[w]] + bcc[ck[w]];
}

// mg_box_lpllsf_gradient on electrode leaf boxes (after the regular
// gradient): faces next to a boundary point get (phi - bc) / (dd dx) from
// cells on the positive side of the level-set function, in the order of the
// stored cells (one thread: later cells overwrite shared faces as in the
// reference's loop); then the field norm of every cell of the box
// (mg_box_field_norm).
template <int D>
__global__ void k_lsf_grad(KTree t, LsfDev L, const int* __restrict__ list, const double* __restrict__ phi,
                           const double* __restrict__ lsfv, double* __restrict__ efc, double* __restrict__ enorm) {
  const int slot = list[blockIdx.x];
  const int q = L.idx[slot], SI = L.SI, nc = t.nc, n2 = t.n2, nf1 = nc + 1;
  const double* p = phi + (size_t)slot * t.S;
  const double* ls = lsfv + (size_t)slot * t.S;
  const double* dd = L.dd + (size_t)q * 2 * D * SI;
  const double* bv = L.bv + (size_t)q * SI;
  if (threadIdx.x == 0) {
    for (int c = 0; c < SI; c++) {
      bool any = false;
      for (int nb = 0; nb < 2 * D; nb++) any = any || dd[(size_t)nb * SI + c] < 1.0;
      if (!any) continue;
      int i, j, k;
      lsf_ijk<D>(nc, c, i, j, k);
      const int x = lsf_at<D>(n2, i, j, k);
      if (!(ls[x] >= 0)) continue;
      const int kk = D == 3 ? k : 1;
      for (int nb = 0; nb < 2 * D; nb++) {
        const double dn = dd[(size_t)nb * SI + c];
        if (!(dn < 1)) continue;
        const int dim = nb >> 1;
        const double inv_dr = -t.idr[slot * D + dim];
        const bool hi = nb & 1;
        int fidx;
        if (dim == 0) fidx = fc_at(nf1, hi ? i + 1 : i, j, kk);
        else if (dim == 1) fidx = fc_at(nf1, i, hi ? j + 1 : j, kk);
        else fidx = fc_at(nf1, i, j, hi ? kk + 1 : kk);
        const double val = hi ? inv_dr * (bv[c] - p[x]) / dn : inv_dr * (p[x] - bv[c]) / dn;
        efc[((size_t)slot * D + dim) * t.NF + fidx] = val;
      }
    }
  }
  __syncthreads();
  const double* F0 = efc + ((size_t)slot * D + 0) * t.NF;
  const double* F1 = efc + ((size_t)slot * D + 1) * t.NF;
  for (int w = threadIdx.x; w < SI; w += blockDim.x) {
    int i, j, k;
    lsf_ijk<D>(nc, w, i, j, k);
    const int kk = D == 3 ? k : 1;
    const double a = F0[fc_at(nf1, i, j, kk)] + F0[fc_at(nf1, i + 1, j, kk)];
    const double b = F1[fc_at(nf1, i, j, kk)] + F1[fc_at(nf1, i, j + 1, kk)];
    double s = a * a + b * b;
    if (D == 3) {
      const double* F2 = efc + ((size_t)slot * D + 2) * t.NF;
      const double cz = F2[fc_at(nf1, i, j, kk)] + F2[fc_at(nf1, i, j, kk + 1)];
      s = s + cz * cz;
    }
    enorm[(size_t)slot * t.S + lsf_at<D>(n2, i, j, k)] = 0.5 * sqrt(s);
  }
}

/* ---- set-up kernels ------------------------------------------------------ */

// set_lsf_box: the level-set value at every cell centre, ghost cells included
template <int D>
__global__ void k_lsf_values(KTree t, const int* __restrict__ list, afg_lsf::Electrode e, double* __restrict__ lsfv) {
  const int slot = list[blockIdx.x];
  const int n2 = t.n2;
  const double* rm = t.r_min + (size_t)slot * D;
  const double* dr = t.dr + (size_t)slot * D;
  for (int x = threadIdx.x; x < t.S; x += blockDim.x) {
    const int ix[3] = {x % n2, (x / n2) % n2, D == 3 ? x / (n2 * n2) : 0};
    double r[3];
    afg_lsf::r_cc(rm, dr, D, ix, r);
    lsfv[(size_t)slot * t.S + x] = afg_lsf::eval(e, r);
  }
}

// number of root-mask cells per box (get_possible_lsf_root_mask)
template <int D>
__global__ void k_lsf_mask(KTree t, const int* __restrict__ list, afg_lsf::Electrode e, int* __restrict__ count) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  const int slot = list[blockIdx.x];
  const int nc = t.nc, SI = D == 2 ? nc * nc : nc * nc * nc;
  const double* rm = t.r_min + (size_t)slot * D;
  const double* dr = t.dr + (size_t)slot * D;
  for (int c = threadIdx.x; c < SI; c += blockDim.x) {
    int i, j, k;
    lsf_ijk<D>(nc, c, i, j, k);
    const int ix[3] = {i, j, k};
    double a[3], g[3];
    afg_lsf::r_cc(rm, dr, D, ix, a);
    const double l = afg_lsf::eval(e, a);
    afg_lsf::numerical_gradient(e, a, g);
    const double al = l < 0 ? -l : l;
    if (al < afg_lsf::norm2(dr, D) * afg_lsf::norm2(g, D) * e.safety) atomicAdd(&cnt, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) count[blockIdx.x] = cnt;
}

// distances of the cells of root-mask boxes: dd[(b * 2D + n) * SI + c];
// any[b] = 1 when a distance is below 1
template <int D>
__global__ void k_lsf_dist(KTree t, const int* __restrict__ list, afg_lsf::Electrode e, double* __restrict__ dd,
                           int* __restrict__ any) {
  const int slot = list[blockIdx.x];
  const int nc = t.nc, SI = D == 2 ? nc * nc : nc * nc * nc;
  const double* rm = t.r_min + (size_t)slot * D;
  const double* dr = t.dr + (size_t)slot * D;
  for (int c = threadIdx.x; c < SI; c += blockDim.x) {
    int i, j, k;
    lsf_ijk<D>(nc, c, i, j, k);
    const int ix[3] = {i, j, k};
    double d[6];
    afg_lsf::cell_distances(e, rm, dr, ix, d);
    bool lt = false;
    for (int n = 0; n < 2 * D; n++) {
      dd[((size_t)blockIdx.x * 2 * D + n) * SI + c] = d[n];
      lt = lt || d[n] < 1.0;
    }
    if (lt) atomicOr(any + blockIdx.x, 1);
  }
}

// stencils of the electrode boxes from their distances: v, f, dd
template <int D>
__global__ void k_lsf_stencil(KTree t, const int* __restrict__ slots, const int* __restrict__ src,
                              const double* __restrict__ dd_tmp, int cyl, double* __restrict__ v,
                              double* __restrict__ f, double* __restrict__ dd) {
  const int q = blockIdx.x, slot = slots[q], b = src[q];
  const int nc = t.nc, SI = D == 2 ? nc * nc : nc * nc * nc;
  const double* rm = t.r_min + (size_t)slot * D;
  const double* dr = t.dr + (size_t)slot * D;
  for (int c = threadIdx.x; c < SI; c += blockDim.x) {
    double d[6], w[7], fv;
    for (int n = 0; n < 2 * D; n++) {
      d[n] = dd_tmp[((size_t)b * 2 * D + n) * SI + c];
      dd[((size_t)q * 2 * D + n) * SI + c] = d[n];
    }
    const int i = c % nc + 1;
    afg_lsf::cell_stencil(D, cyl != 0, rm, dr, i, d, w, fv);
    for (int n = 0; n <= 2 * D; n++) v[((size_t)q * (2 * D + 1) + n) * SI + c] = w[n];
    f[(size_t)q * SI + c] = fv;
  }
}

// boundary values and bcc = f * boundary value
template <int D>
__global__ void k_lsf_bcc(KTree t, const int* __restrict__ slots, afg_lsf::Electrode e, double voltage,
                          const double* __restrict__ f, double* __restrict__ bv, double* __restrict__ bcc) {
  const int q = blockIdx.x, slot = slots[q];
  const int nc = t.nc, SI = D == 2 ? nc * nc : nc * nc * nc;
  const double* rm = t.r_min + (size_t)slot * D;
  const double* dr = t.dr + (size_t)slot * D;
  for (int c = threadIdx.x; c < SI; c += blockDim.x) {
    int i, j, k;
    lsf_ijk<D>(nc, c, i, j, k);
    const int ix[3] = {i, j, k};
    double r[3];
    afg_lsf::r_cc(rm, dr, D, ix, r);
    const double b = afg_lsf::boundary_value(e, r, voltage);
    bv[(size_t)q * SI + c] = b;
    bcc[(size_t)q * SI + c] = f[(size_t)q * SI + c] * b;
  }
}

/* ---- electrode rules of the streamer's densities ----------------------- */

struct DensPtrs {
  int ns;
  double* p[AFG_MAX_SPECIES];
};

// init_cond_set_box's electrode rule (src/m_init_cond.f90:284-288), every
// cell of the listed boxes, ghost cells included
__global__ void k_electrode_init(int S, const int* __restrict__ list, const double* __restrict__ lsfv, DensPtrs dn) {
  const size_t base = (size_t)list[blockIdx.x] * S;
  for (int x = threadIdx.x; x < S; x += blockDim.x)
    if (lsfv[base + x] <= 0.0)
      for (int s = 0; s < dn.ns; s++) dn.p[s][base + x] = 0.0;
}

// electrode_species_bc (src/streamer.f90:598-656) on electrode boxes: cells
// inside the electrode lose their densities; next to a gas cell (and with
// Neumann species boundaries) they take the mean electron density of their
// gas neighbours, the ion density equal to it.  Only cells inside are
// written and only gas cells read, so the cells are independent.
template <int D>
__global__ void k_electrode_species_bc(KTree t, const int* __restrict__ list, const double* __restrict__ lsfv,
                                       DensPtrs dn, int ie, int ii, int neumann) {
  const int slot = list[blockIdx.x];
  const int nc = t.nc, n2 = t.n2, SI = D == 2 ? nc * nc : nc * nc * nc;
  const size_t base = (size_t)slot * t.S;
  for (int c = threadIdx.x; c < SI; c += blockDim.x) {
    int i, j, k;
    lsf_ijk<D>(nc, c, i, j, k);
    const int x = lsf_at<D>(n2, i, j, k);
    if (!(lsfv[base + x] < 0)) continue;
    for (int s = 0; s < dn.ns; s++) dn.p[s][base + x] = 0.0;
    const int st[3] = {1, n2, n2 * n2};
    bool any = false;
    for (int nb = 0; nb < 2 * D; nb++) any = any || lsfv[base + x + ((nb & 1) ? 1 : -1) * st[nb >> 1]] > 0;
    if (!(any && neumann)) continue;
    double sum = 0.0;
    int cnt = 0;
    for (int nb = 0; nb < 2 * D; nb++) {
      const int y = x + ((nb & 1) ? 1 : -1) * st[nb >> 1];
      if (lsfv[base + y] > 0) {
        sum = sum + dn.p[ie][base + y];
        cnt++;
      }
    }
    const double v = sum / (double)cnt;
    dn.p[ie][base + x] = v;
    dn.p[ii][base + x] = v;
  }
}

}  // namespace afg

/* ---- host side: launchers used by the multigrid driver ------------------ */

static afg::LsfDev lsf_dev(const LsfState& L) {
  afg::LsfDev d;
  d.idx = L.d_idx;
  d.v = L.d_v;
  d.bcc = L.d_bcc;
  d.bv = L.d_bv;
  d.dd = L.d_dd;
  d.SI = L.SI;
  return d;
}

// electrode boxes of a level (kind 0: all, 1: parents, 2: leaves)
static const std::vector<int>& lsf_list(const LsfState& L, int kind, int lvl) {
  return kind == 0 ? L.lvl_all[lvl - 1] : kind == 1 ? L.lvl_par[lvl - 1] : L.lvl_leaf[lvl - 1];
}
static const int* lsf_dlist(const LsfState& L, int kind, int lvl) {
  const std::vector<size_t>& off = kind == 0 ? L.off_all : kind == 1 ? L.off_par : L.off_leaf;
  return L.d_lists + off[lvl - 1];
}

static int launch_lsf_gsrb(afg_ctx* ctx, const MgSlot& m, int lvl, double* phi, double* rhs, int rb,
                           const GcDev& g, int otf) {
  const LsfState& L = *m.lsf;
  const int n = (int)lsf_list(L, 0, lvl).size();
  if (n == 0) return AFG_OK;
  KTree t = ktree(ctx);
  if (ctx->D == 3)
    afg::k_lsf_gsrb<3><<<n, 256, 0, ctx->stream>>>(t, lsf_dev(L), lsf_dlist(L, 0, lvl), phi, rhs, rb, g, otf, 1);
  else
    afg::k_lsf_gsrb<2><<<n, 256, 0, ctx->stream>>>(t, lsf_dev(L), lsf_dlist(L, 0, lvl), phi, rhs, rb, g, otf, 1);
  ctx->launches++;
  CKL();
  return AFG_OK;
}

static int launch_lsf_residual(afg_ctx* ctx, const MgSlot& m, int lvl, const double* phi, const double* rhs,
                               double* tmp, const GcDev& g, unsigned long long* maxbits) {
  const LsfState& L = *m.lsf;
  const int n = (int)lsf_list(L, 0, lvl).size();
  if (n == 0) return AFG_OK;
  KTree t = ktree(ctx);
  if (ctx->D == 3)
    afg::k_lsf_residual<3><<<n, 256, 0, ctx->stream>>>(t, lsf_dev(L), lsf_dlist(L, 0, lvl), phi, rhs, tmp, g,
                                                       ctx->d_is_leaf, maxbits, 1);
  else
    afg::k_lsf_residual<2><<<n, 256, 0, ctx->stream>>>(t, lsf_dev(L), lsf_dlist(L, 0, lvl), phi, rhs, tmp, g,
                                                       ctx->d_is_leaf, maxbits, 1);
  ctx->launches++;
  CKL();
  return AFG_OK;
}

static int launch_lsf_rrestrict(afg_ctx* ctx, const MgSlot& m, int lvl, double* phi, const double* rhs,
                                double* tmp, int store_child, const GcDev& g, int otf) {
  const LsfState& L = *m.lsf;
  const int n = (int)lsf_list(L, 0, lvl).size();
  if (n == 0) return AFG_OK;
  KTree t = ktree(ctx);
  const size_t smem = sizeof(double) * L.SI;
  if (ctx->D == 3)
    afg::k_lsf_rrestrict<3, false><<<n, 256, smem, ctx->stream>>>(t, lsf_dev(L), lsf_dlist(L, 0, lvl), phi, rhs, tmp,
                                                                  store_child, g, otf, 1);
  else if (ctx->coord == AFG_CYL)
    afg::k_lsf_rrestrict<2, true><<<n, 256, smem, ctx->stream>>>(t, lsf_dev(L), lsf_dlist(L, 0, lvl), phi, rhs, tmp,
                                                                 store_child, g, otf, 1);
  else
    afg::k_lsf_rrestrict<2, false><<<n, 256, smem, ctx->stream>>>(t, lsf_dev(L), lsf_dlist(L, 0, lvl), phi, rhs, tmp,
                                                                  store_child, g, otf, 1);
  ctx->launches++;
  CKL();
  return AFG_OK;
}

// on the electrode parents of level plvl
static int launch_lsf_coarse_fas(afg_ctx* ctx, const MgSlot& m, int plvl, double* phi, double* rhs, double* tmp,
                                 int copy_tmp, int fill, const GcDev& g) {
  const LsfState& L = *m.lsf;
  const int n = (int)lsf_list(L, 1, plvl).size();
  if (n == 0) return AFG_OK;
  KTree t = ktree(ctx);
  if (ctx->D == 3)
    afg::k_lsf_coarse_fas<3><<<n, 256, 0, ctx->stream>>>(t, lsf_dev(L), lsf_dlist(L, 1, plvl), phi, rhs, tmp, copy_tmp,
                                                         fill, g, 1);
  else
    afg::k_lsf_coarse_fas<2><<<n, 256, 0, ctx->stream>>>(t, lsf_dev(L), lsf_dlist(L, 1, plvl), phi, rhs, tmp, copy_tmp,
                                                         fill, g, 1);
  ctx->launches++;
  CKL();
  return AFG_OK;
}

static int launch_lsf_coarse_bcc(afg_ctx* ctx, const MgSlot& m, double* b) {
  const LsfState& L = *m.lsf;
  if (L.n_cb == 0) return AFG_OK;
  afg::k_lsf_coarse_bcc<<<(L.n_cb + 127) / 128, 128, 0, ctx->stream>>>(L.n_cb, L.d_cb_g, L.d_cb_k, L.d_bcc, b);
  ctx->launches++;
  CKL();
  return AFG_OK;
}

// the electrode slot of the field whose potential is i_phi (null if none)
static const MgSlot* lsf_slot_of(const afg_ctx* ctx, int i_phi) {
  for (const MgSlot& m : ctx->mg)
    if (m.used && m.lsf && m.d.i_phi == i_phi) return &m;
  return nullptr;
}

static int launch_lsf_grad(afg_ctx* ctx, const MgSlot& m, const double* phi, double* efc, double* enorm) {
  const LsfState& L = *m.lsf;
  KTree t = ktree(ctx);
  for (int lvl = 1; lvl <= ctx->highest_lvl; lvl++) {
    const int n = (int)lsf_list(L, 2, lvl).size();
    if (n == 0) continue;
    if (ctx->D == 3)
      afg::k_lsf_grad<3><<<n, 128, 0, ctx->stream>>>(t, lsf_dev(L), lsf_dlist(L, 2, lvl), phi, ctx->cc[L.i_lsf - 1],
                                                     efc, enorm);
    else
      afg::k_lsf_grad<2><<<n, 128, 0, ctx->stream>>>(t, lsf_dev(L), lsf_dlist(L, 2, lvl), phi, ctx->cc[L.i_lsf - 1],
                                                     efc, enorm);
    ctx->launches++;
    CKL();
  }
  return AFG_OK;
}

static int lsf_set_voltage(afg_ctx* ctx, MgSlot& m, double voltage) {
  LsfState& L = *m.lsf;
  L.voltage = voltage;
  if (L.n == 0) return AFG_OK;
  KTree t = ktree(ctx);
  if (ctx->D == 3)
    afg::k_lsf_bcc<3><<<L.n, 128, 0, ctx->stream>>>(t, L.d_slots, L.e, voltage, L.d_f, L.d_bv, L.d_bcc);
  else
    afg::k_lsf_bcc<2><<<L.n, 128, 0, ctx->stream>>>(t, L.d_slots, L.e, voltage, L.d_f, L.d_bv, L.d_bcc);
  ctx->launches++;
  CKL();
  return AFG_OK;
}
