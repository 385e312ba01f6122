// afg_gc_kernels.cuh -- ghost-cell fill of one level's boxes (af_gc_box,
// afivo/src/m_af_ghostcell.f90:64-120).  One CTA per box: face ghosts first
// (same-level copy copy_from_nb 654-669, physical bc_to_gc 173-279, or the
// refinement rule mg_sides_rb m_af_multigrid.f90:294-461 / af_gc_interp
// 394-498 / af_gc_interp_lim 503-612), then in 3D the edge ghosts and finally
// the corners (af_gc_box_corner 125-170 with the extrapolations 860-924).
// Every value is computed with the reference's operation order.
#pragma once
#include "afg_common.cuh"

namespace afg {

template <int D, typename T>
__device__ __forceinline__ T bc_ghost(int type, double bval, double drd, bool low, T x1, T x2) {
  T c0, c1, c2;
  switch (type) {
    case -10: c0 = T(2); c1 = T(-1); c2 = T(0); break;                 // Dirichlet
    case -11: c0 = T(drd * (low ? -1 : 1)); c1 = T(1); c2 = T(0); break; // Neumann
    case -12: c0 = T(0); c1 = T(2); c2 = T(-1); break;                 // continuous
    default: c0 = T(1); c1 = T(0); c2 = T(0); break;                   // dirichlet copy
  }
  return c0 * T(bval) + c1 * x1 + c2 * x2;
}

// Ghost value of face nb at tangential position (p,q) of box `slot`, whose
// neighbour across that face is nbs (a slot, kNbRefine or kNbPhys).
template <int D, typename T>
__device__ __forceinline__ T face_ghost_nb(const KTree& t, const T* __restrict__ v, int slot, int nb, int nbs,
                                           int p, int q, const GcDev& g) {
  const int nc = t.nc, n2 = t.n2, S = t.S, d = nb >> 1;
  const bool low = (nb & 1) == 0;
  const T* a = v + (size_t)slot * S;
  if (nbs >= 0) {
    const T* b = v + (size_t)nbs * S;
    return b[face_at<D>(n2, d, low ? nc : 1, p, q)];
  }
  if (nbs == kNbPhys) {
    const int i1 = low ? 1 : nc, i2 = low ? 2 : nc - 1;
    return bc_ghost<D, T>(gc_type(g, nb), gc_val(g, nb, t, slot), t.dr[slot * D + d], low,
                          a[face_at<D>(n2, d, i1, p, q)], a[face_at<D>(n2, d, i2, p, q)]);
  }
  // refinement boundary: data of the parent's neighbour
  const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
  const int cs = t.pnb[slot * 2 * D + nb];
  const T* C = v + (size_t)cs * S;
  const int off1 = child_offset(t, slot, t1);
  const int off2 = D == 3 ? child_offset(t, slot, t2) : 0;
  const int cx = low ? nc : 1;
  if (g.rb == 0) {
    // mg_sides_rb: slope-corrected coarse value next to the fine cell, then
    // 0.5*gc + 0.75*phi(1) - 0.25*phi(2)
    const int ix = low ? 1 : nc, dix = low ? 1 : -1;
    T gcv;
    if (D == 2) {
      const int i = (p + 1) >> 1;  // tmp index
      const T tm = C[face_at<D>(n2, d, cx, off1 + i - 1, 0)];
      const T t0 = C[face_at<D>(n2, d, cx, off1 + i, 0)];
      const T tp = C[face_at<D>(n2, d, cx, off1 + i + 1, 0)];
      const T grad = T(0.125) * (tp - tm);
      gcv = (p & 1) ? t0 - grad : t0 + grad;
    } else {
      const int i = (p + 1) >> 1, j = (q + 1) >> 1;
      const T t0 = C[face_at<D>(n2, d, cx, off1 + i, off2 + j)];
      const T g1 = T(0.125) * (C[face_at<D>(n2, d, cx, off1 + i + 1, off2 + j)] -
                               C[face_at<D>(n2, d, cx, off1 + i - 1, off2 + j)]);
      const T g2 = T(0.125) * (C[face_at<D>(n2, d, cx, off1 + i, off2 + j + 1)] -
                               C[face_at<D>(n2, d, cx, off1 + i, off2 + j - 1)]);
      const T s1 = (p & 1) ? t0 - g1 : t0 + g1;
      gcv = (q & 1) ? s1 - g2 : s1 + g2;
    }
    return T(0.5) * gcv + T(0.75) * a[face_at<D>(n2, d, ix, p, q)] -
           T(0.25) * a[face_at<D>(n2, d, ix + dix, p, q)];
  }
  // af_gc_interp(_lim)
  const T third = T(1 / 3.0), sixth = T(1 / 6.0);
  const int p1 = off1 + ((p + 1) >> 1), p2 = p1 + 1 - 2 * (p & 1);
  const T f = a[face_at<D>(n2, d, low ? 1 : nc, p, q)];
  T val, c1;
  if (D == 2) {
    c1 = C[face_at<D>(n2, d, cx, p1, 0)];
    const T c2 = C[face_at<D>(n2, d, cx, p2, 0)];
    val = T(0.5) * c1 + sixth * c2 + third * f;
  } else {
    const int q1 = off2 + ((q + 1) >> 1), q2 = q1 + 1 - 2 * (q & 1);
    c1 = C[face_at<D>(n2, d, cx, p1, q1)];
    T c2, c3;
    if (d < 2) {
      c2 = C[face_at<D>(n2, d, cx, p2, q1)];
      c3 = C[face_at<D>(n2, d, cx, p1, q2)];
    } else {
      c2 = C[face_at<D>(n2, d, cx, p1, q2)];
      c3 = C[face_at<D>(n2, d, cx, p2, q1)];
    }
    val = third * c1 + sixth * c2 + sixth * c3 + third * f;
  }
  if (g.rb == 2 && val > T(2) * c1) val = T(2) * c1;
  return val;
}

// face_ghost_nb with the neighbour slot from the tree's table
template <int D, typename T>
__device__ __forceinline__ T face_ghost(const KTree& t, const T* __restrict__ v, int slot, int nb, int p, int q,
                                        const GcDev& g) {
  return face_ghost_nb<D, T>(t, v, slot, nb, t.nbr[slot * 2 * D + nb], p, q, g);
}

__constant__ int c_edge_dim[12] = {0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2};
__constant__ int c_edge_dir[12][3] = {{0, -1, -1}, {0, 1, -1}, {0, -1, 1}, {0, 1, 1},
                                      {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1}, {1, 0, 1},
                                      {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 1, 0}};

__device__ __forceinline__ int nbmat_at(const KTree& t, int slot, int dx, int dy, int dz) {
  const int nm = t.D == 2 ? 9 : 27;
  const int k = (dx + 1) + 3 * (dy + 1) + (t.D == 3 ? 9 * (dz + 1) : 0);
  return t.nbmat[slot * nm + k];
}

// Edge (3D) and corner ghosts of one box; face ghosts must be in place.
// Threads lane, lane + nl, ... of the CTA work on the box (all threads of
// the CTA reach the barrier; active == false: the box is skipped).
template <int D, typename T>
__device__ void corner_ghosts(const KTree& t, T* __restrict__ v, int slot, int lane, int nl, bool active) {
  const int nc = t.nc, n2 = t.n2;
  T* a = v + (size_t)slot * t.S;
  if (D == 3) {
    for (int w = lane; active && w < 12 * nc; w += nl) {
      const int n = w / nc, pp = w % nc + 1;
      const int dim = c_edge_dim[n];
      const int dx = c_edge_dir[n][0], dy = c_edge_dir[n][1], dz = c_edge_dir[n][2];
      // the edge cell (kept in scalars: no dynamically indexed arrays)
      const int x0 = dim == 0 ? pp : (dx == 1) * (nc + 1);
      const int x1 = dim == 1 ? pp : (dy == 1) * (nc + 1);
      const int x2 = dim == 2 ? pp : (dz == 1) * (nc + 1);
      const int c = at3(n2, x0, x1, x2);
      const int nbs = nbmat_at(t, slot, dx, dy, dz);
      if (nbs >= 0) {
        const T* b = v + (size_t)nbs * t.S;
        a[c] = b[at3(n2, x0 - dx * nc, x1 - dy * nc, x2 - dz * nc)];
      } else {
        // steps towards the interior across the two other dimensions o1 =
        // dim+1, o2 = dim+2 (mod 3): a(o1 step) + a(o2 step) - a(both)
        const int s0 = dim == 0 ? 0 : 1 - 2 * (x0 & 1);
        const int s1 = dim == 1 ? 0 : (1 - 2 * (x1 & 1)) * n2;
        const int s2 = dim == 2 ? 0 : (1 - 2 * (x2 & 1)) * n2 * n2;
        const int ua = dim == 0 ? c + s1 : (dim == 1 ? c + s2 : c + s0);
        const int ub = dim == 0 ? c + s2 : (dim == 1 ? c + s0 : c + s1);
        a[c] = a[ua] + a[ub] - a[c + s0 + s1 + s2];
      }
    }
    __syncthreads();
  }
  const int nch = 1 << D;
  for (int n = lane; active && n < nch; n += nl) {
    const int cd0 = n & 1, cd1 = (n >> 1) & 1, cd2 = (n >> 2) & 1;
    const int dx = 2 * cd0 - 1, dy = 2 * cd1 - 1, dz = D == 3 ? 2 * cd2 - 1 : 0;
    const int x = cd0 * (nc + 1), y = cd1 * (nc + 1), z = D == 3 ? cd2 * (nc + 1) : 0;
    const int nbs = nbmat_at(t, slot, dx, dy, dz);
    const int di = 1 - 2 * (x & 1), dj = 1 - 2 * (y & 1), dk = 1 - 2 * (z & 1);
    if (D == 2) {
      if (nbs >= 0) {
        const T* b = v + (size_t)nbs * t.S;
        a[at2(n2, x, y)] = b[at2(n2, x - dx * nc, y - dy * nc)];
      } else {
        a[at2(n2, x, y)] = a[at2(n2, x + di, y)] + a[at2(n2, x, y + dj)] - a[at2(n2, x + di, y + dj)];
      }
    } else {
      if (nbs >= 0) {
        const T* b = v + (size_t)nbs * t.S;
        a[at3(n2, x, y, z)] = b[at3(n2, x - dx * nc, y - dy * nc, z - dz * nc)];
      } else {
        a[at3(n2, x, y, z)] = a[at3(n2, x, y + dj, z + dk)] + a[at3(n2, x + di, y, z + dk)] +
                              a[at3(n2, x + di, y + dj, z)] - T(2) * a[at3(n2, x + di, y + dj, z + dk)];
      }
    }
  }
}

// the whole CTA on one box
template <int D, typename T>
__device__ void corner_ghosts(const KTree& t, T* __restrict__ v, int slot) {
  corner_ghosts<D, T>(t, v, slot, threadIdx.x, blockDim.x, true);
}

// af_gc_lvl on a box list: kGcLanes<D> threads per box, blockDim.x /
// kGcLanes<D> boxes per CTA (a box's ghost work is a few hundred cells in
// dependent phases, so several boxes share a CTA to keep loads in flight).
template <int D>
constexpr int kGcLanes = D == 3 ? 64 : 32;

template <int D, typename T, int NC = 0>
__global__ void __launch_bounds__(256) k_gc(KTree t0, const int* __restrict__ rec, int n, ModeArg<T> v_, GcDev g,
                                            int corners) {
  const KTree t = fix_dims<D, NC>(t0);
  T* __restrict__ v = v_.get();
  constexpr int L = kGcLanes<D>;
  const int e = blockIdx.x * (blockDim.x / L) + threadIdx.x / L, lane = threadIdx.x % L;
  int4 r0 = make_int4(0, 0, 0, 0), r1 = r0;
  bool active = e < n;
  if (active) load_rec(rec, e, r0, r1);
  const int slot = r0.x;
  active = active && !box_frozen(t, slot);
  const int nc = t.nc;
  const int nface = D == 2 ? nc : nc * nc;
  T* a = v + (size_t)slot * t.S;
  // corners: 0 = face ghosts, 1 = faces then edges/corners, 2 = only the
  // edges/corners (face ghosts already valid)
  for (int w = lane; active && corners != 2 && w < 2 * D * nface; w += L) {
    const int nb = w / nface, pq = w - nb * nface;
    const int p = pq % nc + 1, q = D == 3 ? pq / nc + 1 : 0;
    const int d = nb >> 1;
    const bool low = (nb & 1) == 0;
    const T val = face_ghost_nb<D, T>(t, v, slot, nb, rec_nb(r0, r1, nb), p, q, g);
    a[face_at<D>(t.n2, d, low ? 0 : nc + 1, p, q)] = val;
  }
  if (corners) {
    __syncthreads();
    corner_ghosts<D, T>(t, v, slot, lane, L, active);
  }
}

}  // namespace afg
