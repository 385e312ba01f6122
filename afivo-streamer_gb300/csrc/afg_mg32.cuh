// afg_mg32.cuh -- the FP32 correction solve of the mixed-precision multigrid
// (afg_mixed.cuh) on a compact red-black layout of its buffers.
//
// Layout of one FP32 buffer (correction e, its right-hand side r, FAS tmp):
//   [n_boxes][SI] interior blocks, then [n_boxes][S] ghost blocks,
// SI = nc^D, S = (nc+2)^D.  A box's interior block holds two colour halves
// of SI/2 cells, colour (i + j [+ k]) & 1 (1-based indices); inside a half
// the rows (j [, k]) follow each other and a row holds the nc/2 cells of the
// colour in order of i.  The ghost block keeps the (nc+2)^D layout of the
// FP64 variables, of which only the ghost positions are used.
//
// A red-black half sweep updates one colour from the other: per box it reads
// the other colour's half (contiguous, one bulk copy), the updated colour's
// right-hand side half and writes that colour's half -- 1.5 words per cell,
// the algorithmic traffic, with full 32-byte sectors -- where the ghosted
// layout moves whole (nc+2)^D blocks with rows that straddle sectors.
// The stencils, ghost rules and transfer operators are those of
// afg_mg_kernels.cuh / afg_gc_kernels.cuh (afivo/src/m_af_multigrid.f90,
// m_af_stencil.f90, m_af_ghostcell.f90) in the same operation order, so the
// FP32 results equal those of the ghosted layout bit for bit.
#pragma once
#include "afg_common.cuh"
#include "afg_gc_kernels.cuh"
#include "afg_tma.cuh"

namespace afg {

// offset of interior cell (i, j[, k]) in its box's interior block (k = 0 in 2D)
template <int D>
__device__ __forceinline__ int rb_idx(int nc, int i, int j, int k) {
  const int hn = nc >> 1;
  const int sh = D == 2 ? nc * hn : nc * nc * hn;
  const int row = D == 2 ? j - 1 : (k - 1) * nc + (j - 1);
  return (((i + j + k) & 1) ? sh : 0) + row * hn + ((i - 1) >> 1);
}

// cell (i, j[, k]) of colour `col` at position w of the colour's half
template <int D>
__device__ __forceinline__ void rb_cell(int nc, int col, int w, int& i, int& j, int& k) {
  const int hn = nc >> 1;
  const int row = w / hn, m = w - row * hn;
  if (D == 2) {
    j = row + 1;
    k = 0;
  } else {
    j = row % nc + 1;
    k = row / nc + 1;
  }
  i = 2 * m + 2 - ((col + j + k) & 1);
}

template <int D>
__device__ __forceinline__ bool rb_inside(int nc, int i, int j, int k) {
  return (unsigned)(i - 1) < (unsigned)nc && (unsigned)(j - 1) < (unsigned)nc &&
         (D == 2 || (unsigned)(k - 1) < (unsigned)nc);
}

// address of cell (i, j[, k]) of box `slot`, interior or ghost
template <int D, typename T>
__device__ __forceinline__ T* rb_ptr(const KTree& t, T* v, int slot, int i, int j, int k) {
  if (rb_inside<D>(t.nc, i, j, k)) return v + (size_t)slot * t.SI + rb_idx<D>(t.nc, i, j, k);
  return v + (size_t)t.nbox * t.SI + (size_t)slot * t.S + (D == 2 ? at2(t.n2, i, j) : at3(t.n2, i, j, k));
}

// the cell of face_at<D>(n2, d, x, p, q) as indices
template <int D>
__device__ __forceinline__ void face_ijk(int d, int x, int p, int q, int& i, int& j, int& k) {
  if (D == 2) {
    i = d == 0 ? x : p;
    j = d == 0 ? p : x;
    k = 0;
  } else {
    i = d == 0 ? x : p;
    j = d == 0 ? p : (d == 1 ? x : q);
    k = d == 2 ? x : q;
  }
}

// face_ghost_nb (mg_sides_rb rule on refinement faces) on the compact layout
template <int D>
__device__ __forceinline__ float face_ghost_rb(const KTree& t, const float* __restrict__ v, int slot, int nb,
                                               int nbs, int p, int q, const GcDev& g) {
  const int nc = t.nc, d = nb >> 1;
  const bool low = (nb & 1) == 0;
  int i, j, k;
  if (nbs >= 0) {
    face_ijk<D>(d, low ? nc : 1, p, q, i, j, k);
    return v[(size_t)nbs * t.SI + rb_idx<D>(nc, i, j, k)];
  }
  const float* a = v + (size_t)slot * t.SI;
  if (nbs == kNbPhys) {
    int i2, j2, k2;
    face_ijk<D>(d, low ? 1 : nc, p, q, i, j, k);
    face_ijk<D>(d, low ? 2 : nc - 1, p, q, i2, j2, k2);
    return bc_ghost<D, float>(gc_type(g, nb), gc_val(g, nb, t, slot), t.dr[slot * D + d], low,
                              a[rb_idx<D>(nc, i, j, k)], a[rb_idx<D>(nc, i2, j2, k2)]);
  }
  // refinement boundary: slope-corrected value of the parent's neighbour next
  // to the fine cell, then 0.5*gc + 0.75*phi(1) - 0.25*phi(2)
  // (m_af_multigrid.f90:294-461)
  const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
  const int cs = t.pnb[slot * 2 * D + nb];
  const int off1 = child_offset(t, slot, t1);
  const int off2 = D == 3 ? child_offset(t, slot, t2) : 0;
  const int cx = low ? nc : 1;
  const int ix = low ? 1 : nc, dix = low ? 1 : -1;
  auto C = [&](int a1, int a2) {
    int ci, cj, ck;
    face_ijk<D>(d, cx, a1, a2, ci, cj, ck);
    return *rb_ptr<D>(t, v, cs, ci, cj, ck);
  };
  float gcv;
  if (D == 2) {
    const int ii = (p + 1) >> 1;
    const float tm = C(off1 + ii - 1, 0);
    const float t0 = C(off1 + ii, 0);
    const float tp = C(off1 + ii + 1, 0);
    const float grad = 0.125f * (tp - tm);
    gcv = (p & 1) ? t0 - grad : t0 + grad;
  } else {
    const int ii = (p + 1) >> 1, jj = (q + 1) >> 1;
    const float t0 = C(off1 + ii, off2 + jj);
    const float g1 = 0.125f * (C(off1 + ii + 1, off2 + jj) - C(off1 + ii - 1, off2 + jj));
    const float g2 = 0.125f * (C(off1 + ii, off2 + jj + 1) - C(off1 + ii, off2 + jj - 1));
    const float s1 = (p & 1) ? t0 - g1 : t0 + g1;
    gcv = (q & 1) ? s1 - g2 : s1 + g2;
  }
  int i2, j2, k2;
  face_ijk<D>(d, ix, p, q, i, j, k);
  face_ijk<D>(d, ix + dix, p, q, i2, j2, k2);
  return 0.5f * gcv + 0.75f * a[rb_idx<D>(nc, i, j, k)] - 0.25f * a[rb_idx<D>(nc, i2, j2, k2)];
}

// Value of neighbour (i, j[, k]) of an interior cell: interior cells from the
// box itself, cells across a face by the face's ghost rule.
template <int D>
__device__ __forceinline__ float nb_val_rb(const KTree& t, const float* __restrict__ v, int slot, int i, int j, int k,
                                           const GcDev& g, const int4& r0, const int4& r1) {
  const int nc = t.nc;
  int nb = -1, p = 0, q = 0;
  if (i == 0 || i == nc + 1) {
    nb = i == 0 ? 0 : 1;
    p = j;
    q = k;
  } else if (j == 0 || j == nc + 1) {
    nb = j == 0 ? 2 : 3;
    p = i;
    q = k;
  } else if (D == 3 && (k == 0 || k == nc + 1)) {
    nb = k == 0 ? 4 : 5;
    p = i;
    q = j;
  }
  if (nb < 0) return v[(size_t)slot * t.SI + rb_idx<D>(nc, i, j, k)];
  return face_ghost_rb<D>(t, v, slot, nb, rec_nb(r0, r1, nb), p, q, g);
}

// Red-black half sweep, one box per CTA, any box size: the cells of colour
// redblack & 1 from the other colour and the face ghost rules
// (k_gsrb_fused's arithmetic).
template <int D, bool CYL, int NC = 0>
__global__ void __launch_bounds__(256) k_gsrb_rb(KTree t0, const int* __restrict__ rec, ModeArg<float> phi_,
                                                 ModeArg<const float> rhs_, int redblack, ModeCoef<float> mc_,
                                                 GcDev g) {
  const KTree t = fix_dims<D, NC>(t0);
  float* __restrict__ phi = phi_.get();
  const float* __restrict__ rhs = rhs_.get();
  const MgCoef<float> mc = mc_.get();
  int4 r0, r1;
  load_rec(rec, blockIdx.x, r0, r1);
  const int slot = r0.x;
  if (box_frozen(t, slot)) return;
  const int nc = t.nc, col = redblack & 1, sh = t.SI / 2;
  float c[7];
  for (int q = 0; q < 2 * D + 1; q++) c[q] = mc.cb[slot * 8 + q];
  const float inv_c1 = mc.cb[slot * 8 + 7];
  float* out = phi + (size_t)slot * t.SI + col * sh;
  const float* f = rhs + (size_t)slot * t.SI + col * sh;
  for (int w = threadIdx.x; w < sh; w += blockDim.x) {
    int i, j, k;
    rb_cell<D>(nc, col, w, i, j, k);
    const float pw = nb_val_rb<D>(t, phi, slot, i - 1, j, k, g, r0, r1);
    const float pe = nb_val_rb<D>(t, phi, slot, i + 1, j, k, g, r0, r1);
    const float ps = nb_val_rb<D>(t, phi, slot, i, j - 1, k, g, r0, r1);
    const float pn = nb_val_rb<D>(t, phi, slot, i, j + 1, k, g, r0, r1);
    float val;
    if (D == 2) {
      if (CYL) {
        const float* y = mc.cy + ((size_t)slot * nc + (i - 1)) * 4;
        val = (f[w] - y[1] * pw - y[2] * pe - c[3] * ps - c[4] * pn) * y[3];
      } else {
        val = (f[w] - c[1] * pw - c[2] * pe - c[3] * ps - c[4] * pn) * inv_c1;
      }
    } else {
      const float pb = nb_val_rb<D>(t, phi, slot, i, j, k - 1, g, r0, r1);
      const float pf = nb_val_rb<D>(t, phi, slot, i, j, k + 1, g, r0, r1);
      val = (f[w] - c[1] * pw - c[2] * pe - c[3] * ps - c[4] * pn - c[5] * pb - c[6] * pf) * inv_c1;
    }
    // cells of one colour never read each other (a ghost rule reads the
    // updated cell itself, in this thread, before the store)
    out[w] = val;
  }
}

// The same half sweep staged in shared memory for a compile-time box size:
// a persistent grid walks the box records; per box, thread 0 bulk-copies the
// next box's other-colour half and the right-hand sides of its updated colour
// (SI/2 values each, contiguous) into one of two stages while the CTA works
// on the current box.  Before waiting for the current box's copies, each
// thread evaluates its share of the face ghosts next to cells of the updated
// colour (face_ghost_rb on global memory: the values af_gc would store), so
// those loads overlap the copies.  The CTA then spreads
// the staged half and the ghosts into a padded (nc+2)^D block and each thread
// updates CPT cells of the colour from shared memory without branches.  A
// wait that times out (1 s) raises *err; the CTA drains its copies (bounded)
// and returns, raising bit 2 of *err if they did not complete.
template <int D, bool CYL, int NC, int CPT>
__global__ void __launch_bounds__((D == 2 ? NC * NC / 2 : NC * NC * NC / 2) / CPT,
                                  1024 / ((D == 2 ? NC * NC / 2 : NC * NC * NC / 2) / CPT))
    k_gsrb_rb_tma(KTree t0, const int* __restrict__ rec, int n, ModeArg<float> phi_, ModeArg<const float> rhs_,
                  int redblack, ModeCoef<float> mc_, GcDev g, unsigned* err) {
  constexpr int SH = D == 2 ? NC * NC / 2 : NC * NC * NC / 2;
  constexpr int TPB = SH / CPT;
  constexpr int nc = NC, n2 = NC + 2, hn = NC / 2, sk = n2 * n2;
  constexpr int S = D == 2 ? n2 * n2 : n2 * n2 * n2;
  constexpr int SI = 2 * SH;
  constexpr int NGF = D == 2 ? hn : nc * hn;  // ghosts read per face and half sweep
  constexpr int NGT = (2 * D * NGF + TPB - 1) / TPB;  // ghosts per thread
  constexpr unsigned BYTES = SH * sizeof(float);
  static_assert(BYTES % 16 == 0, "bulk copies need 16-byte multiples");
  __shared__ __align__(128) float cst[2][SH];  // other colour
  __shared__ __align__(128) float rst[2][SH];  // right-hand sides of the updated colour
  __shared__ float P[S];
  __shared__ __align__(8) unsigned long long bar[2];
  float* __restrict__ phi = phi_.get();
  const float* __restrict__ rhs = rhs_.get();
  const MgCoef<float> mc = mc_.get();
  const KTree t = fix_dims<D, NC>(t0);
  const int col = redblack & 1, oc = col ^ 1;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int e, int st) {
    const int s = rec[8 * e];
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bar[st], 2 * BYTES);
    bulk_copy_g2s(cst[st], phi + (size_t)s * SI + oc * SH, BYTES, &bar[st]);
    bulk_copy_g2s(rst[st], rhs + (size_t)s * SI + col * SH, BYTES, &bar[st]);
  };
  if (threadIdx.x == 0 && (int)blockIdx.x < n) issue(blockIdx.x, 0);
  int it = 0;
  for (int e = blockIdx.x; e < n; e += gridDim.x, it++) {
    const int st = it & 1;
    const bool next = e + (int)gridDim.x < n;
    if (threadIdx.x == 0 && next) issue(e + gridDim.x, st ^ 1);
    const int4 r0 = reinterpret_cast<const int4*>(rec)[2 * e];
    const int4 r1 = reinterpret_cast<const int4*>(rec)[2 * e + 1];
    const int slot = r0.x;
    const bool active = !box_frozen(t, slot);
    float c[7];
    for (int q = 0; q < 2 * D + 1; q++) c[q] = mc.cb[slot * 8 + q];
    const float inv_c1 = mc.cb[slot * 8 + 7];
    // this thread's cells
    int xs[CPT];
#pragma unroll
    for (int u = 0; u < CPT; u++) {
      const int w = (int)threadIdx.x + u * TPB;
      int i, j, k;
      rb_cell<D>(nc, col, w, i, j, k);
      xs[u] = D == 2 ? at2(n2, i, j) : at3(n2, i, j, k);
    }
    // this thread's face ghosts next to cells of the updated colour: cell
    // (i, j[, k]) is updated when i + j (+ k) + redblack is even
    float gv[NGT];
    int gx[NGT];
#pragma unroll
    for (int u = 0; u < NGT; u++) {
      const int w = (int)threadIdx.x + u * TPB;
      gx[u] = -1;
      gv[u] = 0.0f;
      if (active && w < 2 * D * NGF) {
        const int nb = w / NGF, m = w - nb * NGF, d = nb >> 1;
        const bool low = (nb & 1) == 0;
        const int a = low ? 1 : nc;  // normal index of the adjacent cell
        int pt, qt;
        if (D == 2) {
          qt = 0;
          pt = 2 * m + 1 + ((a + 1 + redblack) & 1);
        } else {
          qt = m / hn + 1;
          pt = 2 * (m - (qt - 1) * hn) + 1 + ((a + 1 + qt + redblack) & 1);
        }
        gx[u] = face_at<D>(n2, d, low ? 0 : nc + 1, pt, qt);
        gv[u] = face_ghost_rb<D>(t, phi, slot, nb, rec_nb(r0, r1, nb), pt, qt, g);
      }
    }
    const bool ok = mbar_wait(&bar[st], (it >> 1) & 1);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        bool drained = mbar_wait(&bar[st], (it >> 1) & 1);
        if (next) drained = mbar_wait(&bar[st ^ 1], ((it + 1) >> 1) & 1) && drained;
        atomicOr(err, drained ? 1u : 3u);
      }
      return;
    }
    // the other colour and the ghosts into the padded block
    for (int w = threadIdx.x; active && w < SH; w += TPB) {
      int i, j, k;
      rb_cell<D>(nc, oc, w, i, j, k);
      P[D == 2 ? at2(n2, i, j) : at3(n2, i, j, k)] = cst[st][w];
    }
#pragma unroll
    for (int u = 0; u < NGT; u++)
      if (gx[u] >= 0) P[gx[u]] = gv[u];
    __syncthreads();
    if (active) {
      float* out = phi + (size_t)slot * SI + col * SH;
      float val[CPT];
#pragma unroll
      for (int u = 0; u < CPT; u++) {
        const int x = xs[u];
        const float fv = rst[st][threadIdx.x + u * TPB];
        if (D == 2) {
          if (CYL) {
            const int i = x % n2;
            const float* y = mc.cy + ((size_t)slot * nc + (i - 1)) * 4;
            val[u] = (fv - y[1] * P[x - 1] - y[2] * P[x + 1] - c[3] * P[x - n2] - c[4] * P[x + n2]) * y[3];
          } else {
            val[u] = (fv - c[1] * P[x - 1] - c[2] * P[x + 1] - c[3] * P[x - n2] - c[4] * P[x + n2]) * inv_c1;
          }
        } else {
          val[u] = (fv - c[1] * P[x - 1] - c[2] * P[x + 1] - c[3] * P[x - n2] - c[4] * P[x + n2] -
                    c[5] * P[x - sk] - c[6] * P[x + sk]) *
                   inv_c1;
        }
      }
#pragma unroll
      for (int u = 0; u < CPT; u++) out[threadIdx.x + u * TPB] = val[u];
    }
    __syncthreads();  // stage st and the padded block are read completely before reuse
  }
}

// Edge (3D) and corner ghosts of one box on the compact layout; the face
// ghosts must be in place (corner_ghosts of afg_gc_kernels.cuh).
template <int D>
__device__ void corner_ghosts_rb(const KTree& t, float* __restrict__ v, int slot, int lane, int nl, bool active) {
  const int nc = t.nc;
  auto at = [&](int b, int i, int j, int k) -> float& { return *rb_ptr<D>(t, v, b, i, j, k); };
  if (D == 3) {
    for (int w = lane; active && w < 12 * nc; w += nl) {
      const int n = w / nc, pp = w % nc + 1;
      const int dim = c_edge_dim[n];
      const int dx = c_edge_dir[n][0], dy = c_edge_dir[n][1], dz = c_edge_dir[n][2];
      const int x0 = dim == 0 ? pp : (dx == 1) * (nc + 1);
      const int x1 = dim == 1 ? pp : (dy == 1) * (nc + 1);
      const int x2 = dim == 2 ? pp : (dz == 1) * (nc + 1);
      const int nbs = nbmat_at(t, slot, dx, dy, dz);
      if (nbs >= 0) {
        at(slot, x0, x1, x2) = at(nbs, x0 - dx * nc, x1 - dy * nc, x2 - dz * nc);
      } else {
        const int s0 = dim == 0 ? 0 : 1 - 2 * (x0 & 1);
        const int s1 = dim == 1 ? 0 : 1 - 2 * (x1 & 1);
        const int s2 = dim == 2 ? 0 : 1 - 2 * (x2 & 1);
        float ua, ub;
        if (dim == 0) {
          ua = at(slot, x0, x1 + s1, x2);
          ub = at(slot, x0, x1, x2 + s2);
        } else if (dim == 1) {
          ua = at(slot, x0, x1, x2 + s2);
          ub = at(slot, x0 + s0, x1, x2);
        } else {
          ua = at(slot, x0 + s0, x1, x2);
          ub = at(slot, x0, x1 + s1, x2);
        }
        at(slot, x0, x1, x2) = ua + ub - at(slot, x0 + s0, x1 + s1, x2 + s2);
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
    if (nbs >= 0) {
      at(slot, x, y, z) = at(nbs, x - dx * nc, y - dy * nc, D == 3 ? z - dz * nc : 0);
    } else if (D == 2) {
      at(slot, x, y, 0) = at(slot, x + di, y, 0) + at(slot, x, y + dj, 0) - at(slot, x + di, y + dj, 0);
    } else {
      at(slot, x, y, z) = at(slot, x, y + dj, z + dk) + at(slot, x + di, y, z + dk) + at(slot, x + di, y + dj, z) -
                          2.0f * at(slot, x + di, y + dj, z + dk);
    }
  }
}

// the whole CTA on one box
template <int D>
__device__ void corner_ghosts_rb(const KTree& t, float* __restrict__ v, int slot) {
  corner_ghosts_rb<D>(t, v, slot, threadIdx.x, blockDim.x, true);
}

// face ghosts (all positions) of one box into its ghost block, by threads
// lane, lane + nl, ...
template <int D>
__device__ __forceinline__ void face_ghosts_rb(const KTree& t, float* __restrict__ v, int slot, const int4& r0,
                                               const int4& r1, const GcDev& g, int lane, int nl) {
  const int nc = t.nc;
  const int nface = D == 2 ? nc : nc * nc;
  for (int w = lane; w < 2 * D * nface; w += nl) {
    const int nb = w / nface, pq = w - nb * nface;
    const int p = pq % nc + 1, q = D == 3 ? pq / nc + 1 : 0;
    const float val = face_ghost_rb<D>(t, v, slot, nb, rec_nb(r0, r1, nb), p, q, g);
    int i, j, k;
    face_ijk<D>(nb >> 1, (nb & 1) ? nc + 1 : 0, p, q, i, j, k);
    *rb_ptr<D>(t, v, slot, i, j, k) = val;
  }
}

template <int D>
__device__ __forceinline__ void face_ghosts_rb(const KTree& t, float* __restrict__ v, int slot, const int4& r0,
                                               const int4& r1, const GcDev& g) {
  face_ghosts_rb<D>(t, v, slot, r0, r1, g, threadIdx.x, blockDim.x);
}

// af_gc_lvl on a box list (k_gc, kGcLanes<D> threads per box): 0 = face
// ghosts, 1 = faces then edges and corners, 2 = only the edges and corners
template <int D, int NC = 0>
__global__ void __launch_bounds__(256) k_gc_rb(KTree t0, const int* __restrict__ rec, int n, ModeArg<float> v_,
                                               GcDev g, int corners) {
  const KTree t = fix_dims<D, NC>(t0);
  float* __restrict__ v = v_.get();
  constexpr int L = kGcLanes<D>;
  const int e = blockIdx.x * (blockDim.x / L) + threadIdx.x / L, lane = threadIdx.x % L;
  int4 r0 = make_int4(0, 0, 0, 0), r1 = r0;
  bool active = e < n;
  if (active) load_rec(rec, e, r0, r1);
  const int slot = r0.x;
  active = active && !box_frozen(t, slot);
  if (active && corners != 2) face_ghosts_rb<D>(t, v, slot, r0, r1, g, lane, L);
  if (corners) {
    __syncthreads();
    corner_ghosts_rb<D>(t, v, slot, lane, L, active);
  }
}

// update_coarse first half (k_residual_restrict with the face neighbours on
// the fly): residual of each child box restricted to its parent's tmp (with
// the cylindrical weights), phi restricted without geometry.  The CTA first
// gathers the box's interior and its face ghosts (face_ghost_rb: the values
// af_gc would store) into a padded (nc+2)^D block in shared memory
// (dynamic, S floats); the stencil then reads shared memory only.
template <int D, bool CYL, int NC = 0>
__global__ void __launch_bounds__(256) k_residual_restrict_rb(KTree t0, const int* __restrict__ rec,
                                                              ModeArg<float> phi_, ModeArg<const float> rhs_,
                                                              ModeArg<float> tmp_, ModeCoef<float> mc_, GcDev g) {
  const KTree t = fix_dims<D, NC>(t0);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* P = reinterpret_cast<float*>(smem_raw);
  float* __restrict__ phi = phi_.get();
  const float* __restrict__ rhs = rhs_.get();
  float* __restrict__ tmp = tmp_.get();
  const MgCoef<float> mc = mc_.get();
  int4 r0, r1;
  load_rec(rec, blockIdx.x, r0, r1);
  const int slot = r0.x;
  if (box_frozen(t, slot)) return;
  const int pslot = t.parent[slot];
  const int nc = t.nc, n2 = t.n2, hnc = nc / 2, sk = n2 * n2;
  const float* p = phi + (size_t)slot * t.SI;
  const float* f = rhs + (size_t)slot * t.SI;
  for (int w = threadIdx.x; w < t.SI; w += blockDim.x) {
    const int col = w >= t.SI / 2;
    int i, j, k;
    rb_cell<D>(nc, col, w - col * (t.SI / 2), i, j, k);
    P[D == 2 ? at2(n2, i, j) : at3(n2, i, j, k)] = p[w];
  }
  const int nface = D == 2 ? nc : nc * nc;
  for (int w = threadIdx.x; w < 2 * D * nface; w += blockDim.x) {
    const int nb = w / nface, pq = w - nb * nface;
    const int pi = pq % nc + 1, qi = D == 3 ? pq / nc + 1 : 0;
    P[face_at<D>(n2, nb >> 1, (nb & 1) ? nc + 1 : 0, pi, qi)] =
        face_ghost_rb<D>(t, phi, slot, nb, rec_nb(r0, r1, nb), pi, qi, g);
  }
  __syncthreads();
  float c[7];
  for (int q = 0; q < 7; q++) c[q] = mc.cb[slot * 8 + q];
  float* pp = phi + (size_t)pslot * t.SI;
  float* pt = tmp + (size_t)pslot * t.SI;
  const int o0 = child_offset(t, slot, 0), o1 = child_offset(t, slot, 1);
  const int o2 = D == 3 ? child_offset(t, slot, 2) : 0;
  const int count = D == 2 ? hnc * hnc : hnc * hnc * hnc;
  for (int w = threadIdx.x; w < count; w += blockDim.x) {
    const int i = w % hnc + 1, r = w / hnc;
    const int j = D == 2 ? r + 1 : r % hnc + 1, k = D == 2 ? 0 : r / hnc + 1;
    const int ic = o0 + i, jc = o1 + j, kc = o2 + k;
    const int fi = 2 * i - 1, fj = 2 * j - 1, fk = D == 3 ? 2 * k - 1 : 0;
    if (D == 2) {
      float res[2][2];  // [dj][di]
      for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) {
          float k1 = 0.0f, k2 = 0.0f, k3 = 0.0f;
          if (CYL) {
            const float* y = mc.cy + ((size_t)slot * nc + (fi + di - 1)) * 4;
            k1 = y[0]; k2 = y[1]; k3 = y[2];
          }
          const int x = at2(n2, fi + di, fj + dj);
          res[dj][di] = f[rb_idx<D>(nc, fi + di, fj + dj, 0)] -
                        lpl_vals<D, CYL, float>(P[x], P[x - 1], P[x + 1], P[x - n2], P[x + n2], 0.0f, 0.0f, c, k1,
                                                k2, k3);
        }
      float rv;
      if (CYL) {
        const double* gw = t.geo + ((size_t)pslot * nc + (ic - 1)) * 4;
        const float w1 = float(gw[2]), w2 = float(gw[3]);
        float s1 = 0.0f, s2 = 0.0f;
        s1 = s1 + res[0][0]; s1 = s1 + res[1][0];
        s2 = s2 + res[0][1]; s2 = s2 + res[1][1];
        rv = 0.25f * (w1 * s1 + w2 * s2);
      } else {
        float s = 0.0f;
        s = s + res[0][0]; s = s + res[0][1]; s = s + res[1][0]; s = s + res[1][1];
        rv = 0.25f * s;
      }
      pt[rb_idx<D>(nc, ic, jc, 0)] = rv;
      float s = 0.0f;
      s = s + P[at2(n2, fi, fj)]; s = s + P[at2(n2, fi + 1, fj)];
      s = s + P[at2(n2, fi, fj + 1)]; s = s + P[at2(n2, fi + 1, fj + 1)];
      pp[rb_idx<D>(nc, ic, jc, 0)] = 0.25f * s;
    } else {
      float sr = 0.0f, sp = 0.0f;
      for (int dk = 0; dk < 2; dk++)
        for (int dj = 0; dj < 2; dj++)
          for (int di = 0; di < 2; di++) {
            const int x = at3(n2, fi + di, fj + dj, fk + dk);
            const float res = f[rb_idx<D>(nc, fi + di, fj + dj, fk + dk)] -
                              lpl_vals<D, false, float>(P[x], P[x - 1], P[x + 1], P[x - n2], P[x + n2], P[x - sk],
                                                        P[x + sk], c, 0.0f, 0.0f, 0.0f);
            sr = sr + res;
            sp = sp + P[x];
          }
      pt[rb_idx<D>(nc, ic, jc, kc)] = 0.125f * sr;
      pp[rb_idx<D>(nc, ic, jc, kc)] = 0.125f * sp;
    }
  }
}

// update_coarse second half on the parents (k_coarse_fas with the parent's
// ghost fill and the copy into tmp): ghost cells of phi filled (faces, then
// edges and corners), rhs = L phi + tmp on interior cells, tmp = phi on the
// whole array.
template <int D, bool CYL, int NC = 0>
__global__ void __launch_bounds__(256) k_coarse_fas_rb(KTree t0, const int* __restrict__ rec, ModeArg<float> phi_,
                                                       ModeArg<float> rhs_, ModeArg<float> tmp_, ModeCoef<float> mc_,
                                                       GcDev g) {
  const KTree t = fix_dims<D, NC>(t0);
  float* __restrict__ phi = phi_.get();
  float* __restrict__ rhs = rhs_.get();
  float* __restrict__ tmp = tmp_.get();
  const MgCoef<float> mc = mc_.get();
  int4 r0, r1;
  load_rec(rec, blockIdx.x, r0, r1);
  const int slot = r0.x;
  if (box_frozen(t, slot)) return;
  const int nc = t.nc, n2 = t.n2;
  face_ghosts_rb<D>(t, phi, slot, r0, r1, g);
  __syncthreads();
  corner_ghosts_rb<D>(t, phi, slot);
  __syncthreads();
  float c[7];
  for (int q = 0; q < 7; q++) c[q] = mc.cb[slot * 8 + q];
  for (int x = threadIdx.x; x < t.S; x += blockDim.x) {
    const int i = x % n2, r = x / n2;
    const int j = D == 2 ? r : r % n2, k = D == 2 ? 0 : r / n2;
    float* o = rb_ptr<D>(t, tmp, slot, i, j, k);
    const float pv = *rb_ptr<D>(t, phi, slot, i, j, k);
    if (rb_inside<D>(nc, i, j, k)) {
      float k1 = 0.0f, k2 = 0.0f, k3 = 0.0f;
      if (CYL) {
        const float* y = mc.cy + ((size_t)slot * nc + (i - 1)) * 4;
        k1 = y[0]; k2 = y[1]; k3 = y[2];
      }
      const float pw = *rb_ptr<D>(t, phi, slot, i - 1, j, k), pe = *rb_ptr<D>(t, phi, slot, i + 1, j, k);
      const float ps = *rb_ptr<D>(t, phi, slot, i, j - 1, k), pn = *rb_ptr<D>(t, phi, slot, i, j + 1, k);
      float pb = 0.0f, pf = 0.0f;
      if (D == 3) {
        pb = *rb_ptr<D>(t, phi, slot, i, j, k - 1);
        pf = *rb_ptr<D>(t, phi, slot, i, j, k + 1);
      }
      const float lp = lpl_vals<D, CYL, float>(pv, pw, pe, ps, pn, pb, pf, c, k1, k2, k3);
      rhs[(size_t)slot * t.SI + rb_idx<D>(nc, i, j, k)] = lp + *o;
    }
    *o = pv;
  }
}

// correct_children on the parents (k_correct): tmp = phi - tmp over the
// whole array, then each child's phi gets the bilinear/trilinear
// prolongation of tmp added.
template <int D, int NC = 0>
__global__ void __launch_bounds__(256) k_correct_rb(KTree t0, const int* __restrict__ list, ModeArg<float> phi_,
                                                    ModeArg<float> tmp_) {
  const KTree t = fix_dims<D, NC>(t0);
  float* __restrict__ phi = phi_.get();
  float* __restrict__ tmp = tmp_.get();
  extern __shared__ unsigned char smem_raw[];
  float* sm = reinterpret_cast<float*>(smem_raw);
  const int slot = list[blockIdx.x];
  if (box_frozen(t, slot)) return;
  const int nc = t.nc, n2 = t.n2;
  for (int x = threadIdx.x; x < t.S; x += blockDim.x) {
    const int i = x % n2, r = x / n2;
    const int j = D == 2 ? r : r % n2, k = D == 2 ? 0 : r / n2;
    float* o = rb_ptr<D>(t, tmp, slot, i, j, k);
    const float v = *rb_ptr<D>(t, phi, slot, i, j, k) - *o;
    *o = v;
    sm[x] = v;
  }
  __syncthreads();
  const int nch = 1 << D;
  const int ncell = D == 2 ? nc * nc : nc * nc * nc;
  for (int w = threadIdx.x; w < nch * ncell; w += blockDim.x) {
    const int ch = w / ncell, cw = w - ch * ncell;
    const int cs = t.children[slot * nch + ch];
    if (cs < 0) continue;
    const int i = cw % nc + 1, r = cw / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 0 : r / nc + 1;
    const int o0 = child_offset(t, cs, 0), o1 = child_offset(t, cs, 1);
    const int i1 = o0 + ((i + 1) >> 1), i2 = i1 + 1 - 2 * (i & 1);
    const int j1 = o1 + ((j + 1) >> 1), j2 = j1 + 1 - 2 * (j & 1);
    float* cp = phi + (size_t)cs * t.SI + rb_idx<D>(nc, i, j, k);
    if (D == 2) {
      *cp = *cp + float(9 / 16.0) * sm[at2(n2, i1, j1)] + float(3 / 16.0) * sm[at2(n2, i2, j1)] +
            float(3 / 16.0) * sm[at2(n2, i1, j2)] + float(1 / 16.0) * sm[at2(n2, i2, j2)];
    } else {
      const int o2 = child_offset(t, cs, 2);
      const int k1 = o2 + ((k + 1) >> 1), k2 = k1 + 1 - 2 * (k & 1);
      *cp = *cp + float(27 / 64.0) * sm[at3(n2, i1, j1, k1)] + float(9 / 64.0) * sm[at3(n2, i2, j1, k1)] +
            float(9 / 64.0) * sm[at3(n2, i1, j2, k1)] + float(3 / 64.0) * sm[at3(n2, i2, j2, k1)] +
            float(9 / 64.0) * sm[at3(n2, i1, j1, k2)] + float(3 / 64.0) * sm[at3(n2, i2, j1, k2)] +
            float(3 / 64.0) * sm[at3(n2, i1, j2, k2)] + float(1 / 64.0) * sm[at3(n2, i2, j2, k2)];
    }
  }
}

// init_phi_rhs on one level (k_init_phi_rhs): phi = 0 on the whole array,
// rhs restricted to the parent with geometry.
template <int D, bool CYL, int NC = 0>
__global__ void __launch_bounds__(256) k_init_phi_rhs_rb(KTree t0, const int* __restrict__ list,
                                                         ModeArg<float> phi_, ModeArg<float> rhs_) {
  const KTree t = fix_dims<D, NC>(t0);
  float* __restrict__ phi = phi_.get();
  float* __restrict__ rhs = rhs_.get();
  const int slot = list[blockIdx.x];
  if (box_frozen(t, slot)) return;
  const int pslot = t.parent[slot];
  const int nc = t.nc, hnc = nc / 2;
  float* pin = phi + (size_t)slot * t.SI;
  float* pgh = phi + (size_t)t.nbox * t.SI + (size_t)slot * t.S;
  for (int x = threadIdx.x; x < t.SI; x += blockDim.x) pin[x] = 0.0f;
  for (int x = threadIdx.x; x < t.S; x += blockDim.x) pgh[x] = 0.0f;
  const float* f = rhs + (size_t)slot * t.SI;
  float* pf = rhs + (size_t)pslot * t.SI;
  const int o0 = child_offset(t, slot, 0), o1 = child_offset(t, slot, 1);
  const int o2 = D == 3 ? child_offset(t, slot, 2) : 0;
  const int count = D == 2 ? hnc * hnc : hnc * hnc * hnc;
  for (int w = threadIdx.x; w < count; w += blockDim.x) {
    const int i = w % hnc + 1, r = w / hnc;
    const int j = D == 2 ? r + 1 : r % hnc + 1, k = D == 2 ? 0 : r / hnc + 1;
    const int ic = o0 + i, jc = o1 + j, kc = o2 + k;
    const int fi = 2 * i - 1, fj = 2 * j - 1, fk = D == 3 ? 2 * k - 1 : 0;
    if (D == 2) {
      float rv;
      if (CYL) {
        const double* gw = t.geo + ((size_t)pslot * nc + (ic - 1)) * 4;
        const float w1 = float(gw[2]), w2 = float(gw[3]);
        float s1 = 0.0f, s2 = 0.0f;
        s1 = s1 + f[rb_idx<D>(nc, fi, fj, 0)]; s1 = s1 + f[rb_idx<D>(nc, fi, fj + 1, 0)];
        s2 = s2 + f[rb_idx<D>(nc, fi + 1, fj, 0)]; s2 = s2 + f[rb_idx<D>(nc, fi + 1, fj + 1, 0)];
        rv = 0.25f * (w1 * s1 + w2 * s2);
      } else {
        float s = 0.0f;
        s = s + f[rb_idx<D>(nc, fi, fj, 0)]; s = s + f[rb_idx<D>(nc, fi + 1, fj, 0)];
        s = s + f[rb_idx<D>(nc, fi, fj + 1, 0)]; s = s + f[rb_idx<D>(nc, fi + 1, fj + 1, 0)];
        rv = 0.25f * s;
      }
      pf[rb_idx<D>(nc, ic, jc, 0)] = rv;
    } else {
      float s = 0.0f;
      for (int dk = 0; dk < 2; dk++)
        for (int dj = 0; dj < 2; dj++)
          for (int di = 0; di < 2; di++) s = s + f[rb_idx<D>(nc, fi + di, fj + dj, fk + dk)];
      pf[rb_idx<D>(nc, ic, jc, kc)] = 0.125f * s;
    }
  }
}

// whole-array copy (interior and ghost blocks) on a box list (k_copy)
__global__ void __launch_bounds__(256) k_copy_rb(KTree t, const int* __restrict__ list, ModeArg<const float> src_,
                                                 ModeArg<float> dst_) {
  const float* __restrict__ src = src_.get();
  float* __restrict__ dst = dst_.get();
  const int slot = list[blockIdx.x];
  if (box_frozen(t, slot)) return;
  const size_t in = (size_t)slot * t.SI, gh = (size_t)t.nbox * t.SI + (size_t)slot * t.S;
  for (int x = threadIdx.x; x < t.SI; x += blockDim.x) dst[in + x] = src[in + x];
  for (int x = threadIdx.x; x < t.S; x += blockDim.x) dst[gh + x] = src[gh + x];
}

}  // namespace afg
