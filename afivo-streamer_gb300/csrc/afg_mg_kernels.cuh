// afg_mg_kernels.cuh -- FAS multigrid stages on box lists (afivo/src/
// m_af_multigrid.f90, m_af_stencil.f90, m_af_restrict.f90).
//
// Every kernel takes a device list of box slots of one level and processes
// one box per CTA.  The arithmetic follows the reference expression by
// expression (left-to-right, no contraction: the library is built with
// --fmad=false) so that the FP64 instantiation reproduces the CPU oracle
// bit for bit; the FP32 instantiation is the inner solver of the mixed path.
#pragma once
#include "afg_common.cuh"
#include "afg_gc_kernels.cuh"
#include "afg_tma.cuh"

namespace afg {

// Operator coefficients mg_box_lpl_stencil (m_af_multigrid.f90:1246-1264):
// c = [-sum(c(2:)) - lambda^2, 1/dx^2, 1/dx^2, 1/dy^2, 1/dy^2(, 1/dz^2 x2)],
// always formed in FP64 and rounded to T.
template <int D>
__device__ __forceinline__ void lpl_coeffs(const KTree& t, int slot, double lambda2, double c[7]) {
  double inv[3];
  for (int d = 0; d < D; d++) {
    const double h = t.dr[slot * D + d];
    inv[d] = 1 / (h * h);
  }
  for (int d = 0; d < D; d++) c[1 + 2 * d] = c[2 + 2 * d] = inv[d];
  double s = 0;
  for (int k = 1; k <= 2 * D; k++) s += c[k];
  c[0] = -s - lambda2;
}

// Cylindrical correction per radial index i (af_cyl_flux_factors,
// m_af_types.f90:1199-1211; m_af_stencil.f90:884-906).
__device__ __forceinline__ void cyl_coeffs(const KTree& t, int slot, int i, const double c[7],
                                           double& k1, double& k2, double& k3) {
  const double rmin = t.r_min[slot * 2], h = t.dr[slot * 2];
  const double r = rmin + (i - 0.5) * h;
  const double inv_r = 1 / r;
  const double f1 = (r - 0.5 * h) * inv_r, f2 = (r + 0.5 * h) * inv_r;
  k2 = f1 * c[1];
  k3 = f2 * c[2];
  k1 = c[0] - (k2 - c[1]) - (k3 - c[2]);
}

// L phi at interior cell (i,j[,k]); stencil_apply_357 (m_af_stencil.f90:367-496)
template <int D, bool CYL, typename T>
__device__ __forceinline__ T apply_lpl(const T* __restrict__ p, int n2, int i, int j, int k,
                                       const T c[7], T k1, T k2, T k3) {
  if (D == 2) {
    const int x = at2(n2, i, j);
    if (CYL)
      return k1 * p[x] + k2 * p[x - 1] + k3 * p[x + 1] + c[3] * p[x - n2] + c[4] * p[x + n2];
    return c[0] * p[x] + c[1] * p[x - 1] + c[2] * p[x + 1] + c[3] * p[x - n2] + c[4] * p[x + n2];
  } else {
    const int x = at3(n2, i, j, k), sk = n2 * n2;
    return c[0] * p[x] + c[1] * p[x - 1] + c[2] * p[x + 1] + c[3] * p[x - n2] + c[4] * p[x + n2] +
           c[5] * p[x - sk] + c[6] * p[x + sk];
  }
}

// L phi from the centre and neighbour values, in apply_lpl's operation order
template <int D, bool CYL, typename T>
__device__ __forceinline__ T lpl_vals(T pc, T pw, T pe, T ps, T pn, T pb, T pf, const T c[7], T k1, T k2, T k3) {
  if (D == 2) {
    if (CYL) return k1 * pc + k2 * pw + k3 * pe + c[3] * ps + c[4] * pn;
    return c[0] * pc + c[1] * pw + c[2] * pe + c[3] * ps + c[4] * pn;
  }
  return c[0] * pc + c[1] * pw + c[2] * pe + c[3] * ps + c[4] * pn + c[5] * pb + c[6] * pf;
}

// apply_lpl with the neighbours across the box faces given by face_ghost,
// i.e. the values af_gc_box would store in the ghost cells at this moment,
// so no ghost-cell fill is needed before the stencil.
template <int D, bool CYL, typename T>
__device__ __forceinline__ T apply_lpl_otf(const KTree& t, const T* __restrict__ phi, const T* __restrict__ p,
                                           int slot, int i, int j, int k, const T c[7], T k1, T k2, T k3,
                                           const GcDev& g, const int4& r0, const int4& r1) {
  const int nc = t.nc, n2 = t.n2;
  if (D == 2) {
    const int x = at2(n2, i, j);
    const T pw = i == 1 ? face_ghost_nb<D, T>(t, phi, slot, 0, r0.y, j, 0, g) : p[x - 1];
    const T pe = i == nc ? face_ghost_nb<D, T>(t, phi, slot, 1, r0.z, j, 0, g) : p[x + 1];
    const T ps = j == 1 ? face_ghost_nb<D, T>(t, phi, slot, 2, r0.w, i, 0, g) : p[x - n2];
    const T pn = j == nc ? face_ghost_nb<D, T>(t, phi, slot, 3, r1.x, i, 0, g) : p[x + n2];
    return lpl_vals<D, CYL, T>(p[x], pw, pe, ps, pn, T(0), T(0), c, k1, k2, k3);
  } else {
    const int x = at3(n2, i, j, k), sk = n2 * n2;
    const T pw = i == 1 ? face_ghost_nb<D, T>(t, phi, slot, 0, r0.y, j, k, g) : p[x - 1];
    const T pe = i == nc ? face_ghost_nb<D, T>(t, phi, slot, 1, r0.z, j, k, g) : p[x + 1];
    const T ps = j == 1 ? face_ghost_nb<D, T>(t, phi, slot, 2, r0.w, i, k, g) : p[x - n2];
    const T pn = j == nc ? face_ghost_nb<D, T>(t, phi, slot, 3, r1.x, i, k, g) : p[x + n2];
    const T pb = k == 1 ? face_ghost_nb<D, T>(t, phi, slot, 4, r1.y, i, j, g) : p[x - sk];
    const T pf = k == nc ? face_ghost_nb<D, T>(t, phi, slot, 5, r1.z, i, j, g) : p[x + sk];
    return lpl_vals<D, CYL, T>(p[x], pw, pe, ps, pn, pb, pf, c, k1, k2, k3);
  }
}

// One red-black half sweep on each box of the list; stencil_gsrb_357
// (m_af_stencil.f90:838-998).  Updated cells satisfy (i+j[+k]+n) even.
template <int D, bool CYL, typename T, int NC = 0>
__global__ void __launch_bounds__(256) k_gsrb(KTree t0, const int* __restrict__ list, T* __restrict__ phi,
                                              const T* __restrict__ rhs, int redblack, MgCoef<T> mc) {
  const KTree t = fix_dims<D, NC>(t0);
  const int slot = list[blockIdx.x];
  if (box_frozen(t, slot) || lsf_box(t, slot)) return;
  const int nc = t.nc, n2 = t.n2, hn = nc / 2;
  T c[7];
  for (int q = 0; q < 7; q++) c[q] = mc.cb[slot * 8 + q];
  const T inv_c1 = mc.cb[slot * 8 + 7];
  T* p = phi + (size_t)slot * t.S;
  const T* f = rhs + (size_t)slot * t.S;
  const int count = D == 2 ? nc * hn : nc * nc * hn;
  for (int w = threadIdx.x; w < count; w += blockDim.x) {
    const int row = w / hn, col = w - row * hn;
    if (D == 2) {
      const int j = row + 1;
      const int i = 2 - ((redblack ^ j) & 1) + 2 * col;
      const int x = at2(n2, i, j);
      if (CYL) {
        const T* y = mc.cy + ((size_t)slot * nc + (i - 1)) * 4;
        p[x] = (f[x] - y[1] * p[x - 1] - y[2] * p[x + 1] - c[3] * p[x - n2] - c[4] * p[x + n2]) * y[3];
      } else {
        p[x] = (f[x] - c[1] * p[x - 1] - c[2] * p[x + 1] - c[3] * p[x - n2] - c[4] * p[x + n2]) * inv_c1;
      }
    } else {
      const int j = row % nc + 1, k = row / nc + 1;
      const int i = 2 - ((redblack ^ (k + j)) & 1) + 2 * col;
      const int x = at3(n2, i, j, k), sk = n2 * n2;
      p[x] = (f[x] - c[1] * p[x - 1] - c[2] * p[x + 1] - c[3] * p[x - n2] - c[4] * p[x + n2] -
              c[5] * p[x - sk] - c[6] * p[x + sk]) *
             inv_c1;
    }
  }
}

// Red-black half sweep with the ghost-cell refresh fused in: a neighbour
// outside the box is evaluated on the fly with the box's ghost rule
// (face_ghost) instead of being read from the ghost layer.  Between half
// sweeps the reference refreshes every ghost cell (gsrb_boxes,
// m_af_multigrid.f90:666-684); the on-the-fly value is the value that refresh
// stores, because each ghost read by a cell of colour c depends only on
// cells of the other colour, on the coarse level, and on the updated cell
// itself before its update.  One ghost fill after the last half sweep then
// leaves memory exactly as the reference does.
template <int D, bool CYL, typename T, int NC = 0>
__global__ void __launch_bounds__(256, 6) k_gsrb_fused(KTree t0, const int* __restrict__ list, ModeArg<T> phi_,
                                                    ModeArg<const T> rhs_, int redblack, ModeCoef<T> mc_,
                                                    GcDev g) {
  const KTree t = fix_dims<D, NC>(t0);
  T* __restrict__ phi = phi_.get();
  const T* __restrict__ rhs = rhs_.get();
  const MgCoef<T> mc = mc_.get();
  const int slot = list[blockIdx.x];
  if (box_frozen(t, slot) || lsf_box(t, slot)) return;
  const int nc = t.nc, n2 = t.n2, hn = nc / 2;
  T c[7];
  for (int q = 0; q < 7; q++) c[q] = mc.cb[slot * 8 + q];
  const T inv_c1 = mc.cb[slot * 8 + 7];
  T* p = phi + (size_t)slot * t.S;
  const T* f = rhs + (size_t)slot * t.S;
  const int count = D == 2 ? nc * hn : nc * nc * hn;
  for (int w = threadIdx.x; w < count; w += blockDim.x) {
    const int row = w / hn, col = w - row * hn;
    if (D == 2) {
      const int j = row + 1;
      const int i = 2 - ((redblack ^ j) & 1) + 2 * col;
      const int x = at2(n2, i, j);
      const T pw = i == 1 ? face_ghost<D, T>(t, phi, slot, 0, j, 0, g) : p[x - 1];
      const T pe = i == nc ? face_ghost<D, T>(t, phi, slot, 1, j, 0, g) : p[x + 1];
      const T ps = j == 1 ? face_ghost<D, T>(t, phi, slot, 2, i, 0, g) : p[x - n2];
      const T pn = j == nc ? face_ghost<D, T>(t, phi, slot, 3, i, 0, g) : p[x + n2];
      if (CYL) {
        const T* y = mc.cy + ((size_t)slot * nc + (i - 1)) * 4;
        p[x] = (f[x] - y[1] * pw - y[2] * pe - c[3] * ps - c[4] * pn) * y[3];
      } else {
        p[x] = (f[x] - c[1] * pw - c[2] * pe - c[3] * ps - c[4] * pn) * inv_c1;
      }
    } else {
      const int j = row % nc + 1, k = row / nc + 1;
      const int i = 2 - ((redblack ^ (k + j)) & 1) + 2 * col;
      const int x = at3(n2, i, j, k), sk = n2 * n2;
      const T pw = i == 1 ? face_ghost<D, T>(t, phi, slot, 0, j, k, g) : p[x - 1];
      const T pe = i == nc ? face_ghost<D, T>(t, phi, slot, 1, j, k, g) : p[x + 1];
      const T ps = j == 1 ? face_ghost<D, T>(t, phi, slot, 2, i, k, g) : p[x - n2];
      const T pn = j == nc ? face_ghost<D, T>(t, phi, slot, 3, i, k, g) : p[x + n2];
      const T pb = k == 1 ? face_ghost<D, T>(t, phi, slot, 4, i, j, g) : p[x - sk];
      const T pf = k == nc ? face_ghost<D, T>(t, phi, slot, 5, i, j, g) : p[x + sk];
      p[x] = (f[x] - c[1] * pw - c[2] * pe - c[3] * ps - c[4] * pn - c[5] * pb - c[6] * pf) * inv_c1;
    }
  }
}

// The same half sweep for a compile-time box size NC: CPT cells of the colour
// per thread, all their loads issued before the stores (cells of one colour
// never read each other), and the box's slot and face neighbours from its
// 32-byte record (one load instead of a list load and neighbour-table loads).
// The arithmetic is that of k_gsrb_fused.
template <int D, bool CYL, typename T, int NC, int CPT>
__global__ void __launch_bounds__((D == 2 ? NC * NC / 2 : NC * NC * NC / 2) / CPT,
                                  1536 / ((D == 2 ? NC * NC / 2 : NC * NC * NC / 2) / CPT))
    k_gsrb_rec(KTree t0, const int* __restrict__ rec, ModeArg<T> phi_, ModeArg<const T> rhs_, int redblack,
               ModeCoef<T> mc_, GcDev g) {
  constexpr int TPB = (D == 2 ? NC * NC / 2 : NC * NC * NC / 2) / CPT;
  constexpr int nc = NC, n2 = NC + 2, hn = NC / 2, sk = n2 * n2;
  const KTree t = fix_dims<D, NC>(t0);
  T* __restrict__ phi = phi_.get();
  const T* __restrict__ rhs = rhs_.get();
  const MgCoef<T> mc = mc_.get();
  const int4 r0 = reinterpret_cast<const int4*>(rec)[2 * blockIdx.x];
  const int4 r1 = reinterpret_cast<const int4*>(rec)[2 * blockIdx.x + 1];
  const int slot = r0.x;
  if (box_frozen(t, slot)) return;
  T c[7];
  for (int q = 0; q < 2 * D + 1; q++) c[q] = mc.cb[slot * 8 + q];
  const T inv_c1 = mc.cb[slot * 8 + 7];
  T* p = phi + (size_t)slot * t.S;
  const T* f = rhs + (size_t)slot * t.S;
  T val[CPT];
  int xs[CPT];
#pragma unroll
  for (int u = 0; u < CPT; u++) {
    const int w = (int)threadIdx.x + u * TPB;
    const int row = w / hn, col = w - row * hn;
    if (D == 2) {
      const int j = row + 1;
      const int i = 2 - ((redblack ^ j) & 1) + 2 * col;
      const int x = at2(n2, i, j);
      const T pw = i == 1 ? face_ghost_nb<D, T>(t, phi, slot, 0, r0.y, j, 0, g) : p[x - 1];
      const T pe = i == nc ? face_ghost_nb<D, T>(t, phi, slot, 1, r0.z, j, 0, g) : p[x + 1];
      const T ps = j == 1 ? face_ghost_nb<D, T>(t, phi, slot, 2, r0.w, i, 0, g) : p[x - n2];
      const T pn = j == nc ? face_ghost_nb<D, T>(t, phi, slot, 3, r1.x, i, 0, g) : p[x + n2];
      if (CYL) {
        const T* y = mc.cy + ((size_t)slot * nc + (i - 1)) * 4;
        val[u] = (f[x] - y[1] * pw - y[2] * pe - c[3] * ps - c[4] * pn) * y[3];
      } else {
        val[u] = (f[x] - c[1] * pw - c[2] * pe - c[3] * ps - c[4] * pn) * inv_c1;
      }
      xs[u] = x;
    } else {
      const int j = row % nc + 1, k = row / nc + 1;
      const int i = 2 - ((redblack ^ (k + j)) & 1) + 2 * col;
      const int x = at3(n2, i, j, k);
      const T pw = i == 1 ? face_ghost_nb<D, T>(t, phi, slot, 0, r0.y, j, k, g) : p[x - 1];
      const T pe = i == nc ? face_ghost_nb<D, T>(t, phi, slot, 1, r0.z, j, k, g) : p[x + 1];
      const T ps = j == 1 ? face_ghost_nb<D, T>(t, phi, slot, 2, r0.w, i, k, g) : p[x - n2];
      const T pn = j == nc ? face_ghost_nb<D, T>(t, phi, slot, 3, r1.x, i, k, g) : p[x + n2];
      const T pb = k == 1 ? face_ghost_nb<D, T>(t, phi, slot, 4, r1.y, i, j, g) : p[x - sk];
      const T pf = k == nc ? face_ghost_nb<D, T>(t, phi, slot, 5, r1.z, i, j, g) : p[x + sk];
      val[u] = (f[x] - c[1] * pw - c[2] * pe - c[3] * ps - c[4] * pn - c[5] * pb - c[6] * pf) * inv_c1;
      xs[u] = x;
    }
  }
#pragma unroll
  for (int u = 0; u < CPT; u++) p[xs[u]] = val[u];
}

// The same half sweep with the boxes staged in shared memory: a persistent
// grid walks the record list, each CTA copying the next box's phi block
// ((nc+2)^D values, ghost layers included; with SR also its rhs block) into
// shared memory with bulk asynchronous copies while it updates the current
// box from the previous copy (two stages, one mbarrier each).  Without SR
// the right-hand side, read once per cell, is loaded from global memory
// before the wait (half the shared memory, more CTAs per SM).  Per box, first the face
// ghosts that this half sweep reads (those next to cells of its colour, half
// of each face) are evaluated cooperatively with face_ghost_nb on global
// memory (the values af_gc would store) into the staged block; then every
// thread updates its cells from shared memory alone, without branches.
// Interior neighbours are cells of the other colour, which no CTA writes in
// a half sweep, so the staged copy is current.  Results go to global memory;
// the arithmetic is that of k_gsrb_rec.  A wait that times out (1 s) sets
// *err; the CTA then waits (bounded) for its copies in flight and returns.
template <int D, bool CYL, typename T, int NC, int CPT, bool SR>
__global__ void __launch_bounds__((D == 2 ? NC * NC / 2 : NC * NC * NC / 2) / CPT)
    k_gsrb_tma(KTree t0, const int* __restrict__ rec, int n, ModeArg<T> phi_, ModeArg<const T> rhs_, int redblack,
               ModeCoef<T> mc_, GcDev g, unsigned* err) {
  T* __restrict__ phi = phi_.get();
  const T* __restrict__ rhs = rhs_.get();
  const MgCoef<T> mc = mc_.get();
  constexpr int TPB = (D == 2 ? NC * NC / 2 : NC * NC * NC / 2) / CPT;
  constexpr int nc = NC, n2 = NC + 2, hn = NC / 2, sk = n2 * n2;
  constexpr int S = D == 2 ? n2 * n2 : n2 * n2 * n2;
  constexpr int NGF = D == 2 ? hn : nc * hn;  // ghosts read per face and half sweep
  constexpr unsigned BYTES = S * sizeof(T);
  static_assert(BYTES % 16 == 0, "bulk copies need 16-byte multiples");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* sphi = reinterpret_cast<T*>(smem_raw);  // [2][S]
  T* srhs = sphi + 2 * S;                     // [2][S] when SR
  __shared__ __align__(8) unsigned long long bar[2];
  const KTree t = fix_dims<D, NC>(t0);
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  // thread 0: copies of list entry e into stage st
  auto issue = [&](int e, int st) {
    const int s = rec[8 * e];
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bar[st], SR ? 2 * BYTES : BYTES);
    bulk_copy_g2s(sphi + st * S, phi + (size_t)s * S, BYTES, &bar[st]);
    if (SR) bulk_copy_g2s(srhs + st * S, rhs + (size_t)s * S, BYTES, &bar[st]);
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
    T c[7];
    for (int q = 0; q < 2 * D + 1; q++) c[q] = mc.cb[slot * 8 + q];
    const T inv_c1 = mc.cb[slot * 8 + 7];
    // this thread's cells and their right-hand sides, loaded before the wait
    const T* f = rhs + (size_t)slot * S;
    T fv[CPT];
    int xs[CPT];
#pragma unroll
    for (int u = 0; u < CPT; u++) {
      const int w = (int)threadIdx.x + u * TPB;
      const int row = w / hn, col = w - row * hn;
      if (D == 2) {
        const int j = row + 1;
        xs[u] = at2(n2, 2 - ((redblack ^ j) & 1) + 2 * col, j);
      } else {
        const int j = row % nc + 1, k = row / nc + 1;
        xs[u] = at3(n2, 2 - ((redblack ^ (k + j)) & 1) + 2 * col, j, k);
      }
      if (!SR) fv[u] = f[xs[u]];
    }
    const bool ok = mbar_wait(&bar[st], (it >> 1) & 1);
    if (__syncthreads_or(!ok)) {
      // give up: drain the copies in flight into both stages (bounded
      // waits); if they do not complete either, bit 2 of *err tells the
      // host that the CTA returned with copies outstanding
      if (threadIdx.x == 0) {
        bool drained = mbar_wait(&bar[st], (it >> 1) & 1);
        if (next) drained = mbar_wait(&bar[st ^ 1], ((it + 1) >> 1) & 1) && drained;
        atomicOr(err, drained ? 1u : 3u);
      }
      return;
    }
    const bool active = !box_frozen(t, slot);
    T* P = sphi + st * S;
    if (SR) {
#pragma unroll
      for (int u = 0; u < CPT; u++) fv[u] = srhs[st * S + xs[u]];
    }
    // face ghosts next to cells of this colour: cell (i, j[, k]) is updated
    // when i + j (+ k) + redblack is even
    for (int w = threadIdx.x; active && w < 2 * D * NGF; w += TPB) {
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
      P[face_at<D>(n2, d, low ? 0 : nc + 1, pt, qt)] =
          face_ghost_nb<D, T>(t, phi, slot, nb, rec_nb(r0, r1, nb), pt, qt, g);
    }
    __syncthreads();
    if (active) {
      T* p = phi + (size_t)slot * S;
      T val[CPT];
#pragma unroll
      for (int u = 0; u < CPT; u++) {
        const int x = xs[u];
        if (D == 2) {
          if (CYL) {
            const int i = x % n2;
            const T* y = mc.cy + ((size_t)slot * nc + (i - 1)) * 4;
            val[u] = (fv[u] - y[1] * P[x - 1] - y[2] * P[x + 1] - c[3] * P[x - n2] - c[4] * P[x + n2]) * y[3];
          } else {
            val[u] = (fv[u] - c[1] * P[x - 1] - c[2] * P[x + 1] - c[3] * P[x - n2] - c[4] * P[x + n2]) * inv_c1;
          }
        } else {
          val[u] = (fv[u] - c[1] * P[x - 1] - c[2] * P[x + 1] - c[3] * P[x - n2] - c[4] * P[x + n2] -
                    c[5] * P[x - sk] - c[6] * P[x + sk]) *
                   inv_c1;
        }
      }
#pragma unroll
      for (int u = 0; u < CPT; u++) p[xs[u]] = val[u];
    }
    __syncthreads();  // stage st is read completely before it is refilled
  }
}

// Residual on interior cells into tmp (residual_box, m_af_multigrid.f90:
// 801-810); the max |r| over the boxes flagged in is_leaf is folded into
// *maxbits (may be null).
template <int D, bool CYL, typename T, int NC = 0>
__global__ void __launch_bounds__(256) k_residual(KTree t0, const int* __restrict__ list, const T* __restrict__ phi,
                                                  const T* __restrict__ rhs, T* __restrict__ tmp, MgCoef<T> mc,
                                                  const unsigned char* __restrict__ is_leaf,
                                                  unsigned long long* maxbits) {
  const KTree t = fix_dims<D, NC>(t0);
  __shared__ T sred[32];
  const int slot = list[blockIdx.x];
  if (box_frozen(t, slot) || lsf_box(t, slot)) return;
  const int nc = t.nc, n2 = t.n2;
  T c[7];
  for (int q = 0; q < 7; q++) c[q] = mc.cb[slot * 8 + q];
  const T* p = phi + (size_t)slot * t.S;
  const T* f = rhs + (size_t)slot * t.S;
  T* o = tmp + (size_t)slot * t.S;
  const int count = D == 2 ? nc * nc : nc * nc * nc;
  T mx = T(0);
  for (int w = threadIdx.x; w < count; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 0 : r / nc + 1;
    T k1 = T(0), k2 = T(0), k3 = T(0);
    if (CYL) {
      const T* y = mc.cy + ((size_t)slot * nc + (i - 1)) * 4;
      k1 = y[0]; k2 = y[1]; k3 = y[2];
    }
    const int x = D == 2 ? at2(n2, i, j) : at3(n2, i, j, k);
    const T res = f[x] - apply_lpl<D, CYL, T>(p, n2, i, j, k, c, k1, k2, k3);
    o[x] = res;
    acc_absmax(mx, res);
  }
  if (maxbits != nullptr && is_leaf[slot]) {
    mx = block_max<T>(mx, sred);
    if (threadIdx.x == 0) atomic_max_nonneg(inst_max(t, maxbits, slot), double(mx));
  }
}

// update_coarse first half (m_af_multigrid.f90:706-719): residual of each
// child box restricted to its parent's tmp (with the cylindrical weights,
// af_restrict_box use_geometry=.true., m_af_restrict.f90:62-136), phi
// restricted without geometry (mg_box_rstr_lpl 1227-1242).  One thread per
// parent cell covered by the child.
template <int D, bool CYL, typename T, int NC = 0>
__global__ void __launch_bounds__(256) k_residual_restrict(KTree t0, const int* __restrict__ rec,
                                                           ModeArg<T> phi_, ModeArg<const T> rhs_, ModeArg<T> tmp_,
                                                           ModeCoef<T> mc_, int store_child_residual, GcDev g,
                                                           int otf) {
  const KTree t = fix_dims<D, NC>(t0);
  T* __restrict__ phi = phi_.get();
  const T* __restrict__ rhs = rhs_.get();
  T* __restrict__ tmp = tmp_.get();
  const MgCoef<T> mc = mc_.get();
  int4 r0, r1;
  load_rec(rec, blockIdx.x, r0, r1);
  const int slot = r0.x;
  if (box_frozen(t, slot) || lsf_box(t, slot)) return;
  const int pslot = t.parent[slot];
  const int nc = t.nc, n2 = t.n2, hnc = nc / 2;
  T c[7];
  for (int q = 0; q < 7; q++) c[q] = mc.cb[slot * 8 + q];
  const T* p = phi + (size_t)slot * t.S;
  const T* f = rhs + (size_t)slot * t.S;
  T* pp = phi + (size_t)pslot * t.S;
  T* pt = tmp + (size_t)pslot * t.S;
  T* ct = tmp + (size_t)slot * t.S;
  const int o0 = child_offset(t, slot, 0), o1 = child_offset(t, slot, 1);
  const int o2 = D == 3 ? child_offset(t, slot, 2) : 0;
  const int count = D == 2 ? hnc * hnc : hnc * hnc * hnc;
  for (int w = threadIdx.x; w < count; w += blockDim.x) {
    const int i = w % hnc + 1, r = w / hnc;
    const int j = D == 2 ? r + 1 : r % hnc + 1, k = D == 2 ? 0 : r / hnc + 1;
    const int ic = o0 + i, jc = o1 + j, kc = o2 + k;
    const int fi = 2 * i - 1, fj = 2 * j - 1, fk = D == 3 ? 2 * k - 1 : 0;
    if (D == 2) {
      T res[2][2];  // [dj][di]
      for (int dj = 0; dj < 2; dj++)
        for (int di = 0; di < 2; di++) {
          T k1 = T(0), k2 = T(0), k3 = T(0);
          if (CYL) {
            const T* y = mc.cy + ((size_t)slot * nc + (fi + di - 1)) * 4;
            k1 = y[0]; k2 = y[1]; k3 = y[2];
          }
          const int x = at2(n2, fi + di, fj + dj);
          res[dj][di] = f[x] - (otf ? apply_lpl_otf<D, CYL, T>(t, phi, p, slot, fi + di, fj + dj, 0, c, k1, k2, k3, g, r0, r1)
                                    : apply_lpl<D, CYL, T>(p, n2, fi + di, fj + dj, 0, c, k1, k2, k3));
          if (store_child_residual) ct[x] = res[dj][di];
        }
      T rv;
      if (CYL) {
        const double* gw = t.geo + ((size_t)pslot * nc + (ic - 1)) * 4;
        const T w1 = T(gw[2]), w2 = T(gw[3]);
        T s1 = T(0), s2 = T(0);
        s1 = s1 + res[0][0]; s1 = s1 + res[1][0];
        s2 = s2 + res[0][1]; s2 = s2 + res[1][1];
        rv = T(0.25) * (w1 * s1 + w2 * s2);
      } else {
        T s = T(0);
        s = s + res[0][0]; s = s + res[0][1]; s = s + res[1][0]; s = s + res[1][1];
        rv = T(0.25) * s;
      }
      pt[at2(n2, ic, jc)] = rv;
      T s = T(0);
      s = s + p[at2(n2, fi, fj)]; s = s + p[at2(n2, fi + 1, fj)];
      s = s + p[at2(n2, fi, fj + 1)]; s = s + p[at2(n2, fi + 1, fj + 1)];
      pp[at2(n2, ic, jc)] = T(0.25) * s;
    } else {
      T sr = T(0), sp = T(0);
      for (int dk = 0; dk < 2; dk++)
        for (int dj = 0; dj < 2; dj++)
          for (int di = 0; di < 2; di++) {
            const int x = at3(n2, fi + di, fj + dj, fk + dk);
            const T res =
                f[x] - (otf ? apply_lpl_otf<D, false, T>(t, phi, p, slot, fi + di, fj + dj, fk + dk, c, T(0), T(0),
                                                         T(0), g, r0, r1)
                            : apply_lpl<D, false, T>(p, n2, fi + di, fj + dj, fk + dk, c, T(0), T(0), T(0)));
            if (store_child_residual) ct[x] = res;
            sr = sr + res;
            sp = sp + p[x];
          }
      pt[at3(n2, ic, jc, kc)] = T(0.125) * sr;
      pp[at3(n2, ic, jc, kc)] = T(0.125) * sp;
    }
  }
}

// update_coarse second half (m_af_multigrid.f90:723-737) on the parents of
// the level: rhs = L phi + tmp (interior), tmp = phi (whole array).  The
// reference also adds tmp to rhs in the ghost cells; rhs ghost cells are
// never read, so they are left untouched.  With copy_tmp = 0 this is the
// rhs part of set_coarse_phi_rhs (742-776).
//
// fill != 0: the parent's ghost cells of phi are filled first (faces, then
// edges and corners: af_gc_box), so the stencil and the copy into tmp see
// them; this replaces the level-wide ghost fill between the restriction and
// this step (leaf boxes of the level need none there: the fused smoother
// computes its own and the level is filled again after its up smoothing).
template <int D, bool CYL, typename T, int NC = 0>
__global__ void __launch_bounds__(256) k_coarse_fas(KTree t0, const int* __restrict__ rec, ModeArg<T> phi_,
                                                    ModeArg<T> rhs_, ModeArg<T> tmp_, ModeCoef<T> mc_, int copy_tmp,
                                                    int fill, GcDev g) {
  const KTree t = fix_dims<D, NC>(t0);
  T* __restrict__ phi = phi_.get();
  T* __restrict__ rhs = rhs_.get();
  T* __restrict__ tmp = tmp_.get();
  const MgCoef<T> mc = mc_.get();
  int4 r0, r1;
  load_rec(rec, blockIdx.x, r0, r1);
  const int slot = r0.x;
  if (box_frozen(t, slot) || lsf_box(t, slot)) return;
  const int nc = t.nc, n2 = t.n2;
  if (fill) {
    T* a = phi + (size_t)slot * t.S;
    const int nface = D == 2 ? nc : nc * nc;
    for (int w = threadIdx.x; w < 2 * D * nface; w += blockDim.x) {
      const int nb = w / nface, pq = w - nb * nface;
      const int pi = pq % nc + 1, qi = D == 3 ? pq / nc + 1 : 0;
      const T val = face_ghost_nb<D, T>(t, phi, slot, nb, rec_nb(r0, r1, nb), pi, qi, g);
      a[face_at<D>(n2, nb >> 1, (nb & 1) ? nc + 1 : 0, pi, qi)] = val;
    }
    __syncthreads();
    corner_ghosts<D, T>(t, phi, slot);
    __syncthreads();
  }
  T c[7];
  for (int q = 0; q < 7; q++) c[q] = mc.cb[slot * 8 + q];
  const T* p = phi + (size_t)slot * t.S;
  T* f = rhs + (size_t)slot * t.S;
  T* o = tmp + (size_t)slot * t.S;
  for (int x = threadIdx.x; x < t.S; x += blockDim.x) {
    const int i = x % n2, r = x / n2;
    const int j = D == 2 ? r : r % n2, k = D == 2 ? 0 : r / n2;
    const bool interior = i >= 1 && i <= nc && j >= 1 && j <= nc && (D == 2 || (k >= 1 && k <= nc));
    if (interior) {
      T k1 = T(0), k2 = T(0), k3 = T(0);
      if (CYL) {
        const T* y = mc.cy + ((size_t)slot * nc + (i - 1)) * 4;
        k1 = y[0]; k2 = y[1]; k3 = y[2];
      }
      const T lp = apply_lpl<D, CYL, T>(p, n2, i, j, k, c, k1, k2, k3);
      f[x] = lp + o[x];
    }
    if (copy_tmp) o[x] = p[x];
  }
}

// correct_children (m_af_multigrid.f90:624-646): on each parent,
// tmp = phi - tmp over the whole array, then each child's phi gets the
// bilinear/trilinear prolongation of tmp added (stencil_prolong_248,
// m_af_stencil.f90:695-815, coefficients 1267-1284).
template <int D, typename T, int NC = 0>
__global__ void __launch_bounds__(256) k_correct(KTree t0, const int* __restrict__ list, ModeArg<T> phi_,
                                                 ModeArg<T> tmp_) {
  const KTree t = fix_dims<D, NC>(t0);
  T* __restrict__ phi = phi_.get();
  T* __restrict__ tmp = tmp_.get();
  extern __shared__ unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const int slot = list[blockIdx.x];
  if (box_frozen(t, slot)) return;
  const int nc = t.nc, n2 = t.n2;
  T* pp = phi + (size_t)slot * t.S;
  T* pt = tmp + (size_t)slot * t.S;
  for (int x = threadIdx.x; x < t.S; x += blockDim.x) {
    const T v = pp[x] - pt[x];
    pt[x] = v;
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
    T* cp = phi + (size_t)cs * t.S;
    if (D == 2) {
      const int x = at2(n2, i, j);
      cp[x] = cp[x] + T(9 / 16.0) * sm[at2(n2, i1, j1)] + T(3 / 16.0) * sm[at2(n2, i2, j1)] +
              T(3 / 16.0) * sm[at2(n2, i1, j2)] + T(1 / 16.0) * sm[at2(n2, i2, j2)];
    } else {
      const int o2 = child_offset(t, cs, 2);
      const int k1 = o2 + ((k + 1) >> 1), k2 = k1 + 1 - 2 * (k & 1);
      const int x = at3(n2, i, j, k);
      cp[x] = cp[x] + T(27 / 64.0) * sm[at3(n2, i1, j1, k1)] + T(9 / 64.0) * sm[at3(n2, i2, j1, k1)] +
              T(9 / 64.0) * sm[at3(n2, i1, j2, k1)] + T(3 / 64.0) * sm[at3(n2, i2, j2, k1)] +
              T(9 / 64.0) * sm[at3(n2, i1, j1, k2)] + T(3 / 64.0) * sm[at3(n2, i2, j1, k2)] +
              T(3 / 64.0) * sm[at3(n2, i1, j2, k2)] + T(1 / 64.0) * sm[at3(n2, i2, j2, k2)];
    }
  }
}

// init_phi_rhs (m_af_multigrid.f90:779-799) on one level: phi = 0 on the
// whole array, rhs restricted to the parent with geometry.
template <int D, bool CYL, typename T, int NC = 0>
__global__ void __launch_bounds__(256) k_init_phi_rhs(KTree t0, const int* __restrict__ list, ModeArg<T> phi_,
                                                      ModeArg<T> rhs_) {
  const KTree t = fix_dims<D, NC>(t0);
  T* __restrict__ phi = phi_.get();
  T* __restrict__ rhs = rhs_.get();
  const int slot = list[blockIdx.x];
  if (box_frozen(t, slot)) return;
  const int pslot = t.parent[slot];
  const int nc = t.nc, n2 = t.n2, hnc = nc / 2;
  T* p = phi + (size_t)slot * t.S;
  const T* f = rhs + (size_t)slot * t.S;
  T* pf = rhs + (size_t)pslot * t.S;
  for (int x = threadIdx.x; x < t.S; x += blockDim.x) p[x] = T(0);
  const int o0 = child_offset(t, slot, 0), o1 = child_offset(t, slot, 1);
  const int o2 = D == 3 ? child_offset(t, slot, 2) : 0;
  const int count = D == 2 ? hnc * hnc : hnc * hnc * hnc;
  for (int w = threadIdx.x; w < count; w += blockDim.x) {
    const int i = w % hnc + 1, r = w / hnc;
    const int j = D == 2 ? r + 1 : r % hnc + 1, k = D == 2 ? 0 : r / hnc + 1;
    const int ic = o0 + i, jc = o1 + j, kc = o2 + k;
    const int fi = 2 * i - 1, fj = 2 * j - 1, fk = D == 3 ? 2 * k - 1 : 0;
    if (D == 2) {
      T rv;
      if (CYL) {
        const double* gw = t.geo + ((size_t)pslot * nc + (ic - 1)) * 4;
        const T w1 = T(gw[2]), w2 = T(gw[3]);
        T s1 = T(0), s2 = T(0);
        s1 = s1 + f[at2(n2, fi, fj)]; s1 = s1 + f[at2(n2, fi, fj + 1)];
        s2 = s2 + f[at2(n2, fi + 1, fj)]; s2 = s2 + f[at2(n2, fi + 1, fj + 1)];
        rv = T(0.25) * (w1 * s1 + w2 * s2);
      } else {
        T s = T(0);
        s = s + f[at2(n2, fi, fj)]; s = s + f[at2(n2, fi + 1, fj)];
        s = s + f[at2(n2, fi, fj + 1)]; s = s + f[at2(n2, fi + 1, fj + 1)];
        rv = T(0.25) * s;
      }
      pf[at2(n2, ic, jc)] = rv;
    } else {
      T s = T(0);
      for (int dk = 0; dk < 2; dk++)
        for (int dj = 0; dj < 2; dj++)
          for (int di = 0; di < 2; di++) s = s + f[at3(n2, fi + di, fj + dj, fk + dk)];
      pf[at3(n2, ic, jc, kc)] = T(0.125) * s;
    }
  }
}

// Whole-array copy of one variable on a box list (af_boxes_copy_cc,
// m_af_utils.f90:579-588).
template <typename T>
__global__ void __launch_bounds__(256) k_copy(KTree t, const int* __restrict__ list, ModeArg<const T> src_,
                                              ModeArg<T> dst_) {
  const T* __restrict__ src = src_.get();
  T* __restrict__ dst = dst_.get();
  const int slot = list[blockIdx.x];
  if (box_frozen(t, slot)) return;
  const int S = t.S;
  for (int x = threadIdx.x; x < S; x += blockDim.x) dst[(size_t)slot * S + x] = src[(size_t)slot * S + x];
}

// Coarse-grid right-hand side with the boundary values folded in
// (coarse_solver_set_rhs_phi, m_coarse_solver.f90:286-338).  Batched trees
// stack one coarse grid of nloc unknowns per instance (n = n_inst * nloc):
// the boundary tables are per local unknown, the values per instance
// (bc_val + instance * bc_stride).
template <typename T>
__global__ void k_coarse_gather(int n, int nloc, int D, const int* __restrict__ cslot, const int* __restrict__ ccell,
                                const double* __restrict__ b2r, const unsigned char* __restrict__ bmask,
                                const double* __restrict__ bc_val, int bc_stride, ModeArg<const T> rhs_, int S,
                                ModeArg<double> b_) {
  const T* __restrict__ rhs = rhs_.get();
  double* __restrict__ b = b_.get();
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const int q = g / nloc, gl = g - q * nloc;
  const double* bv = bc_val + (size_t)q * bc_stride;
  double v = double(rhs[(size_t)cslot[g] * S + ccell[g]]);
  const unsigned m = bmask[gl];
  for (int nb = 0; nb < 2 * D; nb++)
    if (m & (1u << nb)) v = v + b2r[gl * 2 * D + nb] * bv[nb];
  b[g] = v;
}

// x = A^-1 b per instance (the same inverse of nloc x nloc for all), one
// warp per row: 32 strided partial sums then an xor butterfly; the CPU
// oracle uses the same order.
__global__ void k_coarse_matvec(int n, int nloc, ModeArg<const double> ainv_, ModeArg<const double> b_,
                                ModeArg<double> x_) {
  const double* __restrict__ ainv = ainv_.get();
  const double* __restrict__ b = b_.get();
  double* __restrict__ x = x_.get();
  const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const int q = row / nloc, rl = row - q * nloc;
  const double* a = ainv + (size_t)rl * nloc;
  const double* bq = b + (size_t)q * nloc;
  double s = 0.0;
  for (int c = lane; c < nloc; c += 32) s = s + a[c] * bq[c];
  for (int o = 16; o > 0; o >>= 1) s = s + __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) x[row] = s;
}

// (stride: values per box of phi's blocks, the cell index from ccell)
template <typename T>
__global__ void k_coarse_scatter(KTree t, int n, const int* __restrict__ cslot, const int* __restrict__ ccell,
                                 int stride, ModeArg<const double> x_, ModeArg<T> phi_) {
  const double* __restrict__ x = x_.get();
  T* __restrict__ phi = phi_.get();
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const int slot = cslot[g];
  if (box_frozen(t, slot)) return;
  phi[(size_t)slot * stride + ccell[g]] = T(x[g]);
}

// Freeze flags of batched instances as the kernels read them: the converged
// instances (base) and those whose highest level lies outside [lo, hi].  An
// FMG step at level l runs with [l, inf) (instances without level l are
// finished with their FMG) and its residual with [l, l].
__global__ void k_inst_mask(int n, const int* __restrict__ base, const int* __restrict__ hl, int lo, int hi,
                            int* __restrict__ eff) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  eff[q] = (base[q] != 0 || hl[q] < lo || hl[q] > hi) ? 1 : 0;
}

// max |v| over interior cells of the list's boxes
template <int D, typename T, int NC = 0>
__global__ void __launch_bounds__(256) k_maxabs(KTree t0, const int* __restrict__ list, const T* __restrict__ v,
                                                unsigned long long* maxbits) {
  const KTree t = fix_dims<D, NC>(t0);
  __shared__ T sred[32];
  const int slot = list[blockIdx.x];
  const int nc = t.nc, n2 = t.n2;
  const T* a = v + (size_t)slot * t.S;
  const int count = D == 2 ? nc * nc : nc * nc * nc;
  T mx = T(0);
  for (int w = threadIdx.x; w < count; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 0 : r / nc + 1;
    acc_absmax(mx, a[D == 2 ? at2(n2, i, j) : at3(n2, i, j, k)]);
  }
  mx = block_max<T>(mx, sred);
  if (threadIdx.x == 0) atomic_max_nonneg(inst_max(t, maxbits, slot), double(mx));
}


// Coefficient tables (computed once per operator with the formulas of
// lpl_coeffs / cyl_coeffs, so the values are those the reference computes).
template <int D>
__global__ void k_setup_coef(KTree t, int n, double lambda2, int cyl, double* cb64, float* cb32, double* cy64,
                             float* cy32) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= n) return;
  double cd[7];
  lpl_coeffs<D>(t, slot, lambda2, cd);
  for (int q = 0; q < 7; q++) {
    cb64[slot * 8 + q] = q <= 2 * D ? cd[q] : 0.0;
    cb32[slot * 8 + q] = q <= 2 * D ? float(cd[q]) : 0.0f;
  }
  cb64[slot * 8 + 7] = 1 / cd[0];
  cb32[slot * 8 + 7] = float(1 / cd[0]);
  if (cyl) {
    for (int i = 1; i <= t.nc; i++) {
      double k1, k2, k3;
      cyl_coeffs(t, slot, i, cd, k1, k2, k3);
      double* o = cy64 + ((size_t)slot * t.nc + (i - 1)) * 4;
      float* o32 = cy32 + ((size_t)slot * t.nc + (i - 1)) * 4;
      o[0] = k1; o[1] = k2; o[2] = k3; o[3] = 1 / k1;
      o32[0] = float(k1); o32[1] = float(k2); o32[2] = float(k3); o32[3] = float(1 / k1);
    }
  }
}

__global__ void k_setup_geo(int n, int nc, const double* __restrict__ r_min, const double* __restrict__ dr,
                            double* __restrict__ geo) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= n * nc) return;
  const int slot = w / nc, i = w % nc + 1;
  const double h = dr[slot * 2], r = r_min[slot * 2] + (i - 0.5) * h;
  const double inv_r = 1 / r;
  const double tw = 0.25 * h / r;
  double* o = geo + (size_t)w * 4;
  o[0] = (r - 0.5 * h) * inv_r;
  o[1] = (r + 0.5 * h) * inv_r;
  o[2] = 1 - tw;
  o[3] = 1 + tw;
}

}  // namespace afg
