// afg_transport32.cuh -- mixed-precision variants of the transport and field
// kernels (transport precision AFG_MIXED).
//
// GB300 issues FP64 at a small fraction of its FP32 rate, so a kernel that
// does more than about one FP64 instruction per 24 bytes it moves is bound
// by the FP64 pipe, not by HBM.  These kernels keep the state in FP64 (the
// densities, |E|, E and the fluxes are read and written as FP64) but do the
// per-cell arithmetic in FP32, except where it cancels:
//   - fluxes: velocities, diffusion, the Koren reconstruction and the flux
//     itself in FP32 (the two-layer ghost values stay FP64, as written back);
//   - chemistry: rates, products, sources and the dt limit in FP32; the new
//     density is n0 + sum_m w_m (n_m - n0) + dt (sources - div flux), with the
//     differences of states and the final sum in FP64 (weights summing to 1);
//   - field: E = -(phi_1 - phi_0)/dx with the potential difference in FP64,
//     the scaling and |E| in FP32;
//   - charge density: FP64 (n_+ - n_- cancels), interior cells only.
// The same routines of the reference are cited at the FP64 kernels.
#pragma once
#include "afg_tma.cuh"
#include "afg_transport.cuh"

namespace afg {

struct LtDevF {
  const float* y;  // [n_cols][n]
  int n;
  float x_min, inv_fac;
};

__device__ __forceinline__ void lt_loc_f(const LtDevF& lt, float x, int& ix, float& w) {
  const float frac = (x - lt.x_min) * lt.inv_fac;
  if (frac <= 0.0f) {
    ix = 1;
    w = 1.0f;
  } else if (frac >= (float)(lt.n - 1)) {
    ix = lt.n - 1;
    w = 0.0f;
  } else {
    ix = (int)ceilf(frac);
    w = (float)ix - frac;
  }
}
__device__ __forceinline__ float lt_col_f(const LtDevF& lt, int col, int ix, float w) {
  const float* y = lt.y + (size_t)col * lt.n;
  return w * y[ix - 1] + (1.0f - w) * y[ix];
}

__device__ __forceinline__ float koren_f(float a, float b) {
  const float aa = a * a, ab = a * b;
  if (ab <= 0.0f) return 0.0f;
  if (aa <= 0.25f * ab) return 2.0f * a;
  if (aa <= 2.5f * ab) return (b + 2.0f * a) * (1.0f / 3.0f);
  return 2.0f * b;
}

struct FluxArgs32 {
  FluxArgs a;       // pointers and FP64 parameters (ghost layers)
  LtDevF lt;
  float N_inv_td;   // SI_to_Townsend / N
  float N_inv;
  float sign[AFG_MAX_FLUX];
  float mu_ion[AFG_MAX_FLUX];  // ion mobility (ion_mobility_N / N)
};

// flux_upwind_box with FP32 arithmetic (see k_flux for the reference lines)
template <int D, bool CYL, int NC = 0>
__global__ void __launch_bounds__(256) k_flux32(KTree t0, const int* __restrict__ rec, FluxArgs32 a32) {
  const KTree t = fix_dims<D, NC>(t0);
  extern __shared__ float smf[];
  __shared__ float sred[32];
  __shared__ int srec[8];  // the box record, read by the ghost-layer loop
  const FluxArgs& a = a32.a;
  if (threadIdx.x < 8) srec[threadIdx.x] = rec[8 * blockIdx.x + threadIdx.x];
  const int slot = rec[8 * blockIdx.x];
  const int nc = t.nc, n2 = t.n2, m = nc + 4, nf1 = nc + 1;
  const int tile = D == 2 ? m * m : m * m * m;
  const int nfaces = D == 2 ? nc * nf1 : nc * nc * nf1;
  float* big = smf;                      // [nf][tile]
  float* vf = smf + a.nf * tile;         // [D][nfaces]
  float* df = vf + D * nfaces;           // [D][nfaces]
  float* Es = df + D * nfaces;           // [S] cell |E| with ghosts
  for (int s = 0; s < a.nf; s++) {
    const double* src = a.n[s] + (size_t)slot * t.S;
    for (int x = threadIdx.x; x < t.S; x += blockDim.x) {
      const int i = x % n2, r = x / n2;
      const int j = D == 2 ? r : r % n2, k = D == 2 ? 0 : r / n2;
      big[s * tile + big_at<D>(m, i, j, k)] = d2f(src[x]);
    }
  }
  {
    const double* E = a.E + (size_t)slot * t.S;
    for (int x = threadIdx.x; x < t.S; x += blockDim.x) Es[x] = d2f(E[x]);
  }
  __syncthreads();
  const int nface = D == 2 ? nc : nc * nc;
  for (int s = 0; s < a.nf; s++) {
    double* dst = a.n[s] + (size_t)slot * t.S;
    for (int w = threadIdx.x; w < 2 * D * nface * 2; w += blockDim.x) {
      const int layer = w & 1, w2 = w >> 1;
      const int nb = w2 / nface, pq = w2 - nb * nface;
      const int p = pq % nc + 1, q = D == 3 ? pq / nc + 1 : 0;
      const int d = nb >> 1;
      const bool low = (nb & 1) == 0;
      const double val = gc2_value<D>(t, a.n[s], slot, nb, srec[1 + nb], layer, p, q, a.bc, a.limiter);
      const int x = low ? -layer : nc + 1 + layer;
      big[s * tile + big_face<D>(m, d, x, p, q)] = d2f(val);
      if (layer == 0) dst[face_at<D>(n2, d, x, p, q)] = val;  // af_gc2_box writes layer 1 back
    }
  }
  __syncthreads();
  float smax = 0.0f;
  #pragma unroll 2
  for (int w = threadIdx.x; w < D * nfaces; w += blockDim.x) {
    const int dim = w / nfaces, fw = w - dim * nfaces;
    const int f = fw % nf1 + 1, ln = fw / nf1;
    const int jj = ln % nc + 1, kk = D == 3 ? ln / nc + 1 : 1;
    const float inv_dx = t.idrf[slot * D + dim];
    int fidx;
    if (D == 2) fidx = dim == 0 ? fc_at(nf1, f, jj, 1) : fc_at(nf1, jj, f, 1);
    else if (dim == 0) fidx = fc_at(nf1, f, jj, kk);
    else if (dim == 1) fidx = fc_at(nf1, jj, f, kk);
    else fidx = fc_at(nf1, jj, kk, f);
    const float Ex = d2f(a.Efc[((size_t)slot * D + dim) * t.NF + fidx]);
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
    const float td = 0.5f * (Es[cidx(f - 1)] + Es[cidx(f)]) * a32.N_inv_td;
    int ix;
    float lw;
    lt_loc_f(a32.lt, td, ix, lw);
    const float mu = lt_col_f(a32.lt, a.col_mu, ix, lw) * a32.N_inv;
    const float dc = lt_col_f(a32.lt, a.col_dc, ix, lw) * a32.N_inv;
    const float v = -mu * Ex;
    float sigma = 0.0f;
    for (int s = 0; s < a.nf; s++) {
      const float* L = big + s * tile;
      const float lm2 = L[bidx(f - 2)], lm1 = L[bidx(f - 1)], l0 = L[bidx(f)], lp1 = L[bidx(f + 1)];
      const bool pos = a32.sign[s] * Ex > 0.0f;
      const float u = pos ? lm1 + 0.5f * koren_f(l0 - lm1, lm1 - lm2) : l0 - 0.5f * koren_f(l0 - lm1, lp1 - l0);
      float fl;
      if (s == 0) {
        fl = v * u - dc * inv_dx * (l0 - lm1);
        sigma = mu * u;
      } else {
        const float vi = a32.sign[s] * a32.mu_ion[s] * Ex;
        fl = vi * u;
        sigma = sigma + a32.mu_ion[s] * u;
      }
      a.flux[s][((size_t)slot * D + dim) * t.NF + fidx] = f2d(fl);
    }
    smax = sigma > smax ? sigma : smax;
    vf[w] = v;
    df[w] = dc;
  }
  __syncthreads();
  float cmax = 0.0f;
  const int ncell = D == 2 ? nc * nc : nc * nc * nc;
  for (int w = threadIdx.x; w < ncell; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 1 : r / nc + 1;
    float cfl = 0.0f;
    for (int dim = 0; dim < D; dim++) {
      const float inv_dx = t.idrf[slot * D + dim];
      int c, ln;
      if (D == 2) { c = dim == 0 ? i : j; ln = dim == 0 ? j - 1 : i - 1; }
      else if (dim == 0) { c = i; ln = (j - 1) + nc * (k - 1); }
      else if (dim == 1) { c = j; ln = (i - 1) + nc * (k - 1); }
      else { c = k; ln = (i - 1) + nc * (j - 1); }
      const int base = dim * nfaces + ln * nf1;
      const float vmax = fmaxf(fabsf(vf[base + c]), fabsf(vf[base + c - 1]));
      const float dmax = fmaxf(df[base + c], df[base + c - 1]);
      cfl = cfl + (vmax * inv_dx + 2.0f * dmax * (inv_dx * inv_dx));
    }
    cmax = cfl > cmax ? cfl : cmax;
  }
  cmax = block_max<float>(cmax, sred);
  if (threadIdx.x == 0) atomic_max_nonneg(a.max_cfl, f2d(cmax));
  __syncthreads();
  smax = block_max<float>(smax, sred);
  if (threadIdx.x == 0) atomic_max_nonneg(a.max_sigma, f2d(smax));
}

// k_flux32 for a compile-time box size with the box's data staged in shared
// memory: thread 0 bulk-copies |E| and the flux species of the box (whole
// boxes, ghost cells included, contiguous) while every thread evaluates its
// share of the two-layer ghost values (gc2_value on global memory) and loads
// E on its faces, so those loads overlap the copies.  After the wait the
// staged values are converted into the padded FP32 tile (face-ghost cells
// left to the ghost values), the first ghost layer is written back, and the
// faces and cells are done as in k_flux32, with the same arithmetic, so the
// results are bit-identical.  At most NFMAX flux species (NFMAX = 1: exactly one).  The FP32 face
// values and diffusion coefficients reuse the staging buffer.  A wait that
// times out (1 s) raises *err; the CTA drains its copies (bounded) and
// returns, raising bit 2 of *err if they did not complete.
template <int D, bool CYL, int NC, int NFMAX>
__global__ void __launch_bounds__(256, 5) k_flux32s(KTree t0, const int* __restrict__ rec, FluxArgs32 a32,
                                                unsigned* err) {
  constexpr int nc = NC, n2 = NC + 2, m = NC + 4, nf1 = NC + 1;
  constexpr int S = D == 2 ? n2 * n2 : n2 * n2 * n2;
  constexpr int tile = D == 2 ? m * m : m * m * m;
  constexpr int nfaces = D == 2 ? nc * nf1 : nc * nc * nf1;  // per dimension
  constexpr int NFT = (D * nfaces + 255) / 256;               // faces per thread
  constexpr int nface = D == 2 ? nc : nc * nc;                // cells on one box face
  constexpr int NG = 2 * D * nface * 2;                       // two-layer ghosts per species
  constexpr int NGT = (NG + 255) / 256;
  constexpr unsigned SB = S * sizeof(double);
  static_assert(SB % 16 == 0, "bulk copies need 16-byte multiples");
  const KTree t = fix_dims<D, NC>(t0);
  extern __shared__ __align__(16) unsigned char smb[];
  __shared__ float sred[32];
  __shared__ __align__(8) unsigned long long bar;
  const FluxArgs& a = a32.a;
  const int nf = NFMAX == 1 ? 1 : a.nf;
  double* rawE = reinterpret_cast<double*>(smb);  // staged |E|, then the species
  double* rawN = rawE + S;
  float* vf = reinterpret_cast<float*>(smb);      // [D][nfaces], after the conversion
  float* df = vf + D * nfaces;
  const size_t offA = ((size_t)max((int)(SB * (nf + 1)), (int)(8 * D * nfaces)) + 15) & ~(size_t)15;
  float* big = reinterpret_cast<float*>(smb + offA);  // [nf][tile]
  float* Es = big + nf * tile;                         // [S]
  const int4 r0 = reinterpret_cast<const int4*>(rec)[2 * blockIdx.x];
  const int4 r1 = reinterpret_cast<const int4*>(rec)[2 * blockIdx.x + 1];
  const int slot = r0.x;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(&bar, SB * (unsigned)(nf + 1));
    bulk_copy_g2s(rawE, a.E + (size_t)slot * S, SB, &bar);
    for (int q = 0; q < nf; q++) bulk_copy_g2s(rawN + q * S, a.n[q] + (size_t)slot * S, SB, &bar);
  }
  // this thread's ghost values (both layers) and face fields
  double gval[NFMAX][NGT];
#pragma unroll
  for (int q = 0; q < NFMAX; q++)
#pragma unroll
    for (int u = 0; u < NGT; u++) {
      const int w = (int)threadIdx.x + u * 256;
      gval[q][u] = 0.0;
      if (q < nf && w < NG) {
        const int layer = w & 1, w2 = w >> 1;
        const int nb = w2 / nface, pq = w2 - nb * nface;
        const int p = pq % nc + 1, qq = D == 3 ? pq / nc + 1 : 0;
        gval[q][u] = gc2_value<D>(t, a.n[q], slot, nb, rec_nb(r0, r1, nb), layer, p, qq, a.bc, a.limiter);
      }
    }
  float ex[NFT];
#pragma unroll
  for (int u = 0; u < NFT; u++) {
    const int w = (int)threadIdx.x + u * 256;
    ex[u] = 0.0f;
    if (w < D * nfaces) {
      const int dim = w / nfaces, fw = w - dim * nfaces;
      const int f = fw % nf1 + 1, ln = fw / nf1;
      const int jj = ln % nc + 1, kk = D == 3 ? ln / nc + 1 : 1;
      int fidx;
      if (D == 2) fidx = dim == 0 ? fc_at(nf1, f, jj, 1) : fc_at(nf1, jj, f, 1);
      else if (dim == 0) fidx = fc_at(nf1, f, jj, kk);
      else if (dim == 1) fidx = fc_at(nf1, jj, f, kk);
      else fidx = fc_at(nf1, jj, kk, f);
      ex[u] = d2f(a.Efc[((size_t)slot * D + dim) * t.NF + fidx]);
    }
  }
  const bool ok = mbar_wait(&bar, 0);
  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0) atomicOr(err, mbar_wait(&bar, 0) ? 1u : 3u);
    return;
  }
  // staged values into the tile; the face-ghost cells (one index outside)
  // come from the ghost values
  for (int q = 0; q < nf; q++)
    for (int x = threadIdx.x; x < S; x += 256) {
      const int i = x % n2, r = x / n2;
      const int j = D == 2 ? r : r % n2, k = D == 2 ? 0 : r / n2;
      const int out = (i == 0 || i == n2 - 1) + (j == 0 || j == n2 - 1) + (D == 3 && (k == 0 || k == n2 - 1));
      if (out != 1) big[q * tile + big_at<D>(m, i, j, k)] = d2f(rawN[q * S + x]);
    }
  for (int x = threadIdx.x; x < S; x += 256) Es[x] = d2f(rawE[x]);
#pragma unroll
  for (int q = 0; q < NFMAX; q++)
#pragma unroll
    for (int u = 0; u < NGT; u++) {
      const int w = (int)threadIdx.x + u * 256;
      if (q < nf && w < NG) {
        const int layer = w & 1, w2 = w >> 1;
        const int nb = w2 / nface, pq = w2 - nb * nface;
        const int p = pq % nc + 1, qq = D == 3 ? pq / nc + 1 : 0;
        const int d = nb >> 1;
        const bool low = (nb & 1) == 0;
        const int x = low ? -layer : nc + 1 + layer;
        big[q * tile + big_face<D>(m, d, x, p, qq)] = d2f(gval[q][u]);
        if (layer == 0) a.n[q][(size_t)slot * S + face_at<D>(n2, d, x, p, qq)] = gval[q][u];
      }
    }
  __syncthreads();
  float smax = 0.0f;
#pragma unroll
  for (int u = 0; u < NFT; u++) {
    const int w = (int)threadIdx.x + u * 256;
    if (w < D * nfaces) {
    const int dim = w / nfaces, fw = w - dim * nfaces;
    const int f = fw % nf1 + 1, ln = fw / nf1;
    const int jj = ln % nc + 1, kk = D == 3 ? ln / nc + 1 : 1;
    const float inv_dx = t.idrf[slot * D + dim];
    int fidx;
    if (D == 2) fidx = dim == 0 ? fc_at(nf1, f, jj, 1) : fc_at(nf1, jj, f, 1);
    else if (dim == 0) fidx = fc_at(nf1, f, jj, kk);
    else if (dim == 1) fidx = fc_at(nf1, jj, f, kk);
    else fidx = fc_at(nf1, jj, kk, f);
    const float Ex = ex[u];
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
    const float td = 0.5f * (Es[cidx(f - 1)] + Es[cidx(f)]) * a32.N_inv_td;
    int ix;
    float lw;
    lt_loc_f(a32.lt, td, ix, lw);
    const float mu = lt_col_f(a32.lt, a.col_mu, ix, lw) * a32.N_inv;
    const float dc = lt_col_f(a32.lt, a.col_dc, ix, lw) * a32.N_inv;
    const float v = -mu * Ex;
    float sigma = 0.0f;
    for (int q = 0; q < nf; q++) {
      const float* L = big + q * tile;
      const float lm2 = L[bidx(f - 2)], lm1 = L[bidx(f - 1)], l0 = L[bidx(f)], lp1 = L[bidx(f + 1)];
      const bool pos = a32.sign[q] * Ex > 0.0f;
      const float uu = pos ? lm1 + 0.5f * koren_f(l0 - lm1, lm1 - lm2) : l0 - 0.5f * koren_f(l0 - lm1, lp1 - l0);
      float fl;
      if (q == 0) {
        fl = v * uu - dc * inv_dx * (l0 - lm1);
        sigma = mu * uu;
      } else {
        const float vi = a32.sign[q] * a32.mu_ion[q] * Ex;
        fl = vi * uu;
        sigma = sigma + a32.mu_ion[q] * uu;
      }
      a.flux[q][((size_t)slot * D + dim) * t.NF + fidx] = f2d(fl);
    }
    smax = sigma > smax ? sigma : smax;
    vf[w] = v;
    df[w] = dc;
    }
  }
  __syncthreads();
  float cmax = 0.0f;
  constexpr int ncell = D == 2 ? nc * nc : nc * nc * nc;
  for (int w = threadIdx.x; w < ncell; w += 256) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 1 : r / nc + 1;
    float cfl = 0.0f;
    for (int dim = 0; dim < D; dim++) {
      const float inv_dx = t.idrf[slot * D + dim];
      int c, ln;
      if (D == 2) { c = dim == 0 ? i : j; ln = dim == 0 ? j - 1 : i - 1; }
      else if (dim == 0) { c = i; ln = (j - 1) + nc * (k - 1); }
      else if (dim == 1) { c = j; ln = (i - 1) + nc * (k - 1); }
      else { c = k; ln = (i - 1) + nc * (j - 1); }
      const int base = dim * nfaces + ln * nf1;
      const float vmax = fmaxf(fabsf(vf[base + c]), fabsf(vf[base + c - 1]));
      const float dmax = fmaxf(df[base + c], df[base + c - 1]);
      cfl = cfl + (vmax * inv_dx + 2.0f * dmax * (inv_dx * inv_dx));
    }
    cmax = cfl > cmax ? cfl : cmax;
  }
  cmax = block_max<float>(cmax, sred);
  if (threadIdx.x == 0) atomic_max_nonneg(a.max_cfl, f2d(cmax));
  __syncthreads();
  smax = block_max<float>(smax, sred);
  if (threadIdx.x == 0) atomic_max_nonneg(a.max_sigma, f2d(smax));
}

// Reaction in FP32 form: rate = fa * fb * form(Td) (the factors split so that
// a large rate_factor, e.g. N^2 of a three-body reaction, stays in range).
// The update kernel reads the records from shared memory: in_off are the
// input species' offsets in the per-thread columns (species * 128) and the
// n_upd (species offset, coefficient) pairs are the reaction's net effect on
// each species it touches (outputs' multiplicities less the inputs' counts).
struct alignas(16) Reac32 {
  int rate_type, lt_col, n_in, n_upd;
  float fa, fb, c1, c2;
  float c3, pad0, pad1, pad2;
  int in_off[4];
  int upd_off[8];
  float upd_coef[8];
};
static_assert(sizeof(Reac32) == 128, "Reac32 is 32 words");

__device__ __forceinline__ float rate32(const LtDevF& lt, const Reac32& r, float td, int ix, float w) {
  switch (r.rate_type) {
    case AFG_RATE_TABULATED_FIELD: return r.fb * (r.fa * lt_col_f(lt, r.lt_col, ix, w));
    case AFG_RATE_CONSTANT: return r.fa * r.fb;
    case AFG_RATE_LINEAR: return r.fa * r.fb * (td - r.c1);
    case AFG_RATE_EXP_V1: { const float q = r.c1 / (r.c2 + td); return r.fa * r.fb * expf(-(q * q)); }
    case AFG_RATE_EXP_V2: { const float q = td / r.c1; return r.fa * r.fb * expf(-(q * q)); }
    case AFG_RATE_K13: return r.fa * r.fb * expf(-pow_c(r.c1 / (r.c2 + td), r.c3));
    case AFG_RATE_K14: return r.fa * r.fb * expf(-pow_c(td / r.c1, r.c2));
    case AFG_RATE_K1: {
      const float Te = (float)(2 * 1.602176634e-19 / (3 * 1.380649e-23)) * lt_col_f(lt, r.lt_col, ix, w);
      return r.fa * r.fb * pow_c(300.0f / Te, r.c1);
    }
  }
  return 0.0f;
}

struct UpdateArgs32 {
  UpdateArgs a;
  LtDevF lt;
  const Reac32* reactions;
  float N_inv_td;
  float dt;
  float w_rel[4];   // weights of the differences n_m - n_0 (m >= 1)
  float nmin;
  int prev_is_deriv;  // m with s_prev[m] == s_deriv (its values are reused), or -1
};

template <int NSMAX>
__device__ __forceinline__ void add_tof(float (&v)[NSMAX], int s, float x) {
#pragma unroll
  for (int k = 0; k < NSMAX; k++)
    if (k == s) v[k] = v[k] + x;
}

// flux_update_densities + add_source_terms with FP32 sources; the weights of
// the previous states sum to one (forward Euler and Heun stages).  The
// reaction records sit in dynamic shared memory (n_reactions of them); each
// thread keeps its cell's densities and sources in its own shared-memory
// column, since the records index species at run time.  The fluxes and the
// first previous state are loaded before the chemistry, so that their
// latency overlaps it.
template <int D, bool CYL, int NSMAX, int NC = 0>
__global__ void __launch_bounds__(128, NSMAX <= 6 ? 9 : 8) k_update32(KTree t0, const int* __restrict__ list, UpdateArgs32 u) {
  const KTree t = fix_dims<D, NC>(t0);
  __shared__ float sred[32];
  __shared__ float s_dens[NSMAX * 128], s_der[NSMAX * 128];
  __shared__ double s_raw[NSMAX * 128];  // the derivative state as read
  extern __shared__ __align__(16) int s_rwords[];
  const Reac32* rec = reinterpret_cast<const Reac32*>(s_rwords);
  const UpdateArgs& a = u.a;
  const int nr = a.n_reactions;
  {
    const int4* src = reinterpret_cast<const int4*>(u.reactions);
    int4* dst = reinterpret_cast<int4*>(s_rwords);
    for (int x = threadIdx.x; x < nr * 8; x += blockDim.x) dst[x] = src[x];
  }
  __syncthreads();
  const int slot = list[blockIdx.x];
  const int nc = t.nc, n2 = t.n2, nf1 = nc + 1;
  const int ncell = D == 2 ? nc * nc : nc * nc * nc;
  const int tid = threadIdx.x;
  float dt_dr[3];
  for (int q = 0; q < D; q++) dt_dr[q] = u.dt * t.idrf[slot * D + q];
  float my_chem = 3.0e38f;
  const size_t base = (size_t)slot * t.S;
  const bool n0_raw = u.prev_is_deriv == 0;
  // registers for the early load of the first previous state (up to 8 species)
  constexpr bool kPre = NSMAX <= 8;
  for (int w = threadIdx.x; w < ncell; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 0 : r / nc + 1;
    const int x = D == 2 ? at2(n2, i, j) : at3(n2, i, j, k);
    const int kk = D == 3 ? k : 1;
    float* dens = s_dens + tid;  // species s at dens[s * 128]
    float* der = s_der + tid;
    // every global load of the cell first
    double raw[NSMAX], n0v[NSMAX];
#pragma unroll
    for (int s = 0; s < NSMAX; s++) {
      raw[s] = s < a.ns ? a.deriv[s][base + x] : 0.0;
      n0v[s] = (kPre && s < a.ns && !n0_raw) ? a.prev[0][s][base + x] : 0.0;
    }
    const double Ec = a.E[base + x];
    const double phc = a.photo != nullptr ? a.photo[base + x] : 0.0;
    double fx[2 * D];
    {
      const double* F = a.flux[0] + (size_t)slot * D * t.NF;
      if (D == 2) {
        fx[0] = F[fc_at(nf1, i, j, 1)];
        fx[1] = F[fc_at(nf1, i + 1, j, 1)];
        fx[2] = F[t.NF + fc_at(nf1, i, j, 1)];
        fx[3] = F[t.NF + fc_at(nf1, i, j + 1, 1)];
      } else {
        fx[0] = F[fc_at(nf1, i, j, kk)];
        fx[1] = F[fc_at(nf1, i + 1, j, kk)];
        fx[2] = F[t.NF + fc_at(nf1, i, j, kk)];
        fx[3] = F[t.NF + fc_at(nf1, i, j + 1, kk)];
        fx[4] = F[2 * t.NF + fc_at(nf1, i, j, kk)];
        fx[5] = F[2 * t.NF + fc_at(nf1, i, j, kk + 1)];
      }
    }
#pragma unroll
    for (int s = 0; s < NSMAX; s++) {
      if (s < a.ns) {
        s_raw[s * 128 + tid] = raw[s];
        dens[s * 128] = fmaxf(d2f(raw[s]), 0.0f);
        der[s * 128] = 0.0f;
      }
    }
    const float td = u.N_inv_td * d2f(Ec);
    int ix;
    float lw;
    lt_loc_f(u.lt, td, ix, lw);
    for (int n = 0; n < nr; n++) {
      const Reac32& rc = rec[n];
      float rate = rate32(u.lt, rc, td, ix, lw);
      for (int q = 0; q < rc.n_in; q++) rate = rate * dens[rc.in_off[q]];
      for (int q = 0; q < rc.n_upd; q++) der[rc.upd_off[q]] = fmaf(rc.upd_coef[q], rate, der[rc.upd_off[q]]);
    }
    if (a.last_step) {
      const float eps = 1e-30f;
      float tmp = 3.0e38f;
#pragma unroll
      for (int s = 0; s < NSMAX; s++) {
        if (s >= a.ns) continue;
        const float dn = dens[s * 128], dd = der[s * 128];
        if (u.nmin > 0.0f)
          tmp = fminf(tmp, (dn + u.nmin) / fmaxf(fabsf(dd), eps));
        else if (a.limit_loss)
          tmp = fminf(tmp, fmaxf(dn, eps) / fmaxf(-dd, eps));
      }
      my_chem = fminf(my_chem, tmp);
    }
    if (a.photo != nullptr) {
      const float ph = d2f(phc);
      der[a.flux_species[0] * 128] += ph;
      der[a.photoi_species * 128] += ph;
    }
    float inc[NSMAX];
#pragma unroll
    for (int s = 0; s < NSMAX; s++) inc[s] = s < a.ns ? u.dt * der[s * 128] : 0.0f;
    for (int f = 0; f < a.nf; f++) {
      double g[2 * D];
      if (f == 0) {
#pragma unroll
        for (int q = 0; q < 2 * D; q++) g[q] = fx[q];
      } else {
        const double* F = a.flux[f] + (size_t)slot * D * t.NF;
        g[0] = F[fc_at(nf1, i, j, kk)];
        g[1] = F[fc_at(nf1, i + 1, j, kk)];
        g[2] = F[t.NF + fc_at(nf1, i, j, kk)];
        g[3] = F[t.NF + fc_at(nf1, i, j + 1, kk)];
        if (D == 3) {
          g[4] = F[2 * t.NF + fc_at(nf1, i, j, kk)];
          g[5] = F[2 * t.NF + fc_at(nf1, i, j, kk + 1)];
        }
      }
      float div;
      if (D == 2 && CYL) {
        const double* gw = t.geo + ((size_t)slot * nc + (i - 1)) * 4;
        const float f1 = d2f(gw[0]), f2 = d2f(gw[1]);
        div = dt_dr[0] * (f1 * d2f(g[0]) - f2 * d2f(g[1])) + dt_dr[1] * (d2f(g[2]) - d2f(g[3]));
      } else if (D == 2) {
        div = dt_dr[0] * (d2f(g[0]) - d2f(g[1])) + dt_dr[1] * (d2f(g[2]) - d2f(g[3]));
      } else {
        div = dt_dr[0] * (d2f(g[0]) - d2f(g[1])) + dt_dr[1] * (d2f(g[2]) - d2f(g[3])) +
              dt_dr[2] * (d2f(g[4]) - d2f(g[5]));
      }
      add_tof<NSMAX>(inc, a.flux_species[f], div);
    }
#pragma unroll
    for (int s = 0; s < NSMAX; s++) {
      if (s >= a.ns) continue;
      const double n0 = n0_raw ? s_raw[s * 128 + tid] : kPre ? n0v[s] : a.prev[0][s][base + x];
      float d = inc[s];
      for (int mm = 1; mm < a.n_prev; mm++) {
        const double nm = u.prev_is_deriv == mm ? s_raw[s * 128 + tid] : a.prev[mm][s][base + x];
        d = d + u.w_rel[mm] * d2f(nm - n0);
      }
      a.out[s][base + x] = n0 + f2d(d);
    }
  }
  if (a.last_step) {
    for (int o = 16; o > 0; o >>= 1) my_chem = fminf(my_chem, __shfl_xor_sync(0xffffffffu, my_chem, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sred[warp] = my_chem;
    __syncthreads();
    if (threadIdx.x == 0) {
      float v = sred[0];
      for (int q = 1; q < (int)((blockDim.x + 31) >> 5); q++) v = fminf(v, sred[q]);
      atomicMin(a.min_chem, (unsigned long long)__double_as_longlong(f2d(v)));
    }
  }
}

// E on faces and |E| in cells with FP32 scaling (see k_field_grad)
template <int D, int NC = 0>
__global__ void __launch_bounds__(256) k_field_grad32(KTree t0, const int* __restrict__ list,
                                                      const double* __restrict__ phi, double* __restrict__ efc,
                                                      double* __restrict__ enorm) {
  const KTree t = fix_dims<D, NC>(t0);
  extern __shared__ float sef[];  // [D][NF], the fc layout of one box
  const int slot = list[blockIdx.x];
  const int nc = t.nc, n2 = t.n2, nf1 = nc + 1;
  const double* p = phi + (size_t)slot * t.S;
  const int nfaces = D == 2 ? nc * nf1 : nc * nc * nf1;
  #pragma unroll 4
  for (int w = threadIdx.x; w < D * nfaces; w += blockDim.x) {
    const int dim = w / nfaces, fw = w - dim * nfaces;
    const int f = fw % nf1 + 1, ln = fw / nf1;
    const int jj = ln % nc + 1, kk = D == 3 ? ln / nc + 1 : 1;
    const float inv_dr = -t.idrf[slot * D + dim];
    int fidx, c1, c0;
    if (D == 2) {
      if (dim == 0) { fidx = fc_at(nf1, f, jj, 1); c1 = at2(n2, f, jj); c0 = at2(n2, f - 1, jj); }
      else { fidx = fc_at(nf1, jj, f, 1); c1 = at2(n2, jj, f); c0 = at2(n2, jj, f - 1); }
    } else if (dim == 0) { fidx = fc_at(nf1, f, jj, kk); c1 = at3(n2, f, jj, kk); c0 = at3(n2, f - 1, jj, kk); }
    else if (dim == 1) { fidx = fc_at(nf1, jj, f, kk); c1 = at3(n2, jj, f, kk); c0 = at3(n2, jj, f - 1, kk); }
    else { fidx = fc_at(nf1, jj, kk, f); c1 = at3(n2, jj, kk, f); c0 = at3(n2, jj, kk, f - 1); }
    const float e = inv_dr * d2f(p[c1] - p[c0]);
    sef[dim * t.NF + fidx] = e;
    efc[((size_t)slot * D + dim) * t.NF + fidx] = f2d(e);
  }
  __syncthreads();
  const int ncell = D == 2 ? nc * nc : nc * nc * nc;
  #pragma unroll 2
  for (int w = threadIdx.x; w < ncell; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 1 : r / nc + 1;
    const float a = sef[fc_at(nf1, i, j, k)] + sef[fc_at(nf1, i + 1, j, k)];
    const float b = sef[t.NF + fc_at(nf1, i, j, k)] + sef[t.NF + fc_at(nf1, i, j + 1, k)];
    float s = a * a + b * b;
    if (D == 3) {
      const float c = sef[2 * t.NF + fc_at(nf1, i, j, k)] + sef[2 * t.NF + fc_at(nf1, i, j, k + 1)];
      s = s + c * c;
    }
    enorm[(size_t)slot * t.S + (D == 2 ? at2(n2, i, j) : at3(n2, i, j, k))] = f2d(0.5f * sqrtf(s));
  }
}

// Charge density on interior cells (FP64: n_+ - n_- cancels).  `a` holds
// the charged species only (a.ns of them, at most NQ), so that the unrolled
// species loop indexes the parameter arrays statically and every density
// load of a cell is issued before the sums.
template <int D, int NQ, int NC = 0>
__global__ void __launch_bounds__(256) k_field_rhs_interior(KTree t0, const int* __restrict__ list, RhsArgs a,
                                                            unsigned long long* maxbits) {
  const KTree t = fix_dims<D, NC>(t0);
  __shared__ double sred[32];
  const int slot = list[blockIdx.x];
  const int nc = t.nc, n2 = t.n2;
  const int ncell = D == 2 ? nc * nc : nc * nc * nc;
  const size_t base = (size_t)slot * t.S;
  double mx = 0.0;
  // CPT cells per thread, every density load of them issued first
  constexpr int CPT = 4;
  for (int w0 = threadIdx.x; w0 < ncell; w0 += CPT * blockDim.x) {
    double nv[CPT][NQ];
    size_t xs[CPT];
#pragma unroll
    for (int u = 0; u < CPT; u++) {
      const int w = w0 + u * blockDim.x;
      const int i = w % nc + 1, r = w / nc;
      const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 0 : r / nc + 1;
      xs[u] = base + (D == 2 ? at2(n2, i, j) : at3(n2, i, j, k));
#pragma unroll
      for (int s = 0; s < NQ; s++) nv[u][s] = (s < a.ns && w < ncell) ? a.n[s][xs[u]] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < CPT; u++) {
      if (w0 + u * (int)blockDim.x >= ncell) continue;
      double v = 0.0;
#pragma unroll
      for (int s = 0; s < NQ; s++)
        if (s < a.ns) v = fma(a.q[s], nv[u][s], v);
      a.rhs[xs[u]] = v;
      acc_absmax(mx, v);
    }
  }
  // max |rhs| over the leaves (af_tree_maxabs_cc), fused
  if (maxbits != nullptr) {
    mx = block_max<double>(mx, sred);
    if (threadIdx.x == 0) atomic_max_nonneg(inst_max(t, maxbits, slot), mx);
  }
}

// Photon production (see k_photo_source) with FP32 lookup and products
template <int D, int NC = 0>
__global__ void __launch_bounds__(256) k_photo_source32(KTree t0, const int* __restrict__ list,
                                                        const double* __restrict__ E, const double* __restrict__ ne,
                                                        double* __restrict__ rhs, LtDevF lt, int col_alpha,
                                                        int col_mu, float N_inv_td, float coeff_hi, float coeff_lo) {
  const KTree t = fix_dims<D, NC>(t0);
  const int slot = list[blockIdx.x];
  const int nc = t.nc, n2 = t.n2;
  const int ncell = D == 2 ? nc * nc : nc * nc * nc;
  const size_t base = (size_t)slot * t.S;
  for (int w = threadIdx.x; w < ncell; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 0 : r / nc + 1;
    const int x = D == 2 ? at2(n2, i, j) : at3(n2, i, j, k);
    const float fld = d2f(E[base + x]);
    const float td = fld * N_inv_td;
    int ix;
    float w_;
    lt_loc_f(lt, td, ix, w_);
    const float alpha = lt_col_f(lt, col_alpha, ix, w_);
    const float mob = lt_col_f(lt, col_mu, ix, w_);
    float tmp = ((fld * coeff_hi) * mob) * ((alpha * coeff_lo) * d2f(ne[base + x]));
    if (tmp < 0.0f) tmp = 0.0f;
    rhs[base + x] = f2d(tmp);
  }
}

}  // namespace afg
