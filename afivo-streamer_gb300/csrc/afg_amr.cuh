// afg_amr.cuh -- adaptive refinement on the device: the refinement flags of
// default_refinement (src/m_refine.f90:197-298) reduced to box flags as in
// consistent_ref_flags / cell_to_ref_flags (afivo/src/m_af_core.f90:929-991,
// 1095-1149), the limited prolongation af_prolong_limit
// (afivo/src/m_af_prolong.f90:311-420) into new boxes, and the move of all
// variables to a new tree.  Included by afg_runtime.cu after the transport
// API (lookup table, limiters).
#pragma once

namespace afg {

// Box-flag pass: one CTA per box of the list (leaves and parents of
// leaves).  Every cell gets af_do_ref / af_keep_ref / af_rm_ref from the
// alpha*dx criterion, the seed lines, the fixed regions and limits and the
// dx bounds, in the reference's order; the box's flag (do if any cell is do,
// else keep if any is keep, else rm) and af_do_ref for each neighbour next
// to which a flagged cell lies within ref_buffer cells are folded into
// flags[] with atomicMax (the reference takes the maximum over its
// threads' copies).
template <int D>
__global__ void __launch_bounds__(128) k_refine_flags(KTree t, const int* __restrict__ list,
                                                      const double* __restrict__ E, const double* __restrict__ ne,
                                                      LtDev lt, afg_refine_desc a, int* __restrict__ flags,
                                                      const int* __restrict__ lsf_idx) {
  const int slot = list[blockIdx.x];
  const int nc = t.nc, n2 = t.n2;
  __shared__ int s_do, s_keep;
  __shared__ unsigned s_nb;  // bit of neighbor_mat entry (dx+1) + 3 (dy+1) [+ 9 (dz+1)]: a do cell lies in that slab
  if (threadIdx.x == 0) {
    s_do = 0;
    s_keep = 0;
    s_nb = 0u;
  }
  __syncthreads();
  double drv[3], rmin[3], rmax[3];
  double max_dx = t.dr[slot * D], min_dx = t.dr[slot * D];
  for (int d = 0; d < D; d++) {
    drv[d] = t.dr[slot * D + d];
    rmin[d] = t.r_min[slot * D + d];
    rmax[d] = rmin[d] + drv[d] * nc;
    max_dx = fmax(max_dx, drv[d]);
    min_dx = fmin(min_dx, drv[d]);
  }
  // box-level conditions of the fixed regions and limits
  bool in_region = false, in_limit = false;
  for (int n = 0; n < a.n_regions; n++) {
    bool all = max_dx > a.region_dr[n];
    for (int d = 0; d < D; d++) all = all && rmax[d] >= a.region_rmin[n][d] && rmin[d] <= a.region_rmax[n][d];
    in_region = in_region || all;
  }
  for (int n = 0; n < a.n_limits; n++) {
    bool all = max_dx < 2 * a.limit_dr[n];
    for (int d = 0; d < D; d++) all = all && rmin[d] >= a.limit_rmin[n][d] && rmax[d] <= a.limit_rmax[n][d];
    in_limit = in_limit || all;
  }
  const int ncell = D == 2 ? nc * nc : nc * nc * nc;
  bool any_do = false, any_keep = false;
  unsigned nbm = 0u;
  const int hc = nc / 2;
  for (int w = threadIdx.x; w < ncell; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 0 : r / nc + 1;
    const int x = D == 2 ? at2(n2, i, j) : at3(n2, i, j, k);
    const size_t c = (size_t)slot * t.S + x;
    const double fld = E[c] * kSiToTd / a.gas_number_density;
    int ix;
    double wt;
    lt_loc(lt, a.adx_fac * fld, ix, wt);
    double alpha;
    if (a.use_alpha_effective) {
      alpha = (lt_col(lt, a.lt_col_alpha, ix, wt) - lt_col(lt, a.lt_col_eta, ix, wt)) * a.gas_number_density /
              a.adx_fac;
      alpha = fmax(0.0, alpha);
    } else {
      alpha = lt_col(lt, a.lt_col_alpha, ix, wt) * a.gas_number_density / a.adx_fac;
    }
    const double adx = max_dx * alpha;
    int f;
    if (adx > a.adx && ne[c] > a.min_dens)
      f = AFG_REF_DO;
    else if (adx < 0.125 * a.adx && max_dx < a.derefine_dx)
      f = AFG_REF_RM;
    else
      f = AFG_REF_KEEP;
    // refine around the seed lines (GM_dist_line, src/m_geometry.f90:23-51)
    const int cix[3] = {i, j, k};
    double rc[3];
    for (int d = 0; d < D; d++) rc[d] = rmin[d] + (cix[d] - 0.5) * drv[d];
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
      const double dist = sqrt(s2);
      if (dist - a.seed_width[n] < 2 * max_dx && max_dx > a.init_fac * a.seed_width[n]) f = AFG_REF_DO;
    }
    // refine around the electrode: boxes the electrode surface crosses
    if (lsf_idx != nullptr && lsf_idx[slot] >= 0 && a.electrode_dx > 0 && max_dx > a.electrode_dx) f = AFG_REF_DO;
    // fixed regions mark the centre cell, limits turn do into keep
    const bool centre = i == hc && j == hc && (D == 2 || k == hc);
    if (centre && in_region) f = AFG_REF_DO;
    if (in_limit && f == AFG_REF_DO) f = AFG_REF_KEEP;
    if (max_dx > a.max_dx)
      f = AFG_REF_DO;
    else if (min_dx < 2 * a.min_dx && f == AFG_REF_DO)
      f = AFG_REF_KEEP;
    any_do = any_do || f == AFG_REF_DO;
    any_keep = any_keep || f == AFG_REF_KEEP;
    if (f == AFG_REF_DO && a.ref_buffer > 0) {
      // buffer slabs this cell lies in, per direction and dimension
      const int lo = a.ref_buffer, hi = nc - a.ref_buffer + 1;
      for (int dz = (D == 3 ? -1 : 0); dz <= (D == 3 ? 1 : 0); dz++)
        for (int dy = -1; dy <= 1; dy++)
          for (int dx = -1; dx <= 1; dx++) {
            if (dx == 0 && dy == 0 && dz == 0) continue;
            const int dir[3] = {dx, dy, dz};
            bool in = true;
            for (int d = 0; d < D; d++)
              in = in && (dir[d] == 0 || (dir[d] == 1 ? cix[d] >= hi : cix[d] <= lo));
            if (in) nbm |= 1u << ((dx + 1) + 3 * (dy + 1) + (D == 3 ? 9 * (dz + 1) : 0));
          }
    }
  }
  if (any_do) atomicOr(&s_do, 1);
  if (any_keep) atomicOr(&s_keep, 1);
  if (nbm) atomicOr(&s_nb, nbm);
  __syncthreads();
  if (threadIdx.x == 0) {
    const int own = s_do ? AFG_REF_DO : (s_keep ? AFG_REF_KEEP : AFG_REF_RM);
    atomicMax(&flags[slot], own);
    const int nm = D == 2 ? 9 : 27;
    for (int b = 0; b < nm; b++) {
      if (!((s_nb >> b) & 1u)) continue;
      const int nbs = t.nbmat[slot * nm + b];
      if (nbs >= 0) atomicMax(&flags[nbs], AFG_REF_DO);
    }
  }
}

// af_prolong_limit: one CTA per child box, one thread per parent cell of
// the child's quadrant/octant; the 2^D fine cells get f0 +- the limited
// quarter slopes, added to zero as in the reference (add = .false.).
template <int D>
__global__ void __launch_bounds__(128) k_prolong_limit(KTree t, const int* __restrict__ list, double* __restrict__ v,
                                                       int limiter) {
  const int slot = list[blockIdx.x];
  const int pslot = t.parent[slot];
  const int nc = t.nc, n2 = t.n2, hnc = nc / 2;
  const double* P = v + (size_t)pslot * t.S;
  double* Cc = v + (size_t)slot * t.S;
  const int o0 = child_offset(t, slot, 0), o1 = child_offset(t, slot, 1);
  const int o2 = D == 3 ? child_offset(t, slot, 2) : 0;
  const int count = D == 2 ? hnc * hnc : hnc * hnc * hnc;
  const int sy = n2, sz = n2 * n2;
  for (int w = threadIdx.x; w < count; w += blockDim.x) {
    const int i = w % hnc + 1, r = w / hnc;
    const int j = D == 2 ? r + 1 : r % hnc + 1, k = D == 2 ? 0 : r / hnc + 1;
    const int ic = i + o0, jc = j + o1, kc = k + o2;
    const int fi = 2 * i - 1, fj = 2 * j - 1, fk = 2 * k - 1;
    if (D == 2) {
      const int p = at2(n2, ic, jc);
      const double f0 = P[p];
      const double f1 = 0.25 * limiter_apply(P[p] - P[p - 1], P[p + 1] - P[p], limiter);
      const double f2 = 0.25 * limiter_apply(P[p] - P[p - sy], P[p + sy] - P[p], limiter);
      Cc[at2(n2, fi, fj)] = f0 - f1 - f2 + 0.0;
      Cc[at2(n2, fi + 1, fj)] = f0 + f1 - f2 + 0.0;
      Cc[at2(n2, fi, fj + 1)] = f0 - f1 + f2 + 0.0;
      Cc[at2(n2, fi + 1, fj + 1)] = f0 + f1 + f2 + 0.0;
    } else {
      const int p = at3(n2, ic, jc, kc);
      const double f0 = P[p];
      const double f1 = 0.25 * limiter_apply(P[p] - P[p - 1], P[p + 1] - P[p], limiter);
      const double f2 = 0.25 * limiter_apply(P[p] - P[p - sy], P[p + sy] - P[p], limiter);
      const double f3 = 0.25 * limiter_apply(P[p] - P[p - sz], P[p + sz] - P[p], limiter);
      Cc[at3(n2, fi, fj, fk)] = f0 - f1 - f2 - f3 + 0.0;
      Cc[at3(n2, fi + 1, fj, fk)] = f0 + f1 - f2 - f3 + 0.0;
      Cc[at3(n2, fi, fj + 1, fk)] = f0 - f1 + f2 - f3 + 0.0;
      Cc[at3(n2, fi + 1, fj + 1, fk)] = f0 + f1 + f2 - f3 + 0.0;
      Cc[at3(n2, fi, fj, fk + 1)] = f0 - f1 - f2 + f3 + 0.0;
      Cc[at3(n2, fi + 1, fj, fk + 1)] = f0 + f1 - f2 + f3 + 0.0;
      Cc[at3(n2, fi, fj + 1, fk + 1)] = f0 - f1 + f2 + f3 + 0.0;
      Cc[at3(n2, fi + 1, fj + 1, fk + 1)] = f0 + f1 + f2 + f3 + 0.0;
    }
  }
}

// af_prolong_linear with add = .false. (m_af_prolong.f90:531-679): one CTA
// per child box, one thread per parent cell of the child's quadrant/octant.
// Each fine cell sums the weighted parent values in the reference's order
// (centre, x, y, z, xy, xz, yz, xyz neighbour on the fine cell's side) and
// adds the zeroed child value.  Weights 9,3,3,1 /16 in 2D, 27,9,3,1 /64 in
// 3D by the number of offsets; all are exact in binary.
template <int D>
__global__ void __launch_bounds__(128) k_prolong_linear(KTree t, const int* __restrict__ list, double* __restrict__ v) {
  const int slot = list[blockIdx.x];
  const int pslot = t.parent[slot];
  const int nc = t.nc, n2 = t.n2, hnc = nc / 2;
  const double* P = v + (size_t)pslot * t.S;
  double* Cc = v + (size_t)slot * t.S;
  const int o0 = child_offset(t, slot, 0), o1 = child_offset(t, slot, 1);
  const int o2 = D == 3 ? child_offset(t, slot, 2) : 0;
  const int count = D == 2 ? hnc * hnc : hnc * hnc * hnc;
  const int sy = n2, sz = n2 * n2;
  for (int w = threadIdx.x; w < count; w += blockDim.x) {
    const int i = w % hnc + 1, r = w / hnc;
    const int j = D == 2 ? r + 1 : r % hnc + 1, k = D == 2 ? 0 : r / hnc + 1;
    const int ic = i + o0, jc = j + o1, kc = k + o2;
    const int fi = 2 * i - 1, fj = 2 * j - 1, fk = 2 * k - 1;
    if (D == 2) {
      const double f1 = 1 / 16.0, f3 = 3 / 16.0, f9 = 9 / 16.0;
      const int p = at2(n2, ic, jc);
      const double f0 = f9 * P[p];
      const double flx = f3 * P[p - 1], fhx = f3 * P[p + 1];
      const double fly = f3 * P[p - sy], fhy = f3 * P[p + sy];
      const double fll = f1 * P[p - 1 - sy], fhl = f1 * P[p + 1 - sy];
      const double flh = f1 * P[p - 1 + sy], fhh = f1 * P[p + 1 + sy];
      Cc[at2(n2, fi, fj)] = f0 + flx + fly + fll + 0.0;
      Cc[at2(n2, fi + 1, fj)] = f0 + fhx + fly + fhl + 0.0;
      Cc[at2(n2, fi, fj + 1)] = f0 + flx + fhy + flh + 0.0;
      Cc[at2(n2, fi + 1, fj + 1)] = f0 + fhx + fhy + fhh + 0.0;
    } else {
      const double wt[4] = {27 / 64.0, 9 / 64.0, 3 / 64.0, 1 / 64.0};
      const int p = at3(n2, ic, jc, kc);
      for (int oct = 0; oct < 8; oct++) {
        const int di = oct & 1, dj = (oct >> 1) & 1, dk = oct >> 2;
        const int sx1 = di ? 1 : -1, sy1 = dj ? sy : -sy, sz1 = dk ? sz : -sz;
        double s = wt[0] * P[p];
        s = s + wt[1] * P[p + sx1];
        s = s + wt[1] * P[p + sy1];
        s = s + wt[1] * P[p + sz1];
        s = s + wt[2] * P[p + sx1 + sy1];
        s = s + wt[2] * P[p + sx1 + sz1];
        s = s + wt[2] * P[p + sy1 + sz1];
        s = s + wt[3] * P[p + sx1 + sy1 + sz1];
        Cc[at3(n2, fi + di, fj + dj, fk + dk)] = s + 0.0;
      }
    }
  }
}

// new pool slot <- old pool slot (whole box), for boxes that persist
__global__ void __launch_bounds__(256) k_remap_boxes(int n_new, int S, const int* __restrict__ old_slot,
                                                     const double* __restrict__ src, double* __restrict__ dst) {
  const int b = blockIdx.x;
  if (b >= n_new) return;
  const int o = old_slot[b];
  if (o < 0) return;
  for (int x = threadIdx.x; x < S; x += blockDim.x) dst[(size_t)b * S + x] = src[(size_t)o * S + x];
}

}  // namespace afg

extern "C" {

int afg_refine_flags(afg_ctx* ctx, const afg_refine_desc* d, int* box_flags) {
  RC(need_transport(ctx));
  if (!d || !box_flags) return fail(ctx, AFG_ERR_ARG, "null refinement arguments");
  RC(check_var(ctx, d->i_electron));
  RC(check_var(ctx, d->i_electric_fld));
  const afg_transport_desc& td = ctx->tr.d;
  if (d->lt_col_alpha < 0 || d->lt_col_alpha >= td.lt_n_cols || d->lt_col_eta < 0 || d->lt_col_eta >= td.lt_n_cols)
    return fail(ctx, AFG_ERR_ARG, "bad lookup-table column");
  if (d->n_seeds < 0 || d->n_seeds > AFG_MAX_REFINE_ITEMS || d->n_regions < 0 ||
      d->n_regions > AFG_MAX_REFINE_ITEMS || d->n_limits < 0 || d->n_limits > AFG_MAX_REFINE_ITEMS)
    return fail(ctx, AFG_ERR_ARG, "too many refinement seeds, regions or limits");
  if (d->ref_buffer < 0 || d->ref_buffer > ctx->nc) return fail(ctx, AFG_ERR_ARG, "bad ref_buffer");
  if (!(d->gas_number_density > 0) || !(d->adx_fac > 0)) return fail(ctx, AFG_ERR_ARG, "bad gas density or adx_fac");
  // the electrode boxes of the field's slot (box tag mg_lsf_box)
  const int* lidx = nullptr;
  if (d->electrode_mg >= 0 && d->electrode_mg < kMaxMg && ctx->mg[d->electrode_mg].used &&
      ctx->mg[d->electrode_mg].lsf)
    lidx = ctx->mg[d->electrode_mg].lsf->d_idx;
  const int n = ctx->n_boxes;
  // the leaves, and every parent of a leaf once (consistent_ref_flags
  // evaluates it for the first of its children that is not refined)
  std::vector<int> list;
  std::vector<unsigned char> mark(n, 0);
  for (const auto& lv : ctx->lvl_leaves)
    for (int s : lv) {
      list.push_back(s);
      const int p = ctx->h_parent[s];
      if (p >= 0 && !mark[p]) {
        mark[p] = 1;
        list.push_back(p);
      }
    }
  if (list.empty()) {
    for (int b = 0; b < n; b++) box_flags[b] = AFG_REF_KEEP;
    return AFG_OK;
  }
  int *d_list = nullptr, *d_flags = nullptr;
  CK(dalloc(&d_list, list.size()));
  if (dalloc(&d_flags, n) != cudaSuccess) {
    dfree(d_list);
    return fail(ctx, AFG_ERR_NOMEM, "cannot allocate refinement flags");
  }
  std::vector<int> init(n, INT_MIN);
  int rc = AFG_OK;
  if (cudaMemcpy(d_list, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d_flags, init.data(), sizeof(int) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = fail(ctx, AFG_ERR_CUDA, "refinement flag upload failed");
  } else {
    KTree t = ktree(ctx);
    const double* E = ctx->cc[d->i_electric_fld - 1];
    const double* ne = ctx->cc[d->i_electron - 1];
    if (ctx->D == 3)
      k_refine_flags<3><<<(int)list.size(), 128, 0, ctx->stream>>>(t, d_list, E, ne, lt_dev(ctx), *d, d_flags, lidx);
    else
      k_refine_flags<2><<<(int)list.size(), 128, 0, ctx->stream>>>(t, d_list, E, ne, lt_dev(ctx), *d, d_flags, lidx);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(box_flags, d_flags, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = fail(ctx, AFG_ERR_CUDA, "refinement flags: %s", cudaGetErrorString(e));
  }
  dfree(d_list);
  dfree(d_flags);
  if (rc != AFG_OK) return rc;
  for (int b = 0; b < n; b++)
    if (box_flags[b] == INT_MIN) box_flags[b] = AFG_REF_KEEP;
  return AFG_OK;
}

int afg_prolong_limit(afg_ctx* ctx, int iv, int n, const int* ids, int limiter) {
  RC(check_var(ctx, iv));
  if (n < 0 || (n > 0 && !ids)) return fail(ctx, AFG_ERR_ARG, "bad box list");
  if (limiter < AFG_LIMITER_VANLEER || limiter > AFG_LIMITER_GMINMOD43) return fail(ctx, AFG_ERR_ARG, "bad limiter");
  if (n == 0) return AFG_OK;
  std::vector<int> slots(n);
  for (int q = 0; q < n; q++) {
    if (ids[q] < 1 || ids[q] > ctx->n_boxes) return fail(ctx, AFG_ERR_ARG, "bad box id %d", ids[q]);
    slots[q] = ids[q] - 1;
    if (ctx->h_parent[slots[q]] < 0) return fail(ctx, AFG_ERR_ARG, "box %d has no parent", ids[q]);
  }
  int* d_list = nullptr;
  CK(dalloc(&d_list, n));
  cudaError_t e = cudaMemcpy(d_list, slots.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    KTree t = ktree(ctx);
    if (ctx->D == 3)
      k_prolong_limit<3><<<n, 128, 0, ctx->stream>>>(t, d_list, ctx->cc[iv - 1], limiter);
    else
      k_prolong_limit<2><<<n, 128, 0, ctx->stream>>>(t, d_list, ctx->cc[iv - 1], limiter);
    ctx->launches++;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  }
  dfree(d_list);
  if (e != cudaSuccess) return fail(ctx, AFG_ERR_CUDA, "prolongation: %s", cudaGetErrorString(e));
  return AFG_OK;
}

int afg_prolong_linear(afg_ctx* ctx, int iv, int n, const int* ids) {
  RC(check_var(ctx, iv));
  if (n < 0 || (n > 0 && !ids)) return fail(ctx, AFG_ERR_ARG, "bad box list");
  if (n == 0) return AFG_OK;
  std::vector<int> slots(n);
  for (int q = 0; q < n; q++) {
    if (ids[q] < 1 || ids[q] > ctx->n_boxes) return fail(ctx, AFG_ERR_ARG, "bad box id %d", ids[q]);
    slots[q] = ids[q] - 1;
    if (ctx->h_parent[slots[q]] < 0) return fail(ctx, AFG_ERR_ARG, "box %d has no parent", ids[q]);
  }
  int* d_list = nullptr;
  CK(dalloc(&d_list, n));
  cudaError_t e = cudaMemcpy(d_list, slots.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    KTree t = ktree(ctx);
    if (ctx->D == 3)
      k_prolong_linear<3><<<n, 128, 0, ctx->stream>>>(t, d_list, ctx->cc[iv - 1]);
    else
      k_prolong_linear<2><<<n, 128, 0, ctx->stream>>>(t, d_list, ctx->cc[iv - 1]);
    ctx->launches++;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  }
  dfree(d_list);
  if (e != cudaSuccess) return fail(ctx, AFG_ERR_CUDA, "linear prolongation: %s", cudaGetErrorString(e));
  return AFG_OK;
}

int afg_restrict_tree(afg_ctx* ctx, int iv) {
  RC(check_var(ctx, iv));
  KTree t = ktree(ctx);
  const bool cyl = ctx->coord == AFG_CYL;
  double* v = ctx->cc[iv - 1];
  for (int lvl = ctx->highest_lvl; lvl >= 2; lvl--) {
    const int n = (int)ctx->lvl_ids[lvl - 1].size();
    if (n == 0) continue;
    const int* list = lst(ctx, ctx->off_ids[lvl - 1]);
    if (ctx->D == 3)
      AFG_NC3(NCV_, k_restrict_geom<3, false, NCV_><<<n, 64, 0, ctx->stream>>>(t, list, v));
    else if (cyl)
      AFG_NC2(NCV_, k_restrict_geom<2, true, NCV_><<<n, 64, 0, ctx->stream>>>(t, list, v));
    else
      AFG_NC2(NCV_, k_restrict_geom<2, false, NCV_><<<n, 64, 0, ctx->stream>>>(t, list, v));
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, AFG_ERR_CUDA, "restriction: %s", cudaGetErrorString(e));
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return fail(ctx, AFG_ERR_CUDA, "restriction: %s", cudaGetErrorString(e));
  return AFG_OK;
}

int afg_tree_remap(afg_ctx* ctx, const afg_tree_desc* tree, const int* old_id) {
  if (!ctx || !tree || !old_id) return AFG_ERR_ARG;
  if (!ctx->have_tree) return fail(ctx, AFG_ERR_STATE, "no tree to remap from");
  if (ctx->n_inst > 0) return fail(ctx, AFG_ERR_UNSUPPORTED, "remap of batched trees");
  if (tree->ndim != ctx->D || tree->n_cell != ctx->nc) return fail(ctx, AFG_ERR_ARG, "remap needs the same box size");
  const int n_old = ctx->n_boxes, n_new = tree->n_boxes;
  if (n_new <= 0) return fail(ctx, AFG_ERR_ARG, "empty tree");
  std::vector<int> map(n_new);
  for (int b = 0; b < n_new; b++) {
    if (old_id[b] < 0 || old_id[b] > n_old) return fail(ctx, AFG_ERR_ARG, "bad old id of box %d", b + 1);
    map[b] = old_id[b] - 1;
  }
  CK(cudaStreamSynchronize(ctx->stream));
  // keep the old pools out of the tree rebuild
  std::vector<double*> old_cc, old_fc;
  old_cc.swap(ctx->cc);
  old_fc.swap(ctx->fc);
  const int nvc = ctx->n_var, nvf = ctx->n_var_face;
  auto release = [&]() {
    for (auto& p : old_cc) dfree(p);
    for (auto& p : old_fc) dfree(p);
  };
  int rc = afg_tree_sync(ctx, tree, nvc, nvf);
  if (rc != AFG_OK) {
    release();
    return rc;
  }
  int* d_map = nullptr;
  if (dalloc(&d_map, n_new) != cudaSuccess || cudaMemcpy(d_map, map.data(), sizeof(int) * n_new,
                                                         cudaMemcpyHostToDevice) != cudaSuccess) {
    dfree(d_map);
    release();
    return fail(ctx, AFG_ERR_CUDA, "remap table upload failed");
  }
  const int Sf = ctx->D * ctx->NF;
  for (int v = 0; v < nvc; v++) {
    k_remap_boxes<<<n_new, 256, 0, ctx->stream>>>(n_new, ctx->S, d_map, old_cc[v], ctx->cc[v]);
    ctx->launches++;
  }
  for (int v = 0; v < nvf; v++) {
    k_remap_boxes<<<n_new, 256, 0, ctx->stream>>>(n_new, Sf, d_map, old_fc[v], ctx->fc[v]);
    ctx->launches++;
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  dfree(d_map);
  release();
  if (e != cudaSuccess) return fail(ctx, AFG_ERR_CUDA, "remap: %s", cudaGetErrorString(e));
  return AFG_OK;
}

}  // extern "C"
