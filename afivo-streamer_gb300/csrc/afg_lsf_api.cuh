// afg_lsf_api.cuh -- C-ABI of the electrode set-up (afg_lsf.cuh).
// Included by afg_runtime.cu after the multigrid set-up.
#pragma once

namespace {

// get_conical_rod_properties (src/m_field.f90:406-428): the cone's length is
// cone_length_frac (electrode 1's module value, for either electrode) times
// the rod length; the tip sphere's radius and centre follow from the cone
// angle.  Host C library atan/cos/sin, once per set-up.
void conical_props(const double* r0, const double* r1, int D, double radius, double tip_radius, double cone_frac,
                   double* center, double& r_curv) {
  double h[3];
  for (int d = 0; d < D; d++) h[d] = r1[d] - r0[d];
  const double len = afg_lsf::norm2(h, D);
  const double cone_length = cone_frac * len;
  const double angle = std::atan((radius - tip_radius) / cone_length);
  r_curv = tip_radius / std::cos(angle);
  for (int d = 0; d < D; d++) center[d] = r1[d] - std::sin(angle) * r_curv * (r1[d] - r0[d]) / len;
}

}  // namespace

int afg_mg_set_lsf(afg_ctx* ctx, int mg_id, const afg_lsf_desc* d) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (!d) return fail(ctx, AFG_ERR_ARG, "no electrode description");
  if (m->d.precision != AFG_FP64) return fail(ctx, AFG_ERR_UNSUPPORTED, "electrode: FP64 multigrid slots only");
  if (m->d.helmholtz_lambda != 0.0) return fail(ctx, AFG_ERR_UNSUPPORTED, "electrode: Poisson operator only");
  if (ctx->n_inst > 0) return fail(ctx, AFG_ERR_UNSUPPORTED, "electrode on batched instances");
  if (d->i_lsf < 1 || d->i_lsf > ctx->n_var) return fail(ctx, AFG_ERR_ARG, "bad level-set variable %d", d->i_lsf);
  if (d->i_lsf == m->d.i_phi || d->i_lsf == m->d.i_rhs || d->i_lsf == m->d.i_tmp)
    return fail(ctx, AFG_ERR_ARG, "the level-set variable must differ from phi, rhs and tmp");
  if (d->shape < AFG_LSF_SPHERE || d->shape > AFG_LSF_COAXIAL) return fail(ctx, AFG_ERR_ARG, "bad electrode shape");
  if (!(d->radius > 0)) return fail(ctx, AFG_ERR_ARG, "field_rod_radius not set correctly");
  if (!(d->length_scale > 0) || !(d->tol > 0) || !(d->min_rel_distance > 0) || !(d->gradient_safety_factor > 0))
    return fail(ctx, AFG_ERR_ARG, "bad level-set search parameters");
  const int D = ctx->D, nc = ctx->nc;
  afg_lsf::Electrode e{};
  e.shape = d->shape;
  e.D = D;
  e.cyl = ctx->coord == AFG_CYL;
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
  if (e.shape == AFG_LSF_ROD_CONE_TOP || e.shape == AFG_LSF_TWO_ROD_CONE) {
    if (!(e.tip_radius > 0) || e.tip_radius > e.radius || e.cone_frac < 0 || e.cone_frac > 1)
      return fail(ctx, AFG_ERR_ARG, "cone parameters not set correctly");
    conical_props(e.r0, e.r1, D, e.radius, e.tip_radius, e.cone_frac, e.tip_center, e.r_curv);
  }
  if (e.shape == AFG_LSF_TWO_ROD_CONE) {
    if (!(e.tip_radius2 > 0) || e.tip_radius2 > e.radius2 || e.cone_frac2 < 0 || e.cone_frac2 > 1)
      return fail(ctx, AFG_ERR_ARG, "cone2 parameters not set correctly");
    conical_props(e.q0, e.q1, D, e.radius2, e.tip_radius2, e.cone_frac, e.tip_center2, e.r_curv2);
  }
  if ((e.shape == AFG_LSF_ROD_ROD || e.shape == AFG_LSF_SPHERE_ROD || e.shape == AFG_LSF_TWO_ROD_CONE ||
       e.shape == AFG_LSF_COAXIAL) && !(e.radius2 > 0))
    return fail(ctx, AFG_ERR_ARG, "field_rod2_radius not set correctly");
  clear_graphs(ctx);
  delete m->lsf;
  m->lsf = nullptr;
  std::unique_ptr<LsfState> Lp(new LsfState());
  LsfState& L = *Lp;
  L.e = e;
  L.i_lsf = d->i_lsf;
  L.SI = D == 2 ? nc * nc : nc * nc * nc;
  const int SI = L.SI, nall = ctx->n_all;
  KTree t = ktree(ctx);
  t.lsf = nullptr;
  const int* all = lst(ctx, ctx->off_all);
  // level-set values (set_lsf_box), then the root mask per box
  if (D == 3) afg::k_lsf_values<3><<<nall, 128, 0, ctx->stream>>>(t, all, e, ctx->cc[L.i_lsf - 1]);
  else afg::k_lsf_values<2><<<nall, 128, 0, ctx->stream>>>(t, all, e, ctx->cc[L.i_lsf - 1]);
  ctx->launches++;
  CKL();
  int* d_cnt = nullptr;
  CK(dalloc(&d_cnt, nall));
  if (D == 3) afg::k_lsf_mask<3><<<nall, 128, 0, ctx->stream>>>(t, all, e, d_cnt);
  else afg::k_lsf_mask<2><<<nall, 128, 0, ctx->stream>>>(t, all, e, d_cnt);
  ctx->launches++;
  std::vector<int> cnt(nall);
  // (the context's stream does not synchronise with the default stream)
  cudaError_t err = cudaGetLastError();
  if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
  if (err == cudaSuccess) err = cudaMemcpy(cnt.data(), d_cnt, sizeof(int) * nall, cudaMemcpyDeviceToHost);
  dfree(d_cnt);
  if (err != cudaSuccess) return fail(ctx, AFG_ERR_CUDA, "electrode root mask: %s", cudaGetErrorString(err));
  // the all-box list on the host, in the device list's (level) order
  std::vector<int> h_all;
  h_all.reserve(nall);
  for (int l = 0; l < ctx->highest_lvl; l++) h_all.insert(h_all.end(), ctx->lvl_ids[l].begin(), ctx->lvl_ids[l].end());
  std::vector<int> mslots;
  for (int b = 0; b < nall; b++)
    if (cnt[b] > 0) mslots.push_back(h_all[b]);
  // distances of the root-mask boxes; electrode boxes are those with one
  const int nm = (int)mslots.size();
  std::vector<int> any(std::max(1, nm), 0);
  int *d_ms = nullptr, *d_any = nullptr;
  double* d_ddt = nullptr;
  if (nm > 0) {
    CK(dalloc(&d_ms, nm));
    CK(dalloc(&d_any, nm));
    if (dalloc(&d_ddt, (size_t)nm * 2 * D * SI) != cudaSuccess) {
      dfree(d_ms);
      dfree(d_any);
      return fail(ctx, AFG_ERR_NOMEM, "electrode distances of %d boxes", nm);
    }
    err = cudaMemcpyAsync(d_ms, mslots.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, ctx->stream);
    if (err == cudaSuccess) err = cudaMemsetAsync(d_any, 0, sizeof(int) * nm, ctx->stream);
    if (err == cudaSuccess) {
      if (D == 3) afg::k_lsf_dist<3><<<nm, 128, 0, ctx->stream>>>(t, d_ms, e, d_ddt, d_any);
      else afg::k_lsf_dist<2><<<nm, 128, 0, ctx->stream>>>(t, d_ms, e, d_ddt, d_any);
      ctx->launches++;
      err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
    if (err == cudaSuccess) err = cudaMemcpy(any.data(), d_any, sizeof(int) * nm, cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) {
      dfree(d_ms);
      dfree(d_any);
      dfree(d_ddt);
      return fail(ctx, AFG_ERR_CUDA, "electrode distances: %s", cudaGetErrorString(err));
    }
  }
  std::vector<int> src;
  for (int b = 0; b < nm; b++)
    if (any[b]) {
      L.h_slots.push_back(mslots[b]);
      src.push_back(b);
    }
  L.n = (int)L.h_slots.size();
  std::vector<int> idx(ctx->n_boxes, -1);
  for (int q = 0; q < L.n; q++) idx[L.h_slots[q]] = q;
  const int n = std::max(1, L.n);
  CK(dalloc(&L.d_idx, ctx->n_boxes));
  CK(cudaMemcpyAsync(L.d_idx, idx.data(), sizeof(int) * ctx->n_boxes, cudaMemcpyHostToDevice, ctx->stream));
  CK(dalloc(&L.d_slots, n));
  CK(dalloc(&L.d_v, (size_t)n * (2 * D + 1) * SI));
  CK(dalloc(&L.d_f, (size_t)n * SI));
  CK(dalloc(&L.d_bcc, (size_t)n * SI));
  CK(dalloc(&L.d_bv, (size_t)n * SI));
  CK(dalloc(&L.d_dd, (size_t)n * 2 * D * SI));
  if (L.n > 0) {
    int* d_src = nullptr;
    CK(dalloc(&d_src, L.n));
    err = cudaMemcpyAsync(L.d_slots, L.h_slots.data(), sizeof(int) * L.n, cudaMemcpyHostToDevice, ctx->stream);
    if (err == cudaSuccess) err = cudaMemcpyAsync(d_src, src.data(), sizeof(int) * L.n, cudaMemcpyHostToDevice, ctx->stream);
    if (err == cudaSuccess) {
      if (D == 3)
        afg::k_lsf_stencil<3><<<L.n, 128, 0, ctx->stream>>>(t, L.d_slots, d_src, d_ddt, 0, L.d_v, L.d_f, L.d_dd);
      else
        afg::k_lsf_stencil<2><<<L.n, 128, 0, ctx->stream>>>(t, L.d_slots, d_src, d_ddt, e.cyl, L.d_v, L.d_f,
                                                            L.d_dd);
      ctx->launches++;
      err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
    dfree(d_src);
  }
  dfree(d_ms);
  dfree(d_any);
  dfree(d_ddt);
  if (err != cudaSuccess) return fail(ctx, AFG_ERR_CUDA, "electrode stencils: %s", cudaGetErrorString(err));
  // lists per level: all electrode boxes, those with children, leaves
  std::vector<char> leaf(ctx->n_boxes, 0);
  for (const auto& lv : ctx->lvl_leaves)
    for (int s : lv) leaf[s] = 1;
  const int H = ctx->highest_lvl;
  L.lvl_all.assign(H, {});
  L.lvl_par.assign(H, {});
  L.lvl_leaf.assign(H, {});
  for (int l = 0; l < H; l++)
    for (int s : ctx->lvl_ids[l]) {
      if (idx[s] < 0) continue;
      L.lvl_all[l].push_back(s);
      (leaf[s] ? L.lvl_leaf : L.lvl_par)[l].push_back(s);
    }
  if (L.lvl_all[0].empty())
    return fail(ctx, AFG_ERR_ARG, "level set function not resolved on coarse grid (no root on level 1)");
  std::vector<int> lists;
  auto pack = [&](const std::vector<std::vector<int>>& per, std::vector<size_t>& off) {
    off.resize(H);
    for (int l = 0; l < H; l++) {
      off[l] = lists.size();
      lists.insert(lists.end(), per[l].begin(), per[l].end());
    }
  };
  pack(L.lvl_all, L.off_all);
  pack(L.lvl_par, L.off_par);
  pack(L.lvl_leaf, L.off_leaf);
  CK(dalloc(&L.d_lists, std::max<size_t>(1, lists.size())));
  if (!lists.empty())
    CK(cudaMemcpyAsync(L.d_lists, lists.data(), sizeof(int) * lists.size(), cudaMemcpyHostToDevice, ctx->stream));
  // level-1 electrode boxes: stencils for the coarse matrix, and the map of
  // their cells to coarse unknowns for the boundary-value term
  const std::vector<int>& l1 = L.lvl_all[0];
  L.h_v1.resize(l1.size() * (size_t)(2 * D + 1) * SI);
  std::vector<int> cg, ck;
  for (size_t p = 0; p < l1.size(); p++) {
    const int s = l1[p], q = idx[s];
    CK(cudaMemcpy(L.h_v1.data() + p * (size_t)(2 * D + 1) * SI, L.d_v + (size_t)q * (2 * D + 1) * SI,
                  sizeof(double) * (2 * D + 1) * SI, cudaMemcpyDeviceToHost));
    for (int c = 0; c < SI; c++) {
      const int i = c % nc, j = (c / nc) % nc, k = D == 3 ? c / (nc * nc) : 0;
      const long I = (long)(ctx->h_ix[(size_t)s * D] - 1) * nc + i;
      const long J = (long)(ctx->h_ix[(size_t)s * D + 1] - 1) * nc + j;
      const long K = D == 3 ? (long)(ctx->h_ix[(size_t)s * D + 2] - 1) * nc + k : 0;
      cg.push_back((int)(I + ctx->cgs[0] * (J + (long)ctx->cgs[1] * K)));
      ck.push_back(q * SI + c);
    }
  }
  L.n_cb = (int)cg.size();
  CK(dalloc(&L.d_cb_g, std::max(1, L.n_cb)));
  CK(dalloc(&L.d_cb_k, std::max(1, L.n_cb)));
  if (L.n_cb > 0) {
    CK(cudaMemcpyAsync(L.d_cb_g, cg.data(), sizeof(int) * L.n_cb, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(L.d_cb_k, ck.data(), sizeof(int) * L.n_cb, cudaMemcpyHostToDevice, ctx->stream));
  }
  // the coarse-grid matrix with the electrode stencils
  m->lsf = Lp.release();
  dfree(m->d_ainv); dfree(m->d_b); dfree(m->d_x); dfree(m->d_b2r); dfree(m->d_bmask); dfree(m->d_bcval);
  int rc = build_coarse(ctx, *m);
  if (rc == AFG_OK) rc = lsf_set_voltage(ctx, *m, 0.0);
  if (rc == AFG_OK) {
    err = cudaStreamSynchronize(ctx->stream);
    if (err != cudaSuccess) rc = fail(ctx, AFG_ERR_CUDA, "electrode set-up: %s", cudaGetErrorString(err));
  }
  if (rc != AFG_OK) {
    delete m->lsf;
    m->lsf = nullptr;
    m->used = false;
  }
  return rc;
}

int afg_mg_set_lsf_voltage(afg_ctx* ctx, int mg_id, double voltage) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (!m->lsf) return fail(ctx, AFG_ERR_STATE, "slot %d has no electrode", mg_id);
  RC(lsf_set_voltage(ctx, *m, voltage));
  CK(cudaStreamSynchronize(ctx->stream));
  return AFG_OK;
}

int afg_mg_lsf_info(afg_ctx* ctx, int mg_id, int* n_boxes, int* ids, double* v, double* f, double* bcc, double* dd) {
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (!m->lsf) return fail(ctx, AFG_ERR_STATE, "slot %d has no electrode", mg_id);
  const LsfState& L = *m->lsf;
  const int D = ctx->D, SI = L.SI, n = L.n;
  if (n_boxes) *n_boxes = n;
  CK(cudaStreamSynchronize(ctx->stream));
  if (ids)
    for (int q = 0; q < n; q++) ids[q] = L.h_slots[q] + 1;
  if (n > 0) {
    if (v) CK(cudaMemcpy(v, L.d_v, sizeof(double) * (size_t)n * (2 * D + 1) * SI, cudaMemcpyDeviceToHost));
    if (f) CK(cudaMemcpy(f, L.d_f, sizeof(double) * (size_t)n * SI, cudaMemcpyDeviceToHost));
    if (bcc) CK(cudaMemcpy(bcc, L.d_bcc, sizeof(double) * (size_t)n * SI, cudaMemcpyDeviceToHost));
    if (dd) CK(cudaMemcpy(dd, L.d_dd, sizeof(double) * (size_t)n * 2 * D * SI, cudaMemcpyDeviceToHost));
  }
  return AFG_OK;
}

/* ---- the electrode in the species update and the initial state ---------- */

int afg_transport_set_electrode(afg_ctx* ctx, int i_lsf) {
  RC(need_transport(ctx));
  if (i_lsf != 0) RC(check_var(ctx, i_lsf));
  ctx->tr.mask_iv = i_lsf;
  clear_graphs(ctx);
  return AFG_OK;
}

static int electrode_dens(afg_ctx* ctx, afg::DensPtrs& dn) {
  const afg_transport_desc& td = ctx->tr.d;
  dn.ns = td.n_species;
  for (int s = 0; s < td.n_species; s++) {
    RC(check_var(ctx, td.species_iv[s]));
    dn.p[s] = ctx->cc[td.species_iv[s] - 1];
  }
  return AFG_OK;
}

int afg_electrode_init_densities(afg_ctx* ctx, int mg_id, int n, const int* ids) {
  RC(need_transport(ctx));
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (!m->lsf) return fail(ctx, AFG_ERR_STATE, "slot %d has no electrode", mg_id);
  if (n < 0 || (n > 0 && !ids)) return fail(ctx, AFG_ERR_ARG, "bad box list");
  if (n == 0) return AFG_OK;
  afg::DensPtrs dn{};
  RC(electrode_dens(ctx, dn));
  std::vector<int> slots(n);
  for (int q = 0; q < n; q++) {
    if (ids[q] < 1 || ids[q] > ctx->n_boxes) return fail(ctx, AFG_ERR_ARG, "bad box id %d", ids[q]);
    slots[q] = ids[q] - 1;
  }
  int* d_list = nullptr;
  CK(dalloc(&d_list, n));
  cudaError_t e = cudaMemcpyAsync(d_list, slots.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    afg::k_electrode_init<<<n, 128, 0, ctx->stream>>>(ctx->S, d_list, ctx->cc[m->lsf->i_lsf - 1], dn);
    ctx->launches++;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  dfree(d_list);
  if (e != cudaSuccess) return fail(ctx, AFG_ERR_CUDA, "electrode initial densities: %s", cudaGetErrorString(e));
  return AFG_OK;
}

int afg_electrode_species_bc(afg_ctx* ctx, int mg_id, int electron, int ion, int neumann) {
  RC(need_transport(ctx));
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (!m->lsf) return fail(ctx, AFG_ERR_STATE, "slot %d has no electrode", mg_id);
  const afg_transport_desc& td = ctx->tr.d;
  if (electron < 0 || electron >= td.n_species || ion < 0 || ion >= td.n_species)
    return fail(ctx, AFG_ERR_ARG, "bad species index");
  afg::DensPtrs dn{};
  RC(electrode_dens(ctx, dn));
  const LsfState& L = *m->lsf;
  KTree t = ktree(ctx);
  for (int lvl = 1; lvl <= ctx->highest_lvl; lvl++) {
    const int n = (int)L.lvl_all[lvl - 1].size();
    if (n == 0) continue;
    if (ctx->D == 3)
      afg::k_electrode_species_bc<3><<<n, 128, 0, ctx->stream>>>(t, L.d_lists + L.off_all[lvl - 1], ctx->cc[L.i_lsf - 1],
                                                                  dn, electron, ion, neumann);
    else
      afg::k_electrode_species_bc<2><<<n, 128, 0, ctx->stream>>>(t, L.d_lists + L.off_all[lvl - 1], ctx->cc[L.i_lsf - 1],
                                                                  dn, electron, ion, neumann);
    ctx->launches++;
    CKL();
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return AFG_OK;
}
