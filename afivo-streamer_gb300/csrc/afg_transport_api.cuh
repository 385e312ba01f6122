// afg_transport_api.cuh -- host drivers of the transport, field and
// photoionization entry points (included at the end of afg_runtime.cu).
#pragma once
#include "afg_transport32.cuh"

static int need_transport(afg_ctx* ctx) {
  if (!ctx) return AFG_ERR_ARG;
  if (ctx->poisoned) return fail(ctx, AFG_ERR_CUDA, "context unusable after a failed drain of shared-memory copies");
  if (!ctx->have_tree) return fail(ctx, AFG_ERR_STATE, "no tree");
  if (!ctx->tr.ready) return fail(ctx, AFG_ERR_STATE, "afg_transport_setup not called");
  return AFG_OK;
}

static LtDev lt_dev(const afg_ctx* ctx) {
  LtDev lt;
  lt.y = ctx->tr.d_lt;
  lt.n = ctx->tr.d.lt_n_points;
  lt.x_min = ctx->tr.d.lt_x_min;
  lt.inv_fac = ctx->tr.d.lt_inv_fac;
  return lt;
}

static LtDevF lt_dev_f(const afg_ctx* ctx) {
  LtDevF lt;
  lt.y = ctx->tr.d_ltf;
  lt.n = ctx->tr.d.lt_n_points;
  lt.x_min = (float)ctx->tr.d.lt_x_min;
  lt.inv_fac = (float)ctx->tr.d.lt_inv_fac;
  return lt;
}

// species-update launchers (afg_species_update.cu)
namespace afg {
void launch_update32(int D, bool cyl, int nc, int ns, int n, const KTree& t, const int* list, const UpdateArgs32& u,
                     size_t smem, cudaStream_t st);
void launch_update64(int D, bool cyl, int nc, int ns, int n, const KTree& t, const int* list, const UpdateArgs& a,
                     cudaStream_t st);
}  // namespace afg

static bool mixed_transport(const afg_ctx* ctx) { return ctx->tr.ready && ctx->tr.d.precision == AFG_MIXED; }

static GcDev gc_from_desc(const afg_gc_desc& g) {
  GcDev d;
  for (int n = 0; n < 6; n++) {
    d.bc_type[n] = g.bc_type[n];
    d.bc_val[n] = g.bc_val[n];
  }
  d.rb = g.rb;
  return d;
}

static size_t flux32_smem(const afg_ctx* ctx, int n_flux) {
  const int D = ctx->D, nc = ctx->nc, m = nc + 4;
  const int tile = D == 2 ? m * m : m * m * m;
  const int nfaces = D == 2 ? nc * (nc + 1) : nc * nc * (nc + 1);
  return sizeof(float) * ((size_t)n_flux * tile + 2 * (size_t)D * nfaces + ctx->S);
}

// dynamic shared memory of k_flux32s: the staging buffer (|E| and the
// species, FP64; later the FP32 face values and diffusion coefficients),
// the FP32 tiles and |E| in FP32
static size_t flux32s_smem(const afg_ctx* ctx, int n_flux) {
  const int D = ctx->D, nc = ctx->nc, m = nc + 4;
  const int tile = D == 2 ? m * m : m * m * m;
  const size_t nfaces = D == 2 ? (size_t)nc * (nc + 1) : (size_t)nc * nc * (nc + 1);
  const size_t offA = (std::max(sizeof(double) * ctx->S * (n_flux + 1), 2 * sizeof(float) * D * nfaces) + 15) & ~(size_t)15;
  return offA + sizeof(float) * ((size_t)n_flux * tile + ctx->S);
}

extern "C" {

int afg_transport_setup(afg_ctx* ctx, const afg_transport_desc* d) {
  if (!ctx || !d) return AFG_ERR_ARG;
  if (!ctx->have_tree) return fail(ctx, AFG_ERR_STATE, "no tree");
  const afg_transport_desc& t = *d;
  if (t.n_species < 1 || t.n_species > AFG_MAX_SPECIES) return fail(ctx, AFG_ERR_ARG, "bad n_species");
  if (t.n_flux < 1 || t.n_flux > AFG_MAX_FLUX) return fail(ctx, AFG_ERR_ARG, "bad n_flux");
  if (t.n_reactions < 0 || t.n_reactions > AFG_MAX_REACTIONS) return fail(ctx, AFG_ERR_ARG, "bad n_reactions");
  if (t.lt_n_points < 2 || t.lt_n_cols < 1 || !t.lt_data) return fail(ctx, AFG_ERR_ARG, "bad lookup table");
  if (!(t.gas_number_density > 0)) return fail(ctx, AFG_ERR_ARG, "gas_number_density must be > 0");
  for (int c : {t.lt_col_mobility, t.lt_col_diffusion, t.lt_col_alpha})
    if (c < 0 || c >= t.lt_n_cols) return fail(ctx, AFG_ERR_ARG, "lookup-table column out of range");
  for (int s = 0; s < t.n_species; s++)
    if (t.species_iv[s] < 1 || t.species_iv[s] > ctx->n_var) return fail(ctx, AFG_ERR_ARG, "bad species variable");
  for (int f = 0; f < t.n_flux; f++) {
    if (t.flux_species[f] < 0 || t.flux_species[f] >= t.n_species) return fail(ctx, AFG_ERR_ARG, "bad flux species");
    if (t.flux_fc[f] < 1 || t.flux_fc[f] > ctx->n_var_face) return fail(ctx, AFG_ERR_ARG, "bad flux fc variable");
  }
  if (t.i_electric_fld < 1 || t.i_electric_fld > ctx->n_var) return fail(ctx, AFG_ERR_ARG, "bad i_electric_fld");
  if (t.i_efield_fc < 1 || t.i_efield_fc > ctx->n_var_face) return fail(ctx, AFG_ERR_ARG, "bad i_efield_fc");
  if (t.i_photo < 0 || t.i_photo > ctx->n_var) return fail(ctx, AFG_ERR_ARG, "bad i_photo");
  if (t.photoi_species < 0 || t.photoi_species >= t.n_species) return fail(ctx, AFG_ERR_ARG, "bad photoi_species");
  if (t.precision != AFG_FP64 && t.precision != AFG_MIXED) return fail(ctx, AFG_ERR_ARG, "bad precision");
  for (int n = 2 * ctx->D; n < 6; n++) (void)n;
  for (int n = 0; n < 2 * ctx->D; n++)
    if (t.species_gc.bc_type[n] == AFG_BC_CONTINUOUS)
      return fail(ctx, AFG_ERR_UNSUPPORTED, "two-layer ghost cells support Dirichlet/Neumann/copy only");
  for (int r = 0; r < t.n_reactions; r++) {
    const afg_reaction& rc = t.reactions[r];
    const int rt = rc.rate_type;
    if (!(rt == AFG_RATE_TABULATED_FIELD || rt == AFG_RATE_CONSTANT || rt == AFG_RATE_LINEAR ||
          rt == AFG_RATE_EXP_V1 || rt == AFG_RATE_EXP_V2 || rt == AFG_RATE_K13 || rt == AFG_RATE_K14 ||
          rt == AFG_RATE_K1))
      return fail(ctx, AFG_ERR_UNSUPPORTED, "reaction %d: unsupported rate form %d", r + 1, rt);
    if ((rt == AFG_RATE_TABULATED_FIELD || rt == AFG_RATE_K1) && (rc.lt_col < 0 || rc.lt_col >= t.lt_n_cols))
      return fail(ctx, AFG_ERR_ARG, "reaction %d: bad table column", r + 1);
    if (rc.n_in < 0 || rc.n_in > 4 || rc.n_out < 0 || rc.n_out > 4) return fail(ctx, AFG_ERR_ARG, "bad reaction size");
    for (int q = 0; q < rc.n_in; q++)
      if (rc.ix_in[q] < 0 || rc.ix_in[q] >= t.n_species) return fail(ctx, AFG_ERR_ARG, "bad reaction species");
    for (int q = 0; q < rc.n_out; q++)
      if (rc.ix_out[q] < 0 || rc.ix_out[q] >= t.n_species) return fail(ctx, AFG_ERR_ARG, "bad reaction species");
  }
  clear_graphs(ctx);
  {
    // the staged flux kernel keeps 5 CTAs per SM (its register bound) only
    // with the shared-memory carveout at its maximum
    static bool carveout_set = false;
    if (!carveout_set) {
      const int pct = cudaSharedmemCarveoutMaxShared;
      CK(cudaFuncSetAttribute(k_flux32s<3, false, 8, 1>, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
      CK(cudaFuncSetAttribute(k_flux32s<3, false, 8, 2>, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
      CK(cudaFuncSetAttribute(k_flux32s<2, true, 16, 1>, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
      CK(cudaFuncSetAttribute(k_flux32s<2, true, 16, 2>, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
      CK(cudaFuncSetAttribute(k_flux32s<2, false, 16, 1>, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
      CK(cudaFuncSetAttribute(k_flux32s<2, false, 16, 2>, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
      carveout_set = true;
    }
  }
  TransportState& s = ctx->tr;
  transport_free(s);
  s.d = t;
  s.d.lt_data = nullptr;
  CK(dalloc(&s.d_lt, (size_t)t.lt_n_cols * t.lt_n_points));
  CK(cudaMemcpy(s.d_lt, t.lt_data, sizeof(double) * t.lt_n_cols * t.lt_n_points, cudaMemcpyHostToDevice));
  CK(dalloc(&s.d_reactions, std::max(1, t.n_reactions)));
  if (t.n_reactions > 0)
    CK(cudaMemcpy(s.d_reactions, t.reactions, sizeof(afg_reaction) * t.n_reactions, cudaMemcpyHostToDevice));
  {
    // FP32 forms for the mixed-precision kernels
    std::vector<float> ltf((size_t)t.lt_n_cols * t.lt_n_points);
    for (size_t q = 0; q < ltf.size(); q++) ltf[q] = (float)t.lt_data[q];
    CK(dalloc(&s.d_ltf, ltf.size()));
    CK(cudaMemcpy(s.d_ltf, ltf.data(), sizeof(float) * ltf.size(), cudaMemcpyHostToDevice));
    std::vector<Reac32> r32(std::max(1, t.n_reactions));
    for (int r = 0; r < t.n_reactions; r++) {
      const afg_reaction& rc = t.reactions[r];
      Reac32& o = r32[r];
      o.rate_type = rc.rate_type;
      o.lt_col = rc.lt_col;
      if (rc.rate_type == AFG_RATE_TABULATED_FIELD) {
        // rate_factor (up to N^2) split into two factors of FP32 range
        const double h = std::sqrt(std::fabs(rc.rate_factor));
        o.fa = (float)(rc.rate_factor < 0 ? -h : h);
        o.fb = (float)(h > 0 ? std::fabs(rc.rate_factor) / h : 0.0);
      } else {
        o.fa = (float)(rc.rate_factor * rc.c[0]);
        o.fb = 1.0f;
      }
      o.c1 = (float)rc.c[1];
      o.c2 = (float)rc.c[2];
      o.c3 = (float)rc.c[3];
      // inputs as column offsets; the net change of every species touched:
      // each output's multiplicity less one per occurrence as an input
      o.n_in = rc.n_in;
      for (int q = 0; q < rc.n_in; q++) o.in_off[q] = rc.ix_in[q] * 128;
      double coef[AFG_MAX_SPECIES] = {};
      bool touched[AFG_MAX_SPECIES] = {};
      for (int q = 0; q < rc.n_in; q++) {
        coef[rc.ix_in[q]] -= 1.0;
        touched[rc.ix_in[q]] = true;
      }
      for (int q = 0; q < rc.n_out; q++) {
        coef[rc.ix_out[q]] += rc.mult_out[q];
        touched[rc.ix_out[q]] = true;
      }
      o.n_upd = 0;
      for (int sp = 0; sp < t.n_species; sp++)
        if (touched[sp] && coef[sp] != 0.0) {
          o.upd_off[o.n_upd] = sp * 128;
          o.upd_coef[o.n_upd] = (float)coef[sp];
          o.n_upd++;
        }
      if (t.precision == AFG_MIXED && (!std::isfinite(o.fa) || !std::isfinite(o.fb)))
        return fail(ctx, AFG_ERR_UNSUPPORTED, "reaction %d: rate factor outside the FP32 range", r + 1);
    }
    CK(dalloc(&s.d_reac32, r32.size()));
    CK(cudaMemcpy(s.d_reac32, r32.data(), sizeof(Reac32) * r32.size(), cudaMemcpyHostToDevice));
  }
  // task lists
  const int D = ctx->D, nnb = 2 * D, nch = 1 << D;
  std::vector<int> rrb, cflux;
  std::vector<int> h_children((size_t)ctx->n_boxes * nch);
  CK(cudaMemcpy(h_children.data(), ctx->d_children, sizeof(int) * h_children.size(), cudaMemcpyDeviceToHost));
  std::vector<int> h_parent(ctx->n_boxes);
  CK(cudaMemcpy(h_parent.data(), ctx->d_parent, sizeof(int) * ctx->n_boxes, cudaMemcpyDeviceToHost));
  for (int l = 0; l < ctx->highest_lvl; l++)
    for (int sl : ctx->lvl_leaves[l]) {
      if (h_parent[sl] < 0) continue;
      bool rb = false;
      for (int nb = 0; nb < nnb; nb++) rb = rb || ctx->h_nbr[(size_t)sl * nnb + nb] == 0;
      if (rb) rrb.push_back(sl);
    }
  for (int l = 0; l < ctx->highest_lvl - 1; l++)
    for (int sl : ctx->lvl_parents[l])
      for (int nb = 0; nb < nnb; nb++) {
        const int nid = ctx->h_nbr[(size_t)sl * nnb + nb];
        if (nid <= 0) continue;
        bool has_children = false;
        for (int c = 0; c < nch; c++) has_children = has_children || h_children[(size_t)(nid - 1) * nch + c] >= 0;
        if (has_children) continue;
        cflux.push_back(sl);
        cflux.push_back(nb);
      }
  s.n_rrb = (int)rrb.size();
  s.n_cflux = (int)cflux.size() / 2;
  CK(dalloc(&s.d_rrb, rrb.size()));
  CK(dalloc(&s.d_cflux, cflux.size()));
  if (!rrb.empty()) CK(cudaMemcpy(s.d_rrb, rrb.data(), sizeof(int) * rrb.size(), cudaMemcpyHostToDevice));
  if (!cflux.empty()) CK(cudaMemcpy(s.d_cflux, cflux.data(), sizeof(int) * cflux.size(), cudaMemcpyHostToDevice));
  // dynamic shared memory of the flux kernel (set outside graph capture)
  {
    const int nc = ctx->nc, m = nc + 4;
    const int tile = D == 2 ? m * m : m * m * m;
    const int nfaces = D == 2 ? nc * (nc + 1) : nc * nc * (nc + 1);
    const size_t smem = sizeof(double) * ((size_t)t.n_flux * tile + 2 * (size_t)D * nfaces);
    if (smem > 200 * 1024) return fail(ctx, AFG_ERR_UNSUPPORTED, "box too large for the flux kernel");
    const size_t smem32 = flux32_smem(ctx, t.n_flux);
    const cudaFuncAttribute ms = cudaFuncAttributeMaxDynamicSharedMemorySize;
    CK(cudaFuncSetAttribute(k_flux<3, false, 0>, ms, (int)smem));
    CK(cudaFuncSetAttribute(k_flux<3, false, 8>, ms, (int)smem));
    CK(cudaFuncSetAttribute(k_flux<2, true, 0>, ms, (int)smem));
    CK(cudaFuncSetAttribute(k_flux<2, true, 16>, ms, (int)smem));
    CK(cudaFuncSetAttribute(k_flux<2, false, 0>, ms, (int)smem));
    CK(cudaFuncSetAttribute(k_flux<2, false, 16>, ms, (int)smem));
    CK(cudaFuncSetAttribute(k_flux32<3, false, 0>, ms, (int)smem32));
    CK(cudaFuncSetAttribute(k_flux32<3, false, 8>, ms, (int)smem32));
    CK(cudaFuncSetAttribute(k_flux32<2, true, 0>, ms, (int)smem32));
    CK(cudaFuncSetAttribute(k_flux32<2, true, 16>, ms, (int)smem32));
    CK(cudaFuncSetAttribute(k_flux32<2, false, 0>, ms, (int)smem32));
    CK(cudaFuncSetAttribute(k_flux32<2, false, 16>, ms, (int)smem32));
  }
  s.ready = true;
  return AFG_OK;
}

static FluxArgs flux_args(afg_ctx* ctx, int s_deriv) {
  const afg_transport_desc& d = ctx->tr.d;
  FluxArgs a{};
  a.nf = d.n_flux;
  for (int f = 0; f < d.n_flux; f++) {
    a.n[f] = ctx->cc[d.species_iv[d.flux_species[f]] + s_deriv - 1];
    a.flux[f] = ctx->fc[d.flux_fc[f] - 1];
    a.sign[f] = d.flux_charge_sign[f];
    a.mu_ion_N[f] = d.ion_mobility_N[f];
  }
  a.E = ctx->cc[d.i_electric_fld - 1];
  a.Efc = ctx->fc[d.i_efield_fc - 1];
  a.bc = gc_from_desc(d.species_gc);
  a.limiter = d.prolong_limiter;
  a.N_inv = 1 / d.gas_number_density;
  a.lt = lt_dev(ctx);
  a.col_mu = d.lt_col_mobility;
  a.col_dc = d.lt_col_diffusion;
  a.max_cfl = ctx->d_max + 3;
  a.max_sigma = ctx->d_max + 4;
  return a;
}

int afg_flux_upwind(afg_ctx* ctx, int s_deriv, double* dt_lim) {
  RC(need_transport(ctx));
  const afg_transport_desc& d = ctx->tr.d;
  for (int f = 0; f < d.n_flux; f++) {
    const int iv = d.species_iv[d.flux_species[f]] + s_deriv;
    if (iv < 1 || iv > ctx->n_var) return fail(ctx, AFG_ERR_ARG, "bad state s_deriv");
  }
  RC(run_graph(ctx, gkey("flux", s_deriv), [&]() -> int {
    KTree t = ktree(ctx);
    const bool cyl = ctx->coord == AFG_CYL;
    // af_restrict_ref_boundary
    if (ctx->tr.n_rrb > 0) {
      for (int f = 0; f < d.n_flux; f++) {
        double* v = ctx->cc[d.species_iv[d.flux_species[f]] + s_deriv - 1];
        KtScope kts(ctx, AFG_KT_RESTRICT, 8.0 * ctx->tr.n_rrb * t.SI * (1.0 + 1.0 / (1 << ctx->D)));
        if (ctx->D == 3)
          AFG_NC3(NCV_, k_restrict_geom<3, false, NCV_><<<ctx->tr.n_rrb, 64, 0, ctx->stream>>>(t, ctx->tr.d_rrb, v));
        else if (cyl)
          AFG_NC2(NCV_, k_restrict_geom<2, true, NCV_><<<ctx->tr.n_rrb, 64, 0, ctx->stream>>>(t, ctx->tr.d_rrb, v));
        else
          AFG_NC2(NCV_, k_restrict_geom<2, false, NCV_><<<ctx->tr.n_rrb, 64, 0, ctx->stream>>>(t, ctx->tr.d_rrb, v));
        ctx->launches++;
        CKL();
      }
    }
    CK(cudaMemsetAsync(ctx->d_max + 3, 0, 2 * sizeof(unsigned long long), ctx->stream));
    FluxArgs a = flux_args(ctx, s_deriv);
    const int nc = ctx->nc, m = nc + 4;
    const int tile = ctx->D == 2 ? m * m : m * m * m;
    const int nfaces = ctx->D == 2 ? nc * (nc + 1) : nc * nc * (nc + 1);
    const size_t smem = sizeof(double) * ((size_t)d.n_flux * tile + 2 * (size_t)ctx->D * nfaces);
    if (smem > 200 * 1024) return fail(ctx, AFG_ERR_UNSUPPORTED, "box too large for the flux kernel");
    // leaves level by level: refinement-boundary ghosts read the coarse
    // neighbour's ghost layer written by the previous level
    for (int l = 0; l < ctx->highest_lvl; l++) {
      const int n = (int)ctx->lvl_leaves[l].size();
      if (n == 0) continue;
      const int* list = lst(ctx, ctx->off_leaves[l]);
      kt_begin(ctx, AFG_KT_FLUX);
      if (mixed_transport(ctx)) {
        FluxArgs32 a32{};
        a32.a = a;
        a32.lt = lt_dev_f(ctx);
        a32.N_inv_td = (float)(kSiToTd / d.gas_number_density);
        a32.N_inv = (float)(1 / d.gas_number_density);
        for (int f = 0; f < d.n_flux; f++) {
          a32.sign[f] = (float)d.flux_charge_sign[f];
          a32.mu_ion[f] = (float)(d.ion_mobility_N[f] / d.gas_number_density);
        }
        const size_t smem32 = flux32_smem(ctx, d.n_flux);
        const bool staged = ctx->flux_staged && d.n_flux <= 2 &&
                            ((ctx->D == 3 && ctx->nc == 8) || (ctx->D == 2 && ctx->nc == 16));
        if (staged) {
          // the box's |E| and species staged by bulk copies (k_flux32s)
          const size_t sm = flux32s_smem(ctx, d.n_flux);
const int* rl = rec_of(ctx, list);
          if (ctx->D == 3 && d.n_flux == 1)
            k_flux32s<3, false, 8, 1><<<n, 256, sm, ctx->stream>>>(t, rl, a32, ctx->d_err);
          else if (ctx->D == 3)
            k_flux32s<3, false, 8, 2><<<n, 256, sm, ctx->stream>>>(t, rl, a32, ctx->d_err);
          else if (cyl && d.n_flux == 1)
            k_flux32s<2, true, 16, 1><<<n, 256, sm, ctx->stream>>>(t, rl, a32, ctx->d_err);
          else if (cyl)
            k_flux32s<2, true, 16, 2><<<n, 256, sm, ctx->stream>>>(t, rl, a32, ctx->d_err);
          else if (d.n_flux == 1)
            k_flux32s<2, false, 16, 1><<<n, 256, sm, ctx->stream>>>(t, rl, a32, ctx->d_err);
          else
            k_flux32s<2, false, 16, 2><<<n, 256, sm, ctx->stream>>>(t, rl, a32, ctx->d_err);
        } else if (ctx->D == 3)
          AFG_NC3(NCV_, k_flux32<3, false, NCV_><<<n, 256, smem32, ctx->stream>>>(t, rec_of(ctx, list), a32));
        else if (cyl)
          AFG_NC2(NCV_, k_flux32<2, true, NCV_><<<n, 256, smem32, ctx->stream>>>(t, rec_of(ctx, list), a32));
        else
          AFG_NC2(NCV_, k_flux32<2, false, NCV_><<<n, 256, smem32, ctx->stream>>>(t, rec_of(ctx, list), a32));
      } else if (ctx->D == 3) {
        AFG_NC3(NCV_, k_flux<3, false, NCV_><<<n, 256, smem, ctx->stream>>>(t, list, a));
      } else if (cyl) {
        AFG_NC2(NCV_, k_flux<2, true, NCV_><<<n, 256, smem, ctx->stream>>>(t, list, a));
      } else {
        AFG_NC2(NCV_, k_flux<2, false, NCV_><<<n, 256, smem, ctx->stream>>>(t, list, a));
      }
      // per leaf cell: read n (flux species), |E|, E on D faces; write D fluxes per species
      kt_end(ctx, AFG_KT_FLUX, 8.0 * n * box_cells(ctx) * ((d.n_flux + 1 + ctx->D) + ctx->D * d.n_flux));
      ctx->launches++;
      CKL();
    }
    if (ctx->tr.n_cflux > 0) {
      KtScope kts(ctx, AFG_KT_FLUX, 0.0);
      if (ctx->D == 3)
        AFG_NC3(NCV_, k_consistent_flux<3, false, NCV_><<<ctx->tr.n_cflux, 128, 0, ctx->stream>>>(t, ctx->tr.d_cflux, d.n_flux, a));
      else if (cyl)
        AFG_NC2(NCV_, k_consistent_flux<2, true, NCV_><<<ctx->tr.n_cflux, 128, 0, ctx->stream>>>(t, ctx->tr.d_cflux, d.n_flux, a));
      else
        AFG_NC2(NCV_, k_consistent_flux<2, false, NCV_><<<ctx->tr.n_cflux, 128, 0, ctx->stream>>>(t, ctx->tr.d_cflux, d.n_flux, a));
      ctx->launches++;
      CKL();
    }
    return AFG_OK;
  }));
  if (dt_lim) {
    double mc, ms;
    RC(read_max(ctx, 3, &mc));
    RC(read_max(ctx, 4, &ms));
    dt_lim[0] = 1 / mc;
    dt_lim[1] = kEps0 / (kElem * std::max(ms, 1e-100));
  }
  return AFG_OK;
}

int afg_update_densities(afg_ctx* ctx, double dt, int s_deriv, int n_prev, const int* s_prev, const double* w_prev,
                         int s_out, int last_step, double* dt_chem) {
  RC(need_transport(ctx));
  const afg_transport_desc& d = ctx->tr.d;
  if (n_prev < 1 || n_prev > 4 || !s_prev || !w_prev) return fail(ctx, AFG_ERR_ARG, "bad previous states");
  UpdateArgs a{};
  a.ns = d.n_species;
  a.nf = d.n_flux;
  auto var = [&](int s, int st) -> double* {
    const int iv = d.species_iv[s] + st;
    return (iv >= 1 && iv <= ctx->n_var) ? ctx->cc[iv - 1] : nullptr;
  };
  for (int s = 0; s < d.n_species; s++) {
    a.out[s] = var(s, s_out);
    a.deriv[s] = var(s, s_deriv);
    if (!a.out[s] || !a.deriv[s]) return fail(ctx, AFG_ERR_ARG, "bad time state");
    for (int m = 0; m < n_prev; m++) {
      a.prev[m][s] = var(s, s_prev[m]);
      if (!a.prev[m][s]) return fail(ctx, AFG_ERR_ARG, "bad previous state");
    }
  }
  for (int m = 0; m < n_prev; m++) a.w_prev[m] = w_prev[m];
  a.n_prev = n_prev;
  for (int f = 0; f < d.n_flux; f++) {
    a.flux_species[f] = d.flux_species[f];
    a.flux[f] = ctx->fc[d.flux_fc[f] - 1];
  }
  a.E = ctx->cc[d.i_electric_fld - 1];
  a.photo = d.i_photo > 0 ? ctx->cc[d.i_photo - 1] : nullptr;
  a.photoi_species = d.photoi_species;
  a.dt = dt;
  a.N_inv = 1 / d.gas_number_density;
  a.lt = lt_dev(ctx);
  a.reactions = ctx->tr.d_reactions;
  a.n_reactions = d.n_reactions;
  a.last_step = last_step;
  a.nmin = d.dt_chemistry_nmin;
  a.limit_loss = d.dt_chemistry_limit_loss;
  a.min_chem = ctx->d_max + 5;
  a.mask = ctx->tr.mask_iv > 0 ? ctx->cc[ctx->tr.mask_iv - 1] : nullptr;
  if (mixed_transport(ctx) && a.mask != nullptr)
    return fail(ctx, AFG_ERR_UNSUPPORTED, "electrode mask in the FP32 transport update");
  const double big = 1e100;
  unsigned long long bits;
  memcpy(&bits, &big, sizeof(bits));
  CK(cudaMemcpyAsync(ctx->d_max + 5, &bits, sizeof(bits), cudaMemcpyHostToDevice, ctx->stream));
  KTree t = ktree(ctx);
  const int n = ctx->n_all_leaves;
  const int* list = lst(ctx, ctx->off_all_leaves);
  ctx->ctr[2] += (long long)n * (long long)box_cells(ctx) * d.n_species;
  if (n > 0) {
    kt_begin(ctx, AFG_KT_UPDATE);
    const bool cyl = ctx->coord == AFG_CYL;
    double wsum = 0;
    for (int m = 0; m < n_prev; m++) wsum += w_prev[m];
    if (mixed_transport(ctx) && std::fabs(wsum - 1.0) <= 1e-12) {
      UpdateArgs32 u{};
      u.a = a;
      u.lt = lt_dev_f(ctx);
      u.reactions = ctx->tr.d_reac32;
      u.N_inv_td = (float)(kSiToTd / d.gas_number_density);
      u.dt = (float)dt;
      for (int m = 0; m < n_prev; m++) u.w_rel[m] = (float)w_prev[m];
      u.nmin = (float)d.dt_chemistry_nmin;
      u.prev_is_deriv = -1;
      for (int m = 0; m < n_prev; m++)
        if (s_prev[m] == s_deriv) u.prev_is_deriv = m;
      const size_t rsm = sizeof(Reac32) * (size_t)d.n_reactions;  // the records in shared memory
      launch_update32(ctx->D, cyl, ctx->nc, d.n_species, n, t, list, u, rsm, ctx->stream);
    } else {
      launch_update64(ctx->D, cyl, ctx->nc, d.n_species, n, t, list, a, ctx->stream);
    }
    // per leaf cell: read the S densities of every distinct state (s_deriv
    // and the previous states; s_deriv counts once when it is one of them),
    // |E|, D*F fluxes and the photoionization source; write S densities
    int n_states_read = n_prev + 1;
    for (int m = 0; m < n_prev; m++)
      if (s_prev[m] == s_deriv) n_states_read = n_prev;
    kt_end(ctx, AFG_KT_UPDATE, 8.0 * n * box_cells(ctx) *
                                   (d.n_species * n_states_read + ctx->D * d.n_flux + 1 + (d.i_photo > 0) + d.n_species));
    ctx->launches++;
    CKL();
  }
  if (dt_chem) {
    if (last_step)
      RC(read_max(ctx, 5, dt_chem));
    else
      *dt_chem = 1e100;
  }
  return AFG_OK;
}

// field_set_rhs; with maxbits the FP32-path kernel also folds max |rhs|
// over the leaves into *maxbits (reset by the caller)
static int field_set_rhs(afg_ctx* ctx, int i_rhs, int s_in, unsigned long long* maxbits);

int afg_field_set_rhs(afg_ctx* ctx, int i_rhs, int s_in) { return field_set_rhs(ctx, i_rhs, s_in, nullptr); }

static int field_set_rhs(afg_ctx* ctx, int i_rhs, int s_in, unsigned long long* maxbits) {
  RC(need_transport(ctx));
  RC(check_var(ctx, i_rhs));
  const afg_transport_desc& d = ctx->tr.d;
  RhsArgs a{};
  a.ns = d.n_species;
  const double fac = -kElem / kEps0;
  for (int s = 0; s < d.n_species; s++) {
    const int iv = d.species_iv[s] + s_in;
    if (iv < 1 || iv > ctx->n_var) return fail(ctx, AFG_ERR_ARG, "bad state s_in");
    a.n[s] = ctx->cc[iv - 1];
    a.q[s] = d.species_charge[s] != 0 ? d.species_charge[s] * fac : 0.0;
  }
  a.rhs = ctx->cc[i_rhs - 1];
  if (ctx->n_all_leaves > 0) {
    const int* list = lst(ctx, ctx->off_all_leaves);
    KtScope kts(ctx, AFG_KT_FIELD, 8.0 * ctx->n_all_leaves * box_cells(ctx) * (d.n_species + 1));
    if (!mixed_transport(ctx)) {
      k_field_rhs<<<ctx->n_all_leaves, 256, 0, ctx->stream>>>(ctx->S, list, a);
    } else {
      // the charged species only, in order (the sums skip the others)
      RhsArgs q{};
      q.rhs = a.rhs;
      for (int s = 0; s < a.ns; s++)
        if (a.q[s] != 0.0) {
          q.n[q.ns] = a.n[s];
          q.q[q.ns] = a.q[s];
          q.ns++;
        }
      const KTree t = ktree(ctx);
      const int nl = ctx->n_all_leaves;
#define AFG_LAUNCH_RHS(NQ)                                                                                   \
  if (ctx->D == 3)                                                                                           \
    AFG_NC3(NCV_, k_field_rhs_interior<3, NQ, NCV_><<<nl, 128, 0, ctx->stream>>>(t, list, q, maxbits));     \
  else                                                                                                       \
    AFG_NC2(NCV_, k_field_rhs_interior<2, NQ, NCV_><<<nl, 64, 0, ctx->stream>>>(t, list, q, maxbits));
      if (q.ns <= 2) {
        AFG_LAUNCH_RHS(2)
      } else if (q.ns <= 4) {
        AFG_LAUNCH_RHS(4)
      } else if (q.ns <= 6) {
        AFG_LAUNCH_RHS(6)
      } else if (q.ns <= 8) {
        AFG_LAUNCH_RHS(8)
      } else {
        AFG_LAUNCH_RHS(16)
      }
#undef AFG_LAUNCH_RHS
    }
    ctx->launches++;
    CKL();
  }
  return AFG_OK;
}

int afg_field_from_potential(afg_ctx* ctx, int i_phi) {
  RC(need_transport(ctx));
  RC(check_var(ctx, i_phi));
  const afg_transport_desc& d = ctx->tr.d;
  KTree t = ktree(ctx);
  double* efc = ctx->fc[d.i_efield_fc - 1];
  double* en = ctx->cc[d.i_electric_fld - 1];
  if (!ctx->has_method[d.i_electric_fld - 1])
    return fail(ctx, AFG_ERR_STATE, "no ghost-cell methods for the electric field norm");
  return run_graph(ctx, gkey("efield", i_phi), [&]() -> int {
    {
    KtScope kts(ctx, AFG_KT_FIELD, 8.0 * ctx->n_all * box_cells(ctx) * (2.0 + ctx->D));
    if (mixed_transport(ctx)) {
      const int D = ctx->D;
      const size_t smem = sizeof(float) * D * (size_t)ctx->NF;
      if (D == 3)
        AFG_NC3(NCV_, k_field_grad32<3, NCV_><<<ctx->n_all, 256, smem, ctx->stream>>>(t, lst(ctx, ctx->off_all), ctx->cc[i_phi - 1],
                                                                   efc, en));
      else
        AFG_NC2(NCV_, k_field_grad32<2, NCV_><<<ctx->n_all, 256, smem, ctx->stream>>>(t, lst(ctx, ctx->off_all), ctx->cc[i_phi - 1],
                                                                   efc, en));
    } else if (ctx->D == 3)
      AFG_NC3(NCV_, k_field_grad<3, NCV_><<<ctx->n_all, 256, 0, ctx->stream>>>(t, lst(ctx, ctx->off_all), ctx->cc[i_phi - 1], efc, en));
    else
      AFG_NC2(NCV_, k_field_grad<2, NCV_><<<ctx->n_all, 256, 0, ctx->stream>>>(t, lst(ctx, ctx->off_all), ctx->cc[i_phi - 1], efc, en));
    ctx->launches++;
    CKL();
    // faces next to the electrode surface on electrode leaf boxes
    if (const MgSlot* ms = lsf_slot_of(ctx, i_phi)) {
      if (mixed_transport(ctx)) return fail(ctx, AFG_ERR_UNSUPPORTED, "electrode field in an FP32 transport model");
      RC(launch_lsf_grad(ctx, *ms, ctx->cc[i_phi - 1], efc, en));
    }
    }
    return afg_gc(ctx, d.i_electric_fld, 0, 1);
  });
}

int afg_field_compute_inst(afg_ctx* ctx, int mg_id, int s_in, int have_guess, const double* voltage,
                           double domain_len, double max_rel_residual, int num_vcycles, int* n_cycles,
                           double* residual) {
  RC(need_transport(ctx));
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (ctx->n_inst <= 0) return fail(ctx, AFG_ERR_STATE, "not a batched tree");
  if (!voltage) return fail(ctx, AFG_ERR_ARG, "voltage per instance needed");
  const int Q = ctx->n_inst;
  double mx;
  if (mixed_transport(ctx)) {
    RC(reset_max(ctx, 0));
    RC(field_set_rhs(ctx, m->d.i_rhs, s_in, ctx->d_max));
    RC(read_max(ctx, 0, &mx));
  } else {
    RC(field_set_rhs(ctx, m->d.i_rhs, s_in, nullptr));
    RC(afg_maxabs(ctx, m->d.i_rhs, 1, &mx));
  }
  // field_bc_homogeneous per instance, and the threshold of each instance
  // (the rule of the single-tree path with its own rhs maximum, voltage and
  // finest dr)
  std::vector<double> bcv((size_t)Q * 6), thr(Q), r(Q, 0.0);
  std::vector<int> cyc(Q, 0);
  for (int q = 0; q < Q; q++) {
    for (int k = 0; k < 6; k++) bcv[(size_t)q * 6 + k] = m->d.bc_val[k];
    bcv[(size_t)q * 6 + 2 * ctx->D - 1] = voltage[q];
    const double max_rhs = inst_value(ctx, 0, q);
    thr[q] = std::max(std::max(1e-6, max_rhs * max_rel_residual),
                      1e-10 * std::fabs(voltage[q]) / (domain_len * ctx->inst_min_dr[q]));
  }
  RC(afg_mg_set_bc_values_inst(ctx, mg_id, bcv.data()));
  if (!have_guess) {
    const bool fp32_fmg = m->d.precision == AFG_MIXED;
    std::vector<char> done(Q, 0);
    std::vector<std::vector<double>> hist(Q);
    bool all = false;
    for (int i = 0; i < 100 && !all; i++) {
      RC(set_frozen(ctx, done));
      RC(afg_mg_fmg(ctx, mg_id, 1, 1, &mx));
      all = true;
      for (int q = 0; q < Q; q++) {
        if (done[q]) continue;
        const double v = inst_value(ctx, 1, q);
        hist[q].push_back(v);
        cyc[q]++;
        r[q] = v;
        if (v < thr[q]) {
          done[q] = 1;
        } else if (hist[q].size() >= 3) {
          const size_t k = hist[q].size();
          const double mn = std::min(v, std::min(hist[q][k - 2], hist[q][k - 3]));
          const double mxh = std::max(v, std::max(hist[q][k - 2], hist[q][k - 3]));
          const double ratio = mn / mxh;
          if (ratio < 2.0 && ratio > 0.5 && (v < 1e8 || fp32_fmg)) done[q] = 1;
        }
        all = all && done[q];
      }
    }
    std::fill(done.begin(), done.end(), 0);
    RC(set_frozen(ctx, done));
    if (!all) return fail(ctx, AFG_ERR_NOCONV, "no convergence in initial field computation");
  }
  if (num_vcycles > 0) {
    std::vector<int> nv(Q);
    std::vector<double> rv(Q);
    const int rc = mg_solve_inst(ctx, *m, thr.data(), std::min(num_vcycles, 256), nv.data(), rv.data());
    if (rc != AFG_OK && rc != AFG_ERR_NOCONV) return rc;
    for (int q = 0; q < Q; q++) {
      cyc[q] += nv[q];
      if (nv[q] > 0) r[q] = rv[q];
    }
  }
  RC(afg_field_from_potential(ctx, m->d.i_phi));
  for (int q = 0; q < Q; q++) {
    if (n_cycles) n_cycles[q] = cyc[q];
    if (residual) residual[q] = r[q];
  }
  return AFG_OK;
}

int afg_field_compute(afg_ctx* ctx, int mg_id, int s_in, int have_guess, double voltage, double domain_len,
                      double max_rel_residual, int num_vcycles, int* n_cycles, double* residual) {
  RC(need_transport(ctx));
  MgSlot* m;
  RC(get_mg(ctx, mg_id, &m));
  if (ctx->n_inst > 0) {
    // one voltage for all instances; the most cycles and largest residual
    std::vector<double> v(ctx->n_inst, voltage), res(ctx->n_inst);
    std::vector<int> nc(ctx->n_inst);
    RC(afg_field_compute_inst(ctx, mg_id, s_in, have_guess, v.data(), domain_len, max_rel_residual, num_vcycles,
                              nc.data(), res.data()));
    if (n_cycles) *n_cycles = *std::max_element(nc.begin(), nc.end());
    if (residual) *residual = *std::max_element(res.begin(), res.end());
    return AFG_OK;
  }
  double max_rhs;
  if (mixed_transport(ctx)) {
    RC(reset_max(ctx, 0));
    RC(field_set_rhs(ctx, m->d.i_rhs, s_in, ctx->d_max));
  } else {
    RC(field_set_rhs(ctx, m->d.i_rhs, s_in, nullptr));
  }
  // field_bc_homogeneous: Dirichlet `voltage` on the high face of the last dimension
  double bcv[6];
  for (int q = 0; q < 6; q++) bcv[q] = m->d.bc_val[q];
  bcv[2 * ctx->D - 1] = voltage;
  RC(afg_mg_set_bc_values(ctx, mg_id, bcv));
  if (mixed_transport(ctx))
    RC(read_max(ctx, 0, &max_rhs));
  else
    RC(afg_maxabs(ctx, m->d.i_rhs, 1, &max_rhs));
  // af_min_dr: finest dr of the highest level
  std::vector<double> hdr(ctx->D);
  const int s_fine = ctx->lvl_ids[ctx->highest_lvl - 1][0];
  CK(cudaMemcpy(hdr.data(), ctx->d_dr + (size_t)s_fine * ctx->D, sizeof(double) * ctx->D, cudaMemcpyDeviceToHost));
  double min_dr = hdr[0];
  for (int q = 1; q < ctx->D; q++) min_dr = std::min(min_dr, hdr[q]);
  // with an electrode the round-off estimate is less strict (conv_fac
  // 1e-8, m_field.f90:468-473) and the electrode gets the voltage or 0
  // (mg%lsf_boundary_value, 482-487)
  const double conv_fac = m->lsf ? 1e-8 : 1e-10;
  if (m->lsf) RC(lsf_set_voltage(ctx, *m, voltage));
  const double threshold =
      std::max(std::max(1e-6, max_rhs * max_rel_residual), conv_fac * std::fabs(voltage) / (domain_len * min_dr));
  int nc_done = 0;
  double r = 0;
  // A mixed-precision slot runs FMG in FP32, whose residual floor on fine
  // meshes can exceed the 1e8 guard of the stall test; there the FMG only
  // starts the FP64 defect correction below, so a stall ends it at any level.
  const bool fp32_fmg = m->d.precision == AFG_MIXED;
  if (!have_guess) {
    double res[100];
    int i;
    for (i = 0; i < 100; i++) {
      RC(afg_mg_fmg(ctx, mg_id, 1, 1, &res[i]));
      nc_done++;
      if (res[i] < threshold) break;
      if (i >= 2) {
        const double mn = std::min(res[i], std::min(res[i - 1], res[i - 2]));
        const double mx = std::max(res[i], std::max(res[i - 1], res[i - 2]));
        const double ratio = mn / mx;
        if (ratio < 2.0 && ratio > 0.5 && (res[i] < 1e8 || fp32_fmg)) break;
      }
    }
    if (i == 100) return fail(ctx, AFG_ERR_NOCONV, "no convergence in initial field computation");
    r = res[std::min(i, 99)];
  }
  int nv = 0;
  if (num_vcycles > 0) {
    double hist[256];
    const int rc = afg_mg_solve(ctx, mg_id, threshold, std::min(num_vcycles, 256), &nv, hist);
    if (rc != AFG_OK && rc != AFG_ERR_NOCONV) return rc;
    if (nv > 0) r = hist[nv - 1];
  }
  nc_done += nv;
  RC(afg_field_from_potential(ctx, m->d.i_phi));
  if (n_cycles) *n_cycles = nc_done;
  if (residual) *residual = r;
  return AFG_OK;
}

int afg_set_flux_staged(afg_ctx* ctx, int on) {
  if (!ctx) return AFG_ERR_ARG;
  if (ctx->flux_staged != (on != 0)) clear_graphs(ctx);
  ctx->flux_staged = on != 0;
  return AFG_OK;
}

int afg_stage_setup(afg_ctx* ctx, const afg_stage_desc* d) {
  if (!d) return fail(ctx, AFG_ERR_ARG, "null stage descriptor");
  MgSlot* m;
  RC(get_mg(ctx, d->mg_id, &m));
  if (d->num_vcycles < 0 || !(d->domain_len > 0) || !(d->dt_max > 0) || !(d->dt_cfl_number > 0))
    return fail(ctx, AFG_ERR_ARG, "bad stage settings");
  ctx->stage = *d;
  return AFG_OK;
}

// forward_euler (src/m_fluid.f90:21-99); the limits combine as at lines
// 96-98, the chemistry limit counting on the last step only (add_source_terms
// computes it there, 402-418)
int afg_forward_euler(afg_ctx* ctx, double dt, double voltage, int s_deriv, int n_prev, const int* s_prev,
                      const double* w_prev, int s_out, int i_step, int n_steps, double* dt_lim, int* n_cycles) {
  const afg_stage_desc& sd = ctx->stage;
  if (sd.mg_id < 0) return fail(ctx, AFG_ERR_ARG, "afg_stage_setup not called");
  if (i_step < 1 || i_step > n_steps) return fail(ctx, AFG_ERR_ARG, "bad integrator step");
  int nc = 0;
  if (i_step > 1) {
    double res;
    RC(afg_field_compute(ctx, sd.mg_id, s_deriv, 1, voltage, sd.domain_len, sd.max_rel_residual, sd.num_vcycles,
                         &nc, &res));
  }
  double fl[2];
  RC(afg_flux_upwind(ctx, s_deriv, fl));
  const bool last = i_step == n_steps;
  double chem = 1e100;
  RC(afg_update_densities(ctx, dt, s_deriv, n_prev, s_prev, w_prev, s_out, last ? 1 : 0, &chem));
  if (!last) chem = 1e100;
  if (dt_lim) *dt_lim = std::min(sd.dt_max, std::min(std::min(fl[0] * sd.dt_cfl_number, fl[1]), std::min(chem, 1e100)));
  if (n_cycles) *n_cycles = nc;
  return AFG_OK;
}

int afg_photoi_helmh(afg_ctx* ctx, double coeff, int n_modes, const int* mg_ids, const double* coeffs,
                     double max_rel_residual, int max_fmg_cycles) {
  RC(need_transport(ctx));
  const afg_transport_desc& d = ctx->tr.d;
  if (n_modes < 1 || !mg_ids || !coeffs || d.i_photo <= 0) return fail(ctx, AFG_ERR_ARG, "bad photoionization args");
  if (ctx->n_inst > 0) return fail(ctx, AFG_ERR_UNSUPPORTED, "photoionization of batched instances");
  MgSlot* m0;
  RC(get_mg(ctx, mg_ids[0], &m0));
  const int i_rhs = m0->d.i_rhs;
  KTree t = ktree(ctx);
  // photon production on leaves
  if (ctx->n_all_leaves > 0) {
    const double* E = ctx->cc[d.i_electric_fld - 1];
    const double* ne = ctx->cc[d.species_iv[d.flux_species[0]] - 1];
    double* rhs = ctx->cc[i_rhs - 1];
    KtScope kts(ctx, AFG_KT_FIELD, 24.0 * ctx->n_all_leaves * box_cells(ctx));
    if (mixed_transport(ctx)) {
      const float N_inv_td = (float)(kSiToTd / d.gas_number_density);
      const double ch = std::sqrt(std::fabs(coeff));
      const float c_hi = (float)(coeff < 0 ? -ch : ch), c_lo = (float)ch;
      if (ctx->D == 3)
        AFG_NC3(NCV_, k_photo_source32<3, NCV_><<<ctx->n_all_leaves, 256, 0, ctx->stream>>>(t, lst(ctx, ctx->off_all_leaves), E, ne, rhs,
                                                                        lt_dev_f(ctx), d.lt_col_alpha,
                                                                        d.lt_col_mobility, N_inv_td, c_hi, c_lo));
      else
        AFG_NC2(NCV_, k_photo_source32<2, NCV_><<<ctx->n_all_leaves, 256, 0, ctx->stream>>>(t, lst(ctx, ctx->off_all_leaves), E, ne, rhs,
                                                                        lt_dev_f(ctx), d.lt_col_alpha,
                                                                        d.lt_col_mobility, N_inv_td, c_hi, c_lo));
    } else if (ctx->D == 3)
      AFG_NC3(NCV_, k_photo_source<3, NCV_><<<ctx->n_all_leaves, 256, 0, ctx->stream>>>(t, lst(ctx, ctx->off_all_leaves), E, ne, rhs,
                                                                  lt_dev(ctx), d.lt_col_alpha, d.lt_col_mobility,
                                                                  d.gas_number_density, coeff));
    else
      AFG_NC2(NCV_, k_photo_source<2, NCV_><<<ctx->n_all_leaves, 256, 0, ctx->stream>>>(t, lst(ctx, ctx->off_all_leaves), E, ne, rhs,
                                                                  lt_dev(ctx), d.lt_col_alpha, d.lt_col_mobility,
                                                                  d.gas_number_density, coeff));
    ctx->launches++;
    CKL();
  }
  // photoi_helmh_compute
  double* photo = ctx->cc[d.i_photo - 1];
  CK(cudaMemsetAsync(photo, 0, sizeof(double) * (size_t)ctx->n_boxes * ctx->S, ctx->stream));
  double max_rhs;
  RC(afg_maxabs(ctx, i_rhs, 1, &max_rhs));
  max_rhs = std::max(max_rhs, std::sqrt(2.220446049250313e-16));
  bool all_mixed = n_modes <= kMaxBranch && n_modes <= kMaxSlots - kModeSlot;
  for (int n = 0; n < n_modes; n++) {
    MgSlot* m;
    RC(get_mg(ctx, mg_ids[n], &m));
    if (m->d.i_rhs != i_rhs) return fail(ctx, AFG_ERR_ARG, "Helmholtz modes must share i_rhs");
    if (m->d.precision != AFG_MIXED) all_mixed = false;
    for (int q = 0; q < n; q++)
      if (mg_ids[q] == mg_ids[n]) all_mixed = false;
  }
  // Lockstep (multiple right-hand sides in one sweep): modes with the same
  // boundary conditions and cycle counts run every launch of their
  // defect-correction FMG together, blockIdx.y selecting the mode; converged
  // modes leave the set, as in the per-mode loop.  Each mode's arithmetic is
  // the same as alone, so the results are too.
  bool lockstep = all_mixed && ctx->photoi_lockstep && ctx->fused_gsrb && n_modes <= kMaxModes;
  for (int n = 1; lockstep && n < n_modes; n++) {
    const afg_mg_desc &a = ctx->mg[mg_ids[0]].d, &b = ctx->mg[mg_ids[n]].d;
    lockstep = a.n_cycle_down == b.n_cycle_down && a.n_cycle_up == b.n_cycle_up;
    for (int q = 0; q < 6; q++) lockstep = lockstep && a.bc_type[q] == b.bc_type[q] && a.bc_val[q] == b.bc_val[q];
  }
  if (lockstep) {
    std::vector<int> active(n_modes);
    for (int n = 0; n < n_modes; n++) active[n] = n;
    for (int it = 0; it < max_fmg_cycles && !active.empty(); it++) {
      int mask = 0;
      for (int n : active) mask |= 1 << n;
      ModeArg<double> phi, rhs;
      ModeArg<unsigned long long> mx;
      for (size_t q = 0; q < active.size(); q++) {
        MgSlot* m = &ctx->mg[mg_ids[active[q]]];
        ctx->grp[q] = m;
        phi.p[q] = ctx->cc[m->d.i_phi - 1];
        rhs.p[q] = ctx->cc[m->d.i_rhs - 1];
        mx.p[q] = ctx->d_max + kModeSlot + active[q];
      }
      ctx->ky = (int)active.size();
      const int rc = run_graph(ctx, gkey("photoi_lockstep", mask, mg_ids[0], n_modes), [&]() -> int {
        for (int n : active) RC(reset_max(ctx, kModeSlot + n));
        return mixed_fmg(ctx, *ctx->grp[0], phi, rhs, true, true, mx);
      });
      ctx->ky = 1;
      for (auto& g : ctx->grp) g = nullptr;
      RC(rc);
      CK(cudaMemcpyAsync(ctx->h_max + kModeSlot, ctx->d_max + kModeSlot, sizeof(unsigned long long) * n_modes,
                         cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
      std::vector<int> still;
      for (int n : active) {
        double res;
        memcpy(&res, ctx->h_max + kModeSlot + n, sizeof(double));
        if (!(res / max_rhs < max_rel_residual)) still.push_back(n);
      }
      active.swap(still);
    }
  } else if (all_mixed) {
    // Mixed-precision modes own all the buffers they write (phi_n, the FP32
    // correction, right-hand side and tmp, the coarse-solve vectors) and only
    // read the shared source, so their FMG cycles run as parallel branches
    // (side streams forked from and joined to the context's stream, one
    // graph per set of unconverged modes).  Each mode still gets FMG cycles
    // until its own residual criterion holds, as in the sequential loop, so
    // the results are the same.
    std::vector<int> active(n_modes);
    for (int n = 0; n < n_modes; n++) active[n] = n;
    for (int it = 0; it < max_fmg_cycles && !active.empty(); it++) {
      int mask = 0;
      for (int n : active) mask |= 1 << n;
      RC(run_graph(ctx, gkey("photoi_fmg", mask, mg_ids[0], n_modes), [&]() -> int {
        cudaStream_t main = ctx->stream;
        CK(cudaEventRecord(ctx->ev_fork, main));
        for (size_t q = 0; q < active.size(); q++) {
          const int n = active[q];
          MgSlot* m = &ctx->mg[mg_ids[n]];
          CK(cudaStreamWaitEvent(ctx->side[q], ctx->ev_fork, 0));
          ctx->stream = ctx->side[q];
          int rc = reset_max(ctx, kModeSlot + n);
          if (rc == AFG_OK)
            rc = mixed_fmg(ctx, *m, ctx->cc[m->d.i_phi - 1], ctx->cc[m->d.i_rhs - 1], true, true,
                           ctx->d_max + kModeSlot + n);
          ctx->stream = main;
          RC(rc);
          CK(cudaEventRecord(ctx->ev_join[q], ctx->side[q]));
          CK(cudaStreamWaitEvent(main, ctx->ev_join[q], 0));
        }
        return AFG_OK;
      }));
      CK(cudaMemcpyAsync(ctx->h_max + kModeSlot, ctx->d_max + kModeSlot, sizeof(unsigned long long) * n_modes,
                         cudaMemcpyDeviceToHost, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
      std::vector<int> still;
      for (int n : active) {
        double res;
        memcpy(&res, ctx->h_max + kModeSlot + n, sizeof(double));
        if (!(res / max_rhs < max_rel_residual)) still.push_back(n);
      }
      active.swap(still);
    }
  }
  for (int n = 0; n < n_modes; n++) {
    MgSlot* m;
    RC(get_mg(ctx, mg_ids[n], &m));
    for (int i = 0; !all_mixed && i < max_fmg_cycles; i++) {
      double res;
      RC(afg_mg_fmg(ctx, mg_ids[n], 1, 1, &res));
      if (res / max_rhs < max_rel_residual) break;
    }
    if (ctx->n_all_leaves > 0) {
      KtScope kts(ctx, AFG_KT_FIELD, 24.0 * ctx->n_all_leaves * box_cells(ctx));
      k_axpy_boxes<<<ctx->n_all_leaves, 256, 0, ctx->stream>>>(ctx->S, lst(ctx, ctx->off_all_leaves), photo,
                                                              ctx->cc[m->d.i_phi - 1], coeffs[n]);
      ctx->launches++;
      CKL();
    }
  }
  return AFG_OK;
}

}  // extern "C"
