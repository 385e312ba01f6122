// afg_mixed.cuh -- mixed-precision multigrid solve: an FP64 defect-correction
// (iterative refinement) loop around the FP32 FAS V-cycle.
//
//   r = rhs - L(phi)            FP64, all boxes; max |r| over leaves
//   L e = r, e = 0 initially    one FP32 V-cycle, homogeneous boundary values
//   phi = phi + e               FP64, interior and ghost cells
//
// L is affine in phi (boundary and refinement-boundary ghost rules are
// linear), so e's ghost cells, filled by the same rules with zero boundary
// values, are the ghost-cell correction of phi.  The coarsest-level solve
// stays FP64 (the dense inverse), as do phi, rhs and the residual.
// Included by afg_runtime.cu.
#pragma once

namespace afg {

// r (FP64 residual on interior cells) -> r32, e32 = 0 (whole box), max |r|
// over leaves into *maxbits.  Leaves only (the V-cycle's restriction
// overwrites the parents' right-hand side).  Each block first fills its own
// box's face ghosts of phi (face_ghost_nb: same-level copies, boundary and
// refinement rules; boxes flagged as refinement sources were filled before
// the launch and are left alone, since finer boxes' rules read them), then
// applies the stencil to the stored values.  The Cartesian stencil is one
// FMA chain from f with negated coefficients (7 FP64 instructions per cell
// in 3D); r is rounded to FP32 by bit
// truncation and its maximum taken in FP32.  RB: the FP32 buffers have the
// compact red-black layout (afg_mg32.cuh); e's ghost block is cleared only on
// parents and refinement sources, the boxes whose ghost cells the FP32
// V-cycle reads before writing them.
template <int D, bool CYL, int NC = 0, bool RB = false>
__global__ void __launch_bounds__(256) k_defect(KTree t0, const int* __restrict__ rec, ModeArg<double> phi_,
                                                ModeArg<const double> rhs_, ModeArg<float> r32_,
                                                ModeArg<float> e32_, ModeCoef<double> mc_, GcDev g,
                                                const unsigned char* __restrict__ is_leaf,
                                                ModeArg<unsigned long long> maxbits_) {
  const KTree t = fix_dims<D, NC>(t0);
  double* __restrict__ phi = phi_.get();
  const double* __restrict__ rhs = rhs_.get();
  float* __restrict__ r32 = r32_.get();
  float* __restrict__ e32 = e32_.get();
  const MgCoef<double> mc = mc_.get();
  unsigned long long* maxbits = maxbits_.get();
  __shared__ float sred[32];
  int4 r0, r1;
  load_rec(rec, blockIdx.x, r0, r1);
  const int slot = r0.x;
  if (box_frozen(t, slot)) return;
  const int nc = t.nc, n2 = t.n2;
  const bool leaf = is_leaf[slot] != 0;
  if (RB) {
    float* ei = e32 + (size_t)slot * t.SI;
    for (int x = threadIdx.x; x < t.SI; x += blockDim.x) ei[x] = 0.0f;
    if (!leaf || r1.w != 0) {
      float* eg = e32 + (size_t)t.nbox * t.SI + (size_t)slot * t.S;
      for (int x = threadIdx.x; x < t.S; x += blockDim.x) eg[x] = 0.0f;
    }
  } else {
    float* eo = e32 + (size_t)slot * t.S;
    for (int x = threadIdx.x; x < t.S; x += blockDim.x) eo[x] = 0.0f;
  }
  // parents need no defect: the V-cycle's restriction overwrites their rhs
  if (!leaf) return;
  double* pw_ = phi + (size_t)slot * t.S;
  if (r1.w == 0) {
    const int nface = D == 2 ? nc : nc * nc;
    for (int w = threadIdx.x; w < 2 * D * nface; w += blockDim.x) {
      const int nb = w / nface, pq = w - nb * nface;
      const int pi = pq % nc + 1, qi = D == 3 ? pq / nc + 1 : 0;
      const double val = face_ghost_nb<D, double>(t, phi, slot, nb, rec_nb(r0, r1, nb), pi, qi, g);
      pw_[face_at<D>(n2, nb >> 1, (nb & 1) ? nc + 1 : 0, pi, qi)] = val;
    }
  }
  __syncthreads();
  // negated coefficients: r = f - sum c_q p_q as one chain of 2D+1 FMAs
  // starting from f (one FP64 instruction fewer than summing L(phi) first)
  double cd[7];
  for (int q = 0; q < 7; q++) cd[q] = -mc.cb[slot * 8 + q];
  const double* p = pw_;
  const double* f = rhs + (size_t)slot * t.S;
  float* ro = r32 + (size_t)slot * (RB ? t.SI : t.S);
  float mx = 0.0f;
  const int ncell = D == 2 ? nc * nc : nc * nc * nc;
  for (int w = threadIdx.x; w < ncell; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 0 : r / nc + 1;
    double rd;
    int x;
    if (D == 2) {
      x = at2(n2, i, j);
      if (CYL) {
        const double* y = mc.cy + ((size_t)slot * nc + (i - 1)) * 4;
        rd = fma(cd[4], p[x + n2],
                 fma(cd[3], p[x - n2], fma(-y[2], p[x + 1], fma(-y[1], p[x - 1], fma(-y[0], p[x], f[x])))));
      } else {
        rd = fma(cd[4], p[x + n2],
                 fma(cd[3], p[x - n2], fma(cd[2], p[x + 1], fma(cd[1], p[x - 1], fma(cd[0], p[x], f[x])))));
      }
    } else {
      x = at3(n2, i, j, k);
      const int sk = n2 * n2;
      rd = fma(cd[6], p[x + sk],
               fma(cd[5], p[x - sk],
                   fma(cd[4], p[x + n2],
                       fma(cd[3], p[x - n2], fma(cd[2], p[x + 1], fma(cd[1], p[x - 1], fma(cd[0], p[x], f[x])))))));
    }
    const float res = d2f(rd);
    ro[RB ? rb_idx<D>(nc, i, j, k) : x] = res;
    acc_absmax(mx, res);
  }
  mx = block_max<float>(mx, sred);
  if (threadIdx.x == 0) atomic_max_nonneg(inst_max(t, maxbits, slot), f2d(mx));
}

// Whole-box conversions between the FP64 variables and the FP32 buffers
__global__ void __launch_bounds__(256) k_to_f32(int S, const int* __restrict__ list, const double* __restrict__ src,
                                                float* __restrict__ dst) {
  const size_t base = (size_t)list[blockIdx.x] * S;
  for (int x = threadIdx.x; x < S; x += blockDim.x) dst[base + x] = d2f(src[base + x]);
}
__global__ void __launch_bounds__(256) k_to_f64(int S, const int* __restrict__ list, const float* __restrict__ src,
                                                double* __restrict__ dst) {
  const size_t base = (size_t)list[blockIdx.x] * S;
  for (int x = threadIdx.x; x < S; x += blockDim.x) dst[base + x] = f2d(src[base + x]);
}

// phi += e on whole boxes (ghost cells included)
__global__ void __launch_bounds__(256) k_add_correction(KTree t, const int* __restrict__ list, ModeArg<double> phi_,
                                                        ModeArg<const float> e32_) {
  double* __restrict__ phi = phi_.get();
  const float* __restrict__ e32 = e32_.get();
  const int slot = list[blockIdx.x];
  if (box_frozen(t, slot)) return;
  const int S = t.S;
  double* p = phi + (size_t)slot * S;
  const float* e = e32 + (size_t)slot * S;
  for (int x = threadIdx.x; x < S; x += blockDim.x) p[x] = p[x] + f2d(e[x]);
}

// phi += e on the interior cells, e in the compact layout.  The boxes are
// leaves; their ghost cells of phi are filled again before anything reads
// them (mixed_prepare and the defect's own face ghosts, mixed_finish).
template <int D, int NC = 0>
__global__ void __launch_bounds__(256) k_add_correction_rb(KTree t0, const int* __restrict__ list,
                                                           ModeArg<double> phi_, ModeArg<const float> e32_) {
  const KTree t = fix_dims<D, NC>(t0);
  double* __restrict__ phi = phi_.get();
  const float* __restrict__ e32 = e32_.get();
  const int slot = list[blockIdx.x];
  if (box_frozen(t, slot)) return;
  const int nc = t.nc, n2 = t.n2;
  double* p = phi + (size_t)slot * t.S;
  const float* e = e32 + (size_t)slot * t.SI;
  for (int w = threadIdx.x; w < t.SI; w += blockDim.x) {
    const int i = w % nc + 1, r = w / nc;
    const int j = D == 2 ? r + 1 : r % nc + 1, k = D == 2 ? 0 : r / nc + 1;
    const int x = D == 2 ? at2(n2, i, j) : at3(n2, i, j, k);
    p[x] = p[x] + f2d(e[rb_idx<D>(nc, i, j, k)]);
  }
}

}  // namespace afg

// phi += e on the boxes of a list (leaves), every lockstep slot
static int launch_add_correction(afg_ctx* ctx, const int* list, int n, ModeArg<double> phi, ModeArg<const float> e) {
  if (n <= 0) return AFG_OK;
  KtScope kts(ctx, AFG_KT_CORRECT, 20.0 * n * ctx->ky * ktree(ctx).SI);
  const dim3 grid(n, ctx->ky);
  const KTree t = ktree(ctx);
  if (!ctx->rb32)
    k_add_correction<<<grid, 256, 0, ctx->stream>>>(t, list, phi, e);
  else if (ctx->D == 3)
    AFG_NC3(NCV_, k_add_correction_rb<3, NCV_><<<grid, 256, 0, ctx->stream>>>(t, list, phi, e));
  else
    AFG_NC2(NCV_, k_add_correction_rb<2, NCV_><<<grid, 256, 0, ctx->stream>>>(t, list, phi, e));
  ctx->launches++;
  CKL();
  return AFG_OK;
}

// All boxes: the correction starts at zero everywhere (an FMG from zero
// prolongs the change of the level-1 correction, so it must start at zero
// there too); the defect itself is computed on leaves.
static int launch_defect(afg_ctx* ctx, MgSlot& m, ModeArg<double> phi, ModeArg<const double> rhs,
                         ModeArg<unsigned long long> maxbits) {
  const int n = ctx->n_all;
  if (n <= 0) return AFG_OK;
  KtScope kts(ctx, AFG_KT_DEFECT, 24.0 * ctx->n_all_leaves * ctx->ky * ktree(ctx).SI);
  KTree t = ktree(ctx);
  const int* list = rec_of(ctx, lst(ctx, ctx->off_all));
  const GcDev g = mg_gc(ctx, m, false);
  const ModeArg<float> r32 = slot_bufs(ctx, m, &MgSlot::r32), e32 = slot_bufs(ctx, m, &MgSlot::e32);
  const ModeCoef<double> c = coefs<double>(ctx, m);
  const dim3 grid(n, ctx->ky);
  if (ctx->rb32) {
    if (ctx->D == 3)
      AFG_NC3(NCV_, k_defect<3, false, NCV_, true><<<grid, 256, 0, ctx->stream>>>(t, list, phi, rhs, r32, e32, c, g,
                                                                                 ctx->d_is_leaf, maxbits));
    else if (ctx->coord == AFG_CYL)
      AFG_NC2(NCV_, k_defect<2, true, NCV_, true><<<grid, 256, 0, ctx->stream>>>(t, list, phi, rhs, r32, e32, c, g,
                                                                                ctx->d_is_leaf, maxbits));
    else
      AFG_NC2(NCV_, k_defect<2, false, NCV_, true><<<grid, 256, 0, ctx->stream>>>(t, list, phi, rhs, r32, e32, c, g,
                                                                                 ctx->d_is_leaf, maxbits));
  } else if (ctx->D == 3)
    AFG_NC3(NCV_, k_defect<3, false, NCV_><<<grid, 256, 0, ctx->stream>>>(t, list, phi, rhs, r32, e32, c, g, ctx->d_is_leaf,
                                                   maxbits));
  else if (ctx->coord == AFG_CYL)
    AFG_NC2(NCV_, k_defect<2, true, NCV_><<<grid, 256, 0, ctx->stream>>>(t, list, phi, rhs, r32, e32, c, g, ctx->d_is_leaf,
                                                  maxbits));
  else
    AFG_NC2(NCV_, k_defect<2, false, NCV_><<<grid, 256, 0, ctx->stream>>>(t, list, phi, rhs, r32, e32, c, g, ctx->d_is_leaf,
                                                   maxbits));
  ctx->launches++;
  CKL();
  return AFG_OK;
}

// Composite-grid consistency: coarse leaf cells next to a refined region read
// the parent boxes' phi, which the composite discretisation defines as the
// restriction of their children (the FAS fixed point).  Before each defect
// the parents are therefore restricted top-down (without geometry, as
// mg_box_rstr_lpl does for phi) and the ghost cells refreshed.
static int mixed_prepare(afg_ctx* ctx, MgSlot& m, ModeArg<double> phi) {
  KTree t = ktree(ctx);
  for (int lvl = ctx->highest_lvl; lvl >= 2; lvl--) {
    const int n = (int)ctx->lvl_ids[lvl - 1].size();
    if (n == 0) continue;
    const dim3 grid(n, ctx->ky);
    KtScope kts(ctx, AFG_KT_RESTRICT, 8.0 * n * ctx->ky * ktree(ctx).SI * (1.0 + 1.0 / (1 << ctx->D)));
    if (ctx->D == 3)
      AFG_NC3(NCV_, k_restrict_geom<3, false, NCV_><<<grid, 64, 0, ctx->stream>>>(t, lst(ctx, ctx->off_ids[lvl - 1]), phi));
    else
      AFG_NC2(NCV_, k_restrict_geom<2, false, NCV_><<<grid, 64, 0, ctx->stream>>>(t, lst(ctx, ctx->off_ids[lvl - 1]), phi));
    ctx->launches++;
    CKL();
  }
  // The defect fills the face ghosts of the leaves itself, but its
  // refinement-boundary rules read face ghosts of the coarse source boxes;
  // those (level by level, coarse to fine: their own rules read coarser
  // sources) are filled here, before the launch.
  const GcDev g = mg_gc(ctx, m, false);
  for (int lvl = 1; lvl <= ctx->highest_lvl; lvl++)
    RC(launch_gc<double>(ctx, lst(ctx, ctx->off_rbsrc[lvl - 1]), (int)ctx->lvl_rbsrc[lvl - 1].size(), phi, g, 0));
  return AFG_OK;
}

// all ghost cells of phi (faces, edges, corners) when the solve ends
static int mixed_finish(afg_ctx* ctx, MgSlot& m, ModeArg<double> phi) {
  const GcDev g = mg_gc(ctx, m, false);
  for (int lvl = 1; lvl <= ctx->highest_lvl; lvl++) RC(mg_gc_lvl<double>(ctx, lvl, phi, g, 1));
  return AFG_OK;
}

// FMG of a mixed-precision slot as one defect-correction step: the FP64
// defect r = rhs - L(phi) (parents restricted first), an FP32 FMG from zero
// for the correction L e = r with homogeneous boundary values, phi += e, and
// (set_residual) the FP64 defect of the result.  Without a guess phi starts
// from zero, so the first correction is the whole solution.  Repeated calls
// converge like FP64 FMG cycles down to FP64 accuracy: each FP32 FMG only
// has to reduce the current defect, not resolve phi itself.
// (lockstep slots: phi, rhs and maxbits per slot, the FP32 buffers of
// each slot)
static int mixed_fmg(afg_ctx* ctx, MgSlot& m, ModeArg<double> phi, ModeArg<double> rhs, bool set_residual,
                     bool have_guess, ModeArg<unsigned long long> maxbits) {
  const int n = ctx->n_all_leaves;
  if (n <= 0) return AFG_OK;
  // phi += e on the leaves; the parents are restricted from them next
  const int* list = lst(ctx, ctx->off_all_leaves);
  if (!have_guess)
    for (int k = 0; k < ctx->ky; k++)
      CK(cudaMemsetAsync(phi.p[k], 0, sizeof(double) * (size_t)ctx->n_boxes * ctx->S, ctx->stream));
  RC(mixed_prepare(ctx, m, phi));
  RC(reset_max(ctx, 2));
  // the first defect's maximum is not used: every slot folds it into word 2
  RC(launch_defect(ctx, m, phi, rhs, ModeArg<unsigned long long>(ctx->d_max + 2)));
  RC(mg_fmg<float>(ctx, m, slot_bufs(ctx, m, &MgSlot::e32), slot_bufs(ctx, m, &MgSlot::r32),
                   slot_bufs(ctx, m, &MgSlot::t32), false, false, nullptr, true));
  RC(launch_add_correction(ctx, list, n, phi, ModeArg<const float>(slot_bufs(ctx, m, &MgSlot::e32))));
  RC(mixed_prepare(ctx, m, phi));
  if (set_residual) RC(launch_defect(ctx, m, phi, rhs, maxbits));
  return mixed_finish(ctx, m, phi);
}
