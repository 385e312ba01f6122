"""Adaptive refinement on the GPU against the CPU restatement, through the
C-ABI: the box refinement flags of default_refinement + cell_to_ref_flags
(integers, equal), af_prolong_limit into boxes (bit for bit) and the move of
all data to a new tree (persisting boxes bit for bit, new boxes zero)."""
import numpy as np
import pytest

import afivo_gpu as ag
import afivo_tree as at
import oracle
from mgcases import refined_tree
from streamer_cases import initial_state, make_case
from test_oracle_amr import desc

pytestmark = pytest.mark.gpu


def pair_with_field(name):
    tree, model = make_case(name)
    ctx = ag.Context(0)
    ctx.tree_sync(tree, model.n_var_cell, model.n_var_face)
    o = oracle.Oracle(tree, model.n_var_cell, model.n_var_face)
    d = model.transport_desc()
    ctx.transport_setup(d)
    o.transport_setup(d)
    mg = model.field_mg(-3e4)
    for obj in (ctx, o):
        obj.set_cc_methods(model.i_electric_fld, *model.electric_fld_gc())
        obj.mg_setup(0, mg)
    cc, fc = initial_state(tree, model, seed=3)
    o.gc(cc, model.i_phi, 0, True)
    ctx.upload(cc)
    ctx.upload_fc(fc)
    ctx.field_from_potential(model.i_phi)
    o.field_from_potential(cc, fc, model.i_phi)
    return tree, model, ctx, o, cc


@pytest.mark.parametrize("name", ["2d8cyl", "3d8"])
@pytest.mark.parametrize("variant", ["plain", "effective", "seeds_regions"])
def test_refine_flags_equal(name, variant):
    tree, model, ctx, o, cc = pair_with_field(name)
    D = tree.ndim
    L = tree.dr[0] * tree.n_cell * (np.asarray(tree.coarse_grid_size) / tree.n_cell)
    kw = dict(ref_buffer=2, derefine_dx=3e-4, adx=0.5)
    if variant == "effective":
        kw["use_alpha_effective"] = 1
    d = desc(model, **kw)
    if variant == "seeds_regions":
        d.n_seeds, d.n_regions, d.n_limits = 1, 1, 1
        for k in range(D):
            d.seed_r0[0][k] = 0.5 * L[k]
            d.seed_r1[0][k] = 0.6 * L[k]
            d.region_rmin[0][k] = 0.1 * L[k]
            d.region_rmax[0][k] = 0.3 * L[k]
            d.limit_rmin[0][k] = 0.0
            d.limit_rmax[0][k] = 0.45 * L[k]
        d.seed_width[0], d.init_fac = 0.1 * L[0], 0.01
        d.region_dr[0], d.limit_dr[0] = 1e-5, 1.0
    got = ctx.refine_flags(d)
    ref = o.refine_flags(cc, d)
    ctx.close()
    assert np.array_equal(got, ref), np.nonzero(got != ref)
    assert len(set(ref.tolist())) > 1  # the case exercises more than one flag


@pytest.mark.parametrize("name", ["2d16", "3d8"])
def test_prolong_limit_bitexact(name):
    tree, model = make_case(name)
    ctx = ag.Context(0)
    ctx.tree_sync(tree, model.n_var_cell, model.n_var_face)
    o = oracle.Oracle(tree, model.n_var_cell, model.n_var_face)
    cc, fc = initial_state(tree, model, seed=4)
    iv = model.species_iv[0]
    for obj in (ctx, o):
        obj.set_cc_methods(iv, [ag.BC_NEUMANN] * (2 * tree.ndim), None, ag.RB_INTERP_LIM)
    o.gc(cc, iv, 0, True)
    ctx.upload(cc)
    ctx.gc(iv, 0, True)
    # boxes of one level, as after one refinement step (no parent is itself
    # being filled)
    ids = tree.lvl_ids[-1]
    for lim in (ag.LIMITER_MC, ag.LIMITER_GMINMOD43, ag.LIMITER_KOREN):
        ctx.prolong_limit(iv, ids, lim)
        o.prolong_limit(cc, iv, ids, lim)
        out = ag.new_cc(tree, model.n_var_cell)
        ctx.download(out)
        assert np.array_equal(out[:, iv - 1].view(np.uint64), cc[:, iv - 1].view(np.uint64)), lim
    ctx.close()


def test_tree_remap_keeps_data():
    a = refined_tree(2, 8, [16, 16], [1e-2, 1e-2], 5, 2, [0.4e-2, 0.5e-2], 0.8e-3, seed=1, frac=0.1)
    b = refined_tree(2, 8, [16, 16], [1e-2, 1e-2], 5, 2, [0.6e-2, 0.5e-2], 0.8e-3, seed=1, frac=0.1)
    old_id = at.remap_ids(a, b)
    assert 0 < np.count_nonzero(old_id) < b.n_boxes
    ctx = ag.Context(0)
    ctx.tree_sync(a, 3, 1)
    rng = np.random.default_rng(0)
    cc = rng.standard_normal(ag.new_cc(a, 3).shape)
    fc = rng.standard_normal(ag.new_fc(a, 1).shape)
    ctx.upload(cc)
    ctx.upload_fc(fc)
    ctx.tree_remap(b, old_id)
    out, outf = ag.new_cc(b, 3), ag.new_fc(b, 1)
    ctx.download(out)
    ctx.download_fc(outf)
    ctx.close()
    keep = old_id > 0
    assert np.array_equal(out[keep].view(np.uint64), cc[old_id[keep] - 1].view(np.uint64))
    assert np.array_equal(outf[keep].view(np.uint64), fc[old_id[keep] - 1].view(np.uint64))
    assert not np.any(out[~keep]) and not np.any(outf[~keep])
