"""Known answers of the CPU restatement of the refinement flags
(default_refinement + cell_to_ref_flags) and of af_prolong_limit."""
import numpy as np

import afivo_gpu as ag
import afivo_tree as at
import oracle
import streamer_model as sm
from mgcases import centers, refined_tree


def setup(tree):
    model = sm.StreamerModel(tree.ndim, alpha=sm.baseline_alpha, eta=sm.baseline_eta)
    o = oracle.Oracle(tree, model.n_var_cell, model.n_var_face)
    o.transport_setup(model.transport_desc())
    return model, o


def desc(model, **kw):
    d = ag.RefineDesc()
    d.i_electron, d.i_electric_fld = model.species_iv[0], model.i_electric_fld
    d.lt_col_alpha, d.lt_col_eta = model.col_alpha, model.col_eta
    d.gas_number_density = model.N
    d.adx, d.adx_fac, d.min_dens = 0.8, 1.0, 1e13
    d.derefine_dx, d.max_dx, d.min_dx = 1e-4, 1e-2, 1e-7
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def test_flags_uniform_fields():
    tree = refined_tree(2, 8, [16, 16], [1e-2, 1e-2], 4, 1, [0.5e-2, 0.5e-2], 1e-3, seed=1, frac=0.1)
    model, o = setup(tree)
    cc = ag.new_cc(tree, model.n_var_cell)
    leaves = np.concatenate(tree.lvl_leaves) - 1
    # strong field, dense electrons: every leaf refines
    cc[:, model.i_electric_fld - 1] = 1e7
    cc[:, model.species_iv[0] - 1] = 1e18
    f = o.refine_flags(cc, desc(model))
    assert np.all(f[leaves] == ag.REF_DO)
    # no field: derefine where dx < derefine_dx, else keep
    cc[:, model.i_electric_fld - 1] = 0.0
    f = o.refine_flags(cc, desc(model, derefine_dx=1e-3))
    dxmax = tree.dr.max(axis=1)
    assert np.all(f[leaves] == np.where(dxmax[leaves] < 1e-3, ag.REF_RM, ag.REF_KEEP))
    # dx above refine_max_dx: refine whatever the field
    f = o.refine_flags(cc, desc(model, max_dx=1e-5))
    assert np.all(f[leaves] == ag.REF_DO)


def test_flags_buffer_marks_neighbours():
    """A do-flag next to a box face marks the neighbour across it (ref_buffer
    cells), and only then."""
    tree = at.build_tree(2, 8, [16, 8], [2e-2, 1e-2], max_lvl=1)
    model, o = setup(tree)
    cc = ag.new_cc(tree, model.n_var_cell)
    cc[:, model.species_iv[0] - 1] = 1e18
    n2 = tree.n_cell + 2
    E = cc[:, model.i_electric_fld - 1].reshape(tree.n_boxes, n2, n2)
    E[0, 4, 8] = 1e7   # box 1, cell (i=8, j=4): next to the +x face
    f = o.refine_flags(cc, desc(model, ref_buffer=2))
    assert list(f) == [ag.REF_DO, ag.REF_DO]
    f = o.refine_flags(cc, desc(model, ref_buffer=0))
    assert list(f) == [ag.REF_DO, ag.REF_KEEP]


def test_prolong_limit_linear_and_conservative():
    tree = refined_tree(2, 8, [16, 16], [1.0, 1.0], 3, 1, [0.5, 0.5], 0.2, seed=2, frac=0.2)
    model, o = setup(tree)
    cc = ag.new_cc(tree, 1)
    X = centers(tree)
    cc[:, 0] = (2.0 * X[:, 0] - 3.0 * X[:, 1]).reshape(cc[:, 0].shape)
    ids = tree.lvl_ids[-1]
    o2 = oracle.Oracle(tree, 1)
    for lim in (ag.LIMITER_MC, ag.LIMITER_MINMOD, ag.LIMITER_KOREN):
        out = cc.copy()
        o2.prolong_limit(out, 1, ids, lim)
        n2 = tree.n_cell + 2
        inner = (slice(None),) + (slice(1, n2 - 1),) * 2
        assert np.allclose(out[ids - 1, 0][inner], cc[ids - 1, 0][inner], rtol=0, atol=1e-12)


def test_adjust_refinement_keep_and_conservative_prolongation():
    """No flags change: the same tree back, every box mapped to itself.
    Refining leaves and prolonging (Cartesian): the mean of the 2^D new
    cells equals the parent cell (af_prolong_limit is conservative)."""
    tree = refined_tree(2, 8, [16, 16], [1e-2, 1e-2], 4, 1, [0.5e-2, 0.5e-2], 1e-3, seed=3, frac=0.2)
    same = at.adjust_refinement(tree, np.zeros(tree.n_boxes, np.int32), 4)
    assert np.array_equal(at.remap_ids(tree, same), np.arange(1, tree.n_boxes + 1))
    flags = np.zeros(tree.n_boxes, np.int32)
    flags[tree.lvl_leaves[-1] - 1] = ag.REF_DO
    new = at.adjust_refinement(tree, flags, 5)
    old = at.remap_ids(tree, new)
    fresh = np.nonzero(old == 0)[0] + 1
    assert new.highest_lvl == 5 and len(fresh) > 0
    rng = np.random.default_rng(1)
    cc = ag.new_cc(new, 1)
    cc[:] = 1 + rng.random(cc.shape)
    o = oracle.Oracle(new, 1)
    o.set_cc_methods(1, [ag.BC_NEUMANN] * 4, None, ag.RB_INTERP_LIM)
    lv = new.lvl[fresh - 1]
    for lvl in sorted(set(lv.tolist())):
        o.gc(cc, 1, lvl - 1, True)
        o.prolong_limit(cc, 1, fresh[lv == lvl], ag.LIMITER_MC)
    n2, nc = new.n_cell + 2, new.n_cell
    for b in fresh[:20]:
        p = new.parent[b - 1]
        ch = cc[b - 1, 0].reshape(n2, n2)[1:-1, 1:-1]
        ox, oy = ((new.ix[b - 1] - 1) & 1) * (nc // 2)
        par = cc[p - 1, 0].reshape(n2, n2)[1 + oy:1 + oy + nc // 2, 1 + ox:1 + ox + nc // 2]
        mean = 0.25 * (ch[0::2, 0::2] + ch[1::2, 0::2] + ch[0::2, 1::2] + ch[1::2, 1::2])
        assert np.allclose(mean, par, rtol=1e-14, atol=0)
