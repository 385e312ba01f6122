"""Electrode (level-set) multigrid on the GPU against the CPU restatement,
through the C-ABI, FP64: the level-set values of every cell, the electrode
boxes with their stencils, boundary-value factors, distances and
right-hand-side corrections, and the FMG, V-cycle and solve results (phi of
every box, the residual maximum) bit for bit; the electrode field
(mg_box_lpllsf_gradient) bit for bit; mixed precision refused."""
import numpy as np
import pytest

import afivo_gpu as ag
import oracle
from lsfcases import CASES, I_LSF, I_PHI, I_RHS, N_VAR, case, initial, mg_desc_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=CASES)
def pair(request):
    tree, d, volt = case(request.param)
    ctx = ag.Context(0)
    ctx.tree_sync(tree, N_VAR, 0)
    o = oracle.Oracle(tree, N_VAR)
    desc = mg_desc_for(tree)
    yield request.param, tree, d, volt, desc, ctx, o
    ctx.close()


def set_up(tree, d, volt, desc, ctx, o, seed):
    cc = initial(tree, seed)
    ctx.upload(cc)
    ctx.mg_setup(0, desc)
    o.mg_setup(0, desc)
    ctx.mg_set_lsf(0, d)
    o.mg_set_lsf(cc, 0, d)
    ctx.mg_set_lsf_voltage(0, volt)
    o.mg_set_lsf_voltage(0, volt)
    return cc


def download(ctx, tree):
    out = ag.new_cc(tree, N_VAR)
    ctx.download(out)
    return out


def test_setup_bitexact(pair):
    name, tree, d, volt, desc, ctx, o = pair
    cc = set_up(tree, d, volt, desc, ctx, o, 1)
    out = download(ctx, tree)
    assert np.array_equal(out[:, I_LSF - 1], cc[:, I_LSF - 1])
    g = ctx.mg_lsf_info(0, tree.ndim, tree.n_cell)
    r = o.mg_lsf_info(0)
    assert len(g[0]) > 0
    for a, b, what in zip(g, r, ("ids", "v", "f", "bcc", "dd")):
        assert np.array_equal(a, b), what


def test_fmg_vcycles_bitexact(pair):
    name, tree, d, volt, desc, ctx, o = pair
    cc = set_up(tree, d, volt, desc, ctx, o, 2)
    ctx.gc(I_PHI, 0, True)
    o.gc(cc, I_PHI, 0, True)
    rg = ctx.mg_fmg(0, True, False)
    rc = o.mg_fmg(cc, 0, True, False)
    out = download(ctx, tree)
    assert np.array_equal(out[:, I_PHI - 1], cc[:, I_PHI - 1])
    # interior right-hand side, with the in-place +/- bc_correction (the
    # reference also adds the FAS tmp in the ghost cells, which nothing reads)
    inner = (slice(None),) + (slice(1, -1),) * tree.ndim
    assert np.array_equal(out[:, I_RHS - 1][inner], cc[:, I_RHS - 1][inner])
    assert rg == rc
    for _ in range(3):
        rg = ctx.mg_vcycle(0, True)
        rc = o.mg_vcycle(cc, 0, True)
        assert rg == rc
    out = download(ctx, tree)
    assert np.array_equal(out[:, I_PHI - 1], cc[:, I_PHI - 1])
    # FMG with a guess (set_coarse_phi_rhs path)
    rg = ctx.mg_fmg(0, True, True)
    rc = o.mg_fmg(cc, 0, True, True)
    out = download(ctx, tree)
    assert np.array_equal(out[:, I_PHI - 1], cc[:, I_PHI - 1]) and rg == rc


def test_solve_bitexact_and_converges(pair):
    name, tree, d, volt, desc, ctx, o = pair
    cc = set_up(tree, d, volt, desc, ctx, o, 3)
    cc[:, I_PHI - 1] = 0.0
    cc[:, I_RHS - 1] *= 1e-3
    ctx.upload(cc)
    ctx.gc(I_PHI, 0, True)
    o.gc(cc, I_PHI, 0, True)
    thr = 1e-8 * max(o.maxabs(cc, I_RHS), abs(volt) / (tree.dr[0, 0] ** 2))
    ng, resg = ctx.mg_solve(0, thr, 40)
    nc, resc = o.mg_solve(cc, 0, thr, 40)
    out = download(ctx, tree)
    assert ng == nc and np.array_equal(resg, resc)
    assert np.array_equal(out[:, I_PHI - 1], cc[:, I_PHI - 1])
    assert resg[-1] < thr


def test_mixed_slot_refused(pair):
    name, tree, d, volt, desc, ctx, o = pair
    dm = mg_desc_for(tree, precision=ag.MIXED)
    ctx.mg_setup(1, dm)
    with pytest.raises(ag.AfgError):
        ctx.mg_set_lsf(1, d)


@pytest.mark.parametrize("name", ["2d_rod", "2d_cyl_cone", "3d_rod"])
def test_field_with_electrode_bitexact(name):
    """field_from_potential with an electrode: the regular gradient, the
    electrode faces of leaf boxes (mg_box_lpllsf_gradient) and |E|."""
    import streamer_model as sm
    tree, d, volt = case(name)
    model = sm.StreamerModel(tree.ndim, alpha=sm.baseline_alpha, eta=sm.baseline_eta)
    nv = model.n_var_cell + 1
    d.i_lsf = nv
    ctx = ag.Context(0)
    ctx.tree_sync(tree, nv, model.n_var_face)
    o = oracle.Oracle(tree, nv, model.n_var_face)
    td = model.transport_desc()
    ctx.transport_setup(td)
    o.transport_setup(td)
    mg = model.field_mg(volt)
    for obj in (ctx, o):
        obj.set_cc_methods(model.i_electric_fld, *model.electric_fld_gc())
        obj.mg_setup(0, mg)
    rng = np.random.default_rng(4)
    cc = ag.new_cc(tree, nv)
    cc[:, model.i_phi - 1] = rng.standard_normal(cc[:, 0].shape) * volt
    fc = ag.new_fc(tree, model.n_var_face)
    ctx.upload(cc)
    ctx.mg_set_lsf(0, d)
    o.mg_set_lsf(cc, 0, d)
    ctx.mg_set_lsf_voltage(0, volt)
    o.mg_set_lsf_voltage(0, volt)
    o.gc(cc, model.i_phi, 0, True)
    ctx.gc(model.i_phi, 0, True)
    ctx.field_from_potential(model.i_phi)
    o.field_from_potential(cc, fc, model.i_phi)
    out = ag.new_cc(tree, nv)
    ctx.download(out)
    ofc = ag.new_fc(tree, model.n_var_face)
    ctx.download_fc(ofc)
    k = td.i_efield_fc - 1
    assert np.array_equal(ofc[:, k], fc[:, k])
    assert np.array_equal(out[:, model.i_electric_fld - 1], cc[:, model.i_electric_fld - 1])
    ctx.close()
