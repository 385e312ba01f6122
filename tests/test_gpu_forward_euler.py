"""afg_forward_euler (src/m_fluid.f90:21-99) against the same stage composed
of its C calls (afg_field_compute from the second stage on, afg_flux_upwind,
afg_update_densities) on a second context: every variable bit for bit and
the same dt limit, min(dt_max, dt_cfl_number * CFL limit, dielectric
relaxation time, chemistry limit of the last stage), over two Heun steps in
FP64 and mixed precision.  Without afg_stage_setup the call is refused."""
import numpy as np
import pytest

import afivo_gpu as ag
import streamer_model as sm
from mgcases import refined_tree
from test_gpu_step_parity import make
from streamer_cases import initial_state

pytestmark = pytest.mark.gpu


def composed_stage(ctx, run, f, s_deriv, s_prev, w_prev, s_out, i, n):
    if i > 1:
        ctx.field_compute(0, s_deriv, True, run.voltage, run.L, run.rel, run.num_vcycles)
    fl = ctx.flux_upwind(s_deriv)
    chem = ctx.update_densities(f * run.dt, s_deriv, s_prev, w_prev, s_out, last_step=(i == n))
    return min(run.dt_max, min(fl[0] * run.dt_cfl_number, fl[1], chem if i == n else 1e100, 1e100))


@pytest.mark.parametrize("precision", [ag.FP64, ag.MIXED])
def test_forward_euler_equals_composed_calls(precision):
    w, tree, model = make("cyl2d")
    cc, fc = initial_state(tree, model, seed=5, voltage=w.voltage)
    runs = []
    for _ in range(2):
        ctx = ag.Context(0)
        ctx.tree_sync(tree, model.n_var_cell, model.n_var_face)
        ctx.upload(cc)
        ctx.upload_fc(fc)
        run = sm.StreamerRun(ctx, tree, model, w.voltage, w.dt, precision=precision, max_rel_residual=1e-8,
                             num_vcycles=30, dt_cfl_number=0.5, dt_max=1e-11)
        run.setup()
        run.initial_field()
        runs.append((ctx, run))
    stages = sm.INTEGRATORS["heun"]
    for _ in range(2):
        lims = []
        for k, (ctx, run) in enumerate(runs):
            for s in range(len(model.species)):
                ctx.tree_copy_cc(model.species_iv[s], model.species_iv[s] + model.n_states - 1)
            for i, (f, s_deriv, s_prev, w_prev, s_out) in enumerate(stages, 1):
                if k == 0:
                    lim, nc = ctx.forward_euler(f * run.dt, run.voltage, s_deriv, s_prev, w_prev, s_out, i,
                                                len(stages))
                    assert (nc > 0) == (i > 1)
                else:
                    lim = composed_stage(ctx, run, f, s_deriv, s_prev, w_prev, s_out, i, len(stages))
            lims.append(lim)
            run.field(0, True)
        assert lims[0] == lims[1] and 0 < lims[0] <= 1e-11
        outs = []
        for ctx, _ in runs:
            o = ag.new_cc(tree, model.n_var_cell)
            ctx.download(o)
            outs.append(o)
        assert np.array_equal(outs[0].view(np.uint64), outs[1].view(np.uint64))
    for ctx, _ in runs:
        ctx.close()


def test_forward_euler_needs_stage_setup():
    w, tree, model = make("cyl2d")
    ctx = ag.Context(0)
    ctx.tree_sync(tree, model.n_var_cell, model.n_var_face)
    ctx.transport_setup(model.transport_desc())
    with pytest.raises(ag.AfgError):
        ctx.forward_euler(w.dt, w.voltage, 0, [0], [1.0], 1, 1, 2)
    with pytest.raises(ag.AfgError):
        ctx.stage_setup(0, 1.0, 1e-8, 30)  # no solver in slot 0
    ctx.close()


@pytest.mark.parametrize("name", ["cyl2d", "3d", "cyl2d_ion", "3d_ion"])
def test_staged_flux_equals_direct(name):
    """The FP32 fluxes with the box's |E| and densities staged by bulk copies
    (the default; boxes of 16^2 and 8^3 cells, electrons alone or with one
    mobile ion species) and read from global memory give the same bits:
    fluxes, the written-back ghost layer and both limits."""
    w, tree, model = make(name.split("_")[0])
    if name.startswith("cyl2d"):
        tree = refined_tree(2, 16, [16, 32], [1e-2, 2e-2], 4, 2, [0.0, 1.2e-2], 0.8e-3,
                            coord=ag.AFG_CYL, seed=2, frac=0.1)
    if name.endswith("_ion"):
        model = sm.StreamerModel(tree.ndim, alpha=sm.baseline_alpha, eta=sm.baseline_eta,
                                 mobile_ions=[(1, 2.2e-4)], photoi_modes=3)
    cc, fc = initial_state(tree, model, seed=9, voltage=w.voltage)
    ctx = ag.Context(0)
    ctx.tree_sync(tree, model.n_var_cell, model.n_var_face)
    ctx.upload(cc)
    ctx.upload_fc(fc)
    run = sm.StreamerRun(ctx, tree, model, w.voltage, w.dt, precision=ag.MIXED)
    run.setup()
    run.initial_field()
    res = []
    for on in (True, False):
        ctx.set_flux_staged(on)
        lim = ctx.flux_upwind(0)
        o, f = ag.new_cc(tree, model.n_var_cell), ag.new_fc(tree, model.n_var_face)
        ctx.download(o)
        ctx.download_fc(f)
        res.append((lim, o, f))
    ctx.close()
    assert np.array_equal(np.asarray(res[0][0]), np.asarray(res[1][0]))
    for k in (1, 2):
        assert np.array_equal(res[0][k].view(np.uint64), res[1][k].view(np.uint64))
