"""A refinement cycle with the data on the device against the same cycle on
the CPU restatement: a step, then box flags (seed line, buffer cells,
derefinement of fine boxes away from it), the host's new tree, the data
moved by box, prolongation of the new boxes, the field of the new mesh, and
another step.  The flags, the new trees and (FP64 path) the state after the
second step must agree: flags and box maps exactly, densities, potential and
|E| within 1e-10 of their maxima (the reaction rates of this model are
tabulated, but the two field solves of each step run to the same threshold
on both sides)."""
import numpy as np
import pytest

import afivo_gpu as ag
import streamer_model as sm
from oracle_streamer import OracleStreamerRun
from streamer_cases import initial_state
from test_gpu_step_parity import leaf_interior, make

pytestmark = pytest.mark.gpu


def refine_desc(model):
    d = model.refine_desc(ref_buffer=2, derefine_dx=1e-4, n_seeds=1, init_fac=0.01)
    d.seed_r0[0][0], d.seed_r0[0][1] = 0.0, 1.0e-2
    d.seed_r1[0][0], d.seed_r1[0][1] = 0.0, 1.4e-2
    d.seed_width[0] = 5e-4
    return d


def test_refine_cycle_matches_restatement():
    w, tree, model = make("cyl2d")
    photoi = (w.photoi_lambda, w.photoi_coeffs, w.photoi_eta_quench)
    cc, fc = initial_state(tree, model, seed=7, voltage=w.voltage)
    ctx = ag.Context(0)
    ctx.tree_sync(tree, model.n_var_cell, model.n_var_face)
    ctx.upload(cc)
    ctx.upload_fc(fc)
    gpu = sm.StreamerRun(ctx, tree, model, w.voltage, w.dt, precision=ag.FP64, max_rel_residual=1e-8,
                         num_vcycles=30, photoi=photoi)
    gpu.setup()
    cpu = OracleStreamerRun(tree, model, w.voltage, w.dt, max_rel_residual=1e-8, num_vcycles=30, photoi=photoi)
    cpu.setup()
    gpu.initial_field()
    cpu.initial_field(cc, fc)
    gpu.step()
    cpu.step(cc, fc)
    d = refine_desc(model)
    g_flags, g_old = gpu.refine(d, 6)
    cc, fc, c_flags, c_old = cpu.refine(cc, fc, d, 6)
    assert np.array_equal(g_flags, c_flags)
    assert np.array_equal(g_old, c_old)
    assert np.count_nonzero(g_old == 0) > 0 and gpu.tree.n_boxes != tree.n_boxes
    gpu.step()
    cpu.step(cc, fc)
    out = ag.new_cc(gpu.tree, model.n_var_cell)
    ctx.download(out)
    ctx.close()
    for iv in list(model.species_iv) + [model.i_phi, model.i_electric_fld]:
        a, b = leaf_interior(gpu.tree, out[:, iv - 1]), leaf_interior(gpu.tree, cc[:, iv - 1])
        err = np.max(np.abs(a - b))
        assert err <= 1e-10 * np.max(np.abs(b)), f"variable {iv}: {err} vs max {np.max(np.abs(b))}"
