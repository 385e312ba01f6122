"""Repeated runs give identical bits.

The mixed path runs the photoionization modes as concurrent graph branches
and folds maxima with atomics; neither may make results depend on timing.
Two fresh contexts advance the same 3D state (5 species, k13 chemistry,
photoionization in the first step) by 3 steps; every variable must agree
bit for bit, for the FP64 and the mixed path.
"""
import numpy as np
import pytest

import afivo_gpu as ag
import streamer_model as sm
from streamer_cases import initial_state
from test_gpu_step_parity import make

pytestmark = pytest.mark.gpu


def advance(precision):
    w, tree, model = make("3d")
    cc, fc = initial_state(tree, model, seed=11, voltage=w.voltage)
    ctx = ag.Context(0)
    ctx.tree_sync(tree, model.n_var_cell, model.n_var_face)
    ctx.upload(cc)
    ctx.upload_fc(fc)
    run = sm.StreamerRun(ctx, tree, model, w.voltage, w.dt, precision=precision, max_rel_residual=1e-8,
                         num_vcycles=30, photoi=(w.photoi_lambda, w.photoi_coeffs, w.photoi_eta_quench))
    run.setup()
    run.initial_field()
    for _ in range(3):
        run.step()
    out = ag.new_cc(tree, model.n_var_cell)
    ctx.download(out)
    ctx.close()
    return out


@pytest.mark.parametrize("precision", [ag.FP64, ag.MIXED])
def test_bitwise_repeatable(precision):
    a = advance(precision)
    b = advance(precision)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
