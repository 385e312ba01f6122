"""Helmholtz modes of the photoionization solved as multiple right-hand
sides in one sweep (lockstep: every launch of the mixed-precision FMG covers
all modes not yet converged) against the same modes run as parallel graph
branches, one per mode: each mode's arithmetic is the same either way, so
two steps with photoionization must agree bit for bit (2D cylindrical and
3D trees)."""
import numpy as np
import pytest

import afivo_gpu as ag
import streamer_model as sm
from streamer_cases import initial_state
from test_gpu_step_parity import make

pytestmark = pytest.mark.gpu


def advance(name, lockstep):
    w, tree, model = make(name)
    cc, fc = initial_state(tree, model, seed=5, voltage=w.voltage)
    ctx = ag.Context(0)
    ctx.tree_sync(tree, model.n_var_cell, model.n_var_face)
    ctx.upload(cc)
    ctx.upload_fc(fc)
    ctx.set_photoi_lockstep(lockstep)
    run = sm.StreamerRun(ctx, tree, model, w.voltage, w.dt, precision=ag.MIXED, max_rel_residual=1e-8,
                         num_vcycles=30, photoi=(w.photoi_lambda, w.photoi_coeffs, w.photoi_eta_quench),
                         photoi_per_steps=1)
    run.setup()
    run.initial_field()
    c0 = ctx.counters()
    for _ in range(2):
        run.step()
    c1 = ctx.counters()
    out = ag.new_cc(tree, model.n_var_cell)
    ctx.download(out)
    ctx.close()
    return out, c1["smoother_updates"] - c0["smoother_updates"]


@pytest.mark.parametrize("name", ["cyl2d", "3d"])
def test_lockstep_equals_branches(name):
    a, wa = advance(name, True)
    b, wb = advance(name, False)
    assert wa == wb
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
