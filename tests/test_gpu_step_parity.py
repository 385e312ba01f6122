"""Whole time steps on the GPU against the CPU restatement of the step.

Both run the reference's step order (photoionization every 5 steps, state
copy, two Heun stages with a field solve after each) on small trees with the
benchmark's two models: the 2D cylindrical 3-species model with tabulated
rates and the 3D 5-species model whose 8 reactions use the k13 rate form
(exp/pow per cell, the project's own exp and pow on both sides, so the
FP64 evaluations agree bit for bit).  Tolerances: FP64 path 1e-12 of the
variable's maximum after 6 steps; the mixed-precision path
(FP32 V-cycles inside FP64 defect correction, same 1e-8 residual target)
1e-6 of the maximum.  The cell-update accounting of the GPU counters must
equal the restatement's count exactly on the FP64 path.
"""
import numpy as np
import pytest

import afivo_gpu as ag
import workloads as wl
from mgcases import refined_tree
from oracle_streamer import OracleStreamerRun
from streamer_cases import initial_state
import streamer_model as sm

pytestmark = pytest.mark.gpu

N_STEPS = 6


def make(name):
    if name == "cyl2d":
        w = wl.Cyl2d()
        tree = refined_tree(2, 8, [16, 32], [1e-2, 2e-2], 5, 2, [0.0, 1.2e-2], 0.8e-3,
                            coord=ag.AFG_CYL, seed=2, frac=0.1)
    else:
        w = wl.Streamer3d()
        tree = refined_tree(3, 8, [8, 8, 8], [3e-2] * 3, 4, 2, [1.5e-2, 1.5e-2, 1.7e-2], 2e-3,
                            seed=3, frac=0.05)
    return w, tree, w.model()


def leaf_interior(tree, a):
    leaves = np.concatenate(tree.lvl_leaves) - 1
    n2 = tree.n_cell + 2
    return a[leaves][(slice(None),) + (slice(1, n2 - 1),) * tree.ndim]


def run_pair(name, precision):
    w, tree, model = make(name)
    photoi = (w.photoi_lambda, w.photoi_coeffs, w.photoi_eta_quench)
    cc, fc = initial_state(tree, model, seed=7, voltage=w.voltage)
    ctx = ag.Context(0)
    ctx.tree_sync(tree, model.n_var_cell, model.n_var_face)
    ctx.upload(cc)
    ctx.upload_fc(fc)
    gpu = sm.StreamerRun(ctx, tree, model, w.voltage, w.dt, precision=precision, max_rel_residual=1e-8,
                         num_vcycles=30, photoi=photoi)
    gpu.setup()
    cpu = OracleStreamerRun(tree, model, w.voltage, w.dt, max_rel_residual=1e-8, num_vcycles=30, photoi=photoi)
    cpu.setup()
    gpu.initial_field()
    cpu.initial_field(cc, fc)
    works = []
    for _ in range(N_STEPS):
        c0 = ctx.counters()
        gpu.step()
        c1 = ctx.counters()
        g_work = (c1["smoother_updates"] - c0["smoother_updates"]) + \
            (c1["transport_updates"] - c0["transport_updates"])
        works.append((g_work, cpu.step(cc, fc), gpu.last["vcycles"], cpu.last["vcycles"]))
    out = ag.new_cc(tree, model.n_var_cell)
    ctx.download(out)
    ctx.close()
    return tree, model, cc, out, works


@pytest.mark.parametrize("name", ["cyl2d", "3d"])
def test_steps_fp64(name):
    tree, model, ref, got, works = run_pair(name, ag.FP64)
    for g_work, c_work, g_v, c_v in works:
        assert g_v == c_v
        assert g_work == c_work
    for iv in list(model.species_iv) + [model.i_phi, model.i_electric_fld, model.i_photo]:
        a, b = leaf_interior(tree, got[:, iv - 1]), leaf_interior(tree, ref[:, iv - 1])
        err = np.max(np.abs(a - b))
        print(f"{name} FP64 variable {iv}: max |GPU - restatement| / max {err / np.max(np.abs(b)):.3e}")
        assert err <= 1e-12 * np.max(np.abs(b)), f"variable {iv}: {err} vs max {np.max(np.abs(b))}"


@pytest.mark.parametrize("name", ["cyl2d", "3d"])
def test_steps_mixed(name):
    tree, model, ref, got, works = run_pair(name, ag.MIXED)
    for iv in list(model.species_iv) + [model.i_phi, model.i_electric_fld]:
        a, b = leaf_interior(tree, got[:, iv - 1]), leaf_interior(tree, ref[:, iv - 1])
        err = np.max(np.abs(a - b))
        assert err <= 1e-6 * np.max(np.abs(b)), f"variable {iv}: {err} vs max {np.max(np.abs(b))}"
