"""The plain 2D Cartesian configuration at full size against the CPU
restatement: 1 cm^2, uniform 256^2 grid of 16^2-cell boxes (5 levels, 341
boxes), electrons and immobile ions from a Gaussian seed, ionization
alpha(E) through the tabulated rate, forward Euler at dt = 1e-12 s, one
Poisson solve to 1e-10 relative residual per step.

With tabulated rates every operation of the FP64 path is the reference's, so
100 steps must agree bit for bit with the restatement, V-cycle counts
included.  The mixed path (FP32 V-cycles inside FP64 defect correction)
stays within 1e-6 of each variable's maximum.  Every explicit integrator of
af_advance runs a few steps bit for bit on the grid one level coarser."""
import numpy as np
import pytest

import afivo_gpu as ag
import streamer_model as sm
import workloads as wl
from oracle_streamer import OracleStreamerRun

pytestmark = pytest.mark.gpu


def leaf_interior(tree, a):
    leaves = np.concatenate(tree.lvl_leaves) - 1
    n2 = tree.n_cell + 2
    return a[leaves][(slice(None),) + (slice(1, n2 - 1),) * tree.ndim]


def run_pair(precision, n_steps, integrator=None, coarsen=0):
    w = wl.Cart2d()
    if integrator is not None:
        w.integrator = integrator
    tree, model = w.tree(coarsen=coarsen), w.model()
    assert coarsen or (tree.n_boxes == 341 and tree.highest_lvl == 5)
    H, ivs = w.initial_host_state(tree, model)
    cc = ag.new_cc(tree, model.n_var_cell)
    fc = ag.new_fc(tree, model.n_var_face)
    for v, iv in enumerate(ivs):
        cc[:, iv - 1] = H[:, v]
    ctx = ag.Context(0)
    ctx.tree_sync(tree, model.n_var_cell, model.n_var_face)
    ctx.upload(cc)
    ctx.upload_fc(fc)
    gpu = sm.StreamerRun(ctx, tree, model, w.voltage, w.dt, precision=precision, **w.run_kwargs())
    gpu.setup()
    cpu = OracleStreamerRun(tree, model, w.voltage, w.dt, **w.run_kwargs())
    cpu.setup()
    gpu.initial_field()
    cpu.initial_field(cc, fc)
    vc = []
    for _ in range(n_steps):
        gpu.step()
        cpu.step(cc, fc)
        vc.append((gpu.last["vcycles"], cpu.last["vcycles"]))
    out = ag.new_cc(tree, model.n_var_cell)
    ctx.download(out)
    ctx.close()
    return tree, model, cc, out, vc


def test_cart2d_fp64_100_steps_bitexact():
    tree, model, ref, got, vc = run_pair(ag.FP64, 100)
    assert all(g == c for g, c in vc)
    for iv in list(model.species_iv) + [model.i_phi, model.i_electric_fld]:
        a, b = leaf_interior(tree, got[:, iv - 1]), leaf_interior(tree, ref[:, iv - 1])
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), \
            f"variable {iv}: max diff {np.max(np.abs(a - b))} of max {np.max(np.abs(b))}"


def test_cart2d_mixed():
    tree, model, ref, got, vc = run_pair(ag.MIXED, 20)
    for iv in list(model.species_iv) + [model.i_phi, model.i_electric_fld]:
        a, b = leaf_interior(tree, got[:, iv - 1]), leaf_interior(tree, ref[:, iv - 1])
        err = np.max(np.abs(a - b))
        assert err <= 1e-6 * np.max(np.abs(b)), f"variable {iv}: {err} vs max {np.max(np.abs(b))}"


@pytest.mark.parametrize("integrator", sorted(sm.INTEGRATORS))
def test_cart2d_integrators_bitexact(integrator):
    """Every explicit integrator of af_advance, 4 steps on the grid one
    level coarser, FP64 bit for bit."""
    tree, model, ref, got, vc = run_pair(ag.FP64, 4, integrator=integrator, coarsen=1)
    assert all(g == c for g, c in vc)
    for iv in list(model.species_iv) + [model.i_phi, model.i_electric_fld]:
        a, b = leaf_interior(tree, got[:, iv - 1]), leaf_interior(tree, ref[:, iv - 1])
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), f"{integrator} variable {iv}"
