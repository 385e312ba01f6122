"""Batched independent instances (a forest in one context) against runs of
each instance on its own tree.

Six 2D axisymmetric instances of uneven size (32^2 to 128^2 cells, 2 to 4
levels) with their own applied voltages and seed amplitudes advance through
the initial field solve and three Heun steps as one forest.  Every instance
converges to its own threshold and is frozen while the others continue, so
each must end bit for bit where a run of its own tree ends, with the same
V-cycle counts, and the forest's cell-update count must equal the sum of the
single runs' counts; for the FP64 and the mixed-precision path."""
import numpy as np
import pytest

import afivo_gpu as ag
import streamer_model as sm
import workloads as wl

pytestmark = pytest.mark.gpu

N_STEPS = 3


def work(c0, c1):
    return (c1["smoother_updates"] - c0["smoother_updates"]) + (c1["transport_updates"] - c0["transport_updates"])


def advance(ctx, tree, model, H, ivs, voltage, dt, precision, kw, box_inst=None):
    ctx.tree_sync(tree, model.n_var_cell, model.n_var_face, box_inst=box_inst)
    ctx.upload_vars(H, ivs)
    run = sm.StreamerRun(ctx, tree, model, voltage, dt, precision=precision, **kw)
    run.setup()
    c0 = ctx.counters()
    run.initial_field()
    vc = [run.last.get("vcycles_inst", run.last.get("vcycles"))]
    for _ in range(N_STEPS):
        run.step()
        vc.append(run.last.get("vcycles_inst", run.last["vcycles"]))
    c1 = ctx.counters()
    cc = ag.new_cc(tree, model.n_var_cell)
    fc = ag.new_fc(tree, model.n_var_face)
    ctx.download(cc)
    ctx.download_fc(fc)
    return cc, fc, vc, work(c0, c1)


@pytest.mark.parametrize("precision", [ag.FP64, ag.MIXED])
def test_batched_equals_single_runs(precision):
    b = wl.BatchCyl2d(n_inst=6, seed=7, sides=(32, 64, 128))
    model = b.model()
    f, box_inst, trees = b.forest()
    assert len(set(t.highest_lvl for t in trees)) > 1
    H, ivs = b.initial_host_state(trees, model)
    kw = b.run_kwargs()
    ctx = ag.Context(0)
    cc, fc, vc, w = advance(ctx, f, model, H, ivs, b.voltages, b.dt, precision, kw, box_inst)
    assert ctx.n_instances() == len(trees)
    ctx.close()
    offs = np.cumsum([0] + [t.n_boxes for t in trees])
    w_single = 0
    for q, t in enumerate(trees):
        cq = ag.Context(0)
        ccq, fcq, vcq, wq = advance(cq, t, model, H[offs[q]:offs[q + 1]], ivs, float(b.voltages[q]), b.dt,
                                    precision, kw)
        cq.close()
        w_single += wq
        assert [int(v[q]) for v in vc] == [int(v) for v in vcq], f"instance {q}: V-cycle counts"
        assert np.array_equal(cc[offs[q]:offs[q + 1]].view(np.uint64), ccq.view(np.uint64)), f"instance {q}: cc"
        assert np.array_equal(fc[offs[q]:offs[q + 1]].view(np.uint64), fcq.view(np.uint64)), f"instance {q}: fc"
    assert w == w_single
