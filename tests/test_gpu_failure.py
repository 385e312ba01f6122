"""Failure detection on the device without a GPU fault: a kernel whose
bounded mbarrier wait cannot complete (copies announced on the barrier, none
issued) gives up after its 1 s limit, raises the context's error word, and
the host reports it like after any solve iteration; the context stays usable
(a V-cycle afterwards still matches the CPU restatement)."""
import numpy as np
import pytest

import afivo_gpu as ag
import oracle
from mgcases import I_PHI, I_RHS, I_TMP, refined_tree

pytestmark = pytest.mark.gpu


def test_timed_out_wait_is_reported_and_context_survives():
    tree = refined_tree(2, 16, [32, 32], [1e-2, 1e-2], 4, 2, [0.5e-2, 0.5e-2], 1e-3, seed=8, frac=0.1)
    ctx = ag.Context(0)
    ctx.tree_sync(tree, 3)
    rc, ms = ctx.check_bounded_wait()
    assert rc == ag.AFG_ERR_DEVICE, rc
    assert 900.0 <= ms <= 5000.0, ms
    bt = [ag.BC_NEUMANN, ag.BC_NEUMANN, ag.BC_DIRICHLET, ag.BC_DIRICHLET]
    desc = ag.mg_desc(I_PHI, I_RHS, I_TMP, bt, [0, 0, 0, 1.0])
    rng = np.random.default_rng(3)
    cc = ag.new_cc(tree, 3)
    cc[:] = rng.standard_normal(cc.shape)
    o = oracle.Oracle(tree, 3)
    o.mg_setup(0, desc)
    ctx.mg_setup(0, desc)
    ctx.upload(cc)
    ctx.gc(I_PHI, 0, True)
    o.gc(cc, I_PHI, 0, True)
    r_gpu = ctx.mg_vcycle(0, True)
    r_cpu = o.mg_vcycle(cc, 0, True)
    ctx.close()
    assert abs(r_gpu - r_cpu) <= 1e-12 * abs(r_cpu)
