"""afg_maxabs_noalloc: the max-norm reduction for callers that may not
allocate device memory (no context, caller-owned device buffers, scratch in a
static device array).  Two calls in a row must agree with afg_maxabs, the
context-based entry point, on the same data (max is exact, so equality).
Collected last so that a failure here leaves every other test already run."""
import ctypes

import numpy as np
import pytest

import afivo_gpu as ag
from mgcases import refined_tree

pytestmark = pytest.mark.gpu


def test_maxabs_noalloc_matches_context_entry_point(gpu_lib):
    torch = pytest.importorskip("torch")
    tree = refined_tree(2, 16, [32, 32], [1e-2, 1e-2], 5, 2, [0.5e-2, 0.8e-2], 0.6e-3, seed=1, frac=0.1)
    rng = np.random.default_rng(2024)
    cc = ag.new_cc(tree, 2)
    cc[:, 0] = rng.standard_normal(cc[:, 0].shape)
    cc[:, 1] = rng.standard_normal(cc[:, 1].shape) * 1e7
    # ghost cells are excluded by both entry points: make them dominate
    n2 = tree.n_cell + 2
    cc[:, :, 0, :] = 1e30
    ctx = ag.Context(0)
    ctx.tree_sync(tree, 2)
    ctx.upload(cc)
    slots = np.concatenate(tree.lvl_ids).astype(np.int32) - 1
    leaves = np.concatenate(tree.lvl_leaves).astype(np.int32) - 1
    dev = torch.device("cuda:0")
    for iv, sel, leaves_only in ((1, slots, False), (2, leaves, True)):
        pool = torch.from_numpy(np.ascontiguousarray(cc[:, iv - 1].reshape(tree.n_boxes, -1))).to(dev)
        d_slots = torch.from_numpy(sel).to(dev)
        torch.cuda.synchronize()
        got = ag.maxabs_noalloc(pool.data_ptr(), d_slots.data_ptr(), len(sel), tree.ndim, tree.n_cell)
        want = ctx.maxabs(iv, leaves_only)
        assert got == want, (iv, got, want)
        assert got < 1e29
    ctx.close()


def test_maxabs_noalloc_propagates_nan_like_context_entry_point(gpu_lib):
    """A NaN in one interior cell is the result of both entry points (a
    diverged solve must not read as converged), twice in a row."""
    torch = pytest.importorskip("torch")
    tree = refined_tree(2, 16, [32, 32], [1e-2, 1e-2], 4, 2, [0.5e-2, 0.5e-2], 1e-3, seed=5, frac=0.1)
    rng = np.random.default_rng(77)
    cc = ag.new_cc(tree, 1)
    cc[:] = rng.standard_normal(cc.shape)
    leaves = np.concatenate(tree.lvl_leaves).astype(np.int32) - 1
    cc[leaves[len(leaves) // 2], 0, 5, 7] = np.nan
    ctx = ag.Context(0)
    ctx.tree_sync(tree, 1)
    ctx.upload(cc)
    dev = torch.device("cuda:0")
    pool = torch.from_numpy(np.ascontiguousarray(cc[:, 0].reshape(tree.n_boxes, -1))).to(dev)
    d_slots = torch.from_numpy(leaves).to(dev)
    torch.cuda.synchronize()
    for _ in range(2):
        got = ag.maxabs_noalloc(pool.data_ptr(), d_slots.data_ptr(), len(leaves), tree.ndim, tree.n_cell)
        want = ctx.maxabs(1, True)
        assert np.isnan(got) and np.isnan(want), (got, want)
    ctx.close()


def test_maxabs_noalloc_rejects_oversize(gpu_lib):
    """More boxes than the static scratch holds (AFG_NOALLOC_MAX_BOXES) is an
    argument error, reported before any device work."""
    lib = ag.load_library()
    out = ctypes.c_double(0)
    rc = lib.afg_maxabs_noalloc(1, 1, 262144 + 1, 2, 16, None, ctypes.byref(out))
    assert rc == ag.AFG_ERR_ARG
