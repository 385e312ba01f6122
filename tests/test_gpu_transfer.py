"""Host <-> device copies of the C-ABI: the pitched-DMA path (equally spaced
boxes in page-locked memory), the staged gather/scatter path (pageable
memory, several 32 MiB chunks), NULL boxes left untouched, face data."""
import ctypes as C

import numpy as np
import pytest

import afivo_gpu as ag
import afivo_tree as at

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx_tree(gpu_lib):
    # 3D uniform tree with 4096 boxes of 10^3 doubles: 32.8 MB per variable,
    # more than one staging chunk
    tree = at.uniform_tree(3, 8, [128, 128, 128], [1.0, 1.0, 1.0], 1)
    ctx = ag.Context(0)
    ctx.tree_sync(tree, 3, 1)
    yield ctx, tree
    ctx.close()


def host(tree, nvar, seed):
    n2 = tree.n_cell + 2
    return np.random.default_rng(seed).standard_normal((tree.n_boxes, nvar) + (n2,) * tree.ndim)


@pytest.mark.parametrize("locked", [False, True])
def test_roundtrip(ctx_tree, locked):
    ctx, tree = ctx_tree
    a = host(tree, 3, 1)
    b = np.zeros_like(a)
    if locked:
        ctx.host_register(a)
        ctx.host_register(b)
    try:
        ctx.upload_vars(a, [1, 2, 3], cols=[2, 0, 1])
        ctx.download_vars(b, [1, 2, 3], cols=[2, 0, 1])
    finally:
        if locked:
            ctx.host_unregister(a)
            ctx.host_unregister(b)
    assert np.array_equal(a, b)


def test_roundtrip_page_locked_elsewhere(ctx_tree):
    """Page-locked memory the context did not register: the pitched DMA path."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    ctx, tree = ctx_tree
    n2 = tree.n_cell + 2
    shape = (tree.n_boxes, 2) + (n2,) * tree.ndim
    ta = torch.empty(shape, dtype=torch.float64, pin_memory=True)
    tb = torch.zeros(shape, dtype=torch.float64, pin_memory=True)
    a, b = ta.numpy(), tb.numpy()
    a[...] = host(tree, 2, 5)
    ctx.upload_vars(a, [2, 3])
    ctx.download_vars(b, [2, 3])
    assert np.array_equal(a, b)


def test_async_download_overlaps_later_work(ctx_tree):
    """afg_cc_download_async: the copy is ordered after earlier work and
    completes by afg_transfers_wait, while later work on other variables
    proceeds."""
    ctx, tree = ctx_tree
    a = host(tree, 2, 6)
    ctx.upload_vars(a, [1, 2])
    b = np.zeros_like(a)
    ctx.host_register(b)
    try:
        ctx.tree_copy_cc(1, 3)                 # earlier work reading variable 1
        bp = ctx.download_vars_async(b, [1])   # ordered after it
        ctx.tree_copy_cc(2, 3)                 # later work, not writing variable 1
        ctx.transfers_wait()
        ctx.sync()
    finally:
        ctx.host_unregister(b)
    assert np.array_equal(b[:, 0], a[:, 0])
    c = np.zeros((tree.n_boxes, 1) + a.shape[2:])
    ctx.download_vars(c, [3])
    assert np.array_equal(c[:, 0], a[:, 1])


def test_null_boxes_untouched(ctx_tree):
    ctx, tree = ctx_tree
    a = host(tree, 1, 2)
    ctx.upload_vars(a, [1])
    c = host(tree, 1, 3)
    bp = ag.box_pointers(c)
    skip = np.zeros(tree.n_boxes, bool)
    skip[::7] = True
    skip[100:400] = True
    bp.addr[skip] = 0
    ctx.upload_vars(c, [1], bp=bp)
    out = np.zeros_like(a)
    ctx.download_vars(out, [1])
    assert np.array_equal(out[skip], a[skip])
    assert np.array_equal(out[~skip], c[~skip])
    # download with NULL entries writes only the others
    d = np.full_like(a, 5.0)
    bpd = ag.box_pointers(d)
    bpd.addr[skip] = 0
    ctx.download_vars(d, [1], bp=bpd)
    assert np.all(d[skip] == 5.0)
    assert np.array_equal(d[~skip], c[~skip])


def test_face_roundtrip(ctx_tree):
    ctx, tree = ctx_tree
    f = ag.new_fc(tree, 1)
    f[...] = np.random.default_rng(4).standard_normal(f.shape)
    ctx.upload_fc(f)
    g = np.zeros_like(f)
    ctx.download_fc(g)
    assert np.array_equal(f, g)


def test_register_rejects_null(ctx_tree):
    ctx, tree = ctx_tree
    assert ctx.lib.afg_host_register(ctx.ptr, None, 16) == ag.AFG_ERR_ARG
    assert ctx.lib.afg_host_register(ctx.ptr, C.c_void_p(8), 0) == ag.AFG_ERR_ARG
