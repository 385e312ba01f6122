"""Tree tables follow afivo's conventions (afivo/src/m_af_types.f90)."""
import numpy as np
import pytest

import afivo_tree as at
from mgcases import refined_tree


@pytest.mark.parametrize("ndim", [2, 3])
def test_tree_invariants(ndim):
    if ndim == 2:
        t = refined_tree(2, 8, [16, 32], [1.0, 2.0], 6, 2, [0.2, 1.1], 0.05, seed=3, frac=0.1)
    else:
        t = refined_tree(3, 4, [8, 8, 8], [1.0, 1.0, 1.0], 4, 1, [0.3, 0.6, 0.5], 0.1, seed=4, frac=0.1)
    D = ndim
    nb_rev = [1, 0, 3, 2, 5, 4]
    for b in range(t.n_boxes):
        id_ = b + 1
        # children point back to parent, child index from ix parity
        for c in range(2 ** D):
            ch = t.children[b, c]
            if ch > 0:
                assert t.parent[ch - 1] == id_
                assert all(((t.ix[ch - 1, d] - 1) & 1) == ((c >> d) & 1) for d in range(D))
        for n in range(2 * D):
            nb = t.neighbors[b, n]
            if nb > 0:
                assert t.neighbors[nb - 1, nb_rev[n]] == id_
                assert t.lvl[nb - 1] == t.lvl[b]
            elif nb == 0:  # refinement boundary: parent's neighbour exists (2:1 balance)
                assert t.parent[b] > 0 and t.neighbors[t.parent[b] - 1, n] > 0
        # r_min consistent with ix and dr
        assert np.allclose(t.r_min[b], (t.ix[b] - 1) * t.dr[b] * t.n_cell, rtol=1e-12, atol=1e-15)
        # neighbor_mat centre is the box itself
        assert t.neighbor_mat[b, (3 ** D) // 2] == id_
    # level lists
    for l in range(t.highest_lvl):
        ids = t.lvl_ids[l]
        assert np.all(t.lvl[ids - 1] == l + 1)
        assert len(t.lvl_leaves[l]) + len(t.lvl_parents[l]) == len(ids)
    assert sum(len(x) for x in t.lvl_ids) == t.n_boxes


def test_uniform_counts():
    t = at.uniform_tree(2, 16, [16, 16], [1e-2, 1e-2], 5)
    assert t.n_boxes == 341 and t.n_cells(True) == 65536 and t.n_cells() == 87296


def test_forest_tables():
    """Forest of independent trees: ids of tree q shifted by the boxes of
    the trees before it, relations kept inside each tree, level lists
    concatenated, instance of each box."""
    import afivo_tree as at
    t1 = at.build_tree(2, 8, [8, 8], [1.0, 1.0], max_lvl=2)
    t2 = at.build_tree(2, 8, [8, 8], [1.0, 1.0], max_lvl=3)
    f, inst = at.forest([t1, t2])
    assert f.n_boxes == t1.n_boxes + t2.n_boxes and f.highest_lvl == 3
    assert list(inst) == [0] * t1.n_boxes + [1] * t2.n_boxes
    o = t1.n_boxes
    np.testing.assert_array_equal(f.parent[o:], np.where(t2.parent > 0, t2.parent + o, t2.parent))
    np.testing.assert_array_equal(f.neighbors[o:], np.where(t2.neighbors > 0, t2.neighbors + o, t2.neighbors))
    np.testing.assert_array_equal(f.children[:o], t1.children)
    for l in range(3):
        want = ([t1.lvl_ids[l]] if l < 2 else []) + [t2.lvl_ids[l] + o]
        np.testing.assert_array_equal(f.lvl_ids[l], np.concatenate(want))
    for b in range(f.n_boxes):
        for v in list(f.neighbors[b]) + list(f.children[b]) + [f.parent[b]]:
            if v > 0:
                assert inst[v - 1] == inst[b]
