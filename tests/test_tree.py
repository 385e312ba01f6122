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
