"""afg_adjust_refinement (the library's host code) against the Python
restatement of af_adjust_refinement (afivo_tree.adjust_refinement): the same
new tree, array for array, from random box flags applied repeatedly to 2D,
2D cylindrical and 3D trees.  Runs on the CPU: the host code needs no GPU."""
import numpy as np
import pytest

import afivo_gpu as ag
import afivo_tree as at

FIELDS = ["lvl", "ix", "parent", "children", "neighbors", "neighbor_mat", "r_min", "dr", "dr_base"]


def same_tree(a, b):
    assert a.n_boxes == b.n_boxes and a.highest_lvl == b.highest_lvl
    for k in FIELDS:
        x, y = np.asarray(getattr(a, k)), np.asarray(getattr(b, k))
        assert x.shape == y.shape and np.array_equal(x, y), k
    for k in ["lvl_ids", "lvl_leaves", "lvl_parents"]:
        assert len(getattr(a, k)) == len(getattr(b, k))
        for x, y in zip(getattr(a, k), getattr(b, k)):
            assert np.array_equal(np.asarray(x), np.asarray(y)), k


@pytest.fixture(scope="module")
def lib():
    import build_lib
    build_lib.build()
    return ag.load_library()


@pytest.mark.parametrize("case", ["2d", "cyl", "3d"])
def test_native_matches_restatement(lib, case):
    rng = np.random.default_rng({"2d": 1, "cyl": 2, "3d": 3}[case])
    if case == "3d":
        tree = at.uniform_tree(3, 4, [8, 8, 8], [1e-2] * 3, 2)
        max_lvl = 5
    else:
        coord = at.AF_CYL if case == "cyl" else at.AF_XYZ
        tree = at.uniform_tree(2, 8, [16, 16], [1e-2, 1e-2], 2, coord=coord)
        max_lvl = 7
    changed = 0
    for it in range(25):
        # mostly refine early, mostly coarsen later
        p_do = 0.25 if it < 12 else 0.05
        p_rm = 0.1 if it < 12 else 0.6
        u = rng.random(tree.n_boxes)
        flags = np.where(u < p_do, at.AF_DO_REF, np.where(u < p_do + p_rm, at.AF_RM_REF, at.AF_KEEP_REF))
        flags = flags.astype(np.int32)
        py = at.adjust_refinement(tree, flags, max_lvl)
        nat = ag.adjust_refinement(tree, flags, max_lvl)
        if py is tree:
            assert nat is tree
            continue
        changed += 1
        same_tree(py, nat)
        tree = py
    assert changed >= 10


def test_native_rejects_bad_arguments(lib):
    tree = at.uniform_tree(2, 8, [16, 16], [1e-2, 1e-2], 2)
    with pytest.raises(ag.AfgError):
        ag.adjust_refinement(tree, np.zeros(tree.n_boxes, np.int32), 0)


def test_native_rejects_corrupted_descriptor(lib):
    """Level-list offsets that decrease or overrun the box count, box
    indices below 1 and box flags outside remove/keep/refine are argument
    errors, found before any table is indexed."""
    import ctypes as C
    tree = at.uniform_tree(2, 8, [16, 16], [1e-2, 1e-2], 3)
    flags = np.zeros(tree.n_boxes, np.int32)
    L = ag.load_library()

    def call(mutate, f=flags):
        holder = ag.TreeDescHolder(tree)
        mutate(holder)
        out = C.c_void_p()
        fl = np.ascontiguousarray(f, dtype=np.int32)
        return L.afg_adjust_refinement(C.byref(holder.desc), fl.ctypes.data_as(C.POINTER(C.c_int)), 5,
                                       C.byref(out))

    assert call(lambda h: None) == ag.AFG_OK
    assert call(lambda h: h.arrays["ids_off"].__setitem__(1, tree.n_boxes + 7)) == ag.AFG_ERR_ARG
    lo = ag.TreeDescHolder(tree).arrays["leaves_off"]
    assert call(lambda h: h.arrays["leaves_off"].__setitem__(2, lo[3] + 1)) == ag.AFG_ERR_ARG   # decreasing
    assert call(lambda h: h.arrays["parents_off"].__setitem__(0, -1)) == ag.AFG_ERR_ARG
    assert call(lambda h: h.arrays["ix"].__setitem__((3, 0), 0)) == ag.AFG_ERR_ARG
    bad = flags.copy()
    bad[5] = 7
    assert call(lambda h: None, bad) == ag.AFG_ERR_ARG
    bad[5] = -3
    assert call(lambda h: None, bad) == ag.AFG_ERR_ARG
