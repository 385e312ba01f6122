"""The host restatement of the output writers (oracle_output) on known
answers: Fortran E20.8 and NINT, af_interp1 exact on linear data (the
multilinear interpolation reproduces a linear function, ghost cells
included), af_get_id_at returning the leaf that contains the point, the
af_write_vtk mesh layout, af_write_numpy's automatic grid; plus argument
errors of the output entry points without a device."""
import numpy as np
import pytest

import afivo_gpu as ag
import afivo_tree as at
import oracle_output as oo
from mgcases import centers, refined_tree


def test_fortran_e_known_answers():
    # gfortran: write(*, '(E20.8)') x
    assert oo.fortran_e(1.0) == "      0.10000000E+01"
    assert oo.fortran_e(-123.456) == "     -0.12345600E+03"
    assert oo.fortran_e(0.0) == "      0.00000000E+00"
    assert oo.fortran_e(0.5) == "      0.50000000E+00"
    assert oo.fortran_e(2.5e-3) == "      0.25000000E-02"
    assert oo.fortran_e(1e-100) == "      0.10000000E-99"
    assert oo.fortran_e(1e100) == "      0.10000000+101"
    assert oo.fortran_e(0.123456785) == "      0.12345678E+00" or oo.fortran_e(0.123456785) == "      0.12345679E+00"


def test_nint_halves_away_from_zero():
    assert [oo.nint(x) for x in (0.5, 1.5, 2.5, -0.5, -2.5, 0.49999999999999994, 3.0)] == [1, 2, 3, -1, -3, 0, 3]


@pytest.mark.parametrize("D", [2, 3])
def test_interp1_exact_on_linear_data(D):
    if D == 2:
        tree = refined_tree(2, 8, [16, 16], [1.0, 1.0], 4, 1, [0.3, 0.6], 0.1, seed=1, frac=0.1)
    else:
        tree = refined_tree(3, 4, [8, 8, 8], [1.0, 1.0, 1.0], 3, 1, [0.3, 0.6, 0.5], 0.15, seed=2, frac=0.1)
    X = centers(tree)
    coef = [0.7, -1.3, 2.1][:D]
    cc = ag.new_cc(tree, 1)
    cc[:, 0] = 3.0 + sum(coef[d] * X[:, d] for d in range(D))
    rng = np.random.default_rng(0)
    for _ in range(300):
        r = list(rng.random(D))
        (v,), ok = oo.interp1(tree, cc, r, [1])
        assert ok
        assert abs(v - (3.0 + sum(coef[d] * r[d] for d in range(D)))) < 1e-12
    assert oo.interp1(tree, cc, [1.5] * D, [1]) == ([0.0], False)


def test_get_id_at_finds_the_containing_leaf():
    tree = refined_tree(2, 8, [16, 16], [1.0, 1.0], 5, 1, [0.3, 0.6], 0.08, seed=3, frac=0.1)
    rng = np.random.default_rng(1)
    for _ in range(500):
        r = rng.random(2)
        b = oo.get_id_at(tree, r)
        assert b > 0 and not np.any(tree.children[b - 1] > 0)
        lo = tree.r_min[b - 1]
        assert np.all(r >= lo) and np.all(r <= lo + tree.dr[b - 1] * tree.n_cell)
    assert oo.get_id_at(tree, [-0.1, 0.5]) == -1


def test_vtk_layout():
    tree = at.uniform_tree(2, 4, [8, 8], [1.0, 1.0], 2)
    cc = ag.new_cc(tree, 1)
    a = oo.vtk_arrays(tree, cc, [1])
    nl = sum(len(l) for l in tree.lvl_leaves)
    assert len(a["points"]) == nl * 25 and len(a["offsets"]) == nl * 16
    assert list(a["connectivity"][:4]) == [0, 1, 5, 6]
    assert a["offsets"][-1] == 4 * nl * 16 and set(a["types"]) == {8}
    # the first leaf's first node is its r_min, single precision
    b = int(np.concatenate(tree.lvl_leaves)[0])
    assert np.array_equal(a["points"][0, :2], tree.r_min[b - 1].astype(np.float32))


def test_numpy_auto_grid_spacing():
    tree = at.uniform_tree(2, 4, [8, 8], [1.0, 2.0], 3)
    pts, nx, rmin, rmax, dr = oo.numpy_grid(tree)
    # leaves only on level 3: 4x the coarse grid
    assert nx == [32, 32] and rmax == [1.0, 2.0] and len(pts) == 32 * 32
    assert pts[0] == [0.5 * dr[0], 0.5 * dr[1]]


def test_output_entry_points_reject_null_context(gpu_lib):
    lib = ag.load_library()
    assert lib.afg_write_vtk(None, b"x", 0, 0.0, 0, None, None) == ag.AFG_ERR_ARG
    assert lib.afg_interp1(None, 0, None, 0, None, None, None) == ag.AFG_ERR_ARG
    assert lib.afg_leaf_cells(None, 1, None, None) == ag.AFG_ERR_ARG
    assert lib.afg_write_line(None, b"x", 0, None, None, None, None, 2) == ag.AFG_ERR_ARG
    assert lib.afg_write_plane(None, b"x", 0, None, None, None, None, None) == ag.AFG_ERR_ARG
    assert lib.afg_write_numpy(None, b"x.npy", None, None, None, 0, 0.0, 0, None, None) == ag.AFG_ERR_ARG
