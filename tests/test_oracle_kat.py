"""Known-answer tests that pin the CPU oracle (no GPU).

The reference stores no per-kernel golden vectors; its examples check the
multigrid against analytic solutions (afivo/examples/poisson_basic.f90,
poisson_helmholtz.f90, poisson_cyl_analytic.f90) and its ghost-cell test
checks that ghost cells of a zero field stay zero
(afivo/tests/test_ghostcell.f90, answer "Success").  These tests restate
those checks for the oracle: second-order convergence to manufactured
solutions (Cartesian 2D/3D, cylindrical, Helmholtz), V-cycle convergence
factors, exactness of the ghost rules on linear fields, and zero ghosts.
"""
import numpy as np
import pytest

import afivo_gpu as ag
import afivo_tree as at
import oracle
from mgcases import I_PHI, I_RHS, I_TMP, interior, leaf_error, sine_problem, refined_tree, centers


def solve_oracle(tree, lambda2=0.0, cyl=False, rel=1e-10):
    phi_ex, rhs, bc = sine_problem(tree, lambda2, cyl)
    cc = ag.new_cc(tree, 3)
    cc[:, I_RHS - 1] = rhs
    o = oracle.Oracle(tree, 3)
    o.mg_setup(0, ag.mg_desc(I_PHI, I_RHS, I_TMP, bc, lambda2=lambda2))
    o.gc(cc, I_PHI)
    thr = rel * o.maxabs(cc, I_RHS)
    o.mg_fmg(cc, 0, True, False)
    n, res = o.mg_solve(cc, 0, thr, 30)
    assert res[-1] < thr, res
    return leaf_error(tree, cc, phi_ex), res


@pytest.mark.parametrize("lambda2", [0.0, 30.0])
def test_poisson_2d_second_order(lambda2):
    errs = []
    for lv in (3, 4, 5):
        t = at.uniform_tree(2, 8, [16, 16], [1.0, 1.0], lv)
        e, _ = solve_oracle(t, lambda2)
        errs.append(e)
    ratios = [errs[i] / errs[i + 1] for i in range(len(errs) - 1)]
    assert all(3.5 < r < 4.5 for r in ratios), (errs, ratios)


def test_poisson_3d_second_order():
    errs = []
    for lv in (2, 3, 4):
        t = at.uniform_tree(3, 8, [8, 8, 8], [1.0, 1.0, 1.0], lv)
        e, _ = solve_oracle(t)
        errs.append(e)
    ratios = [errs[i] / errs[i + 1] for i in range(len(errs) - 1)]
    assert all(3.3 < r < 4.7 for r in ratios), (errs, ratios)


def test_poisson_cyl_second_order():
    errs = []
    for lv in (3, 4, 5):
        t = at.uniform_tree(2, 8, [8, 16], [1.0, 2.0], lv, coord=ag.AFG_CYL)
        e, _ = solve_oracle(t, cyl=True)
        errs.append(e)
    ratios = [errs[i] / errs[i + 1] for i in range(len(errs) - 1)]
    assert all(3.3 < r < 4.7 for r in ratios), (errs, ratios)


@pytest.mark.parametrize("cyl", [False, True])
def test_amr_tree_converges(cyl):
    coord = ag.AFG_CYL if cyl else ag.AFG_XYZ
    cgs, L = ([8, 16], [1.0, 2.0]) if cyl else ([16, 16], [1.0, 1.0])
    t = refined_tree(2, 8, cgs, L, 6, 3, [0.3, 0.6], 0.08, coord=coord)
    assert any(len(l) > 0 for l in t.lvl_leaves[:-1])  # truly adaptive
    e, res = solve_oracle(t, cyl=cyl)
    # V-cycle convergence factor of afivo's FAS cycle on this problem
    fac = (res[-1] / res[0]) ** (1.0 / max(1, len(res) - 1))
    assert fac < 0.25, res
    assert e < 5e-3


def test_zero_field_zero_ghosts():
    """test_ghostcell.f90: after refinement, ghost cells of zero data are 0."""
    t = refined_tree(2, 8, [16, 16], [1.0, 1.0], 5, 2, [0.5, 0.5], 0.1)
    cc = ag.new_cc(t, 1)
    o = oracle.Oracle(t, 1)
    for rb in (ag.RB_MG_SIDES, ag.RB_INTERP, ag.RB_INTERP_LIM):
        o.set_cc_methods(1, [ag.BC_DIRICHLET, ag.BC_NEUMANN, ag.BC_CONTINUOUS, ag.BC_DIRICHLET_COPY], rb=rb)
        cc[:] = 0
        o.gc(cc, 1, 0, True)
        assert np.all(cc == 0)


@pytest.mark.parametrize("ndim", [2, 3])
def test_linear_field_exact_ghosts(ndim):
    """A linear field is reproduced exactly by same-level copies, the
    continuous boundary rule, mg_sides_rb and af_gc_interp (up to rounding),
    as in afivo/examples/check_ghostcells.f90."""
    if ndim == 2:
        t = refined_tree(2, 8, [16, 16], [1.0, 1.0], 4, 2, [0.4, 0.6], 0.1)
        a = np.array([0.3, -0.7])
    else:
        t = refined_tree(3, 4, [8, 8, 8], [1.0, 1.0, 1.0], 3, 1, [0.4, 0.6, 0.5], 0.15)
        a = np.array([0.3, -0.7, 0.45])
    X = centers(t)
    f = 1.0 + sum(a[d] * X[:, d] for d in range(ndim))
    for rb in (ag.RB_MG_SIDES, ag.RB_INTERP):
        cc = ag.new_cc(t, 1)
        inner = interior(t)
        cc[(slice(None), 0) + inner] = f[(slice(None),) + inner]
        o = oracle.Oracle(t, 1)
        o.set_cc_methods(1, [ag.BC_CONTINUOUS] * (2 * ndim), rb=rb)
        # coarse levels first: refinement ghosts read the parent's neighbours
        o.gc(cc, 1, 0, False)
        face = np.zeros_like(cc[:, 0], dtype=bool)
        n2 = t.n_cell + 2
        for d in range(ndim):
            for x in (0, n2 - 1):
                sl = [slice(1, n2 - 1)] * ndim
                sl[ndim - 1 - d] = x
                face[(slice(None),) + tuple(sl)] = True
        err = np.max(np.abs(cc[:, 0][face] - f[face]))
        assert err < 1e-12, (rb, err)
