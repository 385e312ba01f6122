"""The electrode (level-set) restatement on known answers: concentric
electrodes at the voltage and grounded, whose potential between them is
analytic (2D Cartesian: log r, axisymmetric: 1/r), solved by FMG and
V-cycles; the error in the annulus falls at second order with the grid
spacing.  Plus the set-up's invariants: electrode boxes on level 1, the
stencils' row sums, boundary distances in (0, 1], bc_correction = f * V."""
import numpy as np
import pytest

import afivo_gpu as ag
import oracle
from lsfcases import (I_LSF, I_PHI, N_VAR, coaxial_desc, coaxial_exact, coaxial_tree, mg_desc_for, case)
from mgcases import centers


def solve_coaxial(nref, cyl):
    tree = coaxial_tree(nref, cyl)
    o = oracle.Oracle(tree, N_VAR)
    o.mg_setup(0, mg_desc_for(tree))
    cc = ag.new_cc(tree, N_VAR)
    d, cen = coaxial_desc(cyl)
    o.mg_set_lsf(cc, 0, d)
    o.mg_set_lsf_voltage(0, 1.0)
    o.gc(cc, I_PHI, 0, True)
    res = o.mg_fmg(cc, 0, True, False)
    for _ in range(10):
        res = o.mg_vcycle(cc, 0, True)
    X = centers(tree)
    r = np.sqrt((X[:, 0] - cen[0]) ** 2 + (X[:, 1] - cen[1]) ** 2)
    leaves = np.concatenate(tree.lvl_leaves) - 1
    phi = cc[leaves, I_PHI - 1][:, 1:-1, 1:-1]
    rr = r[leaves][:, 1:-1, 1:-1]
    m = (rr > 0.12) & (rr < 0.38)
    return np.max(np.abs(phi[m] - coaxial_exact(rr[m], cyl))), res


@pytest.mark.parametrize("cyl", [False, True])
def test_concentric_electrodes_converge_to_analytic(cyl):
    errs = []
    for nref in (1, 2, 3):
        err, res = solve_coaxial(nref, cyl)
        assert res < 1e-9
        errs.append(err)
    # second order in dx (ratios ~4, at least 2.5 here), small on the finest
    assert errs[0] / errs[1] > 2.5 and errs[1] / errs[2] > 2.5, errs
    assert errs[2] < (2e-3 if cyl else 5e-4), errs


@pytest.mark.parametrize("name", ["2d_rod", "2d_cyl_cone", "3d_sphere"])
def test_setup_invariants(name):
    tree, d, volt = case(name)
    o = oracle.Oracle(tree, N_VAR)
    o.mg_setup(0, mg_desc_for(tree))
    cc = ag.new_cc(tree, N_VAR)
    o.mg_set_lsf(cc, 0, d)
    o.mg_set_lsf_voltage(0, volt)
    ids, v, f, bcc, dd = o.mg_lsf_info(0)
    assert len(ids) > 0 and any(tree.lvl[i - 1] == 1 for i in ids)
    assert np.all(dd > 0) and np.all(dd <= 1) and np.any(dd < 1)
    # v[0] = -(sum of the neighbours' coefficients before the boundary
    # couplings moved into f = -(their sum)): row sum - f = 0 up to rounding
    rowsum = v.sum(axis=1) - f
    assert np.max(np.abs(rowsum)) <= 1e-9 * np.max(np.abs(v[:, 0]))
    assert np.array_equal(bcc, f * (0.0 if d.grounded else volt))
    # couplings across a boundary point are moved out of the stencil
    D = tree.ndim
    for n in range(2 * D):
        assert np.all(v[:, n + 1][dd[:, n] < 1] == 0)
        if tree.coord != ag.AFG_CYL:  # (on the axis the 1/r term cancels the inner coupling)
            assert np.all(v[:, n + 1][dd[:, n] == 1] != 0)
    # the level-set values are the electrode's: inside negative
    lsf = cc[:, I_LSF - 1]
    assert np.min(lsf) < 0 < np.max(lsf)


def test_no_root_on_level_one_is_an_error():
    tree = coaxial_tree(1)
    o = oracle.Oracle(tree, N_VAR)
    o.mg_setup(0, mg_desc_for(tree))
    cc = ag.new_cc(tree, N_VAR)
    d = ag.lsf_desc(ag.LSF_SPHERE, I_LSF, r0=[5.0, 5.0], radius=0.1)  # outside the domain
    with pytest.raises(RuntimeError):
        o.mg_set_lsf(cc, 0, d)
