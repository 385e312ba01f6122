"""Shared electrode (level-set) problems for the CPU and GPU tests."""
import numpy as np

import afivo_gpu as ag
import afivo_tree as at
from mgcases import refined_tree

I_PHI, I_RHS, I_TMP, I_LSF = 1, 2, 3, 4
N_VAR = 4


def coaxial_tree(nref, cyl=False):
    return at.uniform_tree(2, 8, [16, 16], [1.0, 1.0], nref, coord=ag.AFG_CYL if cyl else ag.AFG_XYZ)


def coaxial_desc(cyl=False, r1=0.1, r2=0.4):
    """Concentric electrodes (coaxial_lsf, src/m_field.f90:846-878): in 2D
    Cartesian coordinates circles about (0.5, 0.5), in axisymmetric ones
    spheres about (0, 0.5) on the axis; the inner one at the voltage."""
    cen = [0.0 if cyl else 0.5, 0.5]
    return ag.lsf_desc(ag.LSF_COAXIAL, I_LSF, r0=[0, 0], radius=r1, radius2=r2, center=cen), cen


def coaxial_exact(r, cyl, r1=0.1, r2=0.4):
    if cyl:
        return (1 / r - 1 / r2) / (1 / r1 - 1 / r2)
    return np.log(r / r2) / np.log(r1 / r2)


def mg_desc_for(tree, precision=ag.FP64):
    D = tree.ndim
    cyl = tree.coord == ag.AFG_CYL
    bt = [ag.BC_NEUMANN if (cyl and k == 0) else ag.BC_DIRICHLET for k in range(2 * D)]
    return ag.mg_desc(I_PHI, I_RHS, I_TMP, bt, [0.0] * (2 * D), precision=precision)


# electrode cases of the parity tests: (tree, electrode description, voltage)
def case(name):
    if name == "2d_rod":
        # test_2d_pos_electrode's rod: from (0.5, 0) to (0.5, 0.15) times the
        # domain, radius 1 mm, in a 32 mm square
        tree = refined_tree(2, 8, [16, 16], [32e-3, 32e-3], 5, 2, [16e-3, 5e-3], 2e-3, seed=5, frac=0.1)
        d = ag.lsf_desc(ag.LSF_ROD, I_LSF, r0=[16e-3, 0.0], r1=[16e-3, 4.8e-3], radius=1e-3)
        return tree, d, 2.5e4
    if name == "2d_cyl_cone":
        tree = refined_tree(2, 8, [16, 32], [16e-3, 32e-3], 5, 2, [0.0, 8e-3], 2e-3, coord=ag.AFG_CYL, seed=6,
                            frac=0.1)
        d = ag.lsf_desc(ag.LSF_ROD_CONE_TOP, I_LSF, r0=[0.0, 0.0], r1=[0.0, 8e-3], radius=1.5e-3,
                        cone_tip_radius=3e-4, cone_length_frac=0.3)
        return tree, d, -3e4
    if name == "2d_coaxial":
        tree = refined_tree(2, 8, [16, 16], [1.0, 1.0], 4, 1, [0.5, 0.6], 0.1, seed=7, frac=0.1)
        d, _ = coaxial_desc(False)
        return tree, d, 1.0
    if name == "2d_rod_rod":
        tree = refined_tree(2, 8, [16, 16], [1.0, 1.0], 4, 2, [0.5, 0.5], 0.08, seed=8, frac=0.1)
        d = ag.lsf_desc(ag.LSF_ROD_ROD, I_LSF, r0=[0.5, 0.0], r1=[0.5, 0.35], radius=0.04,
                        r2_0=[0.5, 0.65], r2_1=[0.5, 1.0], radius2=0.04, grounded2=True)
        return tree, d, 1e4
    if name == "3d_rod":
        tree = refined_tree(3, 8, [16, 16, 16], [16e-3, 16e-3, 16e-3], 4, 2, [8e-3, 8e-3, 5e-3], 1.5e-3, seed=9,
                            frac=0.05)
        d = ag.lsf_desc(ag.LSF_ROD, I_LSF, r0=[8e-3, 8e-3, 0.0], r1=[8e-3, 8e-3, 4e-3], radius=1e-3)
        return tree, d, 2e4
    if name == "3d_sphere":
        tree = refined_tree(3, 8, [16, 16, 16], [1.0, 1.0, 1.0], 3, 1, [0.5, 0.5, 0.5], 0.15, seed=10, frac=0.05)
        d = ag.lsf_desc(ag.LSF_SPHERE, I_LSF, r0=[0.5, 0.5, 0.5], radius=0.2)
        return tree, d, 1.0
    raise KeyError(name)


CASES = ["2d_rod", "2d_cyl_cone", "2d_coaxial", "2d_rod_rod", "3d_rod", "3d_sphere"]


def initial(tree, seed):
    """Random rhs and phi (every cell, ghost cells included)."""
    rng = np.random.default_rng(seed)
    cc = ag.new_cc(tree, N_VAR)
    cc[:, I_PHI - 1] = rng.standard_normal(cc[:, 0].shape)
    cc[:, I_RHS - 1] = rng.standard_normal(cc[:, 0].shape) * 1e6
    return cc
