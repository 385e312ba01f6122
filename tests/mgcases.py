"""Shared problem setups for the multigrid tests (CPU oracle and GPU)."""
import numpy as np

import afivo_gpu as ag
import afivo_tree as at

I_PHI, I_RHS, I_TMP = 1, 2, 3


def interior(tree):
    n2 = tree.n_cell + 2
    return (slice(1, n2 - 1),) * tree.ndim


def centers(tree):
    """cell centres of every box: array [n, D, (k,) j, i] incl. ghost layer"""
    nc, D = tree.n_cell, tree.ndim
    n2 = nc + 2
    idx = np.arange(n2, dtype=np.float64) - 0.5
    out = np.empty((tree.n_boxes, D) + (n2,) * D)
    for d in range(D):
        shape = [1] * D
        shape[D - 1 - d] = n2
        r = tree.r_min[:, d][:, None] + idx[None, :] * tree.dr[:, d][:, None]
        out[:, d] = r.reshape((tree.n_boxes,) + tuple(shape))
    return out


def sine_problem(tree, lambda2=0.0, cyl=False):
    """Manufactured solution vanishing on Dirichlet faces.

    Cartesian: phi = prod_d sin(pi x_d / L_d) (Dirichlet 0 on all faces).
    Cylindrical: phi = cos(pi r / (2R)) sin(pi z / Z) (Neumann on the axis,
    Dirichlet 0 elsewhere).  Returns (phi_exact on cell centres, rhs, bc).
    """
    X = centers(tree)
    D = tree.ndim
    L = tree.dr[0] * tree.n_cell * (tree.coarse_grid_size / tree.n_cell)
    if not cyl:
        phi = np.ones(X.shape[:1] + X.shape[2:])
        for d in range(D):
            phi = phi * np.sin(np.pi * X[:, d] / L[d])
        k2 = sum((np.pi / L[d]) ** 2 for d in range(D))
        rhs = -(k2 + lambda2) * phi
        bc = [ag.BC_DIRICHLET] * (2 * D)
    else:
        r, z = X[:, 0], X[:, 1]
        k, m = np.pi / (2 * L[0]), np.pi / L[1]
        fr, fz = np.cos(k * r), np.sin(m * z)
        phi = fr * fz
        rhs = (-k * k * fr - k * np.sin(k * r) / r) * fz - m * m * fr * fz - lambda2 * phi
        bc = [ag.BC_NEUMANN, ag.BC_DIRICHLET, ag.BC_DIRICHLET, ag.BC_DIRICHLET]
    return phi, rhs, bc


def leaf_error(tree, cc, phi_exact, iv=I_PHI):
    inner = interior(tree)
    leaves = np.concatenate(tree.lvl_leaves) - 1
    a = cc[leaves, iv - 1][(slice(None),) + inner]
    b = phi_exact[leaves][(slice(None),) + inner]
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def random_state(tree, n_var, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    cc = ag.new_cc(tree, n_var)
    cc[:] = rng.standard_normal(cc.shape) * scale
    return cc


def refined_tree(ndim, nc, cgs, L, max_lvl, base_lvl, center, sigma, coord=ag.AFG_XYZ, seed=None, frac=0.0):
    rng = np.random.default_rng(seed) if seed is not None else None
    return at.build_tree(ndim, nc, cgs, L, coord=coord, max_lvl=max_lvl,
                         refine=at.seeded_refinement(center, sigma, base_lvl, rng, frac))
