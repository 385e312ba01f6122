"""Shared streamer-model states for transport tests (CPU oracle and GPU)."""
import numpy as np

import afivo_gpu as ag
import streamer_model as sm
from mgcases import centers, refined_tree


def make_case(name):
    if name == "2d16":
        tree = refined_tree(2, 16, [32, 32], [1e-2, 1e-2], 5, 2, [0.5e-2, 0.8e-2], 0.6e-3, seed=1, frac=0.1)
    elif name == "2d8cyl":
        tree = refined_tree(2, 8, [16, 32], [1e-2, 2e-2], 5, 2, [0.0, 1.2e-2], 0.8e-3,
                            coord=ag.AFG_CYL, seed=2, frac=0.1)
    elif name == "3d8":
        tree = refined_tree(3, 8, [8, 8, 8], [2e-2, 2e-2, 2e-2], 4, 2, [1e-2, 1e-2, 1.2e-2], 1.5e-3,
                            seed=3, frac=0.05)
    else:
        raise KeyError(name)
    ions = [(1, 2.2e-4)] if name == "2d8cyl" else []
    model = sm.StreamerModel(tree.ndim, alpha=sm.baseline_alpha, eta=sm.baseline_eta, mobile_ions=ions,
                             photoi_modes=3)
    return tree, model


def initial_state(tree, model, seed=0, voltage=-3e4):
    """Seeded Gaussian electron/ion seed on a background, potential of a
    uniform field plus noise; E and |E| are derived later."""
    rng = np.random.default_rng(seed)
    cc = ag.new_cc(tree, model.n_var_cell)
    fc = ag.new_fc(tree, model.n_var_face)
    X = centers(tree)
    D = tree.ndim
    L = tree.dr[0] * tree.n_cell * (tree.coarse_grid_size / tree.n_cell)
    r2 = sum((X[:, d] - (0.5 * L[d] if not (tree.coord == ag.AFG_CYL and d == 0) else 0.0)) ** 2
             for d in range(D - 1)) + (X[:, D - 1] - 0.6 * L[D - 1]) ** 2
    seed_n = 1e15 * np.exp(-r2 / (2 * (0.6e-3) ** 2)) + 1e9
    for s in range(len(model.species)):
        base = seed_n if s < 2 else 0.1 * seed_n
        noise = 1 + 0.05 * rng.standard_normal(base.shape)
        cc[:, model.species_iv[s] - 1] = base * noise
    z = X[:, D - 1]
    cc[:, model.i_phi - 1] = voltage * z / L[D - 1] * (1 + 0.02 * rng.standard_normal(z.shape))
    return cc, fc
