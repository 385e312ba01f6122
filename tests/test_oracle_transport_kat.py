"""Known-answer tests of the CPU restatement's transport (no GPU).

A Gaussian electron cloud drifts in a uniform field on a refined 2D tree
(refinement boundaries cut through the cloud), with no reactions:

* the particle count over the leaves is conserved to round-off, which needs
  the consistent coarse fluxes at refinement boundaries
  (af_consistent_fluxes, afivo/src/m_af_core.f90:1257-1402) and the
  conservative update (flux_update_densities,
  afivo/src/m_af_flux_schemes.f90:320-436);
* the centre of mass moves with the drift velocity v = -mu E of the flux
  (src/m_fluid.f90:102-209) within 1%; diffusion leaves it unchanged;
* the density stays non-negative under the returned CFL time-step limit
  (Koren-limited upwinding, afivo/src/m_af_limiters.f90:72-95);
* with no field, the variance grows by 2 D t per dimension (the discrete
  Laplacian grows the second moment exactly by 2 D t on a uniform patch; the
  refinement boundaries the tail crosses allow 2%).
"""
import numpy as np
import pytest

import afivo_gpu as ag
import oracle
import streamer_model as sm
from mgcases import centers, refined_tree

L = 1e-2
V = -1e4                      # phi = V y / L, E_y = -V / L = 1e6 V/m


def setup(voltage=V):
    tree = refined_tree(2, 16, [32, 32], [L, L], 4, 2, [0.5e-2, 0.5e-2], 0.7e-3, seed=5, frac=0.0)
    model = sm.StreamerModel(2)       # no alpha/eta: the reaction rates vanish
    o = oracle.Oracle(tree, model.n_var_cell, model.n_var_face)
    o.transport_setup(model.transport_desc())
    o.set_cc_methods(model.i_electric_fld, *model.electric_fld_gc())
    for s in range(len(model.species)):
        for st in range(model.n_states):
            o.set_cc_methods(model.species_iv[s] + st, [model.bc_species] * 4, None, ag.RB_INTERP_LIM)
    o.mg_setup(0, model.field_mg(voltage))
    cc = ag.new_cc(tree, model.n_var_cell)
    fc = ag.new_fc(tree, model.n_var_face)
    X = centers(tree)
    cc[:, model.i_phi - 1] = voltage * X[:, 1] / L
    r2 = (X[:, 0] - 0.5e-2) ** 2 + (X[:, 1] - 0.5e-2) ** 2
    cc[:, model.species_iv[0] - 1] = 1e15 * np.exp(-r2 / (2 * (0.5e-3) ** 2))
    o.gc(cc, model.i_phi, 0, True)
    o.field_from_potential(cc, fc, model.i_phi)
    return tree, model, o, cc, fc


def leaf_moments(tree, a):
    leaves = np.concatenate(tree.lvl_leaves) - 1
    X = centers(tree)[leaves][:, :, 1:-1, 1:-1]
    n = a[leaves][:, 1:-1, 1:-1]
    vol = (tree.dr[leaves, 0] * tree.dr[leaves, 1])[:, None, None]
    m0 = np.sum(n * vol)
    cy = np.sum(n * vol * X[:, 1]) / m0
    vy = np.sum(n * vol * (X[:, 1] - cy) ** 2) / m0
    return m0, cy, vy, n.min(), n.max()


def advance(voltage, n_steps=20):
    tree, model, o, cc, fc = setup(voltage)
    iv = model.species_iv[0]
    before = leaf_moments(tree, cc[:, iv - 1])
    t = 0.0
    for _ in range(n_steps):
        lim = o.flux_upwind(cc, fc, 0)
        dt = 0.4 * min(lim[0], lim[1])
        o.update_densities(cc, fc, dt, 0, [0], [1.0], 1)
        for s in range(len(model.species)):
            j = model.species_iv[s] - 1
            cc[:, j] = cc[:, j + 1]
        t += dt
    after = leaf_moments(tree, cc[:, iv - 1])
    return model, before, after, t


@pytest.fixture(scope="module")
def run():
    return advance(V)


def test_particles_conserved(run):
    model, before, after, t = run
    assert abs(after[0] - before[0]) <= 1e-12 * before[0]


def test_centre_of_mass_drifts_with_minus_mu_e(run):
    model, before, after, t = run
    v = -model.mu * (-V / L)          # electrons: v = -mu E
    shift = after[1] - before[1]
    assert abs(shift - v * t) <= 0.01 * abs(v * t)


def test_non_negative(run):
    model, before, after, t = run
    assert after[3] >= -1e-12 * after[4]


def test_pure_diffusion_spread():
    model, before, after, t = advance(0.0, 40)
    assert abs(after[0] - before[0]) <= 1e-12 * before[0]
    assert abs(after[1] - before[1]) <= 1e-9 * L
    grow = after[2] - before[2]
    assert abs(grow - 2 * model.dif * t) <= 0.02 * 2 * model.dif * t
