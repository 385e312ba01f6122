"""GPU transport / field / photoionization parity against the CPU oracle
(FP64), through the C-ABI: field from potential, Koren upwind fluxes with
two-layer ghost cells and consistent coarse fluxes, density + chemistry
update (Euler and Heun stages), Poisson right-hand side, field_compute and
the Helmholtz photoionization source.  Tabulated-rate arithmetic is bit
exact; composite solves within 1e-12 relative."""
import numpy as np
import pytest

import afivo_gpu as ag
import oracle
from streamer_cases import initial_state, make_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["2d16", "2d8cyl", "3d8"])
def pair(request, gpu_lib):
    tree, model = make_case(request.param)
    ctx = ag.Context(0)
    ctx.tree_sync(tree, model.n_var_cell, model.n_var_face)
    o = oracle.Oracle(tree, model.n_var_cell, model.n_var_face)
    desc = model.transport_desc()
    ctx.transport_setup(desc)
    o.transport_setup(desc)
    for obj in (ctx, o):
        obj.set_cc_methods(model.i_electric_fld, *model.electric_fld_gc())
        for s in range(len(model.species)):
            for st in range(model.n_states):
                obj.set_cc_methods(model.species_iv[s] + st, [model.bc_species] * (2 * tree.ndim), None,
                                   ag.RB_INTERP_LIM)
        if model.i_photo:
            obj.set_cc_methods(model.i_photo, *model.photo_gc())
    mg = model.field_mg(-3e4)
    ctx.mg_setup(0, mg)
    o.mg_setup(0, mg)
    yield request.param, tree, model, ctx, o
    ctx.close()


def prepared(tree, model, ctx, o, seed=0):
    cc, fc = initial_state(tree, model, seed)
    o.gc(cc, model.i_phi, 0, True)
    ctx.upload(cc)
    ctx.upload_fc(fc)
    ctx.field_from_potential(model.i_phi)
    o.field_from_potential(cc, fc, model.i_phi)
    return cc, fc


def dl(ctx, tree, model):
    cc = ag.new_cc(tree, model.n_var_cell)
    fc = ag.new_fc(tree, model.n_var_face)
    ctx.download(cc)
    ctx.download_fc(fc)
    return cc, fc


def leaf_interior(tree, a):
    leaves = np.concatenate(tree.lvl_leaves) - 1
    n2 = tree.n_cell + 2
    return a[leaves][(slice(None),) + (slice(1, n2 - 1),) * tree.ndim]


def test_field_from_potential_bitexact(pair):
    name, tree, model, ctx, o = pair
    cc, fc = prepared(tree, model, ctx, o)
    gcc, gfc = dl(ctx, tree, model)
    assert np.array_equal(gfc[:, model.f_efield - 1], fc[:, model.f_efield - 1])
    assert np.array_equal(gcc[:, model.i_electric_fld - 1], cc[:, model.i_electric_fld - 1])


def test_flux_and_update_bitexact(pair):
    name, tree, model, ctx, o = pair
    cc, fc = prepared(tree, model, ctx, o, seed=1)
    dt_g = ctx.flux_upwind(0)
    dt_c = o.flux_upwind(cc, fc, 0)
    assert np.array_equal(dt_g, dt_c), (dt_g, dt_c)
    gcc, gfc = dl(ctx, tree, model)
    for f in model.f_flux:
        assert np.array_equal(gfc[:, f - 1], fc[:, f - 1]), f"flux {f}: {np.max(np.abs(gfc[:, f-1] - fc[:, f-1]))}"
    for s in range(len(model.species)):
        iv = model.species_iv[s]
        assert np.array_equal(gcc[:, iv - 1], cc[:, iv - 1]), f"species {s} ghosts/restriction"
    # Euler stage: s_out = 1 from s_prev = 0
    chem_g = ctx.update_densities(1e-12, 0, [0], [1.0], 1, last_step=True)
    chem_c = o.update_densities(cc, fc, 1e-12, 0, [0], [1.0], 1, last_step=True)
    assert chem_g == chem_c
    gcc, _ = dl(ctx, tree, model)
    for s in range(len(model.species)):
        iv = model.species_iv[s] + 1
        a, b = leaf_interior(tree, gcc[:, iv - 1]), leaf_interior(tree, cc[:, iv - 1])
        assert np.array_equal(a, b), f"species {s}: {np.max(np.abs(a - b) / np.abs(b))}"
    # Heun second stage: state 0 = 0.5 * (0 + 1) + dt * f(1)
    ctx.field_set_rhs(model.i_rhs, 1)
    o.field_set_rhs(cc, model.i_rhs, 1)
    dt_g = ctx.flux_upwind(1)
    dt_c = o.flux_upwind(cc, fc, 1)
    assert np.array_equal(dt_g, dt_c)
    ctx.update_densities(0.5e-12, 1, [0, 1], [0.5, 0.5], 0, last_step=False)
    o.update_densities(cc, fc, 0.5e-12, 1, [0, 1], [0.5, 0.5], 0, last_step=False)
    gcc, _ = dl(ctx, tree, model)
    leaves = np.concatenate(tree.lvl_leaves) - 1
    assert np.array_equal(gcc[leaves, model.i_rhs - 1], cc[leaves, model.i_rhs - 1])
    for s in range(len(model.species)):
        iv = model.species_iv[s]
        a, b = leaf_interior(tree, gcc[:, iv - 1]), leaf_interior(tree, cc[:, iv - 1])
        assert np.array_equal(a, b), f"heun species {s}"


def test_field_compute_fp64(pair):
    """field_compute: rhs from charges, FMG start, V-cycles to 1e-10, E."""
    name, tree, model, ctx, o = pair
    cc, fc = prepared(tree, model, ctx, o, seed=2)
    V = -3e4
    L = float(tree.dr[0, -1] * tree.coarse_grid_size[-1])
    n_g, r_g = ctx.field_compute(0, 0, False, V, L, 1e-10, 10)
    # oracle composition of field_compute (src/m_field.f90:448-528)
    o.field_set_rhs(cc, model.i_rhs, 0)
    o.mg_set_bc_values(0, model.field_bc(V)[1])
    max_rhs = o.maxabs(cc, model.i_rhs)
    min_dr = float(np.min(tree.dr[tree.lvl_ids[-1][0] - 1]))
    thr = max(1e-6, max_rhs * 1e-10, 1e-10 * abs(V) / (L * min_dr))
    res = []
    for i in range(100):
        res.append(o.mg_fmg(cc, 0, True, True))
        if res[-1] < thr:
            break
        if i >= 2:
            ratio = min(res[-3:]) / max(res[-3:])
            if 0.5 < ratio < 2.0 and res[-1] < 1e8:
                break
    n_v, _ = o.mg_solve(cc, 0, thr, 10)
    o.field_from_potential(cc, fc, model.i_phi)
    gcc, gfc = dl(ctx, tree, model)
    assert n_g == len(res) + n_v
    leaves = np.concatenate(tree.lvl_leaves) - 1
    a, b = gcc[leaves, model.i_electric_fld - 1], cc[leaves, model.i_electric_fld - 1]
    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))


def test_photoionization_fp64(pair):
    name, tree, model, ctx, o = pair
    cc, fc = prepared(tree, model, ctx, o, seed=3)
    lam = np.array([0.05, 0.15, 0.5]) * 1e3 * 0.1      # 1/(m bar) at 0.1 bar O2 partial pressure
    coeffs = np.array([1e-2, 5e-2, 1e-1]) * 1e6 * 0.01
    mgs = model.helmholtz_mg(lam)
    for n, m in enumerate(mgs):
        ctx.mg_setup(1 + n, m)
        o.mg_setup(1 + n, m)
    coeff = 0.6 * 0.038
    ctx.photoi_helmh(coeff, [1, 2, 3], coeffs, 1e-2, 10)
    # oracle composition of photoi_helmh_compute (src/m_photoi_helmh.f90:162-204)
    o.photoi_source(cc, coeff, model.i_rhs)
    cc[:, model.i_photo - 1] = 0
    max_rhs = max(o.maxabs(cc, model.i_rhs), np.sqrt(np.finfo(float).eps))
    leaves = np.concatenate(tree.lvl_leaves) - 1
    for n in range(3):
        for i in range(10):
            r = o.mg_fmg(cc, 1 + n, True, True)
            if r / max_rhs < 1e-2:
                break
        cc[leaves, model.i_photo - 1] -= coeffs[n] * cc[leaves, model.i_modes[n] - 1]
    gcc, _ = dl(ctx, tree, model)
    a, b = gcc[leaves, model.i_photo - 1], cc[leaves, model.i_photo - 1]
    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
