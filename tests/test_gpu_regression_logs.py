"""Whole runs of the reference's regression configurations on the GPU.

The `streamer` program loop (streamer_program.Program) runs the
reference's regression configurations (standard_2d and standard_3d tests)
with every numerical stage on the device (GpuEngine, through the C-ABI):
field solves, fluxes, updates, refinement flags, restriction, prolongation
into new boxes and the data move to each new mesh.  The FP64 path gives the
CPU restatement's regression rows bit for bit (the same meshes, steps,
rejections and values); both follow the reference's stored logs within the
bounds its pinning test states.  The mixed-precision path (FP32 inner
multigrid and transport, FP64 state) runs the same program; its density
columns stay within per-configuration bounds of the logs.
"""
import functools
import os

import numpy as np
import pytest

import afivo_gpu as ag
import streamer_program as sp

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "standard_2d")
CASES = ["test_2d", "test_cyl", "test_2d_photoi", "test_cyl_chem", "test_2d_photoi_chem",
         "test_cyl_ion_motion", "test_cyl_ion_motion_v2", "test_3d", "test_3d_chem", "test_3d_photoi_chem",
         "test_cyl_photoi_chem"]
# the electrode runs (grounded rod, positive and negative field, without and
# with photoionization): FP64 only, the electrode operator has no FP32 solve
FP64_CASES = CASES + ["test_2d_pos_electrode", "test_2d_neg_electrode", "test_2d_pos_electrode_photoi",
                      "test_2d_neg_electrode_photoi"]

# FP64 GPU rows against the restatement's: identical (every stage is
# bit-exact, the first smoothing of a solve reads the stored ghost cells as
# the reference's does, and the analytic rates use the same exp/pow)
FP64_VS_ORACLE = 0.0
# every row against the reference's logs: the restatement's own bounds
# (test_oracle_regression_logs.CASES), the rows being identical
# mixed precision against the logs, density columns: the observed maximum
# per configuration, rounded up (the axisymmetric runs are the most sensitive:
# the maxima of e and N2+ on the axis at the streamer head).
# The dt column is the step chosen for the next step and is compared for the
# FP64 path only: after a rejected step the mixed run may pick a different
# step size (test_cyl_chem's 1.25 ns row).
MIXED_VS_LOG = {
    "test_2d": 1e-5,
    "test_cyl": 8e-3,
    "test_2d_photoi": 3e-5,
    "test_cyl_chem": 5e-2,
    "test_2d_photoi_chem": 1.5e-3,
    "test_cyl_ion_motion": 3e-4,
    "test_cyl_ion_motion_v2": 5e-3,
    "test_3d": 2e-5,
    "test_3d_chem": 7e-4,
    "test_3d_photoi_chem": 5e-4,
    "test_cyl_photoi_chem": 1e-3,
}


def rel_err(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


def case_paths(name):
    if name.startswith("test_3d"):
        g = os.path.join(os.path.dirname(GOLD), "standard_3d")
        return os.path.join(g, name + ".cfg"), os.path.join(g, name + "_rtest.log"), 3
    return os.path.join(GOLD, name + ".cfg"), os.path.join(GOLD, name + "_rtest.log"), 2


def run(name, factory):
    cfg_path, _, ndim = case_paths(name)
    cfg = sp.ProgramConfig(cfg_path, ndim=ndim)
    prog = sp.Program(cfg, factory)
    prog.set_initial_conditions()
    rows = np.array(prog.run())
    if hasattr(prog.engine, "close"):
        prog.engine.close()
    return prog, rows


@pytest.mark.gpu
@pytest.mark.parametrize("name", FP64_CASES)
def test_fp64_run_matches_restatement_and_log(gpu_lib, name):
    import oracle_program as op
    po, ro = run(name, op.OracleEngine)
    pg, rg = run(name, functools.partial(sp.GpuEngine, precision=ag.FP64))
    head, ref = sp.read_regression_log(case_paths(name)[1])
    assert pg.n_steps == po.n_steps and pg.n_rejected == po.n_rejected
    assert rg.shape == ro.shape == ref.shape
    err = rel_err(rg[:, 1:], ro[:, 1:])
    err[np.abs(ro[:, 1:]) == 0] = np.abs(rg[:, 1:])[np.abs(ro[:, 1:]) == 0]
    print(f"{name}: FP64 GPU vs restatement per row", " ".join(f"{x:.1e}" for x in err.max(axis=1)))
    print(f"{name}: FP64 GPU vs restatement max rel {err.max():.3e}; "
          f"vs log {rel_err(rg[:, 2:], ref[:, 2:])[ref[:, 2:] != 0].max():.3e}")
    assert err.max() <= FP64_VS_ORACLE
    assert np.array_equal(rg, ro)
    from test_oracle_regression_logs import CASES as ORACLE_BOUNDS
    assert np.allclose(rg[:, 2:], ref[:, 2:], rtol=ORACLE_BOUNDS[name], atol=1e-8)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_mixed_run_matches_log(gpu_lib, name):
    pm, rm = run(name, functools.partial(sp.GpuEngine, precision=ag.MIXED))
    head, ref = sp.read_regression_log(case_paths(name)[1])
    assert rm.shape == ref.shape
    assert np.allclose(rm[:, 1], ref[:, 1], rtol=1e-12, atol=0)
    e = rel_err(rm[:, 3:], ref[:, 3:])[ref[:, 3:] != 0]
    print(f"{name}: mixed GPU vs log max rel {e.max():.3e} ({pm.n_steps} steps, {pm.n_rejected} rejected)")
    assert np.allclose(rm[:, 3:], ref[:, 3:], rtol=MIXED_VS_LOG[name], atol=1e-8)

