"""CPU restatement of one time step of the streamer hot path.

Test and baseline infrastructure only: the tests compare the GPU time step
with it, and the benchmark times it as the CPU baseline.  It drives the C++
restatement (``oracle.Oracle``) in the order of the reference's time loop
(src/streamer.f90:181-432):

* photoionization every `photoi_per_steps` steps (photoi_set_src,
  src/streamer.f90:242-248): photon production on the leaves
  (src/m_photoi_helmh.f90:162-204 via photoi_get_source), then per Helmholtz
  mode FMG cycles until the residual drops below 1e-2 of the source maximum,
  and i_photo -= c_n * mode_n on the leaves;
* copy_current_state (src/streamer.f90:659-671);
* an explicit integrator of af_advance (afivo/src/m_af_advance.f90:150-199;
  Heun's method by default) whose stages are forward_euler
  (src/m_fluid.f90:21-99): field_compute (src/m_field.f90:450-520) of the
  stage's input state from the second stage on, fluxes of that state and the
  densities of the stage; then the field of the new state.

`step()` returns the cell-updates of the step with the same accounting as the
GPU counters: smoother updates of every V-cycle ((n_cycle_down + n_cycle_up)
times the cells of levels 2..max_lvl) plus leaf cells x species per stage.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(HERE, "..", "afivo-streamer_gb300"))

import afivo_gpu as ag  # noqa: E402
import afivo_tree as at  # noqa: E402
import oracle  # noqa: E402


_THIRD, _SIXTH = 1 / 3.0, 1 / 6.0

# forward_euler calls of af_advance's explicit integrators
# (afivo/src/m_af_advance.f90:150-199): (dt factor, s_deriv, s_prev, w_prev,
# s_out) per stage
STAGES = {
    "forward_euler": [(1.0, 0, [0], [1.0], 0)],
    "midpoint": [(0.5, 0, [0], [1.0], 1), (1.0, 1, [0], [1.0], 0)],
    "heun": [(1.0, 0, [0], [1.0], 1), (0.5, 1, [0, 1], [0.5, 0.5], 0)],
    "ssprk33": [(1.0, 0, [0], [1.0], 1), (0.25, 1, [0, 1], [0.75, 0.25], 2),
                (2 * _THIRD, 2, [0, 2], [_THIRD, 2 * _THIRD], 0)],
    "ssprk43": [(0.5, 0, [0], [1.0], 1), (0.5, 1, [1], [1.0], 2),
                (_SIXTH, 2, [0, 2], [2 * _THIRD, _THIRD], 3), (0.5, 3, [3], [1.0], 0)],
    "rk4": [(0.5, 0, [0], [1.0], 1), (0.5, 1, [0], [1.0], 2), (1.0, 2, [0], [1.0], 3),
            (_SIXTH, 3, [0, 1, 2, 3], [-_THIRD, _THIRD, 2 * _THIRD, _THIRD], 0)],
}


class OracleStreamerRun:
    def __init__(self, tree, model, voltage, dt, max_rel_residual=1e-8, num_vcycles=30, photoi=None,
                 photoi_per_steps=5, integrator="heun"):
        self.stages = STAGES[integrator]
        self.integrator = integrator
        self.tree, self.m = tree, model
        self.voltage, self.dt = voltage, dt
        self.rel = max_rel_residual
        self.num_vcycles = num_vcycles
        self.photoi = photoi          # (lambdas 1/m, coeffs 1/m^2, eta*quench)
        self.photoi_per_steps = photoi_per_steps
        self.it = 0
        self.L = float(tree.dr[0, -1] * tree.coarse_grid_size[-1])
        self.o = oracle.Oracle(tree, model.n_var_cell, model.n_var_face)
        D, nc = tree.ndim, tree.n_cell
        self.leaves = np.concatenate(tree.lvl_leaves) - 1
        self.ncell_leaf = len(self.leaves) * nc ** D
        self.level_cells = [len(tree.lvl_ids[l]) * nc ** D for l in range(tree.highest_lvl)]
        self.min_dr = float(np.min(tree.dr[tree.lvl_ids[-1][0] - 1]))
        self.last = {}

    def vcycle_updates(self, max_lvl, mg):
        return (mg.n_cycle_down + mg.n_cycle_up) * sum(self.level_cells[1:max_lvl])

    def setup(self):
        o, m = self.o, self.m
        D = self.tree.ndim
        o.transport_setup(m.transport_desc())
        o.set_cc_methods(m.i_electric_fld, *m.electric_fld_gc())
        for s in range(len(m.species)):
            for st in range(m.n_states):
                o.set_cc_methods(m.species_iv[s] + st, [m.bc_species] * (2 * D), None, ag.RB_INTERP_LIM)
        if m.i_photo:
            o.set_cc_methods(m.i_photo, *m.photo_gc())
        self.field_desc = m.field_mg(self.voltage)
        o.mg_setup(0, self.field_desc)
        self.mode_descs = []
        if self.photoi is not None:
            for n, d in enumerate(m.helmholtz_mg(self.photoi[0])):
                o.mg_setup(1 + n, d)
                self.mode_descs.append(d)

    def field(self, cc, fc, s_in, have_guess):
        """field_compute: rhs, residual threshold, FMG start without a guess,
        V-cycles to the threshold, E from the potential."""
        o, m = self.o, self.m
        H = self.tree.highest_lvl
        o.field_set_rhs(cc, m.i_rhs, s_in)
        max_rhs = o.maxabs(cc, m.i_rhs)
        # with an electrode: conv_fac 1e-8 and the electrode at the voltage
        # or grounded (field_compute, src/m_field.f90:468-487)
        conv = 1e-8 if m.electrode else 1e-10
        if m.electrode:
            o.mg_set_lsf_voltage(0, self.voltage)
        thr = max(1e-6, max_rhs * self.rel, conv * abs(self.voltage) / (self.L * self.min_dr))
        work = nv = 0
        if not have_guess:
            res = []
            for i in range(100):
                res.append(o.mg_fmg(cc, 0, True, True))
                nv += 1
                work += sum(self.vcycle_updates(l, self.field_desc) for l in range(1, H + 1))
                if res[-1] < thr:
                    break
                if i >= 2:
                    ratio = min(res[-3:]) / max(res[-3:])
                    if 0.5 < ratio < 2.0 and res[-1] < 1e8:
                        break
        for _ in range(self.num_vcycles):
            r = o.mg_vcycle(cc, 0, True)
            nv += 1
            work += self.vcycle_updates(H, self.field_desc)
            if r < thr:
                break
        o.field_from_potential(cc, fc, m.i_phi)
        self.last["vcycles"] = self.last.get("vcycles", 0) + nv
        return work

    def refine(self, cc, fc, desc, max_lvl, limiter=ag.LIMITER_MC):
        """The refinement cycle of StreamerRun.refine on the restatement:
        flags (orc_refine_flags), the host's new tree (afivo_tree), the data
        moved by box, prolongation of the new boxes level by level, the field
        of the new mesh.  Returns the new state arrays, the flags and the old
        ids."""
        m = self.m
        flags = self.o.refine_flags(cc, desc)
        new = at.adjust_refinement(self.tree, flags, max_lvl)
        old_id = at.remap_ids(self.tree, new)
        keep = old_id > 0
        cc2 = ag.new_cc(new, m.n_var_cell)
        fc2 = ag.new_fc(new, m.n_var_face)
        cc2[keep] = cc[old_id[keep] - 1]
        fc2[keep] = fc[old_id[keep] - 1]
        it = self.it
        self.__init__(new, m, self.voltage, self.dt, max_rel_residual=self.rel, num_vcycles=self.num_vcycles,
                      photoi=self.photoi, photoi_per_steps=self.photoi_per_steps, integrator=self.integrator)
        self.it = it
        self.setup()
        ivs = [m.species_iv[s] for s in range(len(m.species))] + [m.i_phi]
        fresh = np.nonzero(old_id == 0)[0] + 1
        lv = new.lvl[fresh - 1]
        for lvl in sorted(set(lv.tolist())):
            ids = fresh[lv == lvl]
            for iv in ivs:
                self.o.gc(cc2, iv, lvl - 1, True)
                self.o.prolong_limit(cc2, iv, ids, limiter)
        self.field(cc2, fc2, 0, True)
        return cc2, fc2, flags, old_id

    def initial_field(self, cc, fc):
        self.o.gc(cc, self.m.i_phi, 0, True)
        return self.field(cc, fc, 0, False)

    def photoionization(self, cc):
        o, m = self.o, self.m
        lam, coeffs, coeff = self.photoi
        H = self.tree.highest_lvl
        o.photoi_source(cc, coeff, m.i_rhs)
        cc[:, m.i_photo - 1] = 0.0
        max_rhs = max(o.maxabs(cc, m.i_rhs), np.sqrt(np.finfo(float).eps))
        work = 0
        for n, d in enumerate(self.mode_descs):
            for _ in range(10):
                r = o.mg_fmg(cc, 1 + n, True, True)
                work += sum(self.vcycle_updates(l, d) for l in range(1, H + 1))
                if r / max_rhs < 1e-2:
                    break
            cc[self.leaves, m.i_photo - 1] -= coeffs[n] * cc[self.leaves, m.i_modes[n] - 1]
        return work

    def step(self, cc, fc):
        o, m, dt = self.o, self.m, self.dt
        self.last = {"vcycles": 0}
        work = 0
        if self.photoi is not None and self.it % self.photoi_per_steps == 0:
            work += self.photoionization(cc)
        for s in range(len(m.species)):
            cc[:, m.species_iv[s] + m.n_states - 2] = cc[:, m.species_iv[s] - 1]
        cfl = drt = 1e100
        chem = 0.0
        for i, (f, s_deriv, s_prev, w_prev, s_out) in enumerate(self.stages, 1):
            if i > 1:
                work += self.field(cc, fc, s_deriv, True)
            lim = o.flux_upwind(cc, fc, s_deriv)
            cfl, drt = min(cfl, lim[0]), min(drt, lim[1])
            chem = o.update_densities(cc, fc, f * dt, s_deriv, s_prev, w_prev, s_out, i == len(self.stages))
        work += self.field(cc, fc, 0, True)
        work += len(self.stages) * self.ncell_leaf * len(m.species)
        self.last.update(cfl=cfl, drt=drt, chem=chem)
        self.it += 1
        return work
