"""The `streamer` program's engine on the CPU restatement (TEST
INFRASTRUCTURE ONLY).

`OracleEngine` implements the engine interface of
`streamer_program.Program` with the C++ restatement, so a whole run of a
reference configuration (initial refinement, time loop with time-step
control and refinement every few steps) can be compared with the
regression logs the reference's own tests store.  Stages follow:

* forward_euler (src/m_fluid.f90:21-99) under af_advance
  (afivo/src/m_af_advance.f90:121-214): field of the stage input from the
  second stage on, fluxes, update; the stage's limit min(dt_max,
  cfl_number/max cfl_sum, dielectric relaxation time, chemistry limit) with
  the chemistry limit on the last stage only;
* copy_current_state / restore_previous_state (src/streamer.f90:659-683):
  densities and the potential, and on a restore the field from the restored
  potential;
* the refinement step of the time loop (src/streamer.f90:405-428):
  af_restrict_tree + af_gc_tree of the densities, default_refinement flags,
  af_adjust_refinement and auto_prolong (afivo/src/m_af_core.f90:843-881):
  densities and rhs by af_prolong_limit, phi and |E| by af_prolong_linear,
  level by level, then the ghost cells of the new level.
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
import oracle_streamer as osr  # noqa: E402
import streamer_program as sp  # noqa: E402


class OracleEngine:
    def __init__(self, tree, model, voltage, cfg):
        self.m, self.cfg, self.voltage = model, cfg, voltage
        self.stages = osr.STAGES[model.integrator]
        self._use_tree(tree, ag.new_cc(tree, model.n_var_cell), ag.new_fc(tree, model.n_var_face))

    def _use_tree(self, tree, cc, fc):
        m, cfg = self.m, self.cfg
        self.tree, self.cc, self.fc = tree, cc, fc
        self.run = osr.OracleStreamerRun(tree, m, self.voltage, 0.0,
                                         max_rel_residual=cfg.multigrid_max_rel_residual,
                                         num_vcycles=cfg.multigrid_num_vcycles, integrator=m.integrator,
                                         photoi=m.photoi_params, photoi_per_steps=cfg.photoi_per_steps)
        self.run.setup()
        self.o = self.run.o
        # rhs: af_bc_neumann_zero + af_gc_interp (src/streamer.f90:74-79)
        self.o.set_cc_methods(m.i_rhs, [ag.BC_NEUMANN] * (2 * tree.ndim), None, ag.RB_INTERP)
        if m.electrode:
            self.o.mg_set_lsf(cc, 0, sp.electrode_desc(cfg, m.i_lsf))
            self.o.transport_set_electrode(m.i_lsf)

    def electrode_densities(self):
        """set_electrode_densities (src/streamer.f90:590-594)."""
        self.o.electrode_species_bc(self.cc, 0, 0, self.m.ix_pos_ion, True)

    def set_initial(self, ids, e, ion):
        m = self.m
        idx = np.asarray(ids) - 1
        shp = (len(idx),) + self.cc.shape[2:]
        self.cc[idx, m.species_iv[0] - 1] = e.reshape(shp)
        self.cc[idx, m.species_iv[m.ix_pos_ion] - 1] = ion.reshape(shp)
        if m.electrode:
            self.o.electrode_init_densities(self.cc, 0, ids)

    def field(self, have_guess):
        if not have_guess:
            self.o.gc(self.cc, self.m.i_phi, 0, True)
        self.run.field(self.cc, self.fc, 0, have_guess)

    def advance(self, dt):
        m, o, cfg, cc, fc = self.m, self.o, self.cfg, self.cc, self.fc
        for s in range(len(m.species)):
            cc[:, m.species_iv[s] + m.n_states - 2] = cc[:, m.species_iv[s] - 1]
        self.phi_saved = cc[:, m.i_phi - 1].copy()
        lim = 1e100
        for i, (f, s_deriv, s_prev, w_prev, s_out) in enumerate(self.stages, 1):
            if i > 1:
                self.run.field(cc, fc, s_deriv, True)
            fl = o.flux_upwind(cc, fc, s_deriv)
            last = i == len(self.stages)
            chem = o.update_densities(cc, fc, f * dt, s_deriv, s_prev, w_prev, s_out, last)
            lim = min(cfg.dt_max, min(fl[0] * cfg.dt_cfl_number, fl[1], chem if last else 1e100, 1e100))
        return lim

    def photoi(self):
        self.run.photoionization(self.cc)

    def restore(self):
        m, cc = self.m, self.cc
        for s in range(len(m.species)):
            cc[:, m.species_iv[s] - 1] = cc[:, m.species_iv[s] + m.n_states - 2]
        cc[:, m.i_phi - 1] = self.phi_saved
        self.o.field_from_potential(cc, self.fc, m.i_phi)

    def auto_vars(self):
        """(variable, prolongation) of the tree's cc_auto_vars."""
        m = self.m
        out = [(m.species_iv[s], "limit") for s in range(len(m.species))]
        out += [(m.i_phi, "linear"), (m.i_electric_fld, "linear"), (m.i_rhs, "limit")]
        if m.i_photo:
            out.append((m.i_photo, "linear"))
        return out

    def refine(self, desc, restrict_first):
        m, o, tree = self.m, self.o, self.tree
        if restrict_first:
            for s in range(len(m.species)):
                o.restrict_tree(self.cc, m.species_iv[s])
                o.gc(self.cc, m.species_iv[s], 0, True)
        flags = o.refine_flags(self.cc, desc)
        new = at.adjust_refinement(tree, flags, sp.AF_MAX_LVL)
        if new is tree:
            return 0, 0, np.zeros(0, dtype=np.int32)
        old_id = at.remap_ids(tree, new)
        keep = old_id > 0
        n_add = int(np.count_nonzero(~keep))
        n_rm = tree.n_boxes - int(np.count_nonzero(keep))
        if n_add == 0 and n_rm == 0:
            return 0, 0, np.zeros(0, dtype=np.int32)
        cc2 = ag.new_cc(new, m.n_var_cell)
        fc2 = ag.new_fc(new, m.n_var_face)
        cc2[keep] = self.cc[old_id[keep] - 1]
        fc2[keep] = self.fc[old_id[keep] - 1]
        self._use_tree(new, cc2, fc2)
        fresh = np.nonzero(~keep)[0].astype(np.int32) + 1
        lv = new.lvl[fresh - 1]
        for lvl in sorted(set(lv.tolist())):
            ids = fresh[lv == lvl]
            for iv, how in self.auto_vars():
                self.o.gc(cc2, iv, lvl - 1, True)
                if how == "limit":
                    self.o.prolong_limit(cc2, iv, ids, m.transport_desc().prolong_limiter)
                else:
                    self.o.prolong_linear(cc2, iv, ids)
            for iv, _ in self.auto_vars():
                self.o.gc(cc2, iv, lvl, True)
        return n_add, n_rm, fresh

    def leaf_values(self, s):
        t, nc, D = self.tree, self.tree.n_cell, self.tree.ndim
        iv = self.m.species_iv[s] - 1
        sl = (slice(1, nc + 1),) * D
        out = []
        for lvl in range(1, t.highest_lvl + 1):
            ids = np.asarray(t.lvl_leaves[lvl - 1], dtype=np.int64) - 1
            out.append(self.cc[ids, iv][(slice(None),) + sl].reshape(len(ids), nc ** D))
        return out
