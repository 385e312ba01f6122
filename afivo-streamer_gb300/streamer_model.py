"""Host-side setup of the streamer fluid model for the GPU path.

This stands in for the reference's host initialisation, which stays on the
host and outside the hot path: the variable registry (src/m_streamer.f90:
201-476), the transport lookup table (transport_data_initialize,
src/m_transport_data.f90:61-220, and LT_create/table_set_x,
src/lookup_table_fortran/m_lookup_table.f90:186-289), the chemistry
(chemistry_initialize with the standard two-reaction model when no reaction
file is given, src/m_chemistry.f90:222-261) and the multigrid options of
field_initialize / photoi_helmh_initialize (src/m_field.f90:107-395,
src/m_photoi_helmh.f90:44-160).  It produces the C-ABI descriptors.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

import afivo_gpu as ag
import afivo_tree as at

SI_TO_TD = 1e21          # SI_to_Townsend (src/m_gas.f90:39)
TD_TO_SI = 1e-21
ELEM = 1.602176634e-19   # UC_elem_charge
EPS0 = 8.8541878128e-12  # UC_eps0
KB = 1.380649e-23        # UC_boltzmann_const


def gas_number_density(pressure_bar=1.0, temperature=300.0):
    """N = 1e5 * p / (k_B * T), src/m_gas.f90:174-176."""
    return 1e5 * pressure_bar / (KB * temperature)


def table_x(x_min, x_max, n_points):
    """get_x / table_set_x for linear spacing (m_lookup_table.f90:205-289)."""
    tmp = 1.0 / (n_points - 1)
    x = np.arange(n_points, dtype=np.float64) * tmp
    x = x_min + x * (x_max - x_min)
    inv_fac = (n_points - 1) / (x_max - x_min)
    return x, inv_fac


@dataclass
class Species:
    name: str
    charge: float


@dataclass
class StreamerModel:
    """Variables, transport table and chemistry of a streamer run."""
    ndim: int
    n_states: int = 3                 # af_advance_num_steps(heun) + 1 copies
    species: list = field(default_factory=list)
    mobile_ions: list = field(default_factory=list)  # (species index, mobility m^2/Vs)
    photoi_modes: int = 0
    N: float = gas_number_density()
    mu: float = 0.03                  # m^2/(V s)
    dif: float = 0.1                  # m^2/s
    alpha: callable = None            # alpha(E) in 1/m, E in V/m
    eta: callable = None
    reactions: list = field(default_factory=list)  # list of dict (see below)
    table_size: int = 1000
    td_max: float = 1000.0
    bc_species: int = ag.BC_NEUMANN
    photoi_species_index: int = 1     # species that gains the photoionization source with e
    # a transport table read from data (x in Td, its inv_fac, and the columns
    # mobility*N, diffusion*N, alpha/N, eta/N); replaces mu/dif/alpha/eta
    tabulated: dict = None
    electrode: bool = False           # a level-set variable for the field's electrode

    # variable layout (1-based tree indices)
    def __post_init__(self):
        if not self.species:
            self.species = [Species("e", -1.0), Species("M+", 1.0), Species("M-", -1.0)]
        self.i_phi, self.i_electric_fld, self.i_rhs, self.i_tmp = 1, 2, 3, 4
        nxt = 5
        self.species_iv = []
        for _ in self.species:
            self.species_iv.append(nxt)
            nxt += self.n_states
        self.i_photo = 0
        if self.photoi_modes > 0:
            self.i_photo = nxt
            nxt += 1
        self.i_modes = []
        for _ in range(self.photoi_modes):
            self.i_modes.append(nxt)
            nxt += 1
        self.i_lsf = 0
        if self.electrode:
            self.i_lsf = nxt
            nxt += 1
        self.n_var_cell = nxt - 1
        self.f_efield = 1
        self.f_flux = [2 + n for n in range(1 + len(self.mobile_ions))]
        self.n_var_face = 1 + len(self.f_flux)
        self.build_table()

    def build_table(self):
        """Transport lookup table over the reduced field (columns: mu*N,
        D*N, alpha/N, eta/N, then one column per tabulated reaction)."""
        N = self.N
        if self.tabulated is not None:
            x, inv_fac = self.tabulated["x"], self.tabulated["inv_fac"]
            cols = [np.asarray(c, dtype=np.float64) for c in self.tabulated["cols"]]
            has_eta = True
        else:
            x, inv_fac = table_x(0.0, self.td_max, self.table_size)
            E = x * TD_TO_SI * N
            with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
                a = self.alpha(E) if self.alpha else np.zeros_like(E)
                h = self.eta(E) if self.eta else np.zeros_like(E)
            a = np.where(np.isfinite(a), a, 0.0)
            h = np.where(np.isfinite(h), h, 0.0)
            mobN = np.full_like(x, self.mu * N)
            difN = np.full_like(x, self.dif * N)
            cols = [mobN, difN, a / N, h / N]
            has_eta = self.eta is not None
        self.col_mobility, self.col_diffusion, self.col_alpha, self.col_eta = 0, 1, 2, 3
        self.lt_x = x
        self.lt_inv_fac = inv_fac
        # standard model reactions (src/m_chemistry.f90:232-257):
        # y = alpha/N * mu*N * Td * Townsend_to_SI * N
        if not self.reactions:
            self.reactions = [
                dict(type=ag.RATE_TABULATED_FIELD, col=len(cols), ix_in=[0], ix_out=[0, 1], mult=[2, 1]),
            ]
            cols.append(cols[2] * cols[0] * x * TD_TO_SI * N)
            if has_eta and len(self.species) > 2:
                self.reactions.append(
                    dict(type=ag.RATE_TABULATED_FIELD, col=len(cols), ix_in=[0], ix_out=[2], mult=[1]))
                cols.append(cols[3] * cols[0] * x * TD_TO_SI * N)
        self.lt = np.ascontiguousarray(np.stack(cols), dtype=np.float64)  # [n_cols][n_points]

    def transport_desc(self, precision=ag.FP64) -> ag.TransportDesc:
        d = ag.TransportDesc()
        d.n_species = len(self.species)
        for s, sp in enumerate(self.species):
            d.species_iv[s] = self.species_iv[s]
            d.species_charge[s] = sp.charge
        d.n_flux = 1 + len(self.mobile_ions)
        d.flux_species[0] = 0
        d.flux_fc[0] = self.f_flux[0]
        d.flux_charge_sign[0] = -1.0
        for n, (s, mob) in enumerate(self.mobile_ions):
            d.flux_species[1 + n] = s
            d.flux_fc[1 + n] = self.f_flux[1 + n]
            d.flux_charge_sign[1 + n] = float(np.sign(self.species[s].charge))
            # scaled with the gas number density at 300 K and 1 bar
            # (src/m_transport_data.f90:206-208)
            d.ion_mobility_N[1 + n] = mob * (1e5 / (KB * 300))
        d.i_electric_fld = self.i_electric_fld
        d.i_efield_fc = self.f_efield
        d.i_photo = self.i_photo
        d.photoi_species = self.photoi_species_index
        d.gas_number_density = self.N
        d.species_gc = ag.gc_desc([self.bc_species] * (2 * self.ndim), None, ag.RB_INTERP_LIM)
        d.prolong_limiter = ag.LIMITER_MC if self.ndim < 3 else ag.LIMITER_GMINMOD43
        d.lt_n_points = self.lt.shape[1]
        d.lt_x_min = float(self.lt_x[0])
        d.lt_inv_fac = self.lt_inv_fac
        d.lt_n_cols = self.lt.shape[0]
        d.lt_data = self.lt.ctypes.data_as(C.POINTER(C.c_double))
        d.lt_col_mobility = self.col_mobility
        d.lt_col_diffusion = self.col_diffusion
        d.lt_col_alpha = self.col_alpha
        d.n_reactions = len(self.reactions)
        for n, r in enumerate(self.reactions):
            R = d.reactions[n]
            R.rate_type = r["type"]
            R.lt_col = r.get("col", 0)
            R.rate_factor = r.get("factor", 1.0)
            for q, c in enumerate(r.get("c", [])):
                R.c[q] = c
            R.n_in = len(r["ix_in"])
            for q, v in enumerate(r["ix_in"]):
                R.ix_in[q] = v
            R.n_out = len(r["ix_out"])
            for q, v in enumerate(r["ix_out"]):
                R.ix_out[q] = v
                R.mult_out[q] = r["mult"][q]
        d.dt_chemistry_nmin = 0.0
        d.dt_chemistry_limit_loss = 1
        d.precision = precision
        return d

    def refine_desc(self, **kw):
        """default_refinement parameters with the reference's defaults
        (src/m_refine.f90:10-60: refine_buffer_width 4, refine_min_dx 1e-7,
        refine_max_dx 1e-3, refine_adx 1, refine_adx_fac 1, derefine_dx 1e-4,
        refine_min_dens -1e99), this model's lookup-table columns and gas
        density; keyword arguments override fields of afg_refine_desc."""
        d = ag.RefineDesc()
        d.i_electron, d.i_electric_fld = self.species_iv[0], self.i_electric_fld
        d.lt_col_alpha, d.lt_col_eta = self.col_alpha, self.col_eta
        d.gas_number_density = self.N
        d.adx, d.adx_fac, d.min_dens = 1.0, 1.0, -1e99
        d.derefine_dx, d.max_dx, d.min_dx = 1e-4, 1e-3, 1e-7
        d.ref_buffer, d.init_fac = 4, 0.25
        for k, v in kw.items():
            setattr(d, k, v)
        return d

    def field_bc(self, voltage):
        """field_bc_homogeneous (src/m_field.f90:590-610)."""
        D = self.ndim
        bt = [ag.BC_NEUMANN] * (2 * D - 2) + [ag.BC_DIRICHLET, ag.BC_DIRICHLET]
        bv = [0.0] * (2 * D - 1) + [voltage]
        return bt, bv

    def field_mg(self, voltage, precision=ag.FP64):
        bt, bv = self.field_bc(voltage)
        return ag.mg_desc(self.i_phi, self.i_rhs, self.i_tmp, bt, bv, precision=precision)

    def helmholtz_mg(self, lam, precision=ag.FP64):
        """photoi_helmh_bc: Dirichlet 0 in the last dimension, Neumann 0 else."""
        D = self.ndim
        bt = [ag.BC_NEUMANN] * (2 * D - 2) + [ag.BC_DIRICHLET, ag.BC_DIRICHLET]
        out = []
        for n, l in enumerate(lam):
            out.append(ag.mg_desc(self.i_modes[n], self.i_rhs, self.i_tmp, bt, None, lambda2=l * l,
                                  precision=precision))
        return out

    def electric_fld_gc(self):
        """|E|: af_bc_neumann_zero + af_gc_interp (src/m_field.f90:392-393)."""
        return [ag.BC_NEUMANN] * (2 * self.ndim), None, ag.RB_INTERP

    def photo_gc(self):
        """i_photo: photoi_helmh_bc + af_gc_interp (src/m_photoi.f90:115)."""
        D = self.ndim
        return [ag.BC_NEUMANN] * (2 * D - 2) + [ag.BC_DIRICHLET, ag.BC_DIRICHLET], None, ag.RB_INTERP


def baseline_alpha(E):
    """alpha(E) = 4.3e5 * exp(-2e7/|E|) 1/m (the analytic ionization
    coefficient of the synthetic streamer workloads)."""
    E = np.abs(E)
    with np.errstate(divide="ignore", over="ignore"):
        return np.where(E > 0, 4.3e5 * np.exp(-2e7 / np.maximum(E, 1e-300)), 0.0)


def baseline_eta(E):
    return np.full_like(np.asarray(E, dtype=np.float64), 2e3)


_THIRD, _SIXTH = 1 / 3.0, 1 / 6.0

# The explicit integrators of af_advance (afivo/src/m_af_advance.f90:150-199)
# as their forward_euler stages: (dt factor, s_deriv, s_prev, w_prev, s_out).
# The IMEX schemes need an implicit solver and are not on this path.
INTEGRATORS = {
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


def states_needed(integrator):
    """Copies of every density: one per integrator step plus the backup copy
    of copy_current_state (src/streamer.f90:659-671)."""
    return len(INTEGRATORS[integrator]) + 1


class StreamerRun:
    """Time stepping of the hot path through the C-ABI, mirroring the
    reference's time loop (src/streamer.f90:181-432): photoionization every
    `photoi_per_steps` steps (photoi_set_src, 242-248), copy_current_state
    (659-671), af_advance (afivo/src/m_af_advance.f90:121-214) whose stages
    are forward_euler (src/m_fluid.f90:21-99: field of the stage's input
    state from the second stage on, fluxes, densities), and field_compute for
    the new state (327).  Step rejection is not needed at a fixed dt below
    the limits and is left to the caller.

    On a batched context (a forest of independent instances) `voltage` is
    an array with one applied voltage per instance; the field solves then
    converge per instance (afg_field_compute_inst) and last["vcycles_inst"]
    counts each instance's cycles."""

    def __init__(self, ctx, tree, model, voltage, dt, precision=ag.FP64, max_rel_residual=1e-8,
                 num_vcycles=30, photoi=None, photoi_per_steps=5, integrator="heun", dt_cfl_number=0.5,
                 dt_max=1e-11):
        if model.n_states < states_needed(integrator):
            raise ValueError(f"{integrator} needs {states_needed(integrator)} copies of each density")
        self.stages = INTEGRATORS[integrator]
        self.batched = np.ndim(voltage) == 1
        if self.batched and photoi is not None:
            raise ValueError("photoionization of batched instances is not supported")
        self.ctx, self.tree, self.m = ctx, tree, model
        self.voltage, self.dt = voltage, dt
        self.precision = precision
        self.rel = max_rel_residual
        self.num_vcycles = num_vcycles
        self.photoi = photoi          # (lambdas 1/m, coeffs 1/m^2, eta*quench)
        self.photoi_per_steps = photoi_per_steps
        self.dt_cfl_number, self.dt_max = dt_cfl_number, dt_max
        self.it = 0
        self.L = float(tree.dr[0, -1] * tree.coarse_grid_size[-1])
        self.last = {}

    def setup(self):
        ctx, m = self.ctx, self.m
        D = self.tree.ndim
        ctx.transport_setup(m.transport_desc(self.precision))
        ctx.set_cc_methods(m.i_electric_fld, *m.electric_fld_gc())
        for s in range(len(m.species)):
            for st in range(m.n_states):
                ctx.set_cc_methods(m.species_iv[s] + st, [m.bc_species] * (2 * D), None, ag.RB_INTERP_LIM)
        if m.i_photo:
            ctx.set_cc_methods(m.i_photo, *m.photo_gc())
        v0 = float(self.voltage[0]) if self.batched else self.voltage
        ctx.mg_setup(0, m.field_mg(v0, self.precision))
        if not self.batched:
            ctx.stage_setup(0, self.L, self.rel, self.num_vcycles, self.dt_cfl_number, self.dt_max)
        self.mode_ids = []
        if self.photoi is not None:
            lam, coeffs, _ = self.photoi
            for n, d in enumerate(m.helmholtz_mg(lam, self.precision)):
                ctx.mg_setup(1 + n, d)
                self.mode_ids.append(1 + n)

    def field(self, s_in, have_guess):
        if self.batched:
            n, r = self.ctx.field_compute_inst(0, s_in, have_guess, self.voltage, self.L, self.rel,
                                               self.num_vcycles)
            self.last["vcycles_inst"] = self.last.get("vcycles_inst", 0) + n
            self.last["vcycles"] = self.last.get("vcycles", 0) + int(n.max())
            return int(n.max()), float(r.max())
        n, r = self.ctx.field_compute(0, s_in, have_guess, self.voltage, self.L, self.rel, self.num_vcycles)
        self.last.setdefault("vcycles", 0)
        self.last["vcycles"] += n
        return n, r

    def refine(self, desc, max_lvl, limiter=ag.LIMITER_MC):
        """One refinement of the mesh with the data on the device
        (src/streamer.f90:397-428): box flags from afg_refine_flags, the new
        tree from the host's af_adjust_refinement (afg_adjust_refinement), the data moved
        by afg_tree_remap, the new boxes' densities and potential filled by
        afg_prolong_limit level by level (after a ghost fill of the parents'
        level), the operators set up again and the field of the new mesh.
        Returns the box flags and the old id of every new box."""
        ctx, m = self.ctx, self.m
        flags = ctx.refine_flags(desc)
        new = ag.adjust_refinement(self.tree, flags, max_lvl)
        old_id = at.remap_ids(self.tree, new)
        ctx.tree_remap(new, old_id)
        self.tree = new
        self.setup()
        ivs = [m.species_iv[s] for s in range(len(m.species))] + [m.i_phi]
        fresh = np.nonzero(old_id == 0)[0] + 1
        lv = new.lvl[fresh - 1]
        for lvl in sorted(set(lv.tolist())):
            ids = fresh[lv == lvl]
            for iv in ivs:
                ctx.gc(iv, lvl - 1, True)
                ctx.prolong_limit(iv, ids, limiter)
        self.field(0, True)
        return flags, old_id

    def initial_field(self):
        self.ctx.gc(self.m.i_phi, 0, True)
        return self.field(0, False)

    def step(self, after_update=None):
        """One time step; after_update() (optional) is called once the new
        densities are computed and before the field of the new state, which
        writes no density (e.g. to start their download)."""
        ctx, m, dt = self.ctx, self.m, self.dt
        self.last = {"vcycles": 0}
        if self.photoi is not None and self.it % self.photoi_per_steps == 0:
            lam, coeffs, coeff = self.photoi
            ctx.photoi_helmh(coeff, self.mode_ids, coeffs, 1e-2, 10)
        # copy_current_state: densities to the backup copy
        for s in range(len(m.species)):
            ctx.tree_copy_cc(m.species_iv[s], m.species_iv[s] + m.n_states - 1)
        n_st = len(self.stages)
        lim = 1e100
        for i, (f, s_deriv, s_prev, w_prev, s_out) in enumerate(self.stages, 1):
            if not self.batched:
                # the whole stage in one call (afg_forward_euler)
                lim, nc = ctx.forward_euler(f * dt, self.voltage, s_deriv, s_prev, w_prev, s_out, i, n_st)
                self.last["vcycles"] += nc
                continue
            # batched instances: the field converges per instance
            if i > 1:
                self.field(s_deriv, True)
            fl = ctx.flux_upwind(s_deriv)
            chem = ctx.update_densities(f * dt, s_deriv, s_prev, w_prev, s_out, last_step=(i == n_st))
            lim = min(self.dt_max, fl[0] * self.dt_cfl_number, fl[1], chem if i == n_st else 1e100)
        if after_update is not None:
            after_update()
        # field of the new state
        n, r = self.field(0, True)
        self.last.update(dt_lim=lim, residual=r)
        self.it += 1
