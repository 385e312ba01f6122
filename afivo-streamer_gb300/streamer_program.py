"""The reference's `streamer` program around the hot path, for the
configurations this path supports.

This is the caller side of the hot path: it reads a reference configuration
file (`.cfg`, the m_config format), builds the transport lookup table from
the reference's transport-data file, sets the initial conditions, runs the
initial refinement loop and the time loop with the reference's time-step
control, refinement cadence and output times, and writes the regression-log
rows the reference's own tests compare (`output_regression_log`,
src/m_output.f90:787-842).  Every numerical stage runs on an engine: the
GPU engine (`GpuEngine`, through the C-ABI) here, the CPU restatement in the
oracle's tests.  What it restates:

* `.cfg` syntax and the defaults of the keys it reads (m_config; defaults in
  src/m_streamer.f90, m_refine.f90, m_dt.f90, m_field.f90, m_table_data.f90,
  m_init_cond.f90, m_output.f90, m_gas.f90);
* table_from_file (src/m_table_data.f90:86-176), LT_get_spaced_data /
  LT_lin_interp_list (src/lookup_table_fortran/m_lookup_table.f90:142-254),
  the old-style transport table (src/m_transport_data.f90:61-106) and the
  standard two-reaction chemistry (src/m_chemistry.f90:222-257);
* init_cond_set_box (src/m_init_cond.f90:214-293) with GM_density_line
  (src/m_geometry.f90);
* set_initial_conditions (src/streamer.f90:480-533) and the time loop
  (src/streamer.f90:181-432).

Photoionization by the Helmholtz method, chemistry and reaction files and
mobile ions are supported.  Keys whose values would need code outside the
path (electrodes, dielectrics, Monte Carlo photoionization, gas dynamics,
the IMEX integrators, stochastic densities, the energy equation) raise
`Unsupported`.
"""
from __future__ import annotations

import math
import os
import shlex

import numpy as np

import afivo_gpu as ag
import afivo_tree as at
import streamer_model as sm


class Unsupported(ValueError):
    """A configuration value this path does not implement."""


# ---------------------------------------------------------------------------
# configuration files


def read_cfg(path):
    """m_config's file format (src/config_fortran/m_config.f90:288-356):
    `name = value(s)` lines, `#` comments, `[section]` lines; a variable line
    belongs to the last section (its name gets `section%`) only when it
    starts with a tab or at least two spaces, otherwise it is global.  A
    later line overrides an earlier one.  Returns {name: [tokens]}."""
    out = {}
    section = ""
    with open(path) as f:
        for raw in f:
            body = raw.rstrip("\n").split("#", 1)[0]
            line = body.strip()
            if not line:
                continue
            if "=" not in line:
                if line.startswith("[") and "]" in line:
                    section = line[1:line.index("]")].strip()
                    continue
                raise ValueError(f"{path}: cannot parse line: {raw.strip()}")
            if "+=" in line:
                raise Unsupported("'+=' lines in configuration files")
            name, val = body.split("=", 1)
            indented = name.startswith("\t") or name.startswith("  ")
            name = name.strip()
            if section and indented:
                name = section + "%" + name
            out[name] = shlex.split(val.replace(",", " "))
    return out


def _to_float(tok):
    return float(tok.lower().replace("d", "e"))


def _to_bool(tok):
    t = tok.lower().strip(".")
    if t in ("t", "true"):
        return True
    if t in ("f", "false"):
        return False
    raise ValueError(f"not a logical: {tok}")


class ProgramConfig:
    """The settings of one run with the reference's defaults; `path` is a
    `.cfg` file, `overrides` a dict of extra `name: value` entries."""

    def __init__(self, path=None, overrides=None, ndim=2):
        raw = read_cfg(path) if path else {}
        for k, v in (overrides or {}).items():
            raw[k] = [str(x) for x in (v if isinstance(v, (list, tuple)) else [v])]
        self.raw, self.used = raw, set()
        self.base_dir = os.path.dirname(os.path.abspath(path)) if path else os.getcwd()
        D = self.ndim = ndim
        g = self._get
        # m_streamer.f90
        self.cylindrical = g("cylindrical", False, bool)
        self.end_time = g("end_time", 10e-9)
        self.box_size = g("box_size", 8, int)
        self.domain_len = g("domain_len", [16e-3] * D, n=D)
        self.domain_origin = g("domain_origin", [0.0] * D, n=D)
        self.coarse_grid_size = g("coarse_grid_size", [-1] * D, int, n=D)
        self.periodic = g("periodic", [False] * D, bool, n=D)
        self.multigrid_num_vcycles = g("multigrid_num_vcycles", 2, int)
        self.multigrid_max_rel_residual = g("multigrid_max_rel_residual", 1e-4)
        self.prolong_density = g("prolong_density", "limit", str)
        self.species_boundary_condition = g("species_boundary_condition", "neumann_zero", str)
        self.memory_limit_GB = g("memory_limit_GB", 4.0 ** (D - 1))
        # m_gas.f90
        self.gas_pressure = g("gas%pressure", 1.0)
        self.gas_temperature = g("gas%temperature", 300.0)
        self.gas_components = g("gas%components", ["N2", "O2"], str, n=None)
        self.gas_fractions = g("gas%fractions", [0.8, 0.2], n=None)
        # m_field.f90
        self.field_amplitude = g("field_amplitude", None)
        self.field_given_by = g("field_given_by", None, str, n=None)
        self.field_bc_type = g("field_bc_type", "homogeneous", str)
        # electrode (m_streamer.f90:318-326, m_field.f90:196-229)
        self.use_electrode = g("use_electrode", False, bool)
        self.field_electrode_grounded = g("field_electrode_grounded", False, bool)
        self.field_electrode2_grounded = g("field_electrode2_grounded", False, bool)
        self.field_electrode_type = g("field_electrode_type", "rod", str)
        self.field_rod_r0 = g("field_rod_r0", [-1.0e100] * D, n=D)
        self.field_rod_r1 = g("field_rod_r1", [-1.0e100] * D, n=D)
        self.field_rod2_r0 = g("field_rod2_r0", [-1.0e100] * D, n=D)
        self.field_rod2_r1 = g("field_rod2_r1", [-1.0e100] * D, n=D)
        self.field_rod_radius = g("field_rod_radius", -1.0e100)
        self.field_rod2_radius = g("field_rod2_radius", -1.0e100)
        self.cone_tip_radius = g("cone_tip_radius", -1.0e100)
        self.cone_length_frac = g("cone_length_frac", -1.0e100)
        self.cone2_tip_radius = g("cone2_tip_radius", -1.0e100)
        self.cone2_length_frac = g("cone2_length_frac", -1.0e100)
        self.refine_electrode_dx = g("refine_electrode_dx", 1e99)
        self.electrode_derefine_factor = g("electrode_derefine_factor", 1.0)
        # m_transport_data.f90, m_table_data.f90
        self.input_data_file = g("input_data%file", None, str)
        self.input_data_old_style = g("input_data%old_style", False, bool)
        self.mobile_ions = g("input_data%mobile_ions", [], str, n=None)
        self.ion_mobilities = g("input_data%ion_mobilities", [], n=None)
        self.table_size = g("table_data%size", 1000, int)
        self.table_min_townsend = g("table_data%min_townsend", 0.0)
        self.table_max_townsend = g("table_data%max_townsend", -1.0)
        self.input_interpolation = g("table_data%input_interpolation", "linear", str)
        self.table_xspacing = g("table_data%xspacing", "linear", str)
        # m_init_cond.f90
        self.background_density = g("background_density", 0.0)
        self.seed_density = g("seed_density", [], n=None)
        n_seed = len(self.seed_density)
        self.seed_rel_r0 = g("seed_rel_r0", [], n=None)
        self.seed_rel_r1 = g("seed_rel_r1", [], n=None)
        self.seed_charge_type = g("seed_charge_type", [], int, n=None)
        self.seed_width = g("seed_width", [], n=None)
        self.seed_falloff = g("seed_falloff", ["smoothstep"] * n_seed, str, n=None)
        self.seed_density2 = g("seed_density2", list(self.seed_density), n=None)
        # m_refine.f90
        self.refine_buffer_width = g("refine_buffer_width", 4, int)
        self.refine_per_steps = g("refine_per_steps", 2, int)
        self.refine_min_dx = g("refine_min_dx", 1.0e-7)
        self.refine_max_dx = g("refine_max_dx", 1.0e-3)
        self.refine_adx = g("refine_adx", 1.0)
        self.refine_adx_fac = g("refine_adx_fac", 1.0)
        self.derefine_dx = g("derefine_dx", 1e-4)
        self.refine_init_time = g("refine_init_time", 10e-9)
        self.refine_init_fac = g("refine_init_fac", 0.25)
        self.refine_min_dens = g("refine_min_dens", -1.0e99)
        self.refine_use_alpha_effective = g("refine_use_alpha_effective", False, bool)
        # m_dt.f90
        self.dt_max = g("dt_max", 1.0e-11)
        self.dt_min = g("dt_min", 1.0e-14)
        self.dt_safety_factor = g("dt_safety_factor", 0.9)
        self.dt_cfl_number = g("dt_cfl_number", 0.5)
        self.dt_chemistry_nmin = g("dt_chemistry_nmin", -1.0)
        self.dt_chemistry_limit_loss = g("dt_chemistry_limit_loss", True, bool)
        self.dt_max_growth_factor = g("dt_max_growth_factor", 2.0)
        self.time_integrator = g("time_integrator", "heuns_method", str)
        # m_photoi.f90, m_photoi_helmh.f90
        self.photoi_enabled = g("photoi%enabled", False, bool)
        self.photoi_per_steps = g("photoi%per_steps", 5, int)
        self.photoi_method = g("photoi%method", "helmholtz", str)
        self.photoi_eta = g("photoi%eta", 0.05)
        self.photoi_quenching_pressure = g("photoi%quenching_pressure", 40e-3)
        self.photoi_source_type = g("photoi%source_type", "Zheleznyak", str)
        self.photoi_species = g("photoi%species", "O2_plus", str)
        self.photoi_helmh_author = g("photoi_helmh%author", "Bourdon-3", str)
        self.photoi_helmh_lambdas = g("photoi_helmh%lambdas", [], n=None)
        self.photoi_helmh_coeffs = g("photoi_helmh%coeffs", [], n=None)
        self.photoi_helmh_max_rel_residual = g("photoi_helmh%max_rel_residual", 1e-2)
        # m_output.f90
        self.output_dt = g("output%dt", 1.0e-10)
        self.output_name = g("output%name", "output/sim", str)
        self.output_regression_test = g("output%regression_test", False, bool)
        self._check_supported()

    def _get(self, name, default, typ=float, n=1):
        if name not in self.raw:
            return default
        self.used.add(name)
        toks = self.raw[name]
        conv = {float: _to_float, int: int, bool: _to_bool, str: str}[typ]
        vals = [conv(t) for t in toks]
        if n == 1:
            if len(vals) != 1:
                raise ValueError(f"{name}: expected one value, got {toks}")
            return vals[0]
        if n is not None and len(vals) != n:
            raise ValueError(f"{name}: expected {n} values, got {toks}")
        return vals

    # keys that only affect output files or are informational
    _IGNORED = {"output%name", "memory_limit_GB", "output%regression_test", "output%dt", "silo_write"}
    # keys whose given value must equal the supported one
    _FIXED = {
        "use_dielectric": False,
        "gas%dynamics": False, "compute_power_density": False,
    }

    def _check_supported(self):
        for name, want in self._FIXED.items():
            if name in self.raw:
                self.used.add(name)
                if _to_bool(self.raw[name][0]) != want:
                    raise Unsupported(f"{name} = {self.raw[name][0]} is not supported on this path")
        if self.input_interpolation != "linear" or self.table_xspacing != "linear":
            raise Unsupported("only linear table interpolation and spacing are supported")
        if any(self.periodic):
            raise Unsupported("periodic domains are not supported")
        if len(self.mobile_ions) != len(self.ion_mobilities) or any(m < 0 for m in self.ion_mobilities):
            raise ValueError("input_data%mobile_ions and %ion_mobilities must pair up (positive mobilities)")
        if len(self.mobile_ions) + 1 > ag.AFG_MAX_FLUX:
            raise Unsupported("too many mobile ions for the device tables")
        if self.field_bc_type != "homogeneous":
            raise Unsupported("only field_bc_type = homogeneous is supported")
        if self.field_given_by is not None:
            if len(self.field_given_by) != 2 or self.field_given_by[0] not in ("field", "voltage"):
                raise Unsupported("field_given_by other than 'field <V/m>' or 'voltage <V>'")
        elif self.field_amplitude is None:
            raise ValueError("field_amplitude not specified")
        if self.use_electrode:
            if self.field_electrode_type not in ELECTRODE_SHAPES:
                raise Unsupported(f"field_electrode_type = {self.field_electrode_type}")
            if self.electrode_derefine_factor != 1.0:
                raise Unsupported("electrode_derefine_factor other than 1")
        if self.species_boundary_condition != "neumann_zero" or self.prolong_density != "limit":
            raise Unsupported("species_boundary_condition / prolong_density other than the defaults")
        if self.time_integrator not in TIME_INTEGRATORS:
            raise Unsupported(f"time_integrator = {self.time_integrator}")
        if self.photoi_enabled:
            if self.photoi_method != "helmholtz" or self.photoi_source_type != "Zheleznyak":
                raise Unsupported("photoionization other than helmholtz with the Zheleznyak source")
            if self.input_data_old_style and self.photoi_species != "M_plus":
                raise Unsupported("photoi%species must be the standard chemistry's M_plus")
            if self.photoi_helmh_max_rel_residual != 1e-2:
                raise Unsupported("photoi_helmh%max_rel_residual other than 1e-2")
        unknown = set(self.raw) - self.used - self._IGNORED
        if unknown:
            raise Unsupported("configuration keys not supported on this path: " + ", ".join(sorted(unknown)))


# field_electrode_type (src/m_field.f90:255-380) -> afg_lsf_desc shapes
ELECTRODE_SHAPES = {
    "sphere": ag.LSF_SPHERE, "rod": ag.LSF_ROD, "rod_cone_top": ag.LSF_ROD_CONE_TOP, "rod_rod": ag.LSF_ROD_ROD,
    "sphere_rod": ag.LSF_SPHERE_ROD, "two_rod_cone_electrodes": ag.LSF_TWO_ROD_CONE, "coaxial": ag.LSF_COAXIAL,
}


def electrode_desc(cfg, i_lsf):
    """The electrode of field_initialize (src/m_field.f90:255-390): positions
    relative to the domain (times ST_domain_len plus ST_domain_origin),
    mg%lsf_length_scale = field_rod_radius."""
    D = cfg.ndim
    L = np.asarray(cfg.domain_len, dtype=np.float64)
    O = np.asarray(cfg.domain_origin, dtype=np.float64)

    def absolute(rel):
        return list(np.asarray(rel, dtype=np.float64) * L + O)
    if cfg.field_rod_radius <= 0:
        raise ValueError("set field_rod_radius to smallest length scale of electrode")
    center = [0.0, O[1] + 0.5 * L[1]] if cfg.cylindrical else list(O + 0.5 * L)
    return ag.lsf_desc(ELECTRODE_SHAPES[cfg.field_electrode_type], i_lsf,
                       r0=absolute(cfg.field_rod_r0), r1=absolute(cfg.field_rod_r1), radius=cfg.field_rod_radius,
                       r2_0=absolute(cfg.field_rod2_r0), r2_1=absolute(cfg.field_rod2_r1),
                       radius2=cfg.field_rod2_radius, cone_tip_radius=cfg.cone_tip_radius,
                       cone_length_frac=cfg.cone_length_frac, cone2_tip_radius=cfg.cone2_tip_radius,
                       cone2_length_frac=cfg.cone2_length_frac, center=center,
                       grounded=cfg.field_electrode_grounded, grounded2=cfg.field_electrode2_grounded,
                       length_scale=cfg.field_rod_radius)


# af_integrator_names (afivo/src/m_af_advance.f90) -> the stage tables of
# streamer_model.INTEGRATORS
TIME_INTEGRATORS = {
    "forward_euler": "forward_euler", "midpoint_method": "midpoint", "heuns_method": "heun",
    "ssprk33": "ssprk33", "ssprk43": "ssprk43", "rk4": "rk4",
}


# ---------------------------------------------------------------------------
# transport data and lookup tables


def table_from_file(path, data_name):
    """table_from_file (src/m_table_data.f90:86-176): find the line equal to
    `data_name`, read FACTOR:/COMMENT: lines up to a line of dashes, then two
    columns until the next dashes; y is multiplied by the factor."""
    with open(path) as f:
        lines = [ln.rstrip("\n") for ln in f]
    n = 0
    while n < len(lines) and lines[n].rstrip() != data_name:
        n += 1
    if n == len(lines):
        raise ValueError(f"{path}: no data named '{data_name}'")
    n += 1
    factor = 1.0
    while True:
        s = lines[n].strip()
        n += 1
        if s.startswith("-----"):
            break
        if s.startswith("FACTOR:"):
            factor = _to_float(s[7:].split()[0])
        elif not s.startswith("COMMENT:"):
            raise ValueError(f"{path}: unknown statement '{s}'")
    xs, ys = [], []
    while True:
        s = lines[n].strip()
        n += 1
        if s.startswith("-----"):
            break
        if s == "" or s.startswith("#"):
            continue
        a, b = s.split()[:2]
        xs.append(_to_float(a))
        ys.append(_to_float(b))
    return np.array(xs), factor * np.array(ys)


def lin_interp_list(x_list, y_list, x):
    """LT_lin_interp_list with find_index_adaptive (m_lookup_table.f90:
    101-181): clamped at both ends; inside, the first index whose x is >= the
    value and the weights (1 - t, t)."""
    if x <= x_list[0]:
        return y_list[0]
    if x >= x_list[-1]:
        return y_list[-1]
    ix = int(np.searchsorted(x_list, x, side="left"))   # first x_list[ix] >= x
    t = (x - x_list[ix - 1]) / (x_list[ix] - x_list[ix - 1])
    return (1 - t) * y_list[ix - 1] + t * y_list[ix]


def spaced_data(x_in, y_in, new_x):
    """LT_get_spaced_data (m_lookup_table.f90:240-254)."""
    if np.min(np.diff(x_in)) <= 0:
        raise ValueError("transport data x should strictly increase")
    return np.array([lin_interp_list(x_in, y_in, float(x)) for x in new_x])


def old_style_columns(path, N, table_size, td_min, td_max_cfg):
    """The four columns of td_tbl from old-style data
    (src/m_transport_data.f90:68-105): mobility*N, diffusion*N, alpha/N,
    eta/N on a linear table in Td from table_min_townsend to the last field
    of the mobility data (or table_max_townsend)."""
    def rd(name, scale_y):
        x, y = table_from_file(path, name)
        x = x * sm.SI_TO_TD / N
        y = y * N if scale_y else y / N
        return x, y
    xm, ym = rd("efield[V/m]_vs_mu[m2/Vs]", True)
    td_max = xm[-1] if td_max_cfg < 0 else td_max_cfg
    x, inv_fac = sm.table_x(td_min, td_max, table_size)
    cols = [spaced_data(xm, ym, x)]
    for name, up in (("efield[V/m]_vs_dif[m2/s]", True), ("efield[V/m]_vs_alpha[1/m]", False),
                     ("efield[V/m]_vs_eta[1/m]", False)):
        cols.append(spaced_data(*rd(name, up), x))
    return x, inv_fac, cols


def to_simple_ascii(text):
    """to_simple_ascii (src/m_chemistry.f90:1359-1400): '+' -> '_plus',
    '-' -> '_min' (counted as charge outside brackets), '*' -> '_star',
    '^' -> '_hat', "'" -> 'p', '(' -> '_'; 'e' has charge -1."""
    out, charge, br = "", 0, False
    for ch in text:
        if ch == "(":
            br = True
            out += "_"
        elif ch == ")":
            br = False
        elif ch == "*":
            out += "_star"
        elif ch == "+":
            charge += 0 if br else 1
            out += "_plus"
        elif ch == "-":
            charge -= 0 if br else 1
            out += "_min"
        elif ch == "^":
            out += "_hat"
        elif ch == "'":
            out += "p"
        else:
            out += ch
    if out in ("e", "stoch_e"):
        charge = -1
    return out, charge


# rate expressions of read_reactions (src/m_chemistry.f90:1015-1100) that the
# device evaluates: expression -> (AFG rate type, number of coefficients)
RATE_FORMS = {
    "c1": (ag.RATE_CONSTANT, 1),
    "c1*(Td-c2)": (ag.RATE_LINEAR, 2),
    "c1*exp(-(c2/(c3+Td))**2)": (ag.RATE_EXP_V1, 3),
    "c1*exp(-(Td/c2)**2)": (ag.RATE_EXP_V2, 2),
    "c1*exp(-(c2/(c3+Td))**c4)": (ag.RATE_K13, 4),
    "c1*exp(-(Td/c2)**c3)": (ag.RATE_K14, 3),
    "c1*(300/Te)**c2": (ag.RATE_K1, 2),
}

# expressions of the gas temperature only (rate_analytic_k4..k10,
# src/m_chemistry.f90:731-746): constants at the constant gas temperature,
# evaluated on the host as c0 * value
GAS_TEMPERATURE_FORMS = {
    "c1*(Tg/300)**c2*exp(-c3/Tg)": (3, lambda c, T: c[0] * (T / 300) ** c[1] * math.exp(-c[2] / T)),
    "c1*exp(-c2/Tg)": (2, lambda c, T: c[0] * math.exp(-c[1] / T)),
    "c1*Tg**c2": (2, lambda c, T: c[0] * T ** c[1]),
    "c1*(Tg/c2)**c3": (3, lambda c, T: c[0] * (T / c[1]) ** c[2]),
    "c1*(300/Tg)**c2": (2, lambda c, T: c[0] * (300 / T) ** c[1]),
    "c1*exp(-c2*Tg)": (2, lambda c, T: c[0] * math.exp(-c[1] * T)),
}


def read_reactions(path, gas_components, gas_densities, N):
    """read_reactions + parse_reaction (src/m_chemistry.f90:857-1278) for a
    reaction file without groups: the plasma species in
    order of first appearance (simple-ascii names, charges) and per reaction
    its expression, data, input/output species (0-based plasma indices),
    output multiplicities and rate factor (gas densities of gas reactants, N
    for M, the cm unit conversion)."""
    with open(path) as f:
        lines = [ln.rstrip("\n") for ln in f]
    # read_ignored_species (src/m_chemistry.f90:807-854)
    ignored = []
    for q, ln in enumerate(lines):
        if ln.strip() == "ignored_species":
            for ln2 in lines[q + 2:]:
                t = ln2.strip()
                if t.startswith("#"):
                    continue
                if t.startswith("-----"):
                    break
                ignored.append(t.split()[0])
            break
    n = 0
    while lines[n].strip() != "reaction_list":
        n += 1
    n += 1
    if not lines[n].startswith("-----"):
        raise ValueError("reaction_list not followed by -----")
    entries = []
    for ln in lines[n + 1:]:
        ln = ln.strip()
        if ln.startswith("#"):
            continue
        if ln.startswith("-----"):
            break
        if ln.startswith("@"):
            raise Unsupported("reaction groups")
        fields = [x.strip() for x in ln.split(",") if x.strip()]
        if len(fields) < 3 or len(fields) > 4:
            raise ValueError(f"invalid chemistry syntax: {ln}")
        entries.append(fields + ["m"] * (4 - len(fields)))
    names, reactions = [], []
    for text, how, data, unit in entries:
        left, rfac, n_in_total, keep = True, 1.0, 0, True
        ix_in, ix_out, mult = [], [], []
        for comp in text.split():
            if comp == "+":
                continue
            if comp == "->":
                left = False
                continue
            m = 1
            if "1" <= comp[0] <= "9":
                m, comp = int(comp[0]), comp[1:]
            if left:
                n_in_total += m
            if comp in gas_components:
                if left:
                    rfac = rfac * gas_densities[gas_components.index(comp)]
                continue
            if comp == "M":
                if left:
                    rfac = rfac * N
                continue
            if comp in ignored:
                # an ignored reactant drops the reaction, an ignored product
                # is left out
                if left:
                    keep = False
                    break
                continue
            if comp not in names:
                names.append(comp)
            ix = names.index(comp)
            if left:
                ix_in += [ix] * m
            elif ix in ix_out:
                mult[ix_out.index(ix)] += m
            else:
                ix_out.append(ix)
                mult.append(m)
        if not keep:
            continue
        if not ix_in:
            raise ValueError(f"no input species: {text}")
        if unit == "cm":
            rfac = rfac * 1e-6 ** (n_in_total - 1)
        elif unit != "m":
            raise ValueError(f"invalid length unit {unit}")
        reactions.append(dict(text=text, how=how, data=data, ix_in=ix_in, ix_out=ix_out, mult=mult,
                              factor=rfac))
    species = [to_simple_ascii(nm) for nm in names]
    return species, reactions


def photoi_parameters(cfg: ProgramConfig):
    """(lambdas 1/m, coeffs 1/m^2, eta * quenching factor) of the Helmholtz
    photoionization (photoi_helmh_initialize, src/m_photoi_helmh.f90:44-160,
    and photoi_set_src, src/m_photoi.f90:153-205)."""
    p = cfg.gas_pressure
    frac_O2 = 0.0
    if "O2" in cfg.gas_components:
        frac_O2 = cfg.gas_fractions[cfg.gas_components.index("O2")]
    a = cfg.photoi_helmh_author
    tables = {
        "Luque": ([4425.38, 750.06], [337557.38, 19972.14]),
        "Bourdon-2": ([7305.62, 44081.25], [11814508.38, 998607256.0]),
        "Bourdon-3": ([4147.85, 10950.93, 66755.67], [1117314.935, 28692377.5, 2748842283.0]),
    }
    if a in tables:
        if frac_O2 <= 0.0:
            raise ValueError("Photoionization: no oxygen present")
        lam, co = (np.array(v, dtype=np.float64) for v in tables[a])
        if a == "Luque":
            lam = lam * (frac_O2 / 0.2) * p
            f = (frac_O2 / 0.2) * p
            co = co * (f * f)
        else:
            lam = lam * frac_O2 * p
            f = frac_O2 * p
            co = co * (f * f)
    elif a == "custom":
        lam = np.array(cfg.photoi_helmh_lambdas, dtype=np.float64) * p
        co = np.array(cfg.photoi_helmh_coeffs, dtype=np.float64) * (p * p)
        if len(lam) < 1 or len(lam) != len(co):
            raise ValueError("custom photoionization lambdas and coeffs missing")
    else:
        raise Unsupported(f"photoi_helmh%author = {a}")
    quench = cfg.photoi_quenching_pressure / (p + cfg.photoi_quenching_pressure)
    return lam, co, cfg.photoi_eta * quench


def new_style_columns(path, table_size, td_min, td_max_cfg):
    """td_tbl from new-style data (src/m_transport_data.f90:107-137): x in
    Td, columns mobility*N, diffusion*N, alpha/N, eta/N and the mean
    electron energy (eV) as in the file."""
    xm, ym = table_from_file(path, "Mobility *N (1/m/V/s)")
    td_max = xm[-1] if td_max_cfg < 0 else td_max_cfg
    x, inv_fac = sm.table_x(td_min, td_max, table_size)
    cols = [spaced_data(xm, ym, x)]
    for name in ("Diffusion coefficient *N (1/m/s)", "Townsend ioniz. coef. alpha/N (m2)",
                 "Townsend attach. coef. eta/N (m2)", "Mean energy (eV)"):
        cols.append(spaced_data(*table_from_file(path, name), x))
    return x, inv_fac, cols


def model_from_config(cfg: ProgramConfig) -> sm.StreamerModel:
    """The fluid model of a configuration: the integrator's state copies, the
    transport table, and either the standard chemistry (e, M+, M-; old-style
    data) or the reactions of the data file (chemistry_initialize,
    src/m_chemistry.f90:181-380)."""
    N = sm.gas_number_density(cfg.gas_pressure, cfg.gas_temperature)
    path = cfg.input_data_file
    if not os.path.isabs(path):
        path = os.path.join(cfg.base_dir, path)
    integ = TIME_INTEGRATORS[cfg.time_integrator]
    photoi = photoi_parameters(cfg) if cfg.photoi_enabled else None
    kw = {}
    if cfg.input_data_old_style:
        x, inv_fac, cols = old_style_columns(path, N, cfg.table_size, cfg.table_min_townsend,
                                             cfg.table_max_townsend)
        ix_pos = 1
        photoi_ix = 1
    else:
        x, inv_fac, cols = new_style_columns(path, cfg.table_size, cfg.table_min_townsend,
                                             cfg.table_max_townsend)
        gas_dens = [f * N for f in cfg.gas_fractions]
        species, reacts = read_reactions(path, cfg.gas_components, gas_dens, N)
        if species[0][0] != "e":
            raise Unsupported("the first plasma species must be the electron")
        if len(species) > ag.AFG_MAX_SPECIES or len(reacts) > ag.AFG_MAX_REACTIONS:
            raise Unsupported("too many species or reactions for the device tables")
        # chemtbl_fld: the tabulated rates on the transport table's grid
        # (the same x points, src/m_chemistry.f90:348-373)
        rlist = []
        for r in reacts:
            d = dict(ix_in=r["ix_in"], ix_out=r["ix_out"], mult=r["mult"], factor=r["factor"])
            if r["how"] == "field_table":
                xd, yd = table_from_file(path, r["data"])
                d.update(type=ag.RATE_TABULATED_FIELD, col=len(cols))
                cols.append(spaced_data(xd, yd, x))
            elif r["how"] in RATE_FORMS:
                typ, nco = RATE_FORMS[r["how"]]
                c = [_to_float(v) for v in r["data"].split()[:nco]]
                d.update(type=typ, c=c)
                if typ == ag.RATE_K1:
                    d.update(col=4)       # td_energy_eV
            elif r["how"] in GAS_TEMPERATURE_FORMS:
                nco, fn = GAS_TEMPERATURE_FORMS[r["how"]]
                c = [_to_float(v) for v in r["data"].split()[:nco]]
                d.update(type=ag.RATE_CONSTANT, c=[fn(c, cfg.gas_temperature)])
            else:
                raise Unsupported(f"rate expression {r['how']}")
            rlist.append(d)
        kw = dict(species=[sm.Species(nm, float(q)) for nm, q in species], reactions=rlist)
        names = [nm for nm, _ in species]
        ix_pos = next(i for i, (_, q) in enumerate(species) if q == 1)
        if cfg.photoi_enabled and cfg.photoi_species not in names:
            raise Unsupported(f"photoi%species {cfg.photoi_species} is not a species of the chemistry")
        photoi_ix = names.index(cfg.photoi_species) if cfg.photoi_enabled else 1
    if cfg.mobile_ions:
        # transport_data_ions (src/m_transport_data.f90:186-208): mobilities at
        # 1 bar and 300 K, scaled there by the gas density of those conditions
        names = [sp_.name for sp_ in kw.get("species", [])] or ["e", "M_plus", "M_min"]
        missing = [n for n in cfg.mobile_ions if n not in names]
        if missing:
            raise ValueError(f"mobile ions not in the chemistry: {missing}")
        kw["mobile_ions"] = [(names.index(n), mob) for n, mob in zip(cfg.mobile_ions, cfg.ion_mobilities)]
    m = sm.StreamerModel(ndim=cfg.ndim, n_states=sm.states_needed(integ), N=N,
                         tabulated=dict(x=x, inv_fac=inv_fac, cols=cols),
                         photoi_modes=0 if photoi is None else len(photoi[0]),
                         photoi_species_index=photoi_ix, electrode=cfg.use_electrode, **kw)
    m.ix_pos_ion = ix_pos
    m.integrator = integ
    m.photoi_params = photoi
    m.photoi_max_rel_residual = cfg.photoi_helmh_max_rel_residual
    return m


# ---------------------------------------------------------------------------
# initial conditions


def box_centers_with_ghosts(tree, ids):
    """af_r_cc over cells 0..nc+1 of boxes `ids` (1-based): shape
    [len(ids), D, (k,) j, i] (C order, i fastest)."""
    nc, D = tree.n_cell, tree.ndim
    idx = np.arange(0, nc + 2, dtype=np.float64) - 0.5
    out = np.empty((len(ids), D) + (nc + 2,) * D)
    for d in range(D):
        shape = [1] * D
        shape[D - 1 - d] = nc + 2
        r = tree.r_min[ids - 1, d][:, None] + idx[None, :] * tree.dr[ids - 1, d][:, None]
        out[:, d] = r.reshape((len(ids),) + tuple(shape))
    return out


def _dist_vec_line(r, r0, r1):
    """GM_dist_vec_line (src/m_geometry.f90): r has the dimension first."""
    D = r.shape[0]
    line_len2 = 0.0
    for d in range(D):
        line_len2 = line_len2 + (r1[d] - r0[d]) * (r1[d] - r0[d])
    frac = np.zeros(r.shape[1:])
    for d in range(D):
        frac = frac + (r[d] - r0[d]) * (r1[d] - r0[d])
    lo, hi = frac <= 0.0, frac >= line_len2
    dv = np.empty_like(r)
    for d in range(D):
        mid = r[d] - (r0[d] + frac / line_len2 * (r1[d] - r0[d])) if line_len2 > 0 else r[d] - r0[d]
        dv[d] = np.where(lo, r[d] - r0[d], np.where(hi, r[d] - r1[d], mid))
    frac = np.where(lo, 0.0, np.where(hi, 1.0, frac / line_len2 if line_len2 > 0 else 0.0))
    return dv, frac


def density_line(r, r0, r1, n0, n1, width, falloff):
    """GM_density_line (src/m_geometry.f90) for the fall-off types sigmoid,
    gaussian, smoothstep and step; r has the dimension first."""
    dv, frac = _dist_vec_line(r, r0, r1)
    s = np.zeros(r.shape[1:])
    for d in range(r.shape[0]):
        s = s + dv[d] * dv[d]
    dist = np.sqrt(s)
    if falloff == "smoothstep":
        t = dist / width - 1
        val = np.where(dist < width, 1.0,
                       np.where(dist < 2 * width, 1 - (3 * (t * t) - 2 * (t * t * t)), 0.0))
    elif falloff == "gaussian":
        q = dist / width
        val = np.exp(-(q * q))
    elif falloff == "sigmoid":
        tmp = dist / width
        with np.errstate(over="ignore"):
            val = np.where(tmp > math.log(0.5 * np.finfo(np.float64).max), 0.0, 2 / (1 + np.exp(tmp)))
    elif falloff == "step":
        val = np.where(dist < width, 1.0, 0.0)
    else:
        raise Unsupported(f"seed_falloff = {falloff}")
    return val * (frac * n0 + (1 - frac) * n1)


def seeds(cfg: ProgramConfig):
    """Seed end points in metres (src/m_init_cond.f90:98-101)."""
    D = cfg.ndim
    L, O = np.asarray(cfg.domain_len), np.asarray(cfg.domain_origin)
    out = []
    for n in range(len(cfg.seed_density)):
        r0 = np.asarray(cfg.seed_rel_r0[D * n:D * (n + 1)]) * L + O
        r1 = np.asarray(cfg.seed_rel_r1[D * n:D * (n + 1)]) * L + O
        out.append((r0, r1))
    return out


def initial_densities(cfg: ProgramConfig, tree, ids):
    """init_cond_set_box (src/m_init_cond.f90:214-293) for boxes `ids`,
    ghost cells included: (electrons, positive ions), each
    [len(ids), (nc+2)^D]."""
    r = box_centers_with_ghosts(tree, ids)
    n2 = (tree.n_cell + 2) ** tree.ndim
    e = np.full(r.shape[:1] + r.shape[2:], cfg.background_density)
    ion = e.copy()
    rr = np.moveaxis(r, 1, 0)
    for n, (r0, r1) in enumerate(seeds(cfg)):
        dens = density_line(rr, r0, r1, cfg.seed_density[n], cfg.seed_density2[n], cfg.seed_width[n],
                            cfg.seed_falloff[n])
        ct = cfg.seed_charge_type[n]
        if ct == -1:
            e = e + dens
        elif ct == 0:
            ion = ion + dens
            e = e + dens
        elif ct == 1:
            ion = ion + dens
        else:
            raise ValueError("invalid seed_charge_type")
    return e.reshape(len(ids), n2), ion.reshape(len(ids), n2)


def refine_desc(cfg: ProgramConfig, model: sm.StreamerModel, time: float):
    """default_refinement's parameters (src/m_refine.f90:197-298) at `time`:
    the seed rule only while time < refine_init_time."""
    d = model.refine_desc(adx=cfg.refine_adx, adx_fac=cfg.refine_adx_fac, min_dens=cfg.refine_min_dens,
                          derefine_dx=cfg.derefine_dx, max_dx=cfg.refine_max_dx, min_dx=cfg.refine_min_dx,
                          ref_buffer=cfg.refine_buffer_width, init_fac=cfg.refine_init_fac,
                          use_alpha_effective=int(cfg.refine_use_alpha_effective))
    if cfg.use_electrode:
        # current_electrode_dx (src/streamer.f90:216-225; electrode_derefine_factor 1)
        d.electrode_mg, d.electrode_dx = 0, cfg.refine_electrode_dx
    if time < cfg.refine_init_time:
        sd = seeds(cfg)
        if len(sd) > ag.AFG_MAX_REFINE_ITEMS:
            raise Unsupported("too many seeds")
        d.n_seeds = len(sd)
        for n, (r0, r1) in enumerate(sd):
            for k in range(cfg.ndim):
                d.seed_r0[n][k] = r0[k]
                d.seed_r1[n][k] = r1[k]
            d.seed_width[n] = cfg.seed_width[n]
    return d


def total_volume(tree):
    """af_total_volume (afivo/src/m_af_types.f90:805-825): the coarse boxes'
    volume, rings of pi (r1^2 - r0^2) L_z in 2D cylindrical coordinates."""
    box_len = tree.n_cell * np.asarray(tree.dr_base, dtype=np.float64)
    ids = np.asarray(tree.lvl_ids[0]) - 1
    if tree.ndim == 2 and tree.coord == at.AF_CYL:
        vol = 0.0
        for b in ids:
            r0 = float(tree.r_min[b, 0])
            r1 = r0 + box_len[0]
            vol = vol + math.pi * (r1 * r1 - r0 * r0) * box_len[-1]
        return vol
    return len(ids) * float(np.prod(box_len))


def regression_values(tree, leaf_values):
    """output_regression_log's columns (src/m_output.f90:787-842) for one
    species: sum(n)/vol and sum(n^2)/vol over leaves with af_tree_sum_cc's
    level-by-level accumulation (afivo/src/m_af_utils.f90:966-1026; in 2D
    cylindrical coordinates the sum of 2 pi r n per cell, sum_2pr_box), and
    the maximum over leaves.  `leaf_values[l]` holds the interiors of the
    leaves of level l+1 as [n_leaves, nc^D] in the reference's cell order
    (i fastest)."""
    nc, D = tree.n_cell, tree.ndim
    cyl = D == 2 and tree.coord == at.AF_CYL
    twopi = 2 * math.acos(-1.0)
    s1 = s2 = 0.0
    mx = -np.finfo(np.float64).max / 10
    for lvl in range(1, tree.highest_lvl + 1):
        v = leaf_values[lvl - 1]
        if v.size == 0:
            continue
        ids = np.asarray(tree.lvl_leaves[lvl - 1]) - 1
        fac = float(np.prod(tree.dr[ids[0]]))
        for q, b in enumerate(ids):
            x = v[q]
            if cyl:
                r = tree.r_min[b, 0] + (np.arange(1, nc + 1) - 0.5) * tree.dr[b, 0]
                w = np.tile(r, nc)
                t1 = float(np.sum(x * w)) * twopi
                t2 = float(np.sum(x * x * w)) * twopi
            else:
                t1, t2 = float(np.sum(x)), float(np.sum(x * x))
            s1 = s1 + fac * t1
            s2 = s2 + fac * t2
        mx = max(mx, float(v.max()))
    vol = total_volume(tree)
    return s1 / vol, s2 / vol, mx


# ---------------------------------------------------------------------------
# the program


AF_MAX_LVL = 30                     # af_max_lvl (afivo/src/m_af_types.f90)
MAX_ATTEMPTS_PER_TIME_STEP = 10     # src/streamer.f90


class Program:
    """set_initial_conditions and the time loop of the `streamer` program
    (src/streamer.f90:181-432, 480-533) over an engine.

    `engine_factory(tree, model, voltage, cfg)` returns an object with:
    `tree`; `set_initial(ids, electrons, ions)` (state 0 of the first two
    species, ghost cells included); `field(have_guess)` (field_compute of
    state 0); `advance(dt)` (copy_current_state, the integrator's
    forward_euler stages; returns the last stage's dt limit
    min(dt_max, cfl_number/max cfl_sum, dielectric relaxation time,
    chemistry limit)); `restore()` (restore_previous_state: densities and
    phi from the backup, then the field of that phi);
    `refine(desc, restrict_first)` (af_restrict_tree + af_gc_tree of the
    densities when `restrict_first`, the refinement flags, af_adjust_refinement
    with auto_prolong; returns (n_add, n_rm, added ids)); and
    `leaf_values(species)` (interiors of the leaves per level); with
    photoionization `photoi()` (photoi_set_src: the source from alpha and the
    Helmholtz modes).
    """

    def __init__(self, cfg: ProgramConfig, engine_factory, log=None):
        self.cfg = cfg
        self.model = model_from_config(cfg)
        D = cfg.ndim
        L = np.asarray(cfg.domain_len, dtype=np.float64)
        cgs = list(cfg.coarse_grid_size)
        if all(c == -1 for c in cgs):
            cgs = [cfg.box_size * int(round(v / L.min())) for v in L]
        self.cgs = np.asarray(cgs)
        # field_initialize (src/m_field.f90:119-172): field_given_by 'field E'
        # or the deprecated field_amplitude give -domain_len * E
        if cfg.field_given_by is not None:
            kind, val = cfg.field_given_by[0], _to_float(cfg.field_given_by[1])
            self.voltage = -cfg.domain_len[D - 1] * val if kind == "field" else val
        else:
            self.voltage = -cfg.domain_len[D - 1] * cfg.field_amplitude
        self.factory = engine_factory
        self.log = log
        self.rows = []
        self.n_steps = self.n_rejected = 0

    def _say(self, *a):
        if self.log:
            self.log(*a)

    def initial_tree(self):
        """af_init plus af_refine_up_to_lvl to the first level whose grid
        spacing is at most refine_max_dx (src/streamer.f90:486-490)."""
        dr_base = np.asarray(self.cfg.domain_len) / self.cgs
        for lvl in range(1, AF_MAX_LVL):
            if np.all(dr_base / 2.0 ** (lvl - 1) <= self.cfg.refine_max_dx):
                break
        coord = at.AF_CYL if self.cfg.cylindrical else at.AF_XYZ
        return at.uniform_tree(self.cfg.ndim, self.cfg.box_size, self.cgs, self.cfg.domain_len, lvl,
                               coord=coord, r_base=np.asarray(self.cfg.domain_origin, dtype=np.float64))

    def set_initial_conditions(self):
        cfg = self.cfg
        tree = self.initial_tree()
        self.engine = eng = self.factory(tree, self.model, self.voltage, cfg)
        ids = np.arange(1, tree.n_boxes + 1, dtype=np.int32)
        eng.set_initial(ids, *initial_densities(cfg, tree, ids))
        for n in range(100):
            eng.field(False)
            n_add, n_rm, added = eng.refine(refine_desc(cfg, self.model, 0.0), False)
            self._say(f"initial refinement {n}: +{n_add} -{n_rm} boxes, {eng.tree.n_boxes} in use")
            if len(added):
                eng.set_initial(added, *initial_densities(cfg, eng.tree, added))
            if n_add == 0:
                break

    def regression_row(self, cnt, time, dt):
        vals = [self.engine_values(s) for s in range(len(self.model.species))]
        row = [cnt, time, dt] + [v[0] for v in vals] + [v[1] for v in vals] + [v[2] for v in vals]
        self.rows.append(row)
        self._say("row", " ".join(f"{x:.8e}" for x in row[1:]))
        return row

    def engine_values(self, s):
        return regression_values(self.engine.tree, self.engine.leaf_values(s))

    def run(self, end_time=None, max_outputs=None):
        """The time loop until `end_time` (default: the configuration's), or
        until `max_outputs` rows after the initial one; returns the rows of
        the regression log."""
        cfg, eng = self.cfg, self.engine
        end_time = cfg.end_time if end_time is None else end_time
        time = global_time = 0.0
        dt = global_dt = cfg.dt_min
        it = it_last_output = output_cnt = 0
        time_last_output = time
        frac_rejected = 0.0
        self.regression_row(0, global_time, global_dt)
        while True:
            it += 1
            if time >= end_time or (max_outputs is not None and output_cnt >= max_outputs):
                break
            write_out = time + dt >= time_last_output + cfg.output_dt
            if write_out:
                dt = min(dt, max(0.0, time_last_output + cfg.output_dt - time))
            if cfg.photoi_enabled and it % cfg.photoi_per_steps == 0:
                eng.photoi()
            if cfg.use_electrode:
                eng.electrode_densities()
            dt_lim = 1e100
            for n in range(MAX_ATTEMPTS_PER_TIME_STEP):
                lim = eng.advance(dt)
                time = time + dt
                dt_lim = min(dt_lim, lim)
                if dt <= lim:
                    break
                self.n_rejected += 1
                self._say(f"step {it} rejected at t = {global_time:.6e}: dt = {dt:.4e}, limit {lim:.4e}")
                dt = cfg.dt_safety_factor * lim
                time = global_time
                write_out = False
                eng.restore()
            else:
                raise RuntimeError("All time steps were rejected")
            frac_rejected = 0.99 * frac_rejected + (0.01 if n > 0 else 0.0)
            eng.field(True)
            growth = 1.0 if frac_rejected > 0.1 else cfg.dt_max_growth_factor
            dt = min(growth * global_dt, cfg.dt_safety_factor * min(dt_lim, cfg.dt_max))
            global_dt, global_time = dt, time
            self.n_steps += 1
            if global_dt < cfg.dt_min:
                raise RuntimeError(f"dt too small ({global_dt:.4e})")
            if write_out:
                output_cnt += 1
                time_last_output, it_last_output = global_time, it
                self.regression_row(output_cnt, global_time, global_dt)
            if it % cfg.refine_per_steps == 0:
                n_add, n_rm, _ = eng.refine(refine_desc(cfg, self.model, global_time), True)
                if n_add > 0 or n_rm > 0:
                    eng.field(True)
                    if cfg.photoi_enabled:
                        eng.photoi()
        return self.rows


def read_regression_log(path):
    """Rows of a regression log (src/m_output.f90:787-842): header names and
    a float array [n_rows, 3 + 3 * n_species]."""
    with open(path) as f:
        head = f.readline().split()
        rows = [[float(v) for v in ln.split()] for ln in f if ln.strip()]
    return head, np.array(rows)


class GpuEngine:
    """The program's engine on one GPU through the C-ABI.  The state lives on
    the device; the host sees it only for the initial values of new boxes
    (afg_cc_upload of the chosen boxes) and the regression rows (download of
    one density).  `precision` selects the FP64 path (the reference's
    arithmetic) or AFG_MIXED (FP32 inner multigrid and transport with an FP64
    state)."""

    def __init__(self, tree, model, voltage, cfg, precision=ag.FP64, ctx=None):
        self.ctx = ctx if ctx is not None else ag.Context(0)
        self.m, self.cfg, self.voltage, self.precision = model, cfg, voltage, precision
        # one extra variable: the backup of phi kept by copy_current_state
        self.iv_phi_copy = model.n_var_cell + 1
        self.n_var = model.n_var_cell + 1
        self.stages = sm.INTEGRATORS[model.integrator]
        self.tree = tree
        self.ctx.tree_sync(tree, self.n_var, model.n_var_face)
        self.run = sm.StreamerRun(self.ctx, tree, model, voltage, 0.0, precision,
                                  max_rel_residual=cfg.multigrid_max_rel_residual,
                                  num_vcycles=cfg.multigrid_num_vcycles, integrator=model.integrator,
                                  photoi=model.photoi_params, photoi_per_steps=cfg.photoi_per_steps,
                                  dt_cfl_number=cfg.dt_cfl_number, dt_max=cfg.dt_max)
        self._setup()

    def _setup(self):
        m = self.m
        self.run.tree = self.tree
        self.run.setup()
        # rhs: af_bc_neumann_zero + af_gc_interp (src/streamer.f90:74-79)
        self.ctx.set_cc_methods(m.i_rhs, [ag.BC_NEUMANN] * (2 * self.tree.ndim), None, ag.RB_INTERP)
        if m.electrode:
            # the field's electrode on every box (set_lsf_box, mg_set_box_tag)
            # and the update's gas mask
            self.ctx.mg_set_lsf(0, electrode_desc(self.cfg, m.i_lsf))
            self.ctx.transport_set_electrode(m.i_lsf)

    def electrode_densities(self):
        """set_electrode_densities (src/streamer.f90:590-594)."""
        self.ctx.electrode_species_bc(0, 0, self.m.ix_pos_ion, True)

    def set_initial(self, ids, e, ion):
        m, t = self.m, self.tree
        h = ag.new_cc(t, 2)
        idx = np.asarray(ids, dtype=np.int64) - 1
        h[idx, 0] = e.reshape((len(idx),) + h.shape[2:])
        h[idx, 1] = ion.reshape((len(idx),) + h.shape[2:])
        bp = ag.box_pointers(h)
        keep = np.zeros(t.n_boxes, dtype=bool)
        keep[idx] = True
        bp.addr[~keep] = 0
        self.ctx.upload_vars(h, [m.species_iv[0], m.species_iv[m.ix_pos_ion]], bp=bp)
        if m.electrode:
            self.ctx.electrode_init_densities(0, ids)

    def field(self, have_guess):
        if not have_guess:
            self.ctx.gc(self.m.i_phi, 0, True)
        self.run.field(0, have_guess)

    def advance(self, dt):
        ctx, m = self.ctx, self.m
        for s in range(len(m.species)):
            ctx.tree_copy_cc(m.species_iv[s], m.species_iv[s] + m.n_states - 1)
        ctx.tree_copy_cc(m.i_phi, self.iv_phi_copy)
        lim = 1e100
        for i, (f, s_deriv, s_prev, w_prev, s_out) in enumerate(self.stages, 1):
            lim, _ = ctx.forward_euler(f * dt, self.run.voltage, s_deriv, s_prev, w_prev, s_out, i,
                                       len(self.stages))
        return lim

    def photoi(self):
        lam, coeffs, coeff = self.m.photoi_params
        self.ctx.photoi_helmh(coeff, self.run.mode_ids, coeffs, 1e-2, 10)

    def restore(self):
        ctx, m = self.ctx, self.m
        for s in range(len(m.species)):
            ctx.tree_copy_cc(m.species_iv[s] + m.n_states - 1, m.species_iv[s])
        ctx.tree_copy_cc(self.iv_phi_copy, m.i_phi)
        ctx.field_from_potential(m.i_phi)

    def auto_vars(self):
        """(variable, prolongation) of auto_prolong: the densities and rhs by
        af_prolong_limit (ST_prolongation_method), phi and |E| by the default
        af_prolong_linear (src/streamer.f90:60-79, afivo/src/m_af_core.f90:
        343-410)."""
        m = self.m
        out = [(m.species_iv[s], "limit") for s in range(len(m.species))]
        out += [(m.i_phi, "linear"), (m.i_electric_fld, "linear"), (m.i_rhs, "limit")]
        if m.i_photo:
            out.append((m.i_photo, "linear"))
        return out

    def refine(self, desc, restrict_first):
        ctx, m, tree = self.ctx, self.m, self.tree
        if restrict_first:
            for s in range(len(m.species)):
                ctx.restrict_tree(m.species_iv[s])
                ctx.gc(m.species_iv[s], 0, True)
        flags = ctx.refine_flags(desc)
        new = ag.adjust_refinement(tree, flags, AF_MAX_LVL)
        if new is tree:
            return 0, 0, np.zeros(0, dtype=np.int32)
        old_id = at.remap_ids(tree, new)
        keep = old_id > 0
        n_add = int(np.count_nonzero(~keep))
        n_rm = tree.n_boxes - int(np.count_nonzero(keep))
        if n_add == 0 and n_rm == 0:
            return 0, 0, np.zeros(0, dtype=np.int32)
        ctx.tree_remap(new, old_id)
        self.tree = new
        self._setup()
        limiter = m.transport_desc(self.precision).prolong_limiter
        fresh = np.nonzero(~keep)[0].astype(np.int32) + 1
        lv = new.lvl[fresh - 1]
        for lvl in sorted(set(lv.tolist())):
            ids = fresh[lv == lvl]
            for iv, how in self.auto_vars():
                ctx.gc(iv, lvl - 1, True)
                if how == "limit":
                    ctx.prolong_limit(iv, ids, limiter)
                else:
                    ctx.prolong_linear(iv, ids)
            for iv, _ in self.auto_vars():
                ctx.gc(iv, lvl, True)
        return n_add, n_rm, fresh

    def leaf_values(self, s):
        t, nc, D = self.tree, self.tree.n_cell, self.tree.ndim
        h = ag.new_cc(t, 1)
        self.ctx.download_vars(h, [self.m.species_iv[s]])
        sl = (slice(1, nc + 1),) * D
        out = []
        for lvl in range(1, t.highest_lvl + 1):
            ids = np.asarray(t.lvl_leaves[lvl - 1], dtype=np.int64) - 1
            out.append(h[ids, 0][(slice(None),) + sl].reshape(len(ids), nc ** D))
        return out

    def close(self):
        self.ctx.close()


def fortran_e(x, digits=8, exp_digits=3, width=20):
    """One field of the Fortran edit descriptor E20.8e3 (`0.dddddddd E+eee`,
    right-justified), as output_regression_log writes it."""
    if x == 0:
        mant, e = "0." + "0" * digits, 0
    else:
        s = f"{abs(x):.{digits - 1}e}"          # d.ddddddde+XX
        m, ex = s.split("e")
        mant, e = "0." + m.replace(".", ""), int(ex) + 1
    sign = "-" if x < 0 else ""
    es = "+" if e >= 0 else "-"
    return f"{sign}{mant}E{es}{abs(e):0{exp_digits}d}".rjust(width)


def write_regression_log(path, species_names, rows):
    """The log file of output_regression_log (src/m_output.f90:787-842):
    a header line, then per output `I0` and 3 + 3 * n_species E20.8e3."""
    with open(path, "w") as f:
        f.write("it time dt" + "".join(f" sum({n})" for n in species_names)
                + "".join(f" sum({n}^2)" for n in species_names)
                + "".join(f" max({n})" for n in species_names) + "\n")
        for r in rows:
            f.write(f"{int(r[0])}" + "".join(fortran_e(float(v)) for v in r[1:]) + "\n")


def main(argv=None):
    """Run a reference configuration file on the GPU and write its regression
    log, e.g. `python streamer_program.py test_2d.cfg --ndim 2 --log out.log`
    (the reference's tools/compare_logs.py compares such logs)."""
    import argparse
    import functools
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("cfg")
    ap.add_argument("--ndim", type=int, default=2, choices=[2, 3])
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--log", default=None,
                    help="regression log to write (default: <cfg name>_rtest.out.log in the current directory)")
    ap.add_argument("--end-time", type=float, default=None)
    a = ap.parse_args(argv)
    cfg = ProgramConfig(a.cfg, ndim=a.ndim)
    prec = ag.FP64 if a.precision == "fp64" else ag.MIXED
    prog = Program(cfg, functools.partial(GpuEngine, precision=prec), log=print)
    prog.set_initial_conditions()
    rows = prog.run(end_time=a.end_time)
    out = a.log or os.path.splitext(os.path.basename(a.cfg))[0] + "_rtest.out.log"
    write_regression_log(out, [s.name for s in prog.model.species], rows)
    prog.engine.close()
    print(f"{prog.n_steps} steps ({prog.n_rejected} rejected); log written to {out}")


if __name__ == "__main__":
    main()
