"""Python host side of the afivo GPU hot path: ctypes bindings of the C-ABI
(``include/afivo_gpu.h``) and a small object layer that mirrors the Fortran
API of the path (``mg_fas_vcycle``, ``mg_fas_fmg``, ``af_gc_lvl``,
``af_tree_maxabs_cc`` ...; afivo/src/m_af_multigrid.f90:14-38,
afivo/src/m_af_ghostcell.f90:12-20, afivo/src/m_af_utils.f90:773-784).

The compute path is the CUDA library ``libafivo_gpu.so`` built in this
directory; importing this module fails loudly when it is missing, and no
operation has a CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libafivo_gpu.so")

AFG_OK = 0
AFG_ERR_ARG = -1
AFG_ERR_CUDA = -2
AFG_ERR_UNSUPPORTED = -3
AFG_ERR_STATE = -4
AFG_ERR_DEVICE = -5
AFG_ERR_NOCONV = -6
AFG_ERR_NOMEM = -7

AFG_XYZ = 1
AFG_CYL = 2
BC_DIRICHLET = -10
BC_NEUMANN = -11
BC_CONTINUOUS = -12
BC_DIRICHLET_COPY = -13
RB_MG_SIDES = 0
RB_INTERP = 1
RB_INTERP_LIM = 2
FP64 = 0
MIXED = 1
GSRB_STAGED = 16       # smoother variant code flag: shared-memory-staged persistent kernel
GSRB_STAGED_RHS = 32   # ... with the rhs block staged too
CYCLE_DOWN = 1
CYCLE_UP = 3
KT_NONE, KT_GSRB, KT_GHOST, KT_FLUX, KT_UPDATE, KT_RESIDUAL = 0, 1, 2, 3, 4, 5
KT_DEFECT, KT_RESTRICT, KT_CORRECT, KT_COARSE, KT_FIELD, KT_COPY, KT_NCLASS, KT_ALL = 6, 7, 8, 9, 10, 11, 12, 15
KT_NAMES = {KT_GSRB: "gsrb", KT_GHOST: "ghost", KT_FLUX: "flux", KT_UPDATE: "update", KT_RESIDUAL: "residual",
            KT_DEFECT: "defect", KT_RESTRICT: "restrict", KT_CORRECT: "correct", KT_COARSE: "coarse",
            KT_FIELD: "field", KT_COPY: "copy"}

_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)


class TreeDesc(C.Structure):
    _fields_ = [
        ("ndim", C.c_int), ("n_cell", C.c_int), ("coord", C.c_int),
        ("n_boxes", C.c_int), ("highest_lvl", C.c_int),
        ("coarse_grid_size", C.c_int * 3),
        ("lvl", _IP), ("ix", _IP), ("parent", _IP), ("children", _IP),
        ("neighbors", _IP), ("neighbor_mat", _IP),
        ("r_min", _DP), ("dr", _DP),
        ("ids_off", _IP), ("ids", _IP),
        ("leaves_off", _IP), ("leaves", _IP),
        ("parents_off", _IP), ("parents", _IP),
    ]


class GcDesc(C.Structure):
    _fields_ = [("bc_type", C.c_int * 6), ("bc_val", C.c_double * 6),
                ("rb", C.c_int)]


class MgDesc(C.Structure):
    _fields_ = [
        ("i_phi", C.c_int), ("i_rhs", C.c_int), ("i_tmp", C.c_int),
        ("n_cycle_down", C.c_int), ("n_cycle_up", C.c_int),
        ("helmholtz_lambda", C.c_double),
        ("bc_type", C.c_int * 6), ("bc_val", C.c_double * 6),
        ("precision", C.c_int),
    ]


LSF_SPHERE, LSF_ROD, LSF_ROD_CONE_TOP, LSF_ROD_ROD, LSF_SPHERE_ROD, LSF_TWO_ROD_CONE, LSF_COAXIAL = range(1, 8)


class LsfDesc(C.Structure):
    """afg_lsf_desc: the electrode of a field solve (absolute coordinates)."""
    _fields_ = [
        ("shape", C.c_int), ("i_lsf", C.c_int),
        ("r0", C.c_double * 3), ("r1", C.c_double * 3), ("radius", C.c_double),
        ("r2_0", C.c_double * 3), ("r2_1", C.c_double * 3), ("radius2", C.c_double),
        ("cone_tip_radius", C.c_double), ("cone_length_frac", C.c_double),
        ("cone2_tip_radius", C.c_double), ("cone2_length_frac", C.c_double),
        ("center", C.c_double * 3),
        ("grounded", C.c_int), ("grounded2", C.c_int),
        ("length_scale", C.c_double), ("gradient_safety_factor", C.c_double),
        ("tol", C.c_double), ("min_rel_distance", C.c_double),
    ]


def lsf_desc(shape, i_lsf, r0, r1=None, radius=0.0, r2_0=None, r2_1=None, radius2=0.0, cone_tip_radius=0.0,
             cone_length_frac=0.0, cone2_tip_radius=0.0, cone2_length_frac=0.0, center=None, grounded=False,
             grounded2=False, length_scale=None, gradient_safety_factor=1.5, tol=1e-8, min_rel_distance=1e-4):
    """An afg_lsf_desc with the reference's mg_t defaults (m_af_types.f90:
    604-619) and length_scale = radius as src/m_field.f90:389 sets it."""
    d = LsfDesc()
    d.shape, d.i_lsf = shape, i_lsf
    for name, v in (("r0", r0), ("r1", r1), ("r2_0", r2_0), ("r2_1", r2_1), ("center", center)):
        if v is not None:
            arr = getattr(d, name)
            for k, x in enumerate(v):
                arr[k] = x
    d.radius, d.radius2 = radius, radius2
    d.cone_tip_radius, d.cone_length_frac = cone_tip_radius, cone_length_frac
    d.cone2_tip_radius, d.cone2_length_frac = cone2_tip_radius, cone2_length_frac
    d.grounded, d.grounded2 = int(grounded), int(grounded2)
    d.length_scale = radius if length_scale is None else length_scale
    d.gradient_safety_factor, d.tol, d.min_rel_distance = gradient_safety_factor, tol, min_rel_distance
    return d


AFG_MAX_SPECIES = 16
AFG_MAX_REACTIONS = 32
AFG_MAX_FLUX = 8
RATE_TABULATED_FIELD = 1
RATE_CONSTANT = 2
RATE_LINEAR = 3
RATE_EXP_V1 = 4
RATE_EXP_V2 = 5
RATE_K1 = 6
RATE_K13 = 18
RATE_K14 = 19
LIMITER_VANLEER = 1
LIMITER_KOREN = 2
LIMITER_MINMOD = 3
LIMITER_MC = 4
LIMITER_GMINMOD43 = 5


class Reaction(C.Structure):
    _fields_ = [("rate_type", C.c_int), ("lt_col", C.c_int), ("rate_factor", C.c_double),
                ("c", C.c_double * 4), ("n_in", C.c_int), ("ix_in", C.c_int * 4),
                ("n_out", C.c_int), ("ix_out", C.c_int * 4), ("mult_out", C.c_int * 4)]


AFG_MAX_REFINE_ITEMS = 8
REF_RM, REF_KEEP, REF_DO = -1, 0, 1
_R3 = C.c_double * 3


class RefineDesc(C.Structure):
    """afg_refine_desc: parameters of default_refinement (src/m_refine.f90)."""
    _fields_ = [
        ("i_electron", C.c_int), ("i_electric_fld", C.c_int), ("lt_col_alpha", C.c_int),
        ("lt_col_eta", C.c_int), ("use_alpha_effective", C.c_int), ("gas_number_density", C.c_double),
        ("adx", C.c_double), ("adx_fac", C.c_double), ("min_dens", C.c_double), ("derefine_dx", C.c_double),
        ("max_dx", C.c_double), ("min_dx", C.c_double), ("ref_buffer", C.c_int),
        ("n_seeds", C.c_int), ("seed_r0", _R3 * AFG_MAX_REFINE_ITEMS), ("seed_r1", _R3 * AFG_MAX_REFINE_ITEMS),
        ("seed_width", C.c_double * AFG_MAX_REFINE_ITEMS), ("init_fac", C.c_double),
        ("n_regions", C.c_int), ("region_rmin", _R3 * AFG_MAX_REFINE_ITEMS),
        ("region_rmax", _R3 * AFG_MAX_REFINE_ITEMS), ("region_dr", C.c_double * AFG_MAX_REFINE_ITEMS),
        ("n_limits", C.c_int), ("limit_rmin", _R3 * AFG_MAX_REFINE_ITEMS),
        ("limit_rmax", _R3 * AFG_MAX_REFINE_ITEMS), ("limit_dr", C.c_double * AFG_MAX_REFINE_ITEMS),
        ("electrode_mg", C.c_int), ("electrode_dx", C.c_double),
    ]


class TransportDesc(C.Structure):
    _fields_ = [
        ("n_species", C.c_int), ("species_iv", C.c_int * AFG_MAX_SPECIES),
        ("species_charge", C.c_double * AFG_MAX_SPECIES),
        ("n_flux", C.c_int), ("flux_species", C.c_int * AFG_MAX_FLUX),
        ("flux_fc", C.c_int * AFG_MAX_FLUX), ("flux_charge_sign", C.c_double * AFG_MAX_FLUX),
        ("ion_mobility_N", C.c_double * AFG_MAX_FLUX),
        ("i_electric_fld", C.c_int), ("i_efield_fc", C.c_int), ("i_photo", C.c_int),
        ("photoi_species", C.c_int), ("gas_number_density", C.c_double),
        ("species_gc", GcDesc), ("prolong_limiter", C.c_int),
        ("lt_n_points", C.c_int), ("lt_x_min", C.c_double), ("lt_inv_fac", C.c_double),
        ("lt_n_cols", C.c_int), ("lt_data", C.POINTER(C.c_double)),
        ("lt_col_mobility", C.c_int), ("lt_col_diffusion", C.c_int), ("lt_col_alpha", C.c_int),
        ("n_reactions", C.c_int), ("reactions", Reaction * AFG_MAX_REACTIONS),
        ("dt_chemistry_nmin", C.c_double), ("dt_chemistry_limit_loss", C.c_int),
        ("precision", C.c_int),
    ]


class StageDesc(C.Structure):
    """afg_stage_desc: the settings forward_euler reads (m_field's solver and
    convergence settings, m_dt's dt_cfl_number and dt_max)."""
    _fields_ = [
        ("mg_id", C.c_int), ("domain_len", C.c_double), ("max_rel_residual", C.c_double),
        ("num_vcycles", C.c_int), ("dt_cfl_number", C.c_double), ("dt_max", C.c_double),
    ]


def _ip(a):
    return a.ctypes.data_as(_IP)


def _dp(a):
    return a.ctypes.data_as(_DP)


class TreeDescHolder:
    """Keeps the numpy arrays behind a TreeDesc alive."""

    def __init__(self, tree):
        t = tree
        self.arrays = {
            "lvl": np.ascontiguousarray(t.lvl, dtype=np.int32),
            "ix": np.ascontiguousarray(t.ix, dtype=np.int32),
            "parent": np.ascontiguousarray(t.parent, dtype=np.int32),
            "children": np.ascontiguousarray(t.children, dtype=np.int32),
            "neighbors": np.ascontiguousarray(t.neighbors, dtype=np.int32),
            "neighbor_mat": np.ascontiguousarray(t.neighbor_mat, dtype=np.int32),
            "r_min": np.ascontiguousarray(t.r_min, dtype=np.float64),
            "dr": np.ascontiguousarray(t.dr, dtype=np.float64),
        }
        (io, i), (lo, l), (po, p) = t.flat_lists()
        self.arrays.update(ids_off=io, ids=i, leaves_off=lo, leaves=l,
                           parents_off=po, parents=p)
        d = TreeDesc()
        d.ndim = t.ndim
        d.n_cell = t.n_cell
        d.coord = t.coord
        d.n_boxes = t.n_boxes
        d.highest_lvl = t.highest_lvl
        for k in range(3):
            d.coarse_grid_size[k] = int(t.coarse_grid_size[k]) if k < t.ndim else 1
        for name, arr in self.arrays.items():
            setattr(d, name, _dp(arr) if arr.dtype == np.float64 else _ip(arr))
        self.desc = d


def gc_desc(bc_type, bc_val=None, rb=RB_MG_SIDES) -> GcDesc:
    g = GcDesc()
    for n in range(6):
        g.bc_type[n] = int(bc_type[n]) if n < len(bc_type) else BC_NEUMANN
        g.bc_val[n] = float(bc_val[n]) if bc_val is not None and n < len(bc_val) else 0.0
    g.rb = rb
    return g


def mg_desc(i_phi, i_rhs, i_tmp, bc_type, bc_val=None, lambda2=0.0,
            n_cycle_down=2, n_cycle_up=2, precision=FP64) -> MgDesc:
    m = MgDesc()
    m.i_phi, m.i_rhs, m.i_tmp = i_phi, i_rhs, i_tmp
    m.n_cycle_down, m.n_cycle_up = n_cycle_down, n_cycle_up
    m.helmholtz_lambda = float(lambda2)
    for n in range(6):
        m.bc_type[n] = int(bc_type[n]) if n < len(bc_type) else BC_NEUMANN
        m.bc_val[n] = float(bc_val[n]) if bc_val is not None and n < len(bc_val) else 0.0
    m.precision = precision
    return m


_lib = None


def load_library(path: str = LIB_PATH):
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} not found: build it with __graft_entry__.build() "
            "(the GPU path has no CPU fallback)")
    lib = C.CDLL(path)
    P = C.c_void_p
    sig = {
        "afg_init": (C.c_int, [C.c_int, C.POINTER(P)]),
        "afg_finalize": (C.c_int, [P]),
        "afg_last_error": (C.c_char_p, [P]),
        "afg_tree_sync": (C.c_int, [P, C.POINTER(TreeDesc), C.c_int, C.c_int]),
        "afg_tree_sync_batched": (C.c_int, [P, C.POINTER(TreeDesc), C.c_int, C.c_int, C.c_int, _IP]),
        "afg_n_instances": (C.c_int, [P]),
        "afg_mg_set_bc_values_inst": (C.c_int, [P, C.c_int, _DP]),
        "afg_mg_solve_inst": (C.c_int, [P, C.c_int, _DP, C.c_int, _IP, _DP]),
        "afg_field_compute_inst": (C.c_int, [P, C.c_int, C.c_int, C.c_int, _DP, C.c_double, C.c_double,
                                             C.c_int, _IP, _DP]),
        "afg_cc_upload": (C.c_int, [P, C.c_int, C.POINTER(_DP), C.c_longlong]),
        "afg_cc_download": (C.c_int, [P, C.c_int, C.POINTER(_DP), C.c_longlong]),
        "afg_fc_upload": (C.c_int, [P, C.c_int, C.POINTER(_DP), C.c_longlong]),
        "afg_fc_download": (C.c_int, [P, C.c_int, C.POINTER(_DP), C.c_longlong]),
        "afg_set_cc_methods": (C.c_int, [P, C.c_int, C.POINTER(GcDesc)]),
        "afg_gc": (C.c_int, [P, C.c_int, C.c_int, C.c_int]),
        "afg_maxabs": (C.c_int, [P, C.c_int, C.c_int, _DP]),
        "afg_mg_setup": (C.c_int, [P, C.c_int, C.POINTER(MgDesc)]),
        "afg_mg_set_bc_values": (C.c_int, [P, C.c_int, _DP]),
        "afg_mg_vcycle": (C.c_int, [P, C.c_int, C.c_int, C.c_int, _DP]),
        "afg_mg_fmg": (C.c_int, [P, C.c_int, C.c_int, C.c_int, _DP]),
        "afg_mg_solve": (C.c_int, [P, C.c_int, C.c_double, C.c_int, _IP, _DP]),
        "afg_mg_gsrb_lvl": (C.c_int, [P, C.c_int, C.c_int, C.c_int]),
        "afg_mg_update_coarse": (C.c_int, [P, C.c_int, C.c_int]),
        "afg_mg_correct_lvl": (C.c_int, [P, C.c_int, C.c_int]),
        "afg_mg_coarse_solve": (C.c_int, [P, C.c_int]),
        "afg_mg_residual": (C.c_int, [P, C.c_int, C.c_int]),
        "afg_transport_setup": (C.c_int, [P, C.POINTER(TransportDesc)]),
        "afg_flux_upwind": (C.c_int, [P, C.c_int, _DP]),
        "afg_update_densities": (C.c_int, [P, C.c_double, C.c_int, C.c_int, _IP, _DP, C.c_int,
                                           C.c_int, _DP]),
        "afg_field_set_rhs": (C.c_int, [P, C.c_int, C.c_int]),
        "afg_field_from_potential": (C.c_int, [P, C.c_int]),
        "afg_field_compute": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                        C.c_double, C.c_int, _IP, _DP]),
        "afg_photoi_helmh": (C.c_int, [P, C.c_double, C.c_int, _IP, _DP, C.c_double, C.c_int]),
        "afg_tree_copy_cc": (C.c_int, [P, C.c_int, C.c_int]),
        "afg_stage_setup": (C.c_int, [P, C.POINTER(StageDesc)]),
        "afg_set_flux_staged": (C.c_int, [P, C.c_int]),
        "afg_forward_euler": (C.c_int, [P, C.c_double, C.c_double, C.c_int, C.c_int, _IP, _DP, C.c_int,
                                        C.c_int, C.c_int, _DP, _IP]),
        "afg_counters": (C.c_int, [P, C.POINTER(C.c_longlong)]),
        "afg_event_record": (C.c_int, [P, C.c_int]),
        "afg_event_elapsed": (C.c_int, [P, C.c_int, C.c_int, C.POINTER(C.c_float)]),
        "afg_flush_l2": (C.c_int, [P, C.c_longlong]),
        "afg_kernel_timing": (C.c_int, [P, C.c_int]),
        "afg_kernel_stats": (C.c_int, [P, C.POINTER(C.c_longlong), _DP, _DP]),
        "afg_maxabs_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, _DP]),
        "afg_host_register": (C.c_int, [P, C.c_void_p, C.c_size_t]),
        "afg_cc_download_async": (C.c_int, [P, C.c_int, C.POINTER(_DP), C.c_longlong]),
        "afg_transfers_wait": (C.c_int, [P]),
        "afg_autotune": (C.c_int, [P, C.c_int]),
        "afg_tuning": (C.c_int, [P, _IP]),
        "afg_set_tuning": (C.c_int, [P, _IP]),
        "afg_set_fp32_layout": (C.c_int, [P, C.c_int]),
        "afg_kernel_stats_all": (C.c_int, [P, C.POINTER(C.c_longlong), _DP, _DP]),
        "afg_set_photoi_lockstep": (C.c_int, [P, C.c_int]),
        "afg_check_bounded_wait": (C.c_int, [P, _DP]),
        "afg_refine_flags": (C.c_int, [P, C.POINTER(RefineDesc), _IP]),
        "afg_prolong_limit": (C.c_int, [P, C.c_int, C.c_int, _IP, C.c_int]),
        "afg_prolong_linear": (C.c_int, [P, C.c_int, C.c_int, _IP]),
        "afg_restrict_tree": (C.c_int, [P, C.c_int]),
        "afg_adjust_refinement": (C.c_int, [C.POINTER(TreeDesc), _IP, C.c_int, C.POINTER(P)]),
        "afg_tree_new_sizes": (C.c_int, [P, _IP, _IP]),
        "afg_tree_new_get": (C.c_int, [P, _IP, _IP, _IP, _IP, _IP, _IP, _DP, _DP, _DP]),
        "afg_tree_new_free": (None, [P]),
        "afg_tree_remap": (C.c_int, [P, C.POINTER(TreeDesc), _IP]),
        "afg_host_unregister": (C.c_int, [P, C.c_void_p]),
        "afg_sync": (C.c_int, [P]),
        "afg_launch_count": (C.c_longlong, [P]),
        "afg_mg_set_lsf": (C.c_int, [P, C.c_int, C.POINTER(LsfDesc)]),
        "afg_transport_set_electrode": (C.c_int, [P, C.c_int]),
        "afg_electrode_init_densities": (C.c_int, [P, C.c_int, C.c_int, _IP]),
        "afg_electrode_species_bc": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int]),
        "afg_mg_set_lsf_voltage": (C.c_int, [P, C.c_int, C.c_double]),
        "afg_mg_lsf_info": (C.c_int, [P, C.c_int, _IP, _IP, _DP, _DP, _DP, _DP]),
        "afg_write_vtk": (C.c_int, [P, C.c_char_p, C.c_int, C.c_double, C.c_int, _IP, C.POINTER(C.c_char_p)]),
        "afg_leaf_cells": (C.c_int, [P, C.c_int, _DP, C.POINTER(C.c_longlong)]),
        "afg_interp1": (C.c_int, [P, C.c_longlong, _DP, C.c_int, _IP, _DP, _IP]),
        "afg_write_line": (C.c_int, [P, C.c_char_p, C.c_int, _IP, C.POINTER(C.c_char_p), _DP, _DP, C.c_int]),
        "afg_write_plane": (C.c_int, [P, C.c_char_p, C.c_int, _IP, C.POINTER(C.c_char_p), _DP, _DP, _IP]),
        "afg_write_numpy": (C.c_int, [P, C.c_char_p, _DP, _DP, _IP, C.c_int, C.c_double, C.c_int, _IP,
                                      C.POINTER(C.c_char_p)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class AfgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"afivo_gpu error {code}: {msg}")
        self.code = code


class BoxPointers:
    """Per-box pointer array for a host array laid out like the reference's
    boxes: cc[n_boxes, n_var, ...] (box%cc of box id at row id-1).  Holds a
    reference to the array so the pointers stay valid."""

    def __init__(self, cc: np.ndarray):
        self.array = cc
        self.addr = (np.uint64(cc.ctypes.data) +
                     np.arange(cc.shape[0], dtype=np.uint64) * np.uint64(cc.strides[0]))
        self.ptr = self.addr.ctypes.data_as(C.POINTER(_DP))


def box_pointers(cc: np.ndarray):
    return BoxPointers(cc)


def adjust_refinement(tree, flags, max_lvl: int):
    """The mesh after af_adjust_refinement, computed by the library's host
    code (afg_adjust_refinement): from box flags (REF_RM / REF_KEEP / REF_DO
    per box, as afg_refine_flags returns them) to the new afivo_tree.Tree, or
    `tree` itself when the mesh does not change.  Needs no GPU."""
    import afivo_tree as at
    lib = load_library()
    holder = TreeDescHolder(tree)
    f = np.ascontiguousarray(flags, dtype=np.int32)
    out = C.c_void_p()
    rc = lib.afg_adjust_refinement(C.byref(holder.desc), _ip(f), int(max_lvl), C.byref(out))
    if rc != AFG_OK:
        raise AfgError(rc, "afg_adjust_refinement failed")
    if not out.value:
        return tree
    try:
        n, h = C.c_int(0), C.c_int(0)
        lib.afg_tree_new_sizes(out, C.byref(n), C.byref(h))
        D, N = tree.ndim, n.value
        arr = dict(lvl=np.zeros(N, np.int32), ix=np.zeros((N, D), np.int32), parent=np.zeros(N, np.int32),
                   children=np.zeros((N, 2 ** D), np.int32), neighbors=np.zeros((N, 2 * D), np.int32),
                   neighbor_mat=np.zeros((N, 3 ** D), np.int32), r_min=np.zeros((N, D)), dr=np.zeros((N, D)))
        drb = np.zeros(D)
        lib.afg_tree_new_get(out, _ip(arr["lvl"]), _ip(arr["ix"]), _ip(arr["parent"]), _ip(arr["children"]),
                             _ip(arr["neighbors"]), _ip(arr["neighbor_mat"]), _dp(arr["r_min"]), _dp(arr["dr"]),
                             _dp(drb))
    finally:
        lib.afg_tree_new_free(out)
    t = at.Tree(ndim=D, n_cell=tree.n_cell, coord=tree.coord, coarse_grid_size=tree.coarse_grid_size,
                r_base=tree.r_base, dr_base=drb)
    t.n_boxes, t.highest_lvl = N, h.value
    for k, v in arr.items():
        setattr(t, k, v)
    ids = np.arange(1, N + 1, dtype=np.int32)
    has_c = (t.children > 0).any(axis=1)
    t.lvl_ids = [ids[t.lvl == l] for l in range(1, t.highest_lvl + 1)]
    t.lvl_leaves = [x[~has_c[x - 1]] for x in t.lvl_ids]
    t.lvl_parents = [x[has_c[x - 1]] for x in t.lvl_ids]
    return t


class Context:
    """One afivo tree mirrored on one GPU (wraps ``afg_ctx``)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        self.ptr = C.c_void_p()
        rc = self.lib.afg_init(device, C.byref(self.ptr))
        if rc != AFG_OK:
            raise AfgError(rc, "afg_init failed (no CUDA device?)")
        self._tree_holder = None
        self.n_var = 0

    def check(self, rc, what=""):
        if rc != AFG_OK:
            msg = self.lib.afg_last_error(self.ptr)
            raise AfgError(rc, f"{what}: {msg.decode() if msg else ''}")
        return rc

    def close(self):
        if self.ptr:
            self.lib.afg_finalize(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- tree mirror ------------------------------------------------------
    def tree_sync(self, tree, n_var_cell: int, n_var_face: int = 0, box_inst=None):
        """Mirror `tree`; with box_inst (instance of each box, 0-based) the
        tree is a forest of independent instances (afg_tree_sync_batched)."""
        self._tree_holder = TreeDescHolder(tree)
        self.tree = tree
        self.n_var = n_var_cell
        self.n_var_face = n_var_face
        if box_inst is None:
            self.check(self.lib.afg_tree_sync(self.ptr, C.byref(self._tree_holder.desc),
                                              n_var_cell, n_var_face), "afg_tree_sync")
            return
        self._box_inst = np.ascontiguousarray(box_inst, dtype=np.int32)
        n_inst = int(self._box_inst.max()) + 1
        self.check(self.lib.afg_tree_sync_batched(self.ptr, C.byref(self._tree_holder.desc), n_var_cell,
                                                  n_var_face, n_inst, _ip(self._box_inst)),
                   "afg_tree_sync_batched")

    def refine_flags(self, desc):
        """Box refinement flags (REF_RM / REF_KEEP / REF_DO per box)."""
        out = np.zeros(self.tree.n_boxes, dtype=np.int32)
        self.check(self.lib.afg_refine_flags(self.ptr, C.byref(desc), _ip(out)), "afg_refine_flags")
        return out

    def prolong_limit(self, iv, ids, limiter):
        a = np.ascontiguousarray(ids, dtype=np.int32)
        self.check(self.lib.afg_prolong_limit(self.ptr, iv, len(a), _ip(a), limiter), "afg_prolong_limit")

    def prolong_linear(self, iv, ids):
        a = np.ascontiguousarray(ids, dtype=np.int32)
        self.check(self.lib.afg_prolong_linear(self.ptr, iv, len(a), _ip(a)), "afg_prolong_linear")

    def restrict_tree(self, iv):
        self.check(self.lib.afg_restrict_tree(self.ptr, iv), "afg_restrict_tree")

    # ---- output writers (af_write_vtk, af_write_line, af_write_plane,
    # af_write_numpy, af_interp1) ----
    @staticmethod
    def _names(names):
        arr = (C.c_char_p * max(1, len(names)))(*[n.encode() for n in names])
        return arr

    def write_vtk(self, filename, ivs, names, n_cycle=0, time=0.0):
        """filename + '.vtu' of all leaf cells of variables ivs (1-based)."""
        a = np.ascontiguousarray(ivs, dtype=np.int32)
        nm = self._names(names)
        self.check(self.lib.afg_write_vtk(self.ptr, filename.encode(), int(n_cycle), float(time), len(a), _ip(a), nm),
                   "afg_write_vtk")

    def leaf_cells(self, iv):
        n = C.c_longlong(0)
        self.check(self.lib.afg_leaf_cells(self.ptr, iv, None, C.byref(n)), "afg_leaf_cells")
        out = np.empty(n.value, dtype=np.float64)
        self.check(self.lib.afg_leaf_cells(self.ptr, iv, _dp(out), C.byref(n)), "afg_leaf_cells")
        return out

    def interp1(self, points, ivs):
        """af_interp1 at points [n][ndim]: (values [n][len(ivs)], success [n])."""
        r = np.ascontiguousarray(points, dtype=np.float64)
        a = np.ascontiguousarray(ivs, dtype=np.int32)
        n = r.shape[0]
        vals = np.zeros((n, max(1, len(a))), dtype=np.float64)
        ok = np.zeros(n, dtype=np.int32)
        self.check(self.lib.afg_interp1(self.ptr, n, _dp(r), len(a), _ip(a), _dp(vals), _ip(ok)), "afg_interp1")
        return vals[:, :len(a)], ok.astype(bool)

    def write_line(self, filename, ivs, names, r_min, r_max, n_points):
        a = np.ascontiguousarray(ivs, dtype=np.int32)
        r0 = np.ascontiguousarray(r_min, dtype=np.float64)
        r1 = np.ascontiguousarray(r_max, dtype=np.float64)
        self.check(self.lib.afg_write_line(self.ptr, filename.encode(), len(a), _ip(a), self._names(names),
                                           _dp(r0), _dp(r1), int(n_points)), "afg_write_line")

    def write_plane(self, filename, ivs, names, r_min, r_max, n_pixels):
        a = np.ascontiguousarray(ivs, dtype=np.int32)
        r0 = np.ascontiguousarray(r_min, dtype=np.float64)
        r1 = np.ascontiguousarray(r_max, dtype=np.float64)
        npx = np.ascontiguousarray(n_pixels, dtype=np.int32)
        self.check(self.lib.afg_write_plane(self.ptr, filename.encode(), len(a), _ip(a), self._names(names),
                                            _dp(r0), _dp(r1), _ip(npx)), "afg_write_plane")

    def write_numpy(self, filename, ivs, names, r_min=None, r_max=None, n_points=None, n_cycle=0, time=0.0):
        a = np.ascontiguousarray(ivs, dtype=np.int32)
        r0 = None if r_min is None else np.ascontiguousarray(r_min, dtype=np.float64)
        r1 = None if r_max is None else np.ascontiguousarray(r_max, dtype=np.float64)
        npt = None if n_points is None else np.ascontiguousarray(n_points, dtype=np.int32)
        self.check(self.lib.afg_write_numpy(self.ptr, filename.encode(), None if r0 is None else _dp(r0),
                                            None if r1 is None else _dp(r1), None if npt is None else _ip(npt),
                                            int(n_cycle), float(time), len(a), _ip(a), self._names(names)),
                   "afg_write_numpy")

    def tree_remap(self, tree, old_id):
        """Mirror `tree` keeping the data: old_id[b] = id of new box b+1 in
        the previous tree (0 = new box)."""
        holder = TreeDescHolder(tree)
        o = np.ascontiguousarray(old_id, dtype=np.int32)
        self.check(self.lib.afg_tree_remap(self.ptr, C.byref(holder.desc), _ip(o)), "afg_tree_remap")
        self._tree_holder = holder
        self.tree = tree

    def n_instances(self):
        return self.lib.afg_n_instances(self.ptr)

    def upload(self, cc: np.ndarray, ivs=None, first_iv=1):
        """Upload variables ivs (1-based) from host boxes cc[n, n_var, ...];
        column v of cc holds variable first_iv + v."""
        cc = np.ascontiguousarray(cc, dtype=np.float64)
        S = int(np.prod(cc.shape[2:]))
        bp = box_pointers(cc)
        for iv in (ivs if ivs is not None else range(first_iv, first_iv + cc.shape[1])):
            self.check(self.lib.afg_cc_upload(self.ptr, iv, bp.ptr, (iv - first_iv) * S), "afg_cc_upload")

    def download(self, cc: np.ndarray, ivs=None, first_iv=1):
        """Download variables ivs into host boxes cc[n, n_var, ...] (in place);
        column v of cc receives variable first_iv + v."""
        assert cc.flags.c_contiguous and cc.dtype == np.float64
        S = int(np.prod(cc.shape[2:]))
        bp = box_pointers(cc)
        for iv in (ivs if ivs is not None else range(first_iv, first_iv + cc.shape[1])):
            self.check(self.lib.afg_cc_download(self.ptr, iv, bp.ptr, (iv - first_iv) * S), "afg_cc_download")

    def upload_vars(self, cc: np.ndarray, ivs, cols=None, bp=None):
        """Upload column cols[v] (default v) of cc[n, m, ...] into variable ivs[v]."""
        S = int(np.prod(cc.shape[2:]))
        bp = bp or box_pointers(cc)
        for v, iv in enumerate(ivs):
            col = v if cols is None else cols[v]
            self.check(self.lib.afg_cc_upload(self.ptr, iv, bp.ptr, col * S), "afg_cc_upload")

    def download_vars(self, cc: np.ndarray, ivs, cols=None, bp=None):
        """Download variable ivs[v] into column cols[v] (default v) of cc[n, m, ...]."""
        S = int(np.prod(cc.shape[2:]))
        bp = bp or box_pointers(cc)
        for v, iv in enumerate(ivs):
            col = v if cols is None else cols[v]
            self.check(self.lib.afg_cc_download(self.ptr, iv, bp.ptr, col * S), "afg_cc_download")

    def download_vars_async(self, cc: np.ndarray, ivs, cols=None, bp=None):
        """Start downloading variable ivs[v] into column cols[v] of cc (see
        afg_cc_download_async); keep `bp` alive until transfers_wait()."""
        S = int(np.prod(cc.shape[2:]))
        bp = bp or box_pointers(cc)
        for v, iv in enumerate(ivs):
            col = v if cols is None else cols[v]
            self.check(self.lib.afg_cc_download_async(self.ptr, iv, bp.ptr, col * S), "afg_cc_download_async")
        return bp

    def autotune(self, mg_id):
        self.check(self.lib.afg_autotune(self.ptr, mg_id), "afg_autotune")

    def tuning(self):
        """Smoother variants in use (afg_tuning), decoded."""
        out = (C.c_int * 2)()
        self.check(self.lib.afg_tuning(self.ptr, out), "afg_tuning")

        compact = getattr(self, "fp32_compact", True)

        def name(v, fp32=False):
            if fp32 and compact:
                if v & GSRB_STAGED:
                    return (f"compact red-black layout, other colour staged in shared memory (bulk copies), "
                            f"{v & 15} cells/thread")
                return "compact red-black layout, one box per CTA"
            if v <= 0:
                return "generic"
            if v & GSRB_STAGED:
                what = "phi and rhs" if v & GSRB_STAGED_RHS else "phi"
                return f"{what} staged in shared memory (bulk copies), {v & 15} cells/thread"
            return f"{v} cells/thread"
        return {"gsrb_fp32": name(out[0], True), "gsrb_fp64": name(out[1]), "codes": [out[0], out[1]]}

    def check_bounded_wait(self):
        """(status, ms): AFG_ERR_DEVICE when a timed-out device wait was
        detected and reported through the error word."""
        ms = C.c_double(0)
        rc = self.lib.afg_check_bounded_wait(self.ptr, C.byref(ms))
        return rc, ms.value

    def set_photoi_lockstep(self, on):
        self.check(self.lib.afg_set_photoi_lockstep(self.ptr, int(on)), "afg_set_photoi_lockstep")

    def set_tuning(self, fp32, fp64):
        a = np.array([fp32, fp64], dtype=np.int32)
        self.check(self.lib.afg_set_tuning(self.ptr, _ip(a)), "afg_set_tuning")

    def set_fp32_layout(self, compact):
        """afg_set_fp32_layout: FP32 correction buffers of the mixed solves
        in the compact red-black layout (True, the default) or ghosted."""
        self.fp32_compact = bool(compact)
        self.check(self.lib.afg_set_fp32_layout(self.ptr, int(bool(compact))), "afg_set_fp32_layout")

    def transfers_wait(self):
        self.check(self.lib.afg_transfers_wait(self.ptr), "afg_transfers_wait")

    def upload_fc(self, fc: np.ndarray, ivfs=None):
        fc = np.ascontiguousarray(fc, dtype=np.float64)
        F = int(np.prod(fc.shape[2:]))
        bp = box_pointers(fc)
        for iv in (ivfs if ivfs is not None else range(1, fc.shape[1] + 1)):
            self.check(self.lib.afg_fc_upload(self.ptr, iv, bp.ptr, (iv - 1) * F), "afg_fc_upload")

    def download_fc(self, fc: np.ndarray, ivfs=None):
        assert fc.flags.c_contiguous and fc.dtype == np.float64
        F = int(np.prod(fc.shape[2:]))
        bp = box_pointers(fc)
        for iv in (ivfs if ivfs is not None else range(1, fc.shape[1] + 1)):
            self.check(self.lib.afg_fc_download(self.ptr, iv, bp.ptr, (iv - 1) * F), "afg_fc_download")

    def host_register(self, arr: np.ndarray):
        """Page-lock the memory of a C-contiguous host array."""
        assert arr.flags.c_contiguous
        self.check(self.lib.afg_host_register(self.ptr, arr.ctypes.data, arr.nbytes), "afg_host_register")

    def host_unregister(self, arr: np.ndarray):
        self.check(self.lib.afg_host_unregister(self.ptr, arr.ctypes.data), "afg_host_unregister")

    def set_cc_methods(self, iv, bc_type, bc_val=None, rb=RB_MG_SIDES):
        g = gc_desc(bc_type, bc_val, rb)
        self.check(self.lib.afg_set_cc_methods(self.ptr, iv, C.byref(g)), "afg_set_cc_methods")

    def gc(self, iv, lvl=0, corners=True):
        self.check(self.lib.afg_gc(self.ptr, iv, lvl, int(corners)), "afg_gc")

    def maxabs(self, iv, leaves_only=True) -> float:
        out = C.c_double()
        self.check(self.lib.afg_maxabs(self.ptr, iv, int(leaves_only), C.byref(out)), "afg_maxabs")
        return out.value

    # -- multigrid --------------------------------------------------------
    def mg_setup(self, mg_id, desc: MgDesc):
        self.check(self.lib.afg_mg_setup(self.ptr, mg_id, C.byref(desc)), "afg_mg_setup")

    def mg_set_bc_values(self, mg_id, vals):
        a = np.zeros(6)
        a[:len(vals)] = vals
        self.check(self.lib.afg_mg_set_bc_values(self.ptr, mg_id, _dp(a)), "afg_mg_set_bc_values")

    def mg_set_lsf(self, mg_id, desc: LsfDesc):
        self.check(self.lib.afg_mg_set_lsf(self.ptr, mg_id, C.byref(desc)), "afg_mg_set_lsf")

    def transport_set_electrode(self, i_lsf):
        self.check(self.lib.afg_transport_set_electrode(self.ptr, int(i_lsf)), "afg_transport_set_electrode")

    def electrode_init_densities(self, mg_id, ids):
        a = np.ascontiguousarray(ids, dtype=np.int32)
        self.check(self.lib.afg_electrode_init_densities(self.ptr, mg_id, len(a), _ip(a)),
                   "afg_electrode_init_densities")

    def electrode_species_bc(self, mg_id, electron, ion, neumann=True):
        self.check(self.lib.afg_electrode_species_bc(self.ptr, mg_id, electron, ion, int(neumann)),
                   "afg_electrode_species_bc")

    def mg_set_lsf_voltage(self, mg_id, voltage):
        self.check(self.lib.afg_mg_set_lsf_voltage(self.ptr, mg_id, float(voltage)), "afg_mg_set_lsf_voltage")

    def mg_lsf_info(self, mg_id, ndim, n_cell):
        """(ids, v[n][2D+1][SI], f[n][SI], bcc[n][SI], dd[n][2D][SI])"""
        n = C.c_int(0)
        self.check(self.lib.afg_mg_lsf_info(self.ptr, mg_id, C.byref(n), None, None, None, None, None),
                   "afg_mg_lsf_info")
        n = n.value
        SI = n_cell ** ndim
        ids = np.zeros(max(1, n), dtype=np.int32)
        v = np.zeros((max(1, n), 2 * ndim + 1, SI))
        f = np.zeros((max(1, n), SI))
        bcc = np.zeros((max(1, n), SI))
        dd = np.zeros((max(1, n), 2 * ndim, SI))
        self.check(self.lib.afg_mg_lsf_info(self.ptr, mg_id, None, _ip(ids), _dp(v), _dp(f), _dp(bcc), _dp(dd)),
                   "afg_mg_lsf_info")
        return ids[:n], v[:n], f[:n], bcc[:n], dd[:n]

    def mg_set_bc_values_inst(self, mg_id, vals):
        """vals[q][face] per instance of a batched tree."""
        v = np.asarray(vals, dtype=np.float64)
        a = np.zeros((v.shape[0], 6))
        a[:, :v.shape[1]] = v
        self.check(self.lib.afg_mg_set_bc_values_inst(self.ptr, mg_id, _dp(a)), "afg_mg_set_bc_values_inst")

    def mg_solve_inst(self, mg_id, thresholds, max_cycles=50, allow_noconv=False):
        thr = np.ascontiguousarray(thresholds, dtype=np.float64)
        n = np.zeros(len(thr), dtype=np.int32)
        res = np.zeros(len(thr))
        rc = self.lib.afg_mg_solve_inst(self.ptr, mg_id, _dp(thr), max_cycles, _ip(n), _dp(res))
        if not (allow_noconv and rc == AFG_ERR_NOCONV):
            self.check(rc, "afg_mg_solve_inst")
        return n, res

    def mg_vcycle(self, mg_id, set_residual=True, max_lvl=0):
        out = C.c_double(0)
        self.check(self.lib.afg_mg_vcycle(self.ptr, mg_id, int(set_residual), max_lvl, C.byref(out)),
                   "afg_mg_vcycle")
        return out.value

    def mg_fmg(self, mg_id, set_residual=True, have_guess=False):
        out = C.c_double(0)
        self.check(self.lib.afg_mg_fmg(self.ptr, mg_id, int(set_residual), int(have_guess), C.byref(out)),
                   "afg_mg_fmg")
        return out.value

    def mg_solve(self, mg_id, threshold, max_cycles=50, allow_noconv=False):
        n = C.c_int(0)
        res = np.zeros(max_cycles)
        rc = self.lib.afg_mg_solve(self.ptr, mg_id, threshold, max_cycles, C.byref(n), _dp(res))
        if not (allow_noconv and rc == AFG_ERR_NOCONV):
            self.check(rc, "afg_mg_solve")
        return n.value, res[:n.value].copy()

    def mg_gsrb_lvl(self, mg_id, lvl, cycle_type):
        self.check(self.lib.afg_mg_gsrb_lvl(self.ptr, mg_id, lvl, cycle_type), "afg_mg_gsrb_lvl")

    def mg_update_coarse(self, mg_id, lvl):
        self.check(self.lib.afg_mg_update_coarse(self.ptr, mg_id, lvl), "afg_mg_update_coarse")

    def mg_correct_lvl(self, mg_id, lvl):
        self.check(self.lib.afg_mg_correct_lvl(self.ptr, mg_id, lvl), "afg_mg_correct_lvl")

    def mg_coarse_solve(self, mg_id):
        self.check(self.lib.afg_mg_coarse_solve(self.ptr, mg_id), "afg_mg_coarse_solve")

    def mg_residual(self, mg_id, max_lvl=0):
        self.check(self.lib.afg_mg_residual(self.ptr, mg_id, max_lvl), "afg_mg_residual")

    # -- transport, field, photoionization --------------------------------
    def transport_setup(self, desc: TransportDesc):
        self._transport_desc = desc  # keeps lt_data's buffer reachable
        self.check(self.lib.afg_transport_setup(self.ptr, C.byref(desc)), "afg_transport_setup")

    def flux_upwind(self, s_deriv):
        out = np.zeros(2)
        self.check(self.lib.afg_flux_upwind(self.ptr, s_deriv, _dp(out)), "afg_flux_upwind")
        return out

    def update_densities(self, dt, s_deriv, s_prev, w_prev, s_out, last_step=False):
        sp = np.ascontiguousarray(s_prev, dtype=np.int32)
        wp = np.ascontiguousarray(w_prev, dtype=np.float64)
        chem = C.c_double(0)
        self.check(self.lib.afg_update_densities(self.ptr, dt, s_deriv, len(sp), _ip(sp), _dp(wp), s_out,
                                                 int(last_step), C.byref(chem)), "afg_update_densities")
        return chem.value

    def set_flux_staged(self, on):
        self.check(self.lib.afg_set_flux_staged(self.ptr, int(bool(on))), "afg_set_flux_staged")

    def stage_setup(self, mg_id, domain_len, max_rel_residual, num_vcycles, dt_cfl_number=0.5,
                    dt_max=1e-11):
        d = StageDesc(mg_id, domain_len, max_rel_residual, num_vcycles, dt_cfl_number, dt_max)
        self.check(self.lib.afg_stage_setup(self.ptr, C.byref(d)), "afg_stage_setup")

    def forward_euler(self, dt, voltage, s_deriv, s_prev, w_prev, s_out, i_step, n_steps):
        """One forward_euler stage (afg_forward_euler); returns (dt limit,
        field cycles of the stage)."""
        sp = np.ascontiguousarray(s_prev, dtype=np.int32)
        wp = np.ascontiguousarray(w_prev, dtype=np.float64)
        lim = C.c_double(0)
        n = C.c_int(0)
        self.check(self.lib.afg_forward_euler(self.ptr, dt, voltage, s_deriv, len(sp), _ip(sp), _dp(wp), s_out,
                                              i_step, n_steps, C.byref(lim), C.byref(n)), "afg_forward_euler")
        return lim.value, n.value

    def field_set_rhs(self, i_rhs, s_in):
        self.check(self.lib.afg_field_set_rhs(self.ptr, i_rhs, s_in), "afg_field_set_rhs")

    def field_from_potential(self, i_phi):
        self.check(self.lib.afg_field_from_potential(self.ptr, i_phi), "afg_field_from_potential")

    def field_compute(self, mg_id, s_in, have_guess, voltage, domain_len, max_rel_residual, num_vcycles):
        n = C.c_int(0)
        r = C.c_double(0)
        self.check(self.lib.afg_field_compute(self.ptr, mg_id, s_in, int(have_guess), voltage, domain_len,
                                              max_rel_residual, num_vcycles, C.byref(n), C.byref(r)),
                   "afg_field_compute")
        return n.value, r.value

    def field_compute_inst(self, mg_id, s_in, have_guess, voltages, domain_len, max_rel_residual, num_vcycles):
        """field_compute of every instance of a batched tree with its own
        voltage; per-instance cycle counts and final residuals."""
        v = np.ascontiguousarray(voltages, dtype=np.float64)
        n = np.zeros(len(v), dtype=np.int32)
        r = np.zeros(len(v))
        self.check(self.lib.afg_field_compute_inst(self.ptr, mg_id, s_in, int(have_guess), _dp(v), domain_len,
                                                   max_rel_residual, num_vcycles, _ip(n), _dp(r)),
                   "afg_field_compute_inst")
        return n, r

    def photoi_helmh(self, coeff, mg_ids, coeffs, max_rel_residual=1e-2, max_fmg_cycles=10):
        ids = np.ascontiguousarray(mg_ids, dtype=np.int32)
        cs = np.ascontiguousarray(coeffs, dtype=np.float64)
        self.check(self.lib.afg_photoi_helmh(self.ptr, coeff, len(ids), _ip(ids), _dp(cs), max_rel_residual,
                                             max_fmg_cycles), "afg_photoi_helmh")

    def tree_copy_cc(self, iv_from, iv_to):
        self.check(self.lib.afg_tree_copy_cc(self.ptr, iv_from, iv_to), "afg_tree_copy_cc")

    def counters(self):
        out = (C.c_longlong * 4)()
        self.check(self.lib.afg_counters(self.ptr, out), "afg_counters")
        return dict(launches=out[0], smoother_updates=out[1], transport_updates=out[2], vcycles=out[3])

    def event_record(self, slot):
        self.check(self.lib.afg_event_record(self.ptr, slot), "afg_event_record")

    def event_elapsed(self, a, b) -> float:
        ms = C.c_float(0)
        self.check(self.lib.afg_event_elapsed(self.ptr, a, b, C.byref(ms)), "afg_event_elapsed")
        return ms.value

    def flush_l2(self, nbytes=256 << 20):
        self.check(self.lib.afg_flush_l2(self.ptr, nbytes), "afg_flush_l2")

    def kernel_timing(self, cls):
        self.check(self.lib.afg_kernel_timing(self.ptr, cls), "afg_kernel_timing")

    def kernel_stats(self):
        n = C.c_longlong(0)
        ms = C.c_double(0)
        by = C.c_double(0)
        self.check(self.lib.afg_kernel_stats(self.ptr, C.byref(n), C.byref(ms), C.byref(by)), "afg_kernel_stats")
        return n.value, ms.value, by.value

    def kernel_stats_all(self):
        """After kernel_timing(KT_ALL): {class name: (launches, ms, bytes)}."""
        n = (C.c_longlong * KT_NCLASS)()
        ms = np.zeros(KT_NCLASS)
        by = np.zeros(KT_NCLASS)
        self.check(self.lib.afg_kernel_stats_all(self.ptr, n, _dp(ms), _dp(by)), "afg_kernel_stats_all")
        return {KT_NAMES[c]: (int(n[c]), float(ms[c]), float(by[c])) for c in KT_NAMES if n[c] > 0}

    def sync(self):
        self.check(self.lib.afg_sync(self.ptr), "afg_sync")

    def launch_count(self) -> int:
        return int(self.lib.afg_launch_count(self.ptr))


def maxabs_noalloc(d_pool: int, d_slots: int, n_slots: int, ndim: int, n_cell: int, stream: int = 0) -> float:
    """afg_maxabs_noalloc on caller-owned device buffers (raw device
    addresses); raises on a non-zero status."""
    lib = load_library()
    out = C.c_double(0)
    rc = lib.afg_maxabs_noalloc(C.c_void_p(d_pool), C.c_void_p(d_slots), n_slots, ndim, n_cell,
                                C.c_void_p(stream) if stream else None, C.byref(out))
    if rc != AFG_OK:
        raise AfgError(rc, "afg_maxabs_noalloc")
    return out.value


def new_fc(tree, n_var_face) -> np.ndarray:
    """Host face arrays laid out like box%fc: [n_boxes, n_var_face, D, (k,) j, i]
    with nc+1 entries per dimension."""
    n1 = tree.n_cell + 1
    return np.zeros((tree.n_boxes, n_var_face, tree.ndim) + (n1,) * tree.ndim)


def new_cc(tree, n_var) -> np.ndarray:
    """Host boxes laid out like box%cc: [n_boxes, n_var, (k,) j, i]."""
    n2 = tree.n_cell + 2
    return np.zeros((tree.n_boxes, n_var) + (n2,) * tree.ndim)
