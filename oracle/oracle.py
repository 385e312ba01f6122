"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle restates the reference's Fortran algorithms in C++ FP64 with the
reference's operation order (see oracle_common.h).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
checker; the GPU product never calls it.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "afivo-streamer_gb300"))
import afivo_gpu as ag  # noqa: E402  (only for the shared C struct layouts)
from build_oracle import build  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        P = C.c_void_p
        DP = C.POINTER(C.c_double)
        IP = C.POINTER(C.c_int)
        sig = {
            "orc_create": (P, [C.POINTER(ag.TreeDesc), C.c_int, C.c_int]),
            "orc_destroy": (None, [P]),
            "orc_set_num_threads": (C.c_int, [C.c_int]),
            "orc_set_cc_methods": (C.c_int, [P, C.c_int, C.POINTER(ag.GcDesc)]),
            "orc_gc": (C.c_int, [P, DP, C.c_int, C.c_int, C.c_int]),
            "orc_mg_setup": (C.c_int, [P, C.c_int, C.POINTER(ag.MgDesc)]),
            "orc_mg_set_bc_values": (C.c_int, [P, C.c_int, DP]),
            "orc_mg_coarse_inverse": (C.c_int, [P, C.c_int, DP, C.c_int]),
            "orc_mg_gsrb_lvl": (C.c_int, [P, DP, C.c_int, C.c_int, C.c_int]),
            "orc_mg_update_coarse": (C.c_int, [P, DP, C.c_int, C.c_int]),
            "orc_mg_correct_lvl": (C.c_int, [P, DP, C.c_int, C.c_int]),
            "orc_mg_coarse_solve": (C.c_int, [P, DP, C.c_int]),
            "orc_mg_residual": (C.c_int, [P, DP, C.c_int, C.c_int]),
            "orc_mg_vcycle": (C.c_int, [P, DP, C.c_int, C.c_int, C.c_int, DP]),
            "orc_mg_fmg": (C.c_int, [P, DP, C.c_int, C.c_int, C.c_int, DP]),
            "orc_mg_solve": (C.c_int, [P, DP, C.c_int, C.c_double, C.c_int, IP, DP]),
            "orc_maxabs": (C.c_double, [P, DP, C.c_int, C.c_int]),
            "orc_transport_setup": (C.c_int, [P, C.POINTER(ag.TransportDesc)]),
            "orc_flux_upwind": (C.c_int, [P, DP, DP, C.c_int, DP]),
            "orc_update_densities": (C.c_int, [P, DP, DP, C.c_double, C.c_int, C.c_int, IP, DP, C.c_int,
                                               C.c_int, DP]),
            "orc_field_set_rhs": (C.c_int, [P, DP, C.c_int, C.c_int]),
            "orc_field_from_potential": (C.c_int, [P, DP, DP, C.c_int]),
            "orc_photoi_source": (C.c_int, [P, DP, C.c_double, C.c_int]),
            "orc_refine_flags": (C.c_int, [P, DP, C.c_void_p, C.POINTER(C.c_int)]),
            "orc_prolong_limit": (C.c_int, [P, DP, C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int]),
            "orc_prolong_linear": (C.c_int, [P, DP, C.c_int, C.c_int, C.POINTER(C.c_int)]),
            "orc_restrict_tree": (C.c_int, [P, DP, C.c_int]),
            "orc_math_eval": (C.c_int, [C.c_int, C.c_int, DP, DP, DP]),
            "orc_mg_set_lsf": (C.c_int, [P, DP, C.c_int, C.POINTER(ag.LsfDesc)]),
            "orc_transport_set_electrode": (C.c_int, [P, C.c_int]),
            "orc_electrode_init_densities": (C.c_int, [P, DP, C.c_int, C.c_int, IP]),
            "orc_electrode_species_bc": (C.c_int, [P, DP, C.c_int, C.c_int, C.c_int, C.c_int]),
            "orc_mg_set_lsf_voltage": (C.c_int, [P, C.c_int, C.c_double]),
            "orc_mg_lsf_info": (C.c_int, [P, C.c_int, IP, IP, DP, DP, DP, DP]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def set_num_threads(n: int) -> int:
    return lib().orc_set_num_threads(n)


def _dp(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """CPU restatement operating on host boxes cc[n_boxes, n_var, ...]."""

    def __init__(self, tree, n_var, n_var_face=0):
        self.L = lib()
        self.holder = ag.TreeDescHolder(tree)
        self.p = self.L.orc_create(C.byref(self.holder.desc), n_var, n_var_face)
        self.tree = tree
        self.n_var = n_var

    def __del__(self):
        try:
            self.L.orc_destroy(self.p)
        except Exception:
            pass

    def _ck(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"oracle {what} failed: {rc}")

    def set_cc_methods(self, iv, bc_type, bc_val=None, rb=ag.RB_MG_SIDES):
        g = ag.gc_desc(bc_type, bc_val, rb)
        self._ck(self.L.orc_set_cc_methods(self.p, iv, C.byref(g)), "set_cc_methods")

    def gc(self, cc, iv, lvl=0, corners=True):
        self._ck(self.L.orc_gc(self.p, _dp(cc), iv, lvl, int(corners)), "gc")

    def mg_setup(self, mg_id, desc):
        self._ck(self.L.orc_mg_setup(self.p, mg_id, C.byref(desc)), "mg_setup")

    def mg_set_bc_values(self, mg_id, vals):
        a = np.zeros(6)
        a[:len(vals)] = vals
        self._ck(self.L.orc_mg_set_bc_values(self.p, mg_id, _dp(a)), "mg_set_bc_values")

    def mg_set_lsf(self, cc, mg_id, desc):
        self._ck(self.L.orc_mg_set_lsf(self.p, _dp(cc), mg_id, C.byref(desc)), "mg_set_lsf")

    def transport_set_electrode(self, i_lsf):
        self._ck(self.L.orc_transport_set_electrode(self.p, int(i_lsf)), "transport_set_electrode")

    def electrode_init_densities(self, cc, mg_id, ids):
        a = np.ascontiguousarray(ids, dtype=np.int32)
        self._ck(self.L.orc_electrode_init_densities(self.p, _dp(cc), mg_id, len(a),
                                                     a.ctypes.data_as(C.POINTER(C.c_int))), "electrode_init")

    def electrode_species_bc(self, cc, mg_id, electron, ion, neumann=True):
        self._ck(self.L.orc_electrode_species_bc(self.p, _dp(cc), mg_id, electron, ion, int(neumann)),
                 "electrode_species_bc")

    def mg_set_lsf_voltage(self, mg_id, voltage):
        self._ck(self.L.orc_mg_set_lsf_voltage(self.p, mg_id, float(voltage)), "mg_set_lsf_voltage")

    def mg_lsf_info(self, mg_id):
        t = self.tree
        D, SI = t.ndim, t.n_cell ** t.ndim
        n = C.c_int(0)
        self._ck(self.L.orc_mg_lsf_info(self.p, mg_id, C.byref(n), None, None, None, None, None), "lsf_info")
        n = n.value
        ids = np.zeros(max(1, n), dtype=np.int32)
        v = np.zeros((max(1, n), 2 * D + 1, SI))
        f = np.zeros((max(1, n), SI))
        bcc = np.zeros((max(1, n), SI))
        dd = np.zeros((max(1, n), 2 * D, SI))
        IPt = C.POINTER(C.c_int)
        self._ck(self.L.orc_mg_lsf_info(self.p, mg_id, None, ids.ctypes.data_as(IPt), _dp(v), _dp(f), _dp(bcc),
                                        _dp(dd)), "lsf_info")
        return ids[:n], v[:n], f[:n], bcc[:n], dd[:n]

    def coarse_inverse(self, mg_id):
        n = self.L.orc_mg_coarse_inverse(self.p, mg_id, None, 0)
        out = np.zeros((n, n))
        self.L.orc_mg_coarse_inverse(self.p, mg_id, _dp(out), n * n)
        return out

    def mg_gsrb_lvl(self, cc, mg_id, lvl, t):
        self._ck(self.L.orc_mg_gsrb_lvl(self.p, _dp(cc), mg_id, lvl, t), "gsrb")

    def mg_update_coarse(self, cc, mg_id, lvl):
        self._ck(self.L.orc_mg_update_coarse(self.p, _dp(cc), mg_id, lvl), "update_coarse")

    def mg_correct_lvl(self, cc, mg_id, lvl):
        self._ck(self.L.orc_mg_correct_lvl(self.p, _dp(cc), mg_id, lvl), "correct")

    def mg_coarse_solve(self, cc, mg_id):
        self._ck(self.L.orc_mg_coarse_solve(self.p, _dp(cc), mg_id), "coarse_solve")

    def mg_residual(self, cc, mg_id, max_lvl=0):
        self._ck(self.L.orc_mg_residual(self.p, _dp(cc), mg_id, max_lvl), "residual")

    def mg_vcycle(self, cc, mg_id, set_residual=True, max_lvl=0):
        r = C.c_double(0)
        self._ck(self.L.orc_mg_vcycle(self.p, _dp(cc), mg_id, int(set_residual), max_lvl, C.byref(r)), "vcycle")
        return r.value

    def mg_fmg(self, cc, mg_id, set_residual=True, have_guess=False):
        r = C.c_double(0)
        self._ck(self.L.orc_mg_fmg(self.p, _dp(cc), mg_id, int(set_residual), int(have_guess), C.byref(r)), "fmg")
        return r.value

    def mg_solve(self, cc, mg_id, threshold, max_cycles=50):
        n = C.c_int(0)
        res = np.zeros(max_cycles)
        self._ck(self.L.orc_mg_solve(self.p, _dp(cc), mg_id, threshold, max_cycles, C.byref(n), _dp(res)),
                 "solve")
        return n.value, res[:n.value].copy()

    # -- transport ------------------------------------------------------------
    def transport_setup(self, desc):
        self._ck(self.L.orc_transport_setup(self.p, C.byref(desc)), "transport_setup")

    def flux_upwind(self, cc, fc, s_deriv):
        out = np.zeros(2)
        self._ck(self.L.orc_flux_upwind(self.p, _dp(cc), _dp(fc), s_deriv, _dp(out)), "flux_upwind")
        return out

    def update_densities(self, cc, fc, dt, s_deriv, s_prev, w_prev, s_out, last_step=False):
        sp = np.ascontiguousarray(s_prev, dtype=np.int32)
        wp = np.ascontiguousarray(w_prev, dtype=np.float64)
        chem = C.c_double(0)
        self._ck(self.L.orc_update_densities(self.p, _dp(cc), _dp(fc), dt, s_deriv, len(sp),
                                             sp.ctypes.data_as(C.POINTER(C.c_int)), _dp(wp), s_out,
                                             int(last_step), C.byref(chem)), "update_densities")
        return chem.value

    def field_set_rhs(self, cc, i_rhs, s_in):
        self._ck(self.L.orc_field_set_rhs(self.p, _dp(cc), i_rhs, s_in), "field_set_rhs")

    def field_from_potential(self, cc, fc, i_phi):
        self._ck(self.L.orc_field_from_potential(self.p, _dp(cc), _dp(fc), i_phi), "field_from_potential")

    def photoi_source(self, cc, coeff, i_rhs):
        self._ck(self.L.orc_photoi_source(self.p, _dp(cc), coeff, i_rhs), "photoi_source")

    def refine_flags(self, cc, desc):
        out = np.zeros(self.tree.n_boxes, dtype=np.int32)
        self._ck(self.L.orc_refine_flags(self.p, _dp(cc), C.addressof(desc),
                                         out.ctypes.data_as(C.POINTER(C.c_int))), "refine_flags")
        return out

    def prolong_limit(self, cc, iv, ids, limiter):
        a = np.ascontiguousarray(ids, dtype=np.int32)
        self._ck(self.L.orc_prolong_limit(self.p, _dp(cc), iv, len(a), a.ctypes.data_as(C.POINTER(C.c_int)),
                                          limiter), "prolong_limit")

    def prolong_linear(self, cc, iv, ids):
        a = np.ascontiguousarray(ids, dtype=np.int32)
        self._ck(self.L.orc_prolong_linear(self.p, _dp(cc), iv, len(a), a.ctypes.data_as(C.POINTER(C.c_int))),
                 "prolong_linear")

    def restrict_tree(self, cc, iv):
        self._ck(self.L.orc_restrict_tree(self.p, _dp(cc), iv), "restrict_tree")

    def maxabs(self, cc, iv, leaves_only=True):
        return self.L.orc_maxabs(self.p, _dp(cc), iv, int(leaves_only))


def math_eval(which, x, y=None):
    """The project's exp (which 0), log (1) or pow (2) on arrays, through the
    restatement's library (host build of the same code the device runs)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(np.zeros_like(x) if y is None else y, dtype=np.float64)
    out = np.empty_like(x)
    lib().orc_math_eval(which, len(x), _dp(x), _dp(y), _dp(out))
    return out
