"""ctypes binding of ``libzandgpu.so`` (the C ABI in ``include/zandgpu.h``).

The library is mandatory: importing the device path without it raises, there
is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("ZANDGPU_LIB", os.path.join(HERE, "libzandgpu.so"))

ZG_OK, ZG_EINVAL, ZG_ENOMEM, ZG_ECUDA, ZG_ETIMEOUT, ZG_ENONFINITE = range(6)
ZG_PREC_F64, ZG_PREC_MIXED = 0, 1
ZG_DH_NONE, ZG_DH_MATRIX, ZG_DH_HUBBARD = 0, 1, 2
ZG_MAX_LEADS = 16
ZG_MAX_STAGES = 13
ZG_IMPL_SIMT, ZG_IMPL_TC_PRODUCTS, ZG_IMPL_TC_ALL, ZG_IMPL_TC_SPLIT, ZG_IMPL_COUNT = 0, 1, 2, 3, 4
IMPL_NAMES = ["simt", "tc_products", "tc_all", "tc_split"]
ZG_SCHED_LATE, ZG_SCHED_EARLY, ZG_SCHED_COUNT = 0, 1, 2
SCHED_NAMES = ["late", "early"]
PROF_REGIONS = ["gemm", "omega", "final", "combine", "error", "update", "rhs", "prep", "small", "gemm2"]

_NAMES = {ZG_EINVAL: "EINVAL", ZG_ENOMEM: "ENOMEM", ZG_ECUDA: "ECUDA", ZG_ETIMEOUT: "ETIMEOUT",
          ZG_ENONFINITE: "ENONFINITE"}


class ZGError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("libzandgpu %s: %s" % (_NAMES.get(status, status), msg))
        self.status = status


class ZGInvalid(ZGError, AssertionError):
    """Bad argument or shape; an AssertionError like the reference's checks."""


class zg_layout(C.Structure):
    _fields_ = [("n", C.c_int32), ("n_leads", C.c_int32), ("n_modes", C.c_int32), ("n_sourced", C.c_int32),
                ("nc", C.c_int32), ("hbar", C.c_double),
                ("mode_lead", C.c_void_p), ("s_start", C.c_void_p), ("f_start", C.c_void_p),
                ("lead_cols", C.c_void_p), ("colmap", C.c_void_p), ("H0", C.c_void_p),
                ("Xp", C.c_void_p), ("Xm", C.c_void_p), ("GLP", C.c_void_p), ("dGP", C.c_void_p),
                ("dGM", C.c_void_p), ("XI", C.c_void_p), ("IXI", C.c_void_p), ("XIS", C.c_void_p),
                ("XIT2", C.c_void_p)]


ZG_BIAS = {"zero": 0, "exp_ramp": 1, "gauss": 2, "sin": 3, "step": 4, "box": 5}


class zg_bias(C.Structure):
    _fields_ = [("kind", C.c_int32), ("V0", C.c_double), ("tau", C.c_double), ("tc", C.c_double),
                ("sigma", C.c_double), ("f", C.c_double), ("w", C.c_double * ZG_MAX_LEADS)]


ZG_GRAPH_MAX_BATCH = 256


class zg_attempt_rec(C.Structure):
    _fields_ = [("t", C.c_double), ("h", C.c_double), ("TE", C.c_double), ("h_next", C.c_double),
                ("accepted", C.c_int32), ("status", C.c_int32), ("J", C.c_double * ZG_MAX_LEADS)]


_P = C.c_void_p
_SIGS = {
    "zg_stationary_setup": ([_P, C.c_double, _P, C.c_int, C.c_double, _P, _P], C.c_int),
    "zg_stationary_apply": ([_P, _P, _P], C.c_int),
    "zg_stationary_precond": ([_P, _P, _P], C.c_int),
    "zg_graph_prepare": ([_P, C.POINTER(zg_bias), C.c_int, C.c_double], C.c_int),
    "zg_graph_set": ([_P, C.c_double, C.c_double, C.c_double, C.c_double], C.c_int),
    "zg_graph_run": ([_P, C.c_int, _P, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double),
                      C.POINTER(C.c_int)], C.c_int),
    "zg_attempt": ([_P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double, C.POINTER(zg_bias), C.c_int,
                    C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_int), _P], C.c_int),
    "zg_last_error": ([], C.c_char_p),
    "zg_version": ([], C.c_int),
    "zg_launch_count": ([], C.c_longlong),
    "zg_traj_stream": ([_P], C.c_void_p),
    "zg_traj_create": ([C.c_int, C.POINTER(zg_layout), C.c_int, C.POINTER(C.c_void_p)], C.c_int),
    "zg_traj_destroy": ([_P], C.c_int),
    "zg_traj_info": ([_P, _P], C.c_int),
    "zg_set_tableau": ([_P, C.c_int, _P, _P, _P, _P], C.c_int),
    "zg_set_state": ([_P, C.c_int, _P], C.c_int),
    "zg_get_state": ([_P, C.c_int, _P], C.c_int),
    "zg_set_sigma": ([_P, _P], C.c_int),
    "zg_stage_input": ([_P, C.c_int], C.c_int),
    "zg_get_stage_sigma": ([_P, _P], C.c_int),
    "zg_set_dH": ([_P, _P], C.c_int),
    "zg_set_dissipator": ([_P, _P], C.c_int),
    "zg_set_overlap": ([_P, _P, _P], C.c_int),
    "zg_wait_selftest": ([C.c_int, C.c_longlong], C.c_int),
    "zg_rhs": ([_P, C.c_int, C.c_double, C.c_double, _P, C.c_int, C.c_double, _P], C.c_int),
    "zg_error_norm2": ([_P, _P], C.c_int),
    "zg_step_fourth": ([_P], C.c_int),
    "zg_get_sigma": ([_P, C.c_int, _P], C.c_int),
    "zg_profile": ([_P, C.c_int], C.c_int),
    "zg_profile_read": ([_P, _P, _P], C.c_int),
    "zg_measure_peaks": ([C.c_int, _P], C.c_int),
    "zg_measure_fp64_mma": ([C.c_int, C.POINTER(C.c_double)], C.c_int),
    "zg_split_tf32": ([_P, _P, _P, C.c_int64, _P], C.c_int),
    "zg_gemm_tf32x3": ([_P, _P, _P, _P, _P, C.c_int, C.c_int, C.c_int, _P], C.c_int),
    "zg_combine_c128": ([_P, C.c_int64, C.c_int, _P, _P, C.c_int, _P, C.c_int64, _P], C.c_int),
    "zg_terr2_c128": ([_P, C.c_int64, C.c_int, _P, C.c_int64, _P, _P], C.c_int),
    "zg_terr2_c128_noalloc": ([_P, C.c_int64, C.c_int, _P, C.c_int64, _P, _P], C.c_int),
    "zg_step_fourth_c128": ([_P, C.c_int64, C.c_int, _P, C.c_int64, _P], C.c_int),
    "zg_set_impl": ([_P, C.c_int], C.c_int),
    "zg_get_impl": ([_P, C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
    "zg_tune": ([_P, C.c_int, C.POINTER(C.c_int), _P], C.c_int),
    "zg_set_schedule": ([_P, C.c_int], C.c_int),
    "zg_get_schedule": ([_P, C.POINTER(C.c_int)], C.c_int),
    "zg_combine_fermi_skip_c128": ([_P, C.c_int64, C.c_int, _P, _P, C.c_int, _P, _P, _P, _P, _P], C.c_int),
    "zg_outer_subtraction_c128": ([_P, C.c_int, _P, C.c_int, _P, _P, _P, _P], C.c_int),
}

_lib = None


def lib():
    """Load the library (once) and return it with typed entry points."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libzandgpu.so is not built (expected at %s); run "
                               "`python -m zandpack_gb300.build`" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


def check(status):
    if status != ZG_OK:
        msg = lib().zg_last_error().decode(errors="replace")
        if status == ZG_EINVAL:
            raise ZGInvalid(status, msg)
        raise ZGError(status, msg)
