"""ctypes binding of libraytracer_gb300.so (C ABI in include/rt_gb300.h).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when the shared object is missing; a GPU is needed for every
call that computes.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libraytracer_gb300.so")

RT_OK = 0
RT_ERR_ARG, RT_ERR_NOMEM, RT_ERR_CUDA, RT_ERR_GRID, RT_ERR_STATE = -1, -2, -3, -4, -5
RT_FP64 = 0
RT_FP32 = 1

RT_F_XDOT, RT_F_YDOT, RT_F_ZDOT, RT_F_KDOT, RT_F_LDOT, RT_F_MDOT = range(6)
RT_F_LAMBDA_X, RT_F_LAMBDA_Y, RT_F_LAMBDA_Z, RT_F_LAMBDA = 6, 7, 8, 9
RT_FORCING_NONE, RT_FORCING_FLUX, RT_FORCING_RELAX = 0, 1, 2


class RtDims(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("nx", "ny", "nz", "nk", "nl", "nm", "onx")]


class RtParams(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("f0", ctypes.c_double),
                ("sign_of_omega_i", ctypes.c_double),
                ("enable_upper_reflection", ctypes.c_int),
                ("enable_lower_reflection", ctypes.c_int),
                ("precision", ctypes.c_int)]


BUDGET_FIELDS = ("eint", "mflint", "mfl_max", "umax", "vmax", "wmax", "kmax", "lmax", "mmax",
                 "bfl_xs", "bfl_xe", "bfl_ys", "bfl_ye", "bfl_zs", "bfl_ze",
                 "bfl_ks", "bfl_ke", "bfl_ls", "bfl_le", "bfl_ms", "bfl_me",
                 "cfl_x", "cfl_y", "cfl_z", "cfl_k", "cfl_l", "cfl_m", "residual")


class RtBudget(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in BUDGET_FIELDS]


# name -> (restype, argtypes); every symbol declared in include/rt_gb300.h
_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
SIGNATURES = {
    "rt_create": (ctypes.c_int, [ctypes.POINTER(RtDims), ctypes.POINTER(RtParams), ctypes.POINTER(_P)]),
    "rt_destroy": (ctypes.c_int, [_P]),
    "rt_last_error": (ctypes.c_char_p, [_P]),
    "rt_set_grid": (ctypes.c_int, [_P] + [_D] * 9),
    "rt_set_background": (ctypes.c_int, [_P, _D, _D, _D]),
    "rt_calc_parameter": (ctypes.c_int, [_P]),
    "rt_get_field": (ctypes.c_int, [_P, ctypes.c_int, _D]),
    "rt_max_rate": (ctypes.c_int, [_P, _D]),
    "rt_set_dt": (ctypes.c_int, [_P, ctypes.c_double]),
    "rt_set_state": (ctypes.c_int, [_P, _D]),
    "rt_get_state": (ctypes.c_int, [_P, _D]),
    "rt_integrate": (ctypes.c_int, [_P, ctypes.c_int]),
    "rt_set_forcing": (ctypes.c_int, [_P, ctypes.c_int, _D]),
    "rt_get_tendency": (ctypes.c_int, [_P, _D, _D]),
    "rt_tic": (ctypes.c_int, [_P, ctypes.c_char_p]),
    "rt_toc": (ctypes.c_int, [_P, ctypes.c_char_p]),
    "rt_timing_secs": (ctypes.c_int, [_P, ctypes.c_char_p, _D, ctypes.POINTER(ctypes.c_longlong)]),
    "rt_selftest_wait_timeout": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "rt_fp64_rate": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double)]),
    "rt_set_host_access": (ctypes.c_int, [_P, ctypes.c_int]),
    "rt_set_state_interior": (ctypes.c_int, [_P, _P]),
    "rt_get_state_interior": (ctypes.c_int, [_P, _P]),
    "rt_host_direct": (ctypes.c_int, [_P]),
    "rt_integrate_host": (ctypes.c_int, [_P, _D]),
    "rt_diagnose": (ctypes.c_int, [_P, ctypes.POINTER(RtBudget)] + [_D] * 8),
    "rt_set_tuning": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "rt_stream": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "rt_launch_count": (ctypes.c_longlong, [_P]),
    "rt_device_bytes": (ctypes.c_longlong, [_P]),
    "rt_version": (ctypes.c_char_p, []),
    "rt_set_schedule_sweep": (ctypes.c_int, [_P, ctypes.c_int]),
    "rt_sync": (ctypes.c_int, [_P]),
    "rt_step_dry": (ctypes.c_int, [_P, ctypes.c_int]),
    "rt_batch_dry": (ctypes.c_int, [_P, ctypes.c_int]),
    "rt_cells": (ctypes.c_longlong, [_P]),
    "rt_batch_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.POINTER(_P)]),
    "rt_batch_destroy": (ctypes.c_int, [_P]),
    "rt_batch_last_error": (ctypes.c_char_p, [_P]),
    "rt_batch_set_tuning": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "rt_batch_set_persistent": (ctypes.c_int, [_P, ctypes.c_int]),
    "rt_batch_persistent_members": (ctypes.c_int, [_P]),
    "rt_batch_set_slices": (ctypes.c_int, [_P, ctypes.c_int]),
    "rt_batch_set_fused": (ctypes.c_int, [_P, ctypes.c_int]),
    "rt_batch_integrate": (ctypes.c_int, [_P, ctypes.c_int]),
    "rt_batch_sync": (ctypes.c_int, [_P]),
    "rt_batch_stream": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "rt_batch_launch_count": (ctypes.c_longlong, [_P]),
    "rt_batch_cells": (ctypes.c_longlong, [_P]),
    "rt_max_rate_noalloc": (ctypes.c_int, [ctypes.POINTER(RtDims), ctypes.POINTER(_D), ctypes.POINTER(_D),
                                           ctypes.POINTER(_D), _D, _P]),
    "rt_noalloc_last_error": (ctypes.c_char_p, []),
}

_lib = None


class RtError(RuntimeError):
    pass


def load():
    """Load libraytracer_gb300.so once; raise if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RtError("libraytracer_gb300.so not found at %s: run "
                      "`python -c 'import __graft_entry__ as g; g.build()'` first" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc, handle=None, what="call"):
    if rc != RT_OK:
        msg = load().rt_last_error(handle)
        raise RtError("%s failed (%d): %s" % (what, rc, msg.decode() if msg else ""))
    return rc


def dptr(arr):
    """double* of a C- or Fortran-contiguous float64 numpy array."""
    assert arr.dtype.name == "float64" and (arr.flags.f_contiguous or arr.flags.c_contiguous)
    return arr.ctypes.data_as(_D)
