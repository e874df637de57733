"""ctypes binding of libmce_gb300.so (the C ABI in include/mce_c_api.h).

There is no fallback: if the library is not built, or no CUDA device is
visible when an estimator is created, the call raises.
"""
from __future__ import annotations

import ctypes
import os
import re

from . import build as _build

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_longlong)
_vp = ctypes.c_void_p

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "mce_c_api.h")

# name -> (restype, argtypes)
SIGNATURES = {
    "mce_last_error": (ctypes.c_char_p, []),
    "mce_set_reference_num_cpus": (ctypes.c_int, [ctypes.c_int]),
    "mce_draw_reference_constants": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                     _dp, _dp]),
    "mce_batch_create": (_vp, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _ip, _dp, _dp,
                               _dp, _dp, _dp, ctypes.c_int, _ip]),
    "mce_batch_step": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, ctypes.c_int, _ip]),
    "mce_shift_cf_by_bias": (ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    "mce_deterministic_time_prop": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _dp]),
    "mce_finalize_extended_moments": (ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    "mce_cpdf_1d_grid": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_int, _dp, _dp]),
    "mce_cpdf_nd": (ctypes.c_int, [_vp, ctypes.c_int, _dp, ctypes.c_int, _dp]),
    "mce_cpdf_marginal": (ctypes.c_int, [_vp, ctypes.c_int, _ip, ctypes.c_int, _dp, _dp, ctypes.c_int, _dp]),
    "mce_cpdf_2d_grid": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp] + [ctypes.c_double] * 6
                         + [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]),
    "mce_draw_bar_nu": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_int, _dp]),
    "mce_rel2d_create": (_vp, [_vp, ctypes.c_int, _vp, ctypes.c_int, _dp, _dp, ctypes.c_int, ctypes.c_int,
                               ctypes.c_double, _dp, _lp, _ip]),
    "mce_rel2d_grid": (ctypes.c_int, [_vp] + [ctypes.c_double] * 8 + [ctypes.c_int, _dp, _dp, _dp]),
    "mce_rel2d_num_pairs": (ctypes.c_longlong, [_vp]),
    "mce_rel2d_num_terms": (ctypes.c_longlong, [_vp]),
    "mce_rel2d_device_ms": (ctypes.c_double, [_vp, ctypes.c_int]),
    "mce_rel2d_launch_count": (ctypes.c_longlong, [_vp]),
    "mce_rel2d_destroy": (None, [_vp]),
    "mce_batch_step_noalloc": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, ctypes.c_int, _ip]),
    "mce_batch_run": (ctypes.c_int, [_vp, _dp, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp, ctypes.c_int, _dp,
                                     _dp, _dp, _ip, _lp]),
    "mce_create": (_vp, [_dp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp,
                         _dp, _ip]),
    "mce_step": (ctypes.c_int, [_vp, ctypes.c_double, _dp, _dp, _dp, _dp, ctypes.c_double, _dp, _dp]),
    "mce_get_moments": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _dp]),
    "mce_get_raw_moments": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _dp, _dp]),
    "mce_get_errors": (ctypes.c_int, [_vp, ctypes.c_int]),
    "mce_num_terms": (ctypes.c_longlong, [_vp, ctypes.c_int]),
    "mce_terms_per_shape": (ctypes.c_int, [_vp, ctypes.c_int, _ip, ctypes.c_int]),
    "mce_post_mu_terms": (ctypes.c_longlong, [_vp]),
    "mce_host_time_ms": (ctypes.c_double, [_vp, ctypes.c_int]),
    "mce_master_step": (ctypes.c_int, [_vp]),
    "mce_device_errors": (ctypes.c_int, [_vp]),
    "mce_total_cells": (ctypes.c_longlong, [_vp, ctypes.c_int]),
    "mce_dump_terms": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _ip, _dp, _dp, _dp, _ip, _ip, _dp]),
    "mce_trim_memory": (ctypes.c_longlong, [_vp, ctypes.c_longlong]),
    "mce_reset": (ctypes.c_int, [_vp]),
    "mce_reinitialize_start_statistics": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _dp]),
    "mce_set_master_step": (ctypes.c_int, [_vp, ctypes.c_int]),
    "mce_set_window_number": (ctypes.c_int, [_vp, ctypes.c_int]),
    "mce_set_print_basic_info": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    "mce_last_step_ms": (ctypes.c_double, [_vp]),
    "mce_device_time_ms": (ctypes.c_double, [_vp]),
    "mce_launch_count": (ctypes.c_longlong, [_vp]),
    "mce_set_profiling": (ctypes.c_int, [_vp, ctypes.c_int]),
    "mce_clear_profile": (ctypes.c_int, [_vp]),
    "mce_num_kernel_groups": (ctypes.c_int, []),
    "mce_kernel_group_name": (ctypes.c_char_p, [ctypes.c_int]),
    "mce_kernel_group_stats": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _lp, _dp, _dp]),
    "mce_autotune_configure": (ctypes.c_int, [ctypes.c_int]),
    "mce_autotune_table": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float), ctypes.c_int]),
    "mce_autotune_kernel_name": (ctypes.c_char_p, [ctypes.c_int]),
    "mce_destroy": (None, [_vp]),
    "mce_sym_eig": (ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp]),
    "mce_speyers_window_init": (ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double, _dp,
                                               _dp, _dp, _dp]),
    "mce_swm_create": (_vp, [ctypes.c_int] * 7 + [_dp] * 9 + [ctypes.c_double, ctypes.c_int, _vp, _dp, _dp, _dp,
                                                              ctypes.c_int, _ip]),
    "mce_swm_create_nonlin": (_vp, [ctypes.c_int] * 7 + [_dp] * 6 + [ctypes.c_double, ctypes.c_int, _vp, _vp, _vp,
                                                                     _dp, _dp, _dp, ctypes.c_int, _ip]),
    "mce_swm_step": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip]),
    "mce_swm_post_mu_terms": (ctypes.c_longlong, [_vp]),
    "mce_swm_window": (_vp, [_vp, ctypes.c_int]),
    "mce_swm_window_count": (ctypes.c_int, [_vp, ctypes.c_int]),
    "mce_swm_destroy": (None, [_vp]),
    "mce_adjoint_create": (_vp, [ctypes.c_int] * 4 + [_dp] * 5 + [_ip]),
    "mce_adjoint_forward": (ctypes.c_int, [_vp] + [_dp] * 7),
    "mce_adjoint_num_params": (ctypes.c_int, [_vp]),
    "mce_adjoint_backward": (ctypes.c_int, [_vp, _dp, _dp]),
    "mce_adjoint_check": (ctypes.c_int, [_vp, _dp, _dp]),
    "mce_adjoint_timing": (ctypes.c_int, [_vp, _dp]),
    "mce_adjoint_destroy": (None, [_vp]),
    "mce_adjoint_batch_create": (_vp, [ctypes.c_int] * 4 + [_ip] + [_dp] * 5 + [ctypes.c_int, _ip]),
    "mce_adjoint_batch_forward": (ctypes.c_int, [_vp, _dp, ctypes.c_int] + [_dp] * 6),
    "mce_adjoint_batch_forward_ltv": (ctypes.c_int, [_vp, _dp, ctypes.c_int] + [_dp] * 6),
    "mce_adjoint_forward_ltv": (ctypes.c_int, [_vp] + [_dp] * 7),
    "mce_adjoint_batch_backward": (ctypes.c_int, [_vp, _dp, ctypes.c_int, _dp]),
    "mce_adjoint_batch_num_params": (ctypes.c_int, [_vp]),
    "mce_adjoint_batch_set_first_sub": (ctypes.c_int, [_vp, ctypes.c_int]),
    "mce_adjoint_batch_check": (ctypes.c_int, [_vp, _dp, _dp]),
    "mce_adjoint_batch_timing": (ctypes.c_int, [_vp, _dp]),
    "mce_adjoint_batch_destroy": (None, [_vp]),
}

_LIB = None


def header_functions():
    """Function names declared in include/mce_c_api.h."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mce_[a-z0-9_]+)\s*\(", txt)))


def load(build_if_missing=True):
    """Loads the in-tree library, building it first when it is missing."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise OSError("libmce_gb300.so is not built (run cauchyfriendly_gb300.build.build())")
        _build.build()
    lib = ctypes.CDLL(_build.LIB)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def dp(a):
    """A double* to a contiguous float64 array, or NULL for None."""
    return None if a is None else a.ctypes.data_as(_dp)


def last_error():
    return load().mce_last_error().decode(errors="replace")


class MceError(RuntimeError):
    pass


def check(status, what):
    if status < 0:
        raise MceError("%s failed (%d): %s" % (what, status, last_error()))
    return status
