"""Test infrastructure only: the reference's SWIG module ``pycauchy``
rebuilt as a ctypes module over ``ref_pycauchy.cpp`` (the reference's own
scripts/swig/cauchy/pycauchy.hpp, compiled unmodified; SWIG is absent here).

Same function names, argument order and return tuples as the SWIG wrappers
(numpy.i IN_ARRAY1 inputs, ARGOUTVIEWM_ARRAY1 outputs), for the functions the
reference's scripts/swig/cauchy/cauchy_estimator.py calls on the LTI, LTV and
nonlinear paths: single-estimator stepping, reset, reinitialisation
statistics, Speyer's restart, the search-axis ordering and the C++ window
manager.  Importing the
reference's cauchy_estimator.py with this module registered as ``pycauchy``
runs the reference's PyCauchyEstimator / PySlidingWindowManager /
PySlidingWindowManager_CPP on the reference's C++
(tests/golden/make_windows_golden.py).  Needs the reference sources
(oracle.build()).
"""
from __future__ import annotations

import ctypes as ct
import os

import numpy as np

from . import REF_OUT

_dp = ct.POINTER(ct.c_double)
_ip = ct.POINTER(ct.c_int)
_L = None


def lib():
    global _L
    if _L is None:
        path = os.path.join(REF_OUT, "libmce_ref_pycauchy.so")
        if not os.path.exists(path):
            raise RuntimeError("the reference pycauchy shim is not built (needs the reference sources)")
        _L = ct.PyDLL(path)  # holds the GIL: callbacks may run in forked window processes
        for name in ("refpy_initialize_lti", "refpy_initialize_ltv", "refpy_initialize_nonlin"):
            getattr(_L, name).restype = ct.c_void_p
    return _L


def _a(x):
    """A float64 1-D contiguous array (the IN_ARRAY1 typemap) and its size."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1))
    return a, a.size


def _p(a):
    return a.ctypes.data_as(_dp) if a.size else None


class _RefHandle:
    def __init__(self, ptr, n, p, pncc, cmcc, keep):
        self.ptr = ct.c_void_p(ptr)
        self.n, self.p, self.pncc, self.cmcc = n, p, pncc, cmcc
        self._keep = keep


def _flat_args(arrs):
    args = []
    for a, n in arrs:
        args += [_p(a), n]
    return args


def pycauchy_initialize_lti(num_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma, dt, init_step, debug_print):
    arrs = [_a(x) for x in (A0, p0, b0, Phi, Gamma, B, beta, H, gamma)]
    ptr = lib().refpy_initialize_lti(int(num_steps), *_flat_args(arrs), ct.c_double(dt), int(init_step),
                                     int(bool(debug_print)))
    return _RefHandle(ptr, arrs[2][1], arrs[8][1], arrs[6][1], arrs[5][1] // max(arrs[2][1], 1), arrs)


def pycauchy_initialize_ltv(num_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma, f_dyn_update_callback, dt,
                            init_step, debug_print):
    arrs = [_a(x) for x in (A0, p0, b0, Phi, Gamma, B, beta, H, gamma)]
    ptr = lib().refpy_initialize_ltv(int(num_steps), *_flat_args(arrs), ct.c_void_p(int(f_dyn_update_callback)),
                                     ct.c_double(dt), int(init_step), int(bool(debug_print)))
    return _RefHandle(ptr, arrs[2][1], arrs[8][1], arrs[6][1], arrs[5][1] // max(arrs[2][1], 1), arrs)


def pycauchy_single_step_ltiv(h, msmts, controls):
    m, nm = _a(msmts)
    c, nc = _a(controls)
    n, pncc, cmcc = h.n, h.pncc, h.cmcc
    dyn = [np.zeros(max(s, 1)) for s in (n * n, n * pncc, n * cmcc, nm * n, pncc, nm)]
    dyn_ptrs = (_dp * 6)(*[d.ctypes.data_as(_dp) for d in dyn])
    sizes = (ct.c_int * 6)()
    fz, x, P = np.zeros(nm), np.zeros(nm * n), np.zeros(nm * n * n)
    cfz, cx, cP = np.zeros(nm), np.zeros(nm), np.zeros(nm)
    err = np.zeros(nm, dtype=np.int32)
    lib().refpy_single_step_ltiv(h.ptr, _p(m), nm, _p(c), nc, dyn_ptrs, sizes, fz.ctypes.data_as(_dp),
                                 x.ctypes.data_as(_dp), P.ctypes.data_as(_dp), cfz.ctypes.data_as(_dp),
                                 cx.ctypes.data_as(_dp), cP.ctypes.data_as(_dp), err.ctypes.data_as(_ip))
    outs = [d[:s].copy() for d, s in zip(dyn, sizes)]
    return (*outs, fz, x, P, cfz, cx, cP, err)


def pycauchy_initialize_nonlin(num_steps, x0, A0, p0, b0, beta, gamma, f_dyn_update_callback, f_nonlinear_msmt_model,
                               f_extended_msmt_update_callback, cmcc, dt, init_step, debug_print):
    arrs = [_a(x) for x in (x0, A0, p0, b0, beta, gamma)]
    ptr = lib().refpy_initialize_nonlin(int(num_steps), *_flat_args(arrs), ct.c_void_p(int(f_dyn_update_callback)),
                                        ct.c_void_p(int(f_nonlinear_msmt_model)),
                                        ct.c_void_p(int(f_extended_msmt_update_callback)), int(cmcc),
                                        ct.c_double(dt), int(init_step), int(bool(debug_print)))
    return _RefHandle(ptr, arrs[3][1], arrs[5][1], arrs[4][1], int(cmcc), arrs)


def pycauchy_single_step_nonlin(h, msmts, controls, with_propagate):
    m, nm = _a(msmts)
    c, nc = _a(controls)
    n, pncc, cmcc = h.n, h.pncc, h.cmcc
    dsz = [n * n, n * pncc, n * cmcc, nm * n, pncc, nm, nm, nm * n, nm * n * n, nm * n, nm, nm, nm, nm]
    outs = [np.zeros(max(sz, 1)) for sz in dsz] + [np.zeros(max(nm, 1), dtype=np.int32)]
    ptrs = (ct.c_void_p * 15)(*[o.ctypes.data for o in outs])
    sizes = (ct.c_int * 15)()
    lib().refpy_single_step_nonlin(h.ptr, _p(m), nm, _p(c), nc, int(bool(with_propagate)), ptrs, sizes)
    return tuple(o[:sz].copy() for o, sz in zip(outs, sizes))


def pycauchy_single_step_get_number_of_terms(h):
    return int(lib().refpy_get_number_of_terms(h.ptr))


def pycauchy_single_step_set_master_step(h, step):
    lib().refpy_set_master_step(h.ptr, int(step))


def pycauchy_single_step_set_window_number(h, win_num):
    lib().refpy_set_window_number(h.ptr, int(win_num))


def pycauchy_single_step_reset(h, A0, p0, b0, xbar):
    lib().refpy_reset(h.ptr, *_flat_args([_a(x) for x in (A0, p0, b0, xbar)]))


def pycauchy_single_step_shutdown(h):
    lib().refpy_shutdown(h.ptr)


def pycauchy_get_reinitialization_statistics(h, z, xhat, Phat, H, gamma):
    x, nx = _a(xhat)
    P, nP = _a(np.array(Phat, dtype=np.float64))  # the reference boosts it in place
    Hh, nH = _a(H)
    A0, p0, b0 = np.zeros(nx * nx), np.zeros(nx), np.zeros(nx)
    lib().refpy_get_reinitialization_statistics(h.ptr, ct.c_double(z), _p(x), nx, _p(P), nP, _p(Hh), nH,
                                                ct.c_double(gamma), A0.ctypes.data_as(_dp), p0.ctypes.data_as(_dp),
                                                b0.ctypes.data_as(_dp))
    return A0, p0, b0


def pycauchy_speyers_window_init(x1_hat, Var, H, gamma, z):
    x, nx = _a(x1_hat)
    P, nP = _a(np.array(Var, dtype=np.float64))  # the reference boosts it in place
    Hh, nH = _a(H)
    A0, p0, b0 = np.zeros(nx * nx), np.zeros(nx), np.zeros(nx)
    lib().refpy_speyers_window_init(_p(x), nx, _p(P), nP, _p(Hh), nH, ct.c_double(gamma), ct.c_double(z),
                                    A0.ctypes.data_as(_dp), p0.ctypes.data_as(_dp), b0.ctypes.data_as(_dp))
    return A0, p0, b0


def pycauchy_set_tr_search_idxs_ordering(ordering):
    o = np.ascontiguousarray(np.asarray(ordering, dtype=np.int32).reshape(-1))
    return int(lib().refpy_set_tr_search_idxs_ordering(o.ctypes.data_as(_ip), o.size))


_wm_keep = None


def pycauchy_initialize_lti_window_manager(num_windows, num_sim_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma,
                                           debug_print, log_seq, log_full, log_dir, dt, init_step, win_var_boost):
    global _wm_keep
    arrs = [_a(x) for x in (A0, p0, b0, Phi, Gamma, B, beta, H, gamma, win_var_boost)]
    _wm_keep = arrs
    lib().refpy_initialize_lti_window_manager(int(num_windows), int(num_sim_steps), *_flat_args(arrs[:9]),
                                              int(bool(debug_print)), ct.c_double(dt), int(init_step),
                                              _p(arrs[9][0]), arrs[9][1])


def pycauchy_initialize_ltv_window_manager(num_windows, num_sim_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma,
                                           f_dyn_update_callback, debug_print, log_seq, log_full, log_dir, dt,
                                           init_step, win_var_boost):
    global _wm_keep
    arrs = [_a(x) for x in (A0, p0, b0, Phi, Gamma, B, beta, H, gamma, win_var_boost)]
    _wm_keep = arrs
    lib().refpy_initialize_ltv_window_manager(int(num_windows), int(num_sim_steps), *_flat_args(arrs[:9]),
                                              ct.c_void_p(int(f_dyn_update_callback)), int(bool(debug_print)),
                                              ct.c_double(dt), int(init_step), _p(arrs[9][0]), arrs[9][1])


def pycauchy_initialize_nonlin_window_manager(num_windows, num_sim_steps, x0, A0, p0, b0, beta, gamma,
                                              f_dyn_update_callback, f_nonlinear_msmt_model,
                                              f_extended_msmt_update_callback, cmcc, debug_print, log_seq, log_full,
                                              log_dir, dt, init_step, win_var_boost):
    global _wm_keep
    arrs = [_a(x) for x in (x0, A0, p0, b0, beta, gamma, win_var_boost)]
    # pycauchy_step reads the state dimension from _wm_keep[2]
    _wm_keep = [arrs[1], arrs[2], arrs[3]] + arrs
    lib().refpy_initialize_nonlin_window_manager(int(num_windows), int(num_sim_steps), *_flat_args(arrs[:6]),
                                                 ct.c_void_p(int(f_dyn_update_callback)),
                                                 ct.c_void_p(int(f_nonlinear_msmt_model)),
                                                 ct.c_void_p(int(f_extended_msmt_update_callback)), int(cmcc),
                                                 int(bool(debug_print)), ct.c_double(dt), int(init_step),
                                                 _p(arrs[6][0]), arrs[6][1])


def pycauchy_step(msmts, controls):
    m, nm = _a(msmts)
    c, nc = _a(controls)
    n = _wm_keep[2][1]
    fz, cfz, cx, cP = ct.c_double(), ct.c_double(), ct.c_double(), ct.c_double()
    wi, err = ct.c_int(), ct.c_int()
    x, P = np.zeros(n), np.zeros(n * n)
    lib().refpy_step(_p(m), nm, _p(c), nc, ct.byref(fz), x.ctypes.data_as(_dp), P.ctypes.data_as(_dp),
                     ct.byref(cfz), ct.byref(cx), ct.byref(cP), ct.byref(wi), ct.byref(err))
    return fz.value, x, P, cfz.value, cx.value, cP.value, wi.value, err.value


def pycauchy_shutdown():
    lib().refpy_shutdown_window_manager()


# ---- helpers of this harness (not part of the SWIG module) ----------------

def srand(seed):
    lib().refpy_srand(ct.c_uint(seed))


def get_constants(h):
    """(root_point, b_pert) the estimator behind a handle drew at construction."""
    rp = np.zeros(h.n)
    bp = np.zeros(64)
    ms = ct.c_int()
    lib().refpy_get_constants(h.ptr, rp.ctypes.data_as(_dp), bp.ctypes.data_as(_dp), ct.byref(ms))
    return rp, bp[:ms.value].copy()
