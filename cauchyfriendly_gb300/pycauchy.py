"""Drop-in replacement of the reference's SWIG module ``pycauchy`` for the
single-estimator step path, backed by libmce_gb300.so.

Same function names, argument order and return tuples as the SWIG wrappers in
scripts/swig/cauchy/pycauchy.hpp / pycauchy.i, so the reference's
``cauchy_estimator.PyCauchyEstimator`` runs on the GPU when this module is
importable as ``pycauchy``.  Numpy arrays come in flattened (the numpy.i
IN_ARRAY1 typemaps) and go out as float64 / int32 arrays (ARGOUTVIEWM_ARRAY1).

Covered:
* single estimators: pycauchy_initialize_lti / _ltv / _nonlin,
  pycauchy_single_step_ltiv / _nonlin / _deterministic_transform,
  _get_number_of_terms, _set_master_step, _set_window_number, _get_duc,
  _reset, _shutdown;
* window restarts: pycauchy_get_reinitialization_statistics,
  pycauchy_speyers_window_init (Speyer's statistics, computed by the
  library's C++ with the reference's eigen-solver);
* the C++ window manager: pycauchy_initialize_lti_window_manager / _ltv_ /
  _nonlin_, pycauchy_step (8-tuple), pycauchy_shutdown -- one manager per
  process, as the reference's globals allow;
* pdf grids: pycauchy_get_marginal_1D/2D_pointwise_cpdf, _get_1D/2D_;
  the relative system: pycauchy_single_step_eval_2d_rsys_cpdf;
* pycauchy_set_tr_search_idxs_ordering (accepted, no effect: see its
  docstring).
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from .estimator import CauchyEstimator


class C_CauchyDynamicsUpdateContainer(ct.Structure):
    """Layout of CauchyDynamicsUpdateContainer (include/dynamic_models.hpp:62-80),
    the struct LTV callbacks receive."""
    _fields_ = [("x", ct.POINTER(ct.c_double)), ("u", ct.POINTER(ct.c_double)), ("dt", ct.c_double),
                ("step", ct.c_int), ("n", ct.c_int), ("cmcc", ct.c_int), ("pncc", ct.c_int), ("p", ct.c_int),
                ("Phi", ct.POINTER(ct.c_double)), ("Gamma", ct.POINTER(ct.c_double)), ("B", ct.POINTER(ct.c_double)),
                ("H", ct.POINTER(ct.c_double)), ("beta", ct.POINTER(ct.c_double)), ("gamma", ct.POINTER(ct.c_double)),
                ("is_xbar_set_for_ece", ct.c_bool), ("other_stuff", ct.c_void_p)]


_CALLBACK = ct.CFUNCTYPE(None, ct.POINTER(C_CauchyDynamicsUpdateContainer))
_MSMT_CALLBACK = ct.CFUNCTYPE(None, ct.POINTER(C_CauchyDynamicsUpdateContainer), ct.POINTER(ct.c_double))


class _Handle:
    """What pycauchy_initialize_* returns: the estimator plus the dynamics
    container (pycauchy.hpp:240-280 PyCauchyDataHandler)."""

    def __init__(self, num_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma, dt, init_step, debug_print,
                 est_cmcc=None):
        n = int(np.asarray(b0).size)
        self.n = n
        self.pncc = int(np.asarray(beta).size)
        self.cmcc = int(np.asarray(B).size) // n
        self.p = int(np.asarray(gamma).size)
        f = lambda a, size: (np.zeros(size) if a is None or np.asarray(a).size == 0
                             else np.array(a, dtype=np.float64).reshape(-1))
        # dynamics container storage (owned here, pointed to by the C struct)
        self.x = np.zeros(n)
        self.u = np.zeros(max(self.cmcc, 1))
        self.Phi = f(Phi, n * n)
        self.Gamma = f(Gamma, n * self.pncc)
        self.B = f(B, n * self.cmcc)
        self.H = f(H, self.p * n)
        self.beta = f(beta, self.pncc)
        self.gamma = f(gamma, self.p)
        self.duc = C_CauchyDynamicsUpdateContainer()
        P = lambda a: a.ctypes.data_as(ct.POINTER(ct.c_double))
        self.duc.x, self.duc.u = P(self.x), P(self.u)
        self.duc.dt, self.duc.step = float(dt), int(init_step)
        self.duc.n, self.duc.cmcc, self.duc.pncc, self.duc.p = n, self.cmcc, self.pncc, self.p
        self.duc.Phi, self.duc.Gamma, self.duc.B = P(self.Phi), P(self.Gamma), P(self.B)
        self.duc.H, self.duc.beta, self.duc.gamma = P(self.H), P(self.beta), P(self.gamma)
        self.duc.is_xbar_set_for_ece = False
        self.duc.other_stuff = None
        self.callback = None
        self.est = CauchyEstimator(np.asarray(A0, dtype=np.float64).reshape(n, n), p0, b0, int(num_steps), n,
                                   self.cmcc if est_cmcc is None else int(est_cmcc), self.pncc, self.p,
                                   bool(debug_print))


def pycauchy_initialize_lti(num_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma, dt, init_step, debug_print):
    """pycauchy.hpp:295-328"""
    return _Handle(num_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma, dt, init_step, debug_print)


def pycauchy_initialize_ltv(num_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma, f_dyn_update_callback, dt,
                            init_step, debug_print):
    """pycauchy.hpp:330-363; the callback is a raw C function pointer (int)."""
    h = _Handle(num_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma, dt, init_step, debug_print)
    h.callback = _CALLBACK(int(f_dyn_update_callback))
    return h


def pycauchy_initialize_nonlin(num_steps, x0, A0, p0, b0, beta, gamma, f_dyn_update_callback, f_nonlinear_msmt_model,
                               f_extended_msmt_update_callback, cmcc, dt, init_step, debug_print):
    """pycauchy.hpp:365-396: an estimator (no controls) whose linearised
    dynamics and measurement models come from three callbacks, raw C function
    pointers (ints) taking the dynamics container."""
    n = int(np.asarray(b0).size)
    pncc = int(np.asarray(beta).size)
    p = int(np.asarray(gamma).size)
    h = _Handle(num_steps, A0, p0, b0, None, np.zeros(n * pncc), np.zeros(n * int(cmcc)), beta, np.zeros(p * n),
                gamma, dt, init_step, debug_print, est_cmcc=0)
    h.x[:] = np.asarray(x0, dtype=np.float64).reshape(n)
    h.f_dyn = _CALLBACK(int(f_dyn_update_callback))
    h.f_msmt = _MSMT_CALLBACK(int(f_nonlinear_msmt_model))
    h.f_ext = _CALLBACK(int(f_extended_msmt_update_callback))
    return h


def pycauchy_single_step_nonlin(h, msmts, controls, with_propagate):
    """pycauchy.hpp:545-652: propagate x_bar through the dynamics callback
    (unless with_propagate is false), then for each of the last len(msmts)
    measurements: the nonlinear measurement model gives z_bar, the extended
    update callback sets H, the estimator takes z - z_bar, and
    finalize_extended_moments moves x_bar to the new estimate.  Returns
    (Phi, Gamma, B, H, beta, gamma, fz, xhat, Phat, xbar, zbar, cerr_fz,
    cerr_xhat, cerr_Phat, err_code)."""
    msmts = np.atleast_1d(np.asarray(msmts, dtype=np.float64)).reshape(-1)
    controls = np.atleast_1d(np.asarray(controls, dtype=np.float64)).reshape(-1)
    n, p, pncc, cmcc, k = h.n, h.p, h.pncc, h.cmcc, msmts.size
    assert p >= k
    if cmcc > 0 and controls.size:
        h.u[:cmcc] = controls[:cmcc]
    out_Phi, out_Gamma, out_B = np.zeros(n * n), np.zeros(n * pncc), np.zeros(n * cmcc)
    out_beta, out_H, out_gamma = np.zeros(pncc), np.zeros(k * n), np.zeros(k)
    if with_propagate:
        h.duc.is_xbar_set_for_ece = False
        h.f_dyn(ct.pointer(h.duc))
        assert h.duc.is_xbar_set_for_ece
        out_Phi[:], out_B[:], out_Gamma[:], out_beta[:] = h.Phi, h.B, h.Gamma, h.beta
    fz, xhat, Phat = np.zeros(k), np.zeros(k * n), np.zeros(k * n * n)
    xbar, zbar_out = np.zeros(k * n), np.zeros(k)
    cfz, cx, cP, err = np.zeros(k), np.zeros(k), np.zeros(k), np.zeros(k, dtype=np.int32)
    start = p - k
    zbar = np.zeros(p)
    for i in range(k):
        idx = start + i
        h.f_msmt(ct.pointer(h.duc), zbar.ctypes.data_as(ct.POINTER(ct.c_double)))
        h.f_ext(ct.pointer(h.duc))
        xbar[i * n:(i + 1) * n] = h.x
        zbar_out[i] = zbar[idx]
        out_H[i * n:(i + 1) * n] = h.H[idx * n:(idx + 1) * n]
        out_gamma[i] = h.gamma[idx]
        err[i] = h.est.step(msmts[i] - zbar[idx], h.Phi.reshape(n, n), h.Gamma.reshape(n, pncc) if pncc else None,
                            h.beta if pncc else None, h.H[idx * n:(idx + 1) * n], h.gamma[idx])
        h.x[:] = h.est.finalize_extended_moments(h.x)
        mo = h.est.moments()
        fz[i], cfz[i] = mo["fz"].real, mo["fz"].imag
        xhat[i * n:(i + 1) * n] = mo["mean"].real
        Phat[i * n * n:(i + 1) * n * n] = mo["cov"].real.reshape(-1)
        cx[i] = np.max(np.abs(mo["mean"].imag))
        cP[i] = np.max(np.abs(mo["cov"].imag))
        err[i] = h.est.errors()
    h.duc.step += 1
    return (out_Phi, out_Gamma, out_B, out_H, out_beta, out_gamma, fz, xhat, Phat, xbar, zbar_out, cfz, cx, cP, err)


def pycauchy_single_step_ltiv(h, msmts, controls):
    """pycauchy.hpp:461-543: steps the estimator through len(msmts) scalar
    measurements (the last len(msmts) of the p per step) and returns
    (Phi, Gamma, B, H, beta, gamma, fz, xhat, Phat, cerr_fz, cerr_xhat,
    cerr_Phat, err_code)."""
    msmts = np.atleast_1d(np.asarray(msmts, dtype=np.float64)).reshape(-1)
    controls = np.atleast_1d(np.asarray(controls, dtype=np.float64)).reshape(-1)
    n, p, k = h.n, h.p, msmts.size
    assert p >= k
    if h.cmcc > 0:
        h.u[:h.cmcc] = controls[:h.cmcc]
    start = p - k
    empty = np.array([], dtype=np.float64)
    outs = [empty] * 6
    if h.callback is not None:
        h.x[:] = np.real(h.est.moments()["mean"]) if h.est.master_step() > 0 else h.x
        h.callback(ct.pointer(h.duc))
        outs = [h.Phi.copy(), h.Gamma.copy(), h.B.copy(), h.H[start * n:(start + k) * n].copy(), h.beta.copy(),
                h.gamma[start:start + k].copy()]
    fz = np.zeros(k)
    xhat = np.zeros(k * n)
    Phat = np.zeros(k * n * n)
    cfz = np.zeros(k)
    cx = np.zeros(k)
    cP = np.zeros(k)
    err = np.zeros(k, dtype=np.int32)
    Phi = h.Phi.reshape(n, n)
    Gamma = h.Gamma.reshape(n, h.pncc) if h.pncc else None
    B = h.B.reshape(n, h.cmcc) if h.cmcc else None
    u = h.u[:h.cmcc] if h.cmcc else None
    for i in range(k):
        idx = start + i
        err[i] = h.est.step(msmts[i], Phi, Gamma, h.beta if h.pncc else None, h.H[idx * n:(idx + 1) * n],
                            h.gamma[idx], B, u)
        mo = h.est.moments()
        fz[i] = mo["fz"].real
        cfz[i] = mo["fz"].imag
        xhat[i * n:(i + 1) * n] = mo["mean"].real
        Phat[i * n * n:(i + 1) * n * n] = mo["cov"].real.reshape(-1)
        cx[i] = np.max(np.abs(mo["mean"].imag))
        cP[i] = np.max(np.abs(mo["cov"].imag))
    return (*outs, fz, xhat, Phat, cfz, cx, cP, err)


def pycauchy_single_step_get_number_of_terms(h):
    """pycauchy.hpp:666"""
    return h.est.num_terms()


def pycauchy_single_step_set_master_step(h, step):
    """pycauchy.hpp:767"""
    h.est.set_master_step(int(step))


def pycauchy_single_step_set_window_number(h, win_num):
    """pycauchy.hpp:779"""
    h.est.set_win_num(int(win_num))


def pycauchy_single_step_get_duc(h):
    """pycauchy.hpp:791: address of the dynamics container."""
    return ct.addressof(h.duc)


def pycauchy_single_step_reset(h, A0, p0, b0, xbar):
    """pycauchy.hpp:798-819: new start statistics (empty arrays keep the old
    ones), optional xbar into the container, then reset."""
    n = h.n
    A0 = np.asarray(A0, dtype=np.float64).reshape(-1)
    p0 = np.asarray(p0, dtype=np.float64).reshape(-1)
    b0 = np.asarray(b0, dtype=np.float64).reshape(-1)
    xbar = np.asarray(xbar, dtype=np.float64).reshape(-1)
    if A0.size or p0.size or b0.size:
        cur = h.est
        a = A0 if A0.size else None
        pp = p0 if p0.size else None
        bb = b0 if b0.size else None
        if a is None or pp is None or bb is None:
            raise ValueError("partial start statistics are not supported; pass A0, p0 and b0")
        cur.reinitialize_start_statistics(a.reshape(n, n), pp, bb)
    if xbar.size:
        h.x[:] = xbar
    h.est.reset()


def pycauchy_single_step_deterministic_transform(h, Trans, bias):
    """pycauchy.hpp:654-663: deterministic_time_prop(Trans) then shift_cf_by_bias(bias)."""
    h.est.deterministic_time_prop(np.asarray(Trans, dtype=np.float64).reshape(h.n, h.n))
    h.est.shift_cf_by_bias(np.asarray(bias, dtype=np.float64).reshape(h.n))


def pycauchy_get_marginal_2D_pointwise_cpdf(h, marg_idx1, marg_idx2, gridx_low, gridx_high, gridx_resolution,
                                            gridy_low, gridy_high, gridy_resolution, log_dir=None, reset_cache=True):
    """pycauchy.hpp:822-862: the grid as (x, y, z) triples, flattened, and its
    x and y sizes."""
    X, Y, Z = h.est.get_marginal_2D_pointwise_cpdf(int(marg_idx1), int(marg_idx2), gridx_low, gridx_high,
                                                   gridx_resolution, gridy_low, gridy_high, gridy_resolution,
                                                   reset_cache=reset_cache)
    pts = np.empty(3 * X.size)
    pts[0::3], pts[1::3], pts[2::3] = X.reshape(-1), Y.reshape(-1), Z.reshape(-1)
    return pts, int(X.shape[1]), int(X.shape[0])


def pycauchy_get_2D_pointwise_cpdf(h, gridx_low, gridx_high, gridx_resolution, gridy_low, gridy_high,
                                   gridy_resolution, log_dir=None, reset_cache=True):
    """pycauchy.hpp:864-887"""
    return pycauchy_get_marginal_2D_pointwise_cpdf(h, 0, 1, gridx_low, gridx_high, gridx_resolution, gridy_low,
                                                   gridy_high, gridy_resolution, log_dir, reset_cache)


def pycauchy_single_step_eval_2d_rsys_cpdf(Trel, s_pcdh, p_pcdh, RSYS_APPROX_EPS, xlow, xhigh, delta_x, ylow, yhigh,
                                           delta_y):
    """pycauchy.hpp:672-747: the relative system secondary - primary projected
    by Trel (2 x n, flattened), term approximation at RSYS_APPROX_EPS, its
    moments and its pdf on the grid offset by the relative mean.  Returns
    (fz[1], xhat[2], Phat[4], cerr_fz[1], cerr_xhat[2], cerr_Phat[4],
    cpdf points as flattened (x, y, z) triples, num_gridx, num_gridy).  The
    terms are taken in the reference's single-thread order."""
    from .estimator import RelativeSystem2D
    n = p_pcdh.n
    rs = RelativeSystem2D(p_pcdh.est, s_pcdh.est, np.asarray(Trel, dtype=np.float64).reshape(2, n),
                          full_solve=False, get_relative_moments=True, with_term_approx=True,
                          term_approx_eps=float(RSYS_APPROX_EPS))
    try:
        m = rs.moments
        fz = np.array([m["fz"].real])
        cerr_fz = np.array([m["fz"].imag])
        xhat, cerr_xhat = m["mean"].real.copy(), m["mean"].imag.copy()
        Phat, cerr_Phat = m["cov"].real.reshape(-1).copy(), m["cov"].imag.reshape(-1).copy()
        X, Y, Z, nx, ny = rs.grid(xlow + xhat[0], xhigh + xhat[0], delta_x, ylow + xhat[1], yhigh + xhat[1],
                                  delta_y)
    finally:
        rs.close()
    pts = np.empty(3 * X.size)
    pts[0::3], pts[1::3], pts[2::3] = X, Y, Z
    return fz, xhat, Phat, cerr_fz, cerr_xhat, cerr_Phat, pts, nx, ny


def pycauchy_get_marginal_1D_pointwise_cpdf(h, marg_idx1, gridx_low, gridx_high, gridx_resolution, log_dir=None):
    """pycauchy.hpp:890-931: the grid as (x, y) pairs, flattened, and its size.
    The pdf object (and its rand() draws) is made on the first call."""
    X, Y = h.est.get_marginal_1D_pointwise_cpdf(int(marg_idx1), gridx_low, gridx_high, gridx_resolution)
    pts = np.empty(2 * X.size)
    pts[0::2], pts[1::2] = X, Y
    return pts, int(X.size)


def pycauchy_get_1D_pointwise_cpdf(h, gridx_low, gridx_high, gridx_resolution, log_dir=None):
    """pycauchy.hpp:934-944"""
    return pycauchy_get_marginal_1D_pointwise_cpdf(h, 0, gridx_low, gridx_high, gridx_resolution, log_dir)


def pycauchy_single_step_shutdown(h):
    """pycauchy.hpp:752"""
    h.est.close()


def pycauchy_set_tr_search_idxs_ordering(ordering):
    """pycauchy.hpp:994.  The ordering only says which axis of b the
    reference searches first and in which order it prunes the others
    (include/term_reduction.hpp:159-276): a candidate survives iff
    b_i - eps < b_j <= b_i + eps on every axis, which no order changes, and
    each survivor gets the same root whatever the order it is visited in.
    The reduction groups, and so every result, are therefore the same for
    every ordering (the reference's own runs under two orderings give the same
    doubles: tests/golden/tr_ordering_three_state.npz); this build's term
    reduction (grid buckets over all axes) has no ordering, and the call is
    accepted with no effect.  Returns 1 for more than 12 axes, as the
    reference does."""
    ordering = np.asarray(ordering).reshape(-1)
    if ordering.size > 12:
        return 1
    return 0


def pycauchy_get_reinitialization_statistics(h, z, xhat, Phat, H, gamma):
    """pycauchy.hpp:948-971: Speyer's restart statistics (A0 flattened, p0,
    b0) about the estimate (xhat, Phat) and the measurement z with model row
    H and scale gamma."""
    return pycauchy_speyers_window_init(xhat, Phat, H, gamma, z)


def pycauchy_speyers_window_init(x1_hat, Var, H, gamma, z):
    """pycauchy.hpp:973-992 (speyers_window_init, cauchy_util.hpp:23-113):
    (A0 flattened, p0, b0).  The caller's Var is not modified (the
    reference raises its diagonal in place when it is indefinite)."""
    from .windows import speyers_window_init
    A0, p0, b0 = speyers_window_init(x1_hat, Var, H, gamma, z)
    return A0.reshape(-1), p0, b0


# The reference keeps its C++ window manager in a global (pycauchy.hpp:8):
# one manager per process.
_SWM = None


def _init_window_manager(num_windows, num_sim_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma, dt, init_step,
                         win_var_boost, callback):
    global _SWM
    from .windows import CppSlidingWindowManager
    n = int(np.asarray(b0).size)
    if _SWM is not None:
        _SWM.close()
    f = lambda a: None if a is None or np.asarray(a).size == 0 else np.asarray(a, dtype=np.float64).reshape(1, -1)
    wvb = None if win_var_boost is None or np.asarray(win_var_boost).size == 0 else win_var_boost
    _SWM = CppSlidingWindowManager(num_windows, num_sim_steps, np.asarray(A0, dtype=np.float64).reshape(1, n, n),
                                   f(p0), f(b0), f(Phi), f(Gamma), f(B), f(beta), f(H), f(gamma), dt=float(dt),
                                   init_step=int(init_step), dyn_callback=callback, win_var_boost=wvb)


def pycauchy_initialize_lti_window_manager(num_windows, num_sim_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma,
                                           debug_print, log_seq, log_full, log_dir, dt, init_step, win_var_boost):
    """pycauchy.hpp:80-113: the C++ SlidingWindowManager over an LTI model
    (the logging options have no counterpart and are ignored).  The windows'
    root point and b_pert are drawn from the process's rand() state, once,
    as the reference's forked windows each draw the same values."""
    _init_window_manager(num_windows, num_sim_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma, dt, init_step,
                         win_var_boost, None)


def pycauchy_initialize_ltv_window_manager(num_windows, num_sim_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma,
                                           f_dyn_update_callback, debug_print, log_seq, log_full, log_dir, dt,
                                           init_step, win_var_boost):
    """pycauchy.hpp:116-149: as the LTI manager, with the dynamics callback
    (a raw C function pointer, int) that every window and the manager call on
    their own copy of the dynamics container."""
    _init_window_manager(num_windows, num_sim_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma, dt, init_step,
                         win_var_boost, int(f_dyn_update_callback))


def pycauchy_initialize_nonlin_window_manager(num_windows, num_sim_steps, x0, A0, p0, b0, beta, gamma,
                                              f_dyn_update_callback, f_nonlinear_msmt_model,
                                              f_extended_msmt_update_callback, cmcc, debug_print, log_seq, log_full,
                                              log_dir, dt, init_step, win_var_boost):
    """pycauchy.hpp:152-184: the C++ SlidingWindowManager in extended mode,
    x0 = x_bar_0 and the three callbacks raw C function pointers (ints).  The
    window estimators take no controls; the callbacks see cmcc controls."""
    global _SWM
    from .windows import CppSlidingWindowManager
    n = int(np.asarray(b0).size)
    if _SWM is not None:
        _SWM.close()
    f = lambda a: None if a is None or np.asarray(a).size == 0 else np.asarray(a, dtype=np.float64).reshape(1, -1)
    wvb = None if win_var_boost is None or np.asarray(win_var_boost).size == 0 else win_var_boost
    _SWM = CppSlidingWindowManager(num_windows, num_sim_steps, np.asarray(A0, dtype=np.float64).reshape(1, n, n),
                                   f(p0), f(b0), None, None, None, f(beta), None, f(gamma), dt=float(dt),
                                   init_step=int(init_step), dyn_callback=int(f_dyn_update_callback),
                                   win_var_boost=wvb, x0=f(x0), msmt_model_callback=int(f_nonlinear_msmt_model),
                                   extended_update_callback=int(f_extended_msmt_update_callback), cmcc=int(cmcc))


def pycauchy_step(msmts, controls):
    """pycauchy.hpp:187-221: one step of the window manager; returns
    (fz, xhat, Phat, cerr_fz, cerr_xhat, cerr_Phat, win_idx, err_code) of the
    window chosen at this step."""
    if _SWM is None:
        raise RuntimeError("pycauchy_step: no window manager (call pycauchy_initialize_*_window_manager first)")
    fz, x, P, cfz, cx, cP, wi, err = _SWM.step(msmts, controls)[0]
    return float(fz), x.copy(), P.reshape(-1).copy(), float(cfz), float(cx), float(cP), wi, err


def pycauchy_shutdown():
    """pycauchy.hpp:223-228"""
    global _SWM
    if _SWM is not None:
        _SWM.close()
        _SWM = None
