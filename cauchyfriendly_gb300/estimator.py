"""Host-side mirror of the reference's C++ estimator interface.

``CauchyEstimator`` follows ``struct CauchyEstimator``
(include/cauchy_estimator.hpp:47-1432): same constructor arguments, ``step``
semantics (one scalar measurement, returns the numeric-moment error bitmask)
and public fields (``fz``, ``conditional_mean``, ``conditional_variance``,
``Nt``, ``master_step``, ``terms_per_shape``, ``G_SCALE_FACTOR``).
``BatchedCauchyEstimator`` steps many independent estimators in lock-step on
one GPU.  All compute runs in libmce_gb300.so.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_longlong)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _p(a, kind=_dp):
    return None if a is None else a.ctypes.data_as(kind)


def max_shape(steps, d, pncc):
    """Largest hyperplane count a term can reach (cauchy_estimator.hpp:96)."""
    return (steps - 1) * pncc + d if d > 1 else d + pncc


class BatchedCauchyEstimator:
    """n_est independent estimators stepped together.

    A0 (n_est,d,d), p0 (n_est,d), b0 (n_est,d), steps (n_est,); root_point
    (n_est,d) and b_pert (n_est, stride) default to the reference's libc
    rand() draws."""

    def __init__(self, A0, p0, b0, steps, d, cmcc, pncc, p, root_point=None, b_pert=None):
        self._lib = _lib.load()
        self.d, self.cmcc, self.pncc, self.p = int(d), int(cmcc), int(pncc), int(p)
        self.steps = np.ascontiguousarray(steps, dtype=np.int32).reshape(-1)
        self.n_est = int(self.steps.size)
        A0, p0, b0 = _f64(A0), _f64(p0), _f64(b0)
        rp, bp = _f64(root_point), _f64(b_pert)
        stride = 0 if bp is None else int(bp.reshape(self.n_est, -1).shape[1])
        st = ctypes.c_int(0)
        self._h = self._lib.mce_batch_create(self.n_est, self.d, self.cmcc, self.pncc, self.p,
                                             _p(self.steps, _ip), _p(A0), _p(p0), _p(b0), _p(rp), _p(bp), stride,
                                             ctypes.byref(st))
        if not self._h:
            raise _lib.MceError("mce_batch_create failed (%d): %s" % (st.value, _lib.last_error()))
        self.max_shape = max_shape(int(self.steps.max()), self.d, self.pncc)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mce_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- stepping ------------------------------------------------------------
    def step(self, msmts, Phi, Gamma, beta, H, gamma, B=None, u=None, shared_model=None):
        """One measurement update for every estimator.  With shared_model the
        model arrays hold one copy; otherwise they are stacked per estimator."""
        msmts = _f64(msmts).reshape(self.n_est)
        Phi, Gamma, beta, H, gamma, B, u = map(_f64, (Phi, Gamma, beta, H, gamma, B, u))
        if shared_model is None:
            shared_model = Phi.ndim == 2
        err = np.zeros(self.n_est, dtype=np.int32)
        rc = self._lib.mce_batch_step(self._h, _p(msmts), _p(Phi), _p(Gamma), _p(beta), _p(H), _p(gamma), _p(B),
                                      _p(u), 1 if shared_model else 0, _p(err, _ip))
        _lib.check(rc, "mce_batch_step")
        return err

    def run(self, msmts, Phi, Gamma, beta, H, gamma, B=None, u=None, shared_model=False, outputs=True):
        """Whole measurement histories msmts (n_est, max_steps, p)."""
        msmts = _f64(msmts)
        max_steps = msmts.shape[1]
        Phi, Gamma, beta, H, gamma, B, u = map(_f64, (Phi, Gamma, beta, H, gamma, B, u))
        nu = int(self.p * self.steps.max())
        out = None
        if outputs:
            d = self.d
            out = {"fz": np.zeros((self.n_est, nu, 2)), "mean": np.zeros((self.n_est, nu, 2 * d)),
                   "cov": np.zeros((self.n_est, nu, 2 * d * d)), "err": np.zeros((self.n_est, nu), np.int32),
                   "nt": np.zeros((self.n_est, nu), np.int64)}
        rc = self._lib.mce_batch_run(self._h, _p(msmts), max_steps, _p(Phi), _p(Gamma), _p(beta), _p(H), _p(gamma),
                                     _p(B), _p(u), 1 if shared_model else 0,
                                     _p(out["fz"]) if out else None, _p(out["mean"]) if out else None,
                                     _p(out["cov"]) if out else None, _p(out["err"], _ip) if out else None,
                                     _p(out["nt"], _lp) if out else None)
        _lib.check(rc, "mce_batch_run")
        return out

    # -- read-out ------------------------------------------------------------
    def moments(self, e=0):
        d = self.d
        fz, mean, cov = np.zeros(2), np.zeros(2 * d), np.zeros(2 * d * d)
        rfz, rmean, rcov, gs = np.zeros(2), np.zeros(2 * d), np.zeros(2 * d * d), np.zeros(1)
        _lib.check(self._lib.mce_get_moments(self._h, e, _p(fz), _p(mean), _p(cov)), "mce_get_moments")
        _lib.check(self._lib.mce_get_raw_moments(self._h, e, _p(rfz), _p(rmean), _p(rcov), _p(gs)),
                   "mce_get_raw_moments")
        c = lambda a: a[0::2] + 1j * a[1::2]
        return {"fz": complex(*fz), "mean": c(mean), "cov": c(cov).reshape(d, d), "raw_fz": complex(*rfz),
                "raw_mean": c(rmean), "raw_cov": c(rcov).reshape(d, d), "gscale": float(gs[0])}

    def errors(self, e=0):
        return int(self._lib.mce_get_errors(self._h, e))

    def num_terms(self, e=0):
        return int(self._lib.mce_num_terms(self._h, e))

    def terms_per_shape(self, e=0):
        out = np.zeros(self.max_shape + 1, dtype=np.int32)
        _lib.check(self._lib.mce_terms_per_shape(self._h, e, _p(out, _ip), out.size), "mce_terms_per_shape")
        return out

    def post_mu_terms(self):
        return int(self._lib.mce_post_mu_terms(self._h))

    def master_step(self):
        return int(self._lib.mce_master_step(self._h))

    def device_errors(self):
        return int(self._lib.mce_device_errors(self._h))

    def last_step_ms(self):
        return float(self._lib.mce_last_step_ms(self._h))

    def dump_terms(self, e=0, max_shape=None):
        """Terms of estimator e in (shape, index) order with their g-tables."""
        ms = max_shape or self.max_shape
        nt = self.num_terms(e)
        tc = int(self._lib.mce_total_cells(self._h, e))
        d = self.d
        shape = np.zeros(nt, np.int32)
        A = np.zeros(nt * ms * d)
        p = np.zeros(nt * ms)
        b = np.zeros(nt * d)
        cells = np.zeros(nt, np.int32)
        keys = np.zeros(max(tc, 1), np.int32)
        g = np.zeros(2 * max(tc, 1))
        _lib.check(self._lib.mce_dump_terms(self._h, e, ms, _p(shape, _ip), _p(A), _p(p), _p(b), _p(cells, _ip),
                                            _p(keys, _ip), _p(g)), "mce_dump_terms")
        return {"shape": shape, "A": A.reshape(nt, ms, d), "p": p.reshape(nt, ms), "b": b.reshape(nt, d),
                "cells": cells, "keys": keys[:tc], "g": (g[0::2] + 1j * g[1::2])[:tc]}

    def reset(self):
        _lib.check(self._lib.mce_reset(self._h), "mce_reset")

    def trim_memory(self, min_bytes=0):
        """Frees the device buffers that grow with the term count (between a
        reset and the next step) when they hold at least min_bytes; returns
        the bytes released."""
        return _lib.check(self._lib.mce_trim_memory(self._h, int(min_bytes)), "mce_trim_memory")

    def reinitialize_start_statistics(self, A0, p0, b0, e=0):
        A0, p0, b0 = _f64(A0), _f64(p0), _f64(b0)
        _lib.check(self._lib.mce_reinitialize_start_statistics(self._h, e, _p(A0), _p(p0), _p(b0)),
                   "mce_reinitialize_start_statistics")

    def set_master_step(self, ms):
        _lib.check(self._lib.mce_set_master_step(self._h, int(ms)), "mce_set_master_step")

    def set_print_basic_info(self, on, e=-1):
        """The constructor's print_basic_info for estimator e (every one for
        e < 0): after each update that rebuilds the tables the reported fz,
        moments and G_SCALE_FACTOR are the post-reduction ones of
        compute_moments(false) (include/cauchy_estimator.hpp:524-602)."""
        _lib.check(self._lib.mce_set_print_basic_info(self._h, int(e), int(bool(on))), "mce_set_print_basic_info")

    def set_win_num(self, w):
        _lib.check(self._lib.mce_set_window_number(self._h, int(w)), "mce_set_window_number")

    # -- extended (nonlinear) mode helpers, cauchy_estimator.hpp:1312-1394 ---
    def shift_cf_by_bias(self, bias, e=0):
        b = _f64(bias).reshape(self.d)
        _lib.check(self._lib.mce_shift_cf_by_bias(self._h, int(e), _p(b)), "mce_shift_cf_by_bias")

    def deterministic_time_prop(self, Phi, B=None, u=None, e=0):
        Phi = _f64(Phi).reshape(self.d, self.d)
        B = None if B is None else _f64(B)
        u = None if u is None else _f64(u)
        _lib.check(self._lib.mce_deterministic_time_prop(self._h, int(e), _p(Phi), _p(B), _p(u)),
                   "mce_deterministic_time_prop")

    def finalize_extended_moments(self, x_bar, e=0):
        """Shifts the terms by -Re(mean), sets mean += x_bar; returns the new x_bar = Re(mean)."""
        x = _f64(x_bar).reshape(self.d).copy()
        _lib.check(self._lib.mce_finalize_extended_moments(self._h, int(e), _p(x)), "mce_finalize_extended_moments")
        return x

    def cpdf_2d_grid(self, e, marg_idx1, marg_idx2, gridx, gridy, bar_nu, reset_cache=True):
        """Marginal 2-D conditional pdf of estimator e on gridx = (low, high,
        resolution) by gridy (CauchyCPDFGridDispatcher2D,
        include/cpdf_ndim.hpp:1774-1919); returns flat (X, Y, Z), x fastest."""
        nu = _f64(bar_nu).reshape(self.d)
        g = [float(v) for v in gridx] + [float(v) for v in gridy]
        n = self._lib.mce_cpdf_2d_grid(self._h, int(e), int(marg_idx1), int(marg_idx2), _p(nu), *g,
                                       int(bool(reset_cache)), 0, None, None, None)
        _lib.check(n, "mce_cpdf_2d_grid")
        X, Y, Z = np.zeros(n), np.zeros(n), np.zeros(n)
        n = self._lib.mce_cpdf_2d_grid(self._h, int(e), int(marg_idx1), int(marg_idx2), _p(nu), *g,
                                       int(bool(reset_cache)), n, _p(X), _p(Y), _p(Z))
        _lib.check(n, "mce_cpdf_2d_grid")
        return X, Y, Z

    def cpdf_nd(self, x, e=0):
        """The conditional pdf of estimator e at the points x ([n][d] or [d]):
        PointWiseNDimCauchyCPDF::evaluate_cpdf (include/cpdf_ndim.hpp:677-904)
        for every point at once; complex values (the imaginary parts are
        rounding)."""
        X = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1, self.d))
        out = np.zeros(2 * X.shape[0])
        _lib.check(self._lib.mce_cpdf_nd(self._h, int(e), _p(X), X.shape[0], _p(out)), "mce_cpdf_nd")
        return out[0::2] + 1j * out[1::2]

    def cpdf_marginal(self, x, marg_idxs, nu_bar=None, e=0):
        """The marginal pdf of the states marg_idxs (ascending, fewer than d)
        of estimator e at the points x ([n][len(marg_idxs)]):
        PointWiseNDimCauchyCPDF::evaluate_marginal_cpdf
        (include/cpdf_ndim.hpp:918-1230); complex values.  nu_bar
        (d - len(marg_idxs) values) stands for the reference's rand() draws;
        by default a fixed point off the hyperplanes (the value does not
        depend on it beyond rounding)."""
        idx = np.ascontiguousarray(np.asarray(marg_idxs, dtype=np.int32).reshape(-1))
        nz = self.d - len(idx)
        if nu_bar is None:
            nu_bar = np.cos(1.0 + 2.3 * np.arange(max(nz, 0)))
        nu = np.ascontiguousarray(np.asarray(nu_bar, dtype=np.float64).reshape(-1))
        X = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1, len(idx)))
        out = np.zeros(2 * X.shape[0])
        _lib.check(self._lib.mce_cpdf_marginal(self._h, int(e), idx.ctypes.data_as(_lib._ip), len(idx), _p(nu), _p(X),
                                               X.shape[0], _p(out)), "mce_cpdf_marginal")
        return out[0::2] + 1j * out[1::2]

    def cpdf_1d_grid(self, e, marg_idx, gridx_low, gridx_high, gridx_resolution, bar_nu):
        """Marginal 1-D conditional pdf of estimator e on the grid
        gridx_low..gridx_high step gridx_resolution
        (CauchyCPDFGridDispatcher1D, include/cpdf_ndim.hpp:2017-2139);
        returns (X, Y)."""
        nu = _f64(bar_nu).reshape(self.d)
        n = self._lib.mce_cpdf_1d_grid(self._h, int(e), int(marg_idx), _p(nu), float(gridx_low),
                                       float(gridx_high), float(gridx_resolution), 0, None, None)
        _lib.check(n, "mce_cpdf_1d_grid")
        X, Y = np.zeros(n), np.zeros(n)
        n = self._lib.mce_cpdf_1d_grid(self._h, int(e), int(marg_idx), _p(nu), float(gridx_low),
                                       float(gridx_high), float(gridx_resolution), n, _p(X), _p(Y))
        _lib.check(n, "mce_cpdf_1d_grid")
        return X, Y


def autotune_configure(enabled=True):
    """Drops every tuned block size and turns the process-wide block-size
    autotuner of the thread-per-item kernels on or off (off: fixed sizes)."""
    _lib.check(_lib.load().mce_autotune_configure(1 if enabled else 0), "mce_autotune_configure")


def autotune_table():
    """The settled autotuner keys: dicts of kernel, d, hyperplane capacity
    (mc), log2 of the launch's item count, the chosen block size and the
    fastest sample's device ms."""
    lib = _lib.load()
    n = lib.mce_autotune_table(None, None, 0)
    _lib.check(n, "mce_autotune_table")
    if n == 0:
        return []
    rows = (ctypes.c_int * (5 * n))()
    ms = (ctypes.c_float * n)()
    got = min(n, lib.mce_autotune_table(rows, ms, n))
    return [dict(kernel=lib.mce_autotune_kernel_name(rows[5 * i]).decode(), d=rows[5 * i + 1], mc=rows[5 * i + 2],
                 log2_items=rows[5 * i + 3], block=rows[5 * i + 4], ms=float(ms[i])) for i in range(got)]


def draw_bar_nu(d, seed=-1):
    """The d draws of PointWiseNDimCauchyCPDF's constructor
    (include/cpdf_ndim.hpp:385-389) from libc rand(); seed >= 0 seeds it first."""
    out = np.zeros(int(d))
    _lib.check(_lib.load().mce_draw_bar_nu(int(seed), int(d), _p(out)), "mce_draw_bar_nu")
    return out



def draw_rel_bar_nu(d, seed=-1):
    """The d draws of get_marg2d_relative_and_transformed_cpdf
    (include/cauchy_prediction.hpp:697-698): 2 u - 1 with u from libc rand()
    as random_uniform_open; seed >= 0 seeds it first."""
    return draw_bar_nu(d, seed) - 1.0


class RelativeSystem2D:
    """The relative-then-transformed 2-D system of two estimators: rel =
    secondary - primary projected by the 2 x d matrix Trel, one cached 2-D
    term per (primary term, secondary term) pair, on the GPU
    (get_marg2d_relative_and_transformed_cpdf,
    include/cauchy_prediction.hpp:653-971, single-thread term order).

    primary / secondary: (BatchedCauchyEstimator, index) pairs or
    CauchyEstimator objects.  bar_nu_full defaults to the reference's own
    rand() draw.  After construction: moments (fz, mean, cov, complex, when
    get_relative_moments), pairs, terms (kept) and approxed_out; grid()
    evaluates the pdf."""

    def __init__(self, primary, secondary, Trel, full_solve=False, get_relative_moments=True,
                 with_term_approx=False, term_approx_eps=1e-8, bar_nu_full=None):
        (pe, pi), (se, si) = (self._split(primary), self._split(secondary))
        self._lib = _lib.load()
        d = pe.d
        self.full_solve = bool(full_solve)
        T = _f64(Trel).reshape(2, d)
        nu = draw_rel_bar_nu(d) if bar_nu_full is None else _f64(bar_nu_full).reshape(d)
        self.bar_nu_full = nu.copy()
        mom = np.zeros(14) if get_relative_moments else None
        counts = np.zeros(2, dtype=np.int64)
        st = ctypes.c_int(0)
        self._h = self._lib.mce_rel2d_create(pe._h, int(pi), se._h, int(si), _p(T), _p(nu), int(self.full_solve),
                                             int(bool(with_term_approx)), float(term_approx_eps), _p(mom),
                                             counts.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                                             ctypes.byref(st))
        if not self._h:
            _lib.check(st.value if st.value < 0 else -1, "mce_rel2d_create")
        self.pairs, self.approxed_out = int(counts[0]), int(counts[1])
        self.terms = self.pairs - self.approxed_out
        self.moments = None
        if mom is not None:
            c = mom[0::2] + 1j * mom[1::2]
            self.moments = {"fz": c[0], "mean": c[1:3], "cov": c[3:7].reshape(2, 2)}
        # norm factors the reference passes to the grid: the reported fz of each
        self.norm_factor_prim = float(pe.moments(pi)["fz"].real)
        self.norm_factor_sec = float(se.moments(si)["fz"].real)

    @staticmethod
    def _split(x):
        if isinstance(x, tuple):
            return x[0], int(x[1])
        return x, 0

    def grid(self, xlow, xhigh, delta_x, ylow, yhigh, delta_y, norm_factor_prim=None, norm_factor_sec=None):
        """grid_eval_marg2d_relative_and_transformed_cpdf
        (include/cauchy_prediction.hpp:1091-1186): flat (X, Y, Z), x outermost,
        and the point counts nx, ny."""
        nfp = self.norm_factor_prim if norm_factor_prim is None else float(norm_factor_prim)
        nfs = self.norm_factor_sec if norm_factor_sec is None else float(norm_factor_sec)
        g = [float(v) for v in (xlow, xhigh, delta_x, ylow, yhigh, delta_y)]
        n = self._lib.mce_rel2d_grid(self._h, *g, nfp, nfs, 0, None, None, None)
        _lib.check(n, "mce_rel2d_grid")
        X, Y, Z = np.zeros(n), np.zeros(n), np.zeros(n)
        n = self._lib.mce_rel2d_grid(self._h, *g, nfp, nfs, n, _p(X), _p(Y), _p(Z))
        _lib.check(n, "mce_rel2d_grid")
        ny = int(np.ceil((g[4] - g[3]) / g[5] + 1))
        return X, Y, Z, n // ny, ny

    def device_ms(self):
        """Device time (ms) of the pair kernel and of the kept-pair compaction
        with the moment sums of the construction, and of the last grid."""
        return {k: float(self._lib.mce_rel2d_device_ms(self._h, i)) for i, k in enumerate(("pairs", "moments", "grid"))}

    def launch_count(self):
        """Kernels launched by the construction and the grids so far."""
        return int(self._lib.mce_rel2d_launch_count(self._h))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mce_rel2d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

class CauchyEstimator(BatchedCauchyEstimator):
    """CauchyEstimator(A0, p0, b0, steps, d, cmcc, pncc, p, print_basic_info)
    (include/cauchy_estimator.hpp:87): a batch of one."""

    def __init__(self, A0, p0, b0, steps, d, cmcc, pncc, p, print_basic_info=False, root_point=None,
                 b_pert=None):
        d = int(d)
        A0 = _f64(A0).reshape(1, d, d)
        p0 = _f64(p0).reshape(1, d)
        b0 = _f64(b0).reshape(1, d)
        rp = None if root_point is None else _f64(root_point).reshape(1, d)
        bp = None if b_pert is None else _f64(b_pert).reshape(1, -1)
        super().__init__(A0, p0, b0, [int(steps)], d, cmcc, pncc, p, rp, bp)
        self.print_basic_info = bool(print_basic_info)
        if self.print_basic_info:
            self.set_print_basic_info(True)

    def step(self, msmt, Phi, Gamma, beta, H, gamma, B=None, u=None):
        """CauchyEstimator::step (include/cauchy_estimator.hpp:1211): returns
        numeric_moment_errors."""
        d = self.d
        Phi = _f64(Phi).reshape(d, d)
        Gamma = None if Gamma is None else _f64(Gamma).reshape(d, -1)
        beta = None if beta is None else _f64(beta).reshape(-1)
        H = _f64(H).reshape(d)
        B = None if B is None else _f64(B).reshape(d, -1)
        u = None if u is None else _f64(u).reshape(-1)
        rc = self._lib.mce_step(self._h, float(msmt), _p(Phi), _p(Gamma), _p(beta), _p(H), float(gamma), _p(B), _p(u))
        return _lib.check(rc, "mce_step")

    @property
    def fz(self):
        return self.moments()["fz"]

    @property
    def conditional_mean(self):
        return self.moments()["mean"]

    @property
    def conditional_variance(self):
        return self.moments()["cov"]

    @property
    def G_SCALE_FACTOR(self):
        return self.moments()["gscale"]

    @property
    def Nt(self):
        return self.num_terms()

    @property
    def numeric_moment_errors(self):
        return self.errors()

    def get_marginal_1D_pointwise_cpdf(self, marg_idx, gridx_low, gridx_high, gridx_resolution, log_dir=None):
        """CauchyEstimator.get_marginal_1D_pointwise_cpdf
        (scripts/swig/cauchy/cauchy_estimator.py:1003-1031): (X, Y) on the
        grid.  The pdf's random direction bar_nu is drawn from libc rand() on
        the first call, as the reference's pdf object is."""
        if getattr(self, "_bar_nu", None) is None:
            self._bar_nu = draw_bar_nu(self.d)
        return self.cpdf_1d_grid(0, marg_idx, gridx_low, gridx_high, gridx_resolution, self._bar_nu)

    def get_marginal_2D_pointwise_cpdf(self, marg_idx1, marg_idx2, gridx_low, gridx_high, gridx_resolution,
                                       gridy_low, gridy_high, gridy_resolution, log_dir=None, reset_cache=True):
        """CauchyEstimator.get_marginal_2D_pointwise_cpdf
        (scripts/swig/cauchy/cauchy_estimator.py:954-993): (X, Y, Z) as
        (num_gridy, num_gridx) arrays."""
        if getattr(self, "_bar_nu", None) is None:
            self._bar_nu = draw_bar_nu(self.d)
        X, Y, Z = self.cpdf_2d_grid(0, marg_idx1, marg_idx2, (gridx_low, gridx_high, gridx_resolution),
                                    (gridy_low, gridy_high, gridy_resolution), self._bar_nu, reset_cache)
        nx = int(np.sum(Y == Y[0]))
        return X.reshape(-1, nx), Y.reshape(-1, nx), Z.reshape(-1, nx)

    def get_2D_pointwise_cpdf(self, gridx_low, gridx_high, gridx_resolution, gridy_low, gridy_high, gridy_resolution,
                              log_dir=None, reset_cache=True):
        """The 2-state case of get_marginal_2D_pointwise_cpdf."""
        if self.d != 2:
            raise ValueError("get_2D_pointwise_cpdf needs a 2-state estimator")
        return self.get_marginal_2D_pointwise_cpdf(0, 1, gridx_low, gridx_high, gridx_resolution, gridy_low,
                                                   gridy_high, gridy_resolution, log_dir, reset_cache)

    def get_1D_pointwise_cpdf(self, gridx_low, gridx_high, gridx_resolution, log_dir=None):
        """The 1-state case of get_marginal_1D_pointwise_cpdf (cauchy_estimator.py:1033-1043)."""
        if self.d != 1:
            raise ValueError("get_1D_pointwise_cpdf needs a 1-state estimator")
        return self.get_marginal_1D_pointwise_cpdf(0, gridx_low, gridx_high, gridx_resolution, log_dir)
