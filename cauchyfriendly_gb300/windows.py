"""Sliding-window MCE over the GPU step path.

Two managers, as the reference has two:

* ``SlidingWindowManager`` mirrors the reference's in-process window manager
  ``PySlidingWindowManager`` (scripts/swig/cauchy/cauchy_estimator.py:1092-1335):
  W estimators of W steps each, started one step apart; every step the active
  windows take the new measurements, the fullest window whose covariance is
  usable gives the estimate, the empty window is restarted about it with
  Speyer's initialisation (include/cauchy_util.hpp:23-113) and processes the
  last measurement, and the full window is reset.
* ``CppSlidingWindowManager`` is the C++ front end's SlidingWindowManager
  (include/cauchy_windows.hpp:729-1165), run by the library's C++
  (``mce_swm_*``); pycauchy's window-manager entry points use it.

Batching: ``n_mgr`` independent window managers advance in lock-step, so the
windows in the same slot of every manager are always in the same phase; each
slot is one batched estimator handle, i.e. one GPU launch sequence per slot
and measurement instead of one per window.

Speyer's restart statistics come from the library's C++
(``mce_speyers_window_init``), which uses the reference's eigen-solver so the
restarted window's hyperplanes come in the reference's order and signs.
"""
from __future__ import annotations

import ctypes

import numpy as np

COV_UNSTABLE = 2   # ERROR_COVARIANCE_UNSTABLE_CURRENT_STEP_FINAL_MSMT bit
COV_DNE = 8        # ERROR_COVARIANCE_AT_CURRENT_STEP_DNE bit
COV_EIGENVALUE_TOLERANCE = -1e-5


def sym_eig(A):
    """Eigen-decomposition of a symmetric matrix as the reference's sym_eig
    computes it (include/eig_solve.hpp:404: Householder tridiagonalisation and
    implicit-shift QL, in the library's C++): (eigenvalues, eigenvectors as
    columns), in the solver's order and signs."""
    from . import _lib
    A = np.ascontiguousarray(np.asarray(A, dtype=np.float64))
    n = A.shape[0]
    w, V = np.zeros(n), np.zeros((n, n))
    _lib.check(_lib.load().mce_sym_eig(n, _lib.dp(A), _lib.dp(w), _lib.dp(V)), "mce_sym_eig")
    return w, V


def speyers_window_init(x1_hat, Var, H, gamma, z1, var_boost=None):
    """Restart statistics (A0, p0, b0) of a window about an estimate
    (include/cauchy_util.hpp:23-113, computed by the library's C++
    mce_speyers_window_init): A0 rows are the eigenvectors of
    Var + Var H^T H Var / s with s = gamma^2 + (z1 - H x1)^2, b0 = x1 - Var H^T
    (z1 - H x1)/s and p0_i = lambda_i |v_i . H| gamma / (s + H Var H^T).  A
    covariance with an eigenvalue below -1e-5 has its diagonal raised first.
    The eigen-pairs come in the reference solver's order and signs, which fix
    the restarted window's term order and cell keys."""
    from . import _lib
    x1_hat = np.ascontiguousarray(np.asarray(x1_hat, dtype=np.float64).reshape(-1))
    n = x1_hat.size
    Var = np.ascontiguousarray(np.asarray(Var, dtype=np.float64).reshape(n, n))
    H = np.ascontiguousarray(np.asarray(H, dtype=np.float64).reshape(n))
    boost = None if var_boost is None else np.ascontiguousarray(np.asarray(var_boost, dtype=np.float64).reshape(n))
    A0, p0, b0 = np.zeros((n, n)), np.zeros(n), np.zeros(n)
    _lib.check(_lib.load().mce_speyers_window_init(n, _lib.dp(x1_hat), _lib.dp(Var), _lib.dp(H), float(gamma),
                                                   float(z1), _lib.dp(boost), _lib.dp(A0), _lib.dp(p0), _lib.dp(b0)),
               "mce_speyers_window_init")
    return A0, p0, b0


class _GpuSlot:
    """One window slot: a batched GPU estimator over n_mgr managers."""

    def __init__(self, A0, p0, b0, steps, d, cmcc, pncc, p, root_point=None, b_pert=None):
        from .estimator import BatchedCauchyEstimator
        n = A0.shape[0]
        self.est = BatchedCauchyEstimator(A0, p0, b0, np.full(n, steps, np.int32), d, cmcc, pncc, p, root_point,
                                          b_pert)

    def step(self, z, Phi, Gamma, beta, H, gamma):
        return self.est.step(z, Phi, Gamma, beta, H, gamma, shared_model=False)

    def moments(self, i):
        return self.est.moments(i)

    def errors(self, i):
        return self.est.errors(i)

    def num_terms(self, i):
        return self.est.num_terms(i)

    def reset(self):
        # a window restarts from one term: buffers of a gigabyte or more go back to the device
        self.est.reset()
        self.est.trim_memory(1 << 30)

    def reinit(self, i, A0, p0, b0):
        self.est.reinitialize_start_statistics(A0, p0, b0, i)

    def set_master_step(self, ms):
        self.est.set_master_step(ms)

    def post_mu_terms(self):
        return self.est.post_mu_terms()

    def close(self):
        self.est.close()


class SlidingWindowManager:
    """n_mgr independent copies of the reference's PySlidingWindowManager
    (scripts/swig/cauchy/cauchy_estimator.py:1092-1335), W windows each.

    A0, p0, b0: (n_mgr, d, d), (n_mgr, d), (n_mgr, d) initial statistics.
    root_point / b_pert: None (drawn with rand(), window after window, as the
    reference's windows draw them when they are made), or per window slot
    (W, n_mgr, d) / (W, n_mgr, stride).
    step(msmts (n_mgr, p), Phi (n_mgr, d, d), Gamma (n_mgr, d, pncc),
         beta (n_mgr, pncc), H (n_mgr, p, d), gamma (n_mgr, p))
    returns each manager's (xhat, Phat, window index, error code) of the best
    window, as PySlidingWindowManager.step / _best_window_est choose it;
    ``last`` holds the step's fz, cerr_fz, cerr_x, cerr_P and the weighted
    average estimate (_weighted_average_win_est) per manager.
    """

    def __init__(self, num_windows, A0, p0, b0, d, pncc, p, cmcc=0, slot_factory=None, root_point=None,
                 b_pert=None, no_window="raise"):
        assert num_windows >= 2
        # a step where every window of a manager has an error code: "raise"
        # as the reference does (it exits), or "fullest": take the fullest
        # window anyway and count the step in no_window_steps
        assert no_window in ("raise", "fullest")
        self.no_window = no_window
        self.no_window_steps = 0
        self.W = int(num_windows)
        self.d, self.pncc, self.p, self.cmcc = int(d), int(pncc), int(p), int(cmcc)
        A0 = np.asarray(A0, dtype=np.float64)
        self.n_mgr = A0.shape[0]
        p0 = np.asarray(p0, dtype=np.float64)
        b0 = np.asarray(b0, dtype=np.float64)
        if slot_factory is None:
            self.slots = []
            for w in range(self.W):
                rp = None if root_point is None else np.asarray(root_point)[w]
                bp = None if b_pert is None else np.asarray(b_pert)[w]
                self.slots.append(_GpuSlot(A0, p0, b0, self.W, self.d, self.cmcc, self.pncc, self.p,
                                           root_point=rp, b_pert=bp))
        else:
            self.slots = [slot_factory(A0, p0, b0, self.W, self.d, self.cmcc, self.pncc, self.p)
                          for _ in range(self.W)]
        self.win_counts = np.zeros(self.W, dtype=np.int64)
        self.step_idx = 0
        self.post_mu_terms = 0
        self.history = []
        self.last = None
        # window-boundary checkpoints: every window life's start (slot, step,
        # and each manager's A0, p0, b0), the restarts being Speyer's statistics
        self.starts = [{"slot": 0, "step": 0, "A0": A0.copy(), "p0": p0.copy(), "b0": b0.copy()}]

    def _step_slot(self, w, msmts, Phi, Gamma, beta, H, gamma):
        errs = None
        for j in range(self.p):
            errs = self.slots[w].step(msmts[:, j], Phi, Gamma, beta, H[:, j, :], gamma[:, j])
        return errs

    def _best_windows(self):
        """_best_window_est (cauchy_estimator.py:1181-1216) per manager: the
        fullest window whose covariance is usable (error bits 2 and 8 clear on
        the step's last measurement; ties to the later window), and which
        windows are usable."""
        best = np.zeros(self.n_mgr, dtype=np.int64)
        okay = np.zeros((self.n_mgr, self.W), dtype=bool)
        for m in range(self.n_mgr):
            cands = []
            for w in range(self.W):
                if self.win_counts[w] > 0:
                    err = self.slots[w].errors(m)
                    if not ((err & COV_UNSTABLE) or (err & COV_DNE)):
                        cands.append((w, self.win_counts[w]))
                        okay[m, w] = True
            if self.step_idx == 0:
                okay[m, 0] = True
                continue
            forced = not cands
            if forced:
                if self.no_window == "raise":
                    raise RuntimeError("no window is available without an error code (manager %d)" % m)
                cands = [(w, self.win_counts[w]) for w in range(self.W) if self.win_counts[w] > 0]
                self.no_window_steps += 1
            best[m] = list(reversed(sorted(cands, key=lambda x: x[1])))[0][0]
            if forced:
                okay[m, best[m]] = True  # the weighted average is then that window's estimate
        return best, okay

    def _weighted_average(self, m, okay, moms):
        """_weighted_average_win_est (cauchy_estimator.py:1218-1259): the usable
        windows' estimates weighted by their step counts."""
        n = self.d
        x, P, norm = np.zeros(n), np.zeros((n, n)), 0.0
        for w in range(self.W):
            if self.win_counts[w] > 0 and okay[m, w]:
                f = self.win_counts[w] / self.W
                norm += f
                x += moms[w]["mean"].real * f
                P += moms[w]["cov"].real * f
        return x / norm, P / norm

    def step(self, msmts, Phi, Gamma, beta, H, gamma):
        msmts = np.asarray(msmts, dtype=np.float64).reshape(self.n_mgr, self.p)
        H = np.asarray(H, dtype=np.float64).reshape(self.n_mgr, self.p, self.d)
        gamma = np.asarray(gamma, dtype=np.float64).reshape(self.n_mgr, self.p)
        if self.step_idx == 0:
            self._step_slot(0, msmts, Phi, Gamma, beta, H, gamma)
            self.win_counts[0] += 1
            min_idx = max_idx = None
        else:
            max_idx = int(np.argmax(self.win_counts))
            min_idx = int(np.argmin(self.win_counts))
            for w in range(self.W):
                if self.win_counts[w] > 0:
                    self._step_slot(w, msmts, Phi, Gamma, beta, H, gamma)
                    self.win_counts[w] += 1
        best, okay = self._best_windows()
        out, last = [], []
        for m in range(self.n_mgr):
            moms = {w: self.slots[w].moments(m) for w in range(self.W) if self.win_counts[w] > 0}
            mo = moms[int(best[m])]
            out.append((mo["mean"].real.copy(), mo["cov"].real.copy(), int(best[m]), self.slots[best[m]].errors(m)))
            wx, wP = self._weighted_average(m, okay, moms)
            last.append({"fz": float(mo["fz"].real), "cerr_fz": float(mo["fz"].imag),
                         "cerr_x": float(np.max(np.abs(mo["mean"].imag))),
                         "cerr_P": float(np.max(np.abs(mo["cov"].imag))), "wavg_xhat": wx, "wavg_Phat": wP})
        if self.step_idx > 0:
            # restart the empty window about each manager's best window with the
            # last measurement of this step (reset_about_estimator, msmt_idx = p-1)
            j = self.p - 1
            slot = self.slots[min_idx]
            st = {"slot": min_idx, "step": self.step_idx, "A0": np.zeros((self.n_mgr, self.d, self.d)),
                  "p0": np.zeros((self.n_mgr, self.d)), "b0": np.zeros((self.n_mgr, self.d))}
            for m in range(self.n_mgr):
                xh, Ph = out[m][0], out[m][1]
                A0, p0, b0 = speyers_window_init(xh, Ph, H[m, j], gamma[m, j], msmts[m, j])
                slot.reinit(m, A0, p0, b0)
                st["A0"][m], st["p0"][m], st["b0"][m] = A0, p0, b0
            self.starts.append(st)
            self.post_mu_terms += slot.post_mu_terms()  # a reset clears the slot's count
            slot.reset()  # pycauchy_single_step_reset: new start statistics, then reset
            slot.step(msmts[:, j], Phi, Gamma, beta, H[:, j, :], gamma[:, j])
            slot.set_master_step(self.p)
            self.win_counts[min_idx] += 1
            if self.win_counts[max_idx] == self.W:
                self.post_mu_terms += self.slots[max_idx].post_mu_terms()
                self.slots[max_idx].reset()
                self.win_counts[max_idx] = 0
        self.step_idx += 1
        self.history.append(out)
        self.last = last
        return out

    def total_post_mu_terms(self):
        """Terms present after every MU of every window since construction."""
        return self.post_mu_terms + sum(s.post_mu_terms() for s in self.slots)

    def close(self):
        for s in self.slots:
            s.close()


class CppSlidingWindowManager:
    """The C++ front end's SlidingWindowManager (include/cauchy_windows.hpp:
    729-1165) for n_mgr managers stepped together, run by the library's C++
    (mce_swm_*): the window schedule, best-window choice (fullest window whose
    fz, mean and covariance exist), Speyer restarts and, for LTV models, the
    dynamics callback are those of the reference's manager and its window
    processes.

    A0, p0, b0 and the model arrays are stacked per manager (A0 (n_mgr, d, d),
    Phi (n_mgr, d, d), Gamma (n_mgr, d, pncc), B (n_mgr, d, cmcc), beta
    (n_mgr, pncc), H (n_mgr, p, d), gamma (n_mgr, p)).  dyn_callback is a raw C
    function pointer (int) taking the reference's CauchyDynamicsUpdateContainer,
    or None (LTI).  With msmt_model_callback and extended_update_callback
    (raw C function pointers too) and x0 (n_mgr, d) the manager runs in
    extended (nonlinear) mode; Phi, Gamma, B and H may then be None (the
    callbacks set them) and cmcc gives the controls the callbacks see.  step(msmts (n_mgr, p), controls) returns, per manager, the
    pycauchy_step tuple (fz, xhat, Phat, cerr_fz, cerr_xhat, cerr_Phat,
    win_idx, err_code)."""

    def __init__(self, num_windows, num_sim_steps, A0, p0, b0, Phi, Gamma, B, beta, H, gamma, dt=0.0, init_step=0,
                 dyn_callback=None, win_var_boost=None, root_point=None, b_pert=None, x0=None,
                 msmt_model_callback=None, extended_update_callback=None, cmcc=None):
        from . import _lib
        self._L = _lib.load()
        A0 = np.ascontiguousarray(np.asarray(A0, dtype=np.float64))
        self.n_mgr, self.d = A0.shape[0], A0.shape[1]
        f = lambda a: None if a is None or np.asarray(a).size == 0 else np.ascontiguousarray(
            np.asarray(a, dtype=np.float64).reshape(self.n_mgr, -1))
        self._keep = [f(x) for x in (A0, p0, b0, Phi, Gamma, B, beta, H, gamma)]
        self.pncc = 0 if self._keep[6] is None else self._keep[6].shape[1]
        self.p = self._keep[8].shape[1]
        self.cmcc = 0 if self._keep[5] is None else self._keep[5].shape[1] // self.d
        if cmcc is not None:
            self.cmcc = int(cmcc)
        boost = None if win_var_boost is None or np.asarray(win_var_boost).size == 0 else \
            np.ascontiguousarray(np.asarray(win_var_boost, dtype=np.float64).reshape(self.d))
        rp = None if root_point is None else np.ascontiguousarray(np.asarray(root_point, dtype=np.float64))
        bp = None if b_pert is None else np.ascontiguousarray(np.asarray(b_pert, dtype=np.float64))
        stride = 0 if bp is None else bp.reshape(self.n_mgr, -1).shape[1]
        self._boost = boost
        st = ctypes.c_int(0)
        cb = lambda c: None if c is None else int(c)
        if msmt_model_callback is not None:
            # extended (nonlinear) mode: x0 is x_bar at the first step
            self._x0 = f(x0)
            k = self._keep
            self._h = self._L.mce_swm_create_nonlin(
                self.n_mgr, int(num_windows), int(num_sim_steps), self.d, self.cmcc, self.pncc, self.p,
                _lib.dp(self._x0), _lib.dp(k[0]), _lib.dp(k[1]), _lib.dp(k[2]), _lib.dp(k[6]), _lib.dp(k[8]),
                float(dt), int(init_step), cb(dyn_callback), cb(msmt_model_callback), cb(extended_update_callback),
                _lib.dp(boost), _lib.dp(rp), _lib.dp(bp), stride, ctypes.byref(st))
        else:
            self._h = self._L.mce_swm_create(self.n_mgr, int(num_windows), int(num_sim_steps), self.d, self.cmcc,
                                             self.pncc, self.p, *[_lib.dp(x) for x in self._keep], float(dt),
                                             int(init_step), cb(dyn_callback), _lib.dp(boost), _lib.dp(rp),
                                             _lib.dp(bp), stride, ctypes.byref(st))
        if not self._h:
            raise _lib.MceError("mce_swm_create failed (%d): %s" % (st.value, _lib.last_error()))
        self.W = int(num_windows)

    def step(self, msmts, controls=None):
        from . import _lib
        nm, d = self.n_mgr, self.d
        z = np.ascontiguousarray(np.asarray(msmts, dtype=np.float64).reshape(nm, self.p))
        u = None
        if self.cmcc and controls is not None and np.asarray(controls).size:
            u = np.ascontiguousarray(np.asarray(controls, dtype=np.float64).reshape(nm, self.cmcc))
        fz, cfz, cx, cP = np.zeros(nm), np.zeros(nm), np.zeros(nm), np.zeros(nm)
        x, P = np.zeros((nm, d)), np.zeros((nm, d, d))
        wi, err = np.zeros(nm, dtype=np.int32), np.zeros(nm, dtype=np.int32)
        ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        _lib.check(self._L.mce_swm_step(self._h, _lib.dp(z), _lib.dp(u), _lib.dp(fz), _lib.dp(x), _lib.dp(P),
                                        _lib.dp(cfz), _lib.dp(cx), _lib.dp(cP), ip(wi), ip(err)), "mce_swm_step")
        return [(fz[m], x[m], P[m], cfz[m], cx[m], cP[m], int(wi[m]), int(err[m])) for m in range(nm)]

    def window_count(self, j):
        return int(self._L.mce_swm_window_count(self._h, int(j)))

    def num_terms(self, j, m=0):
        return int(self._L.mce_num_terms(self._L.mce_swm_window(self._h, int(j)), int(m)))

    def total_post_mu_terms(self):
        return int(self._L.mce_swm_post_mu_terms(self._h))

    def close(self):
        if getattr(self, "_h", None):
            self._L.mce_swm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
