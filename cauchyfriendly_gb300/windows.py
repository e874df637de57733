"""Sliding-window MCE over the GPU step path.

Mirrors the reference's in-process window manager ``PySlidingWindowManager``
(scripts/swig/cauchy/cauchy_estimator.py:1092-1335): W estimators of W steps
each, started one step apart; every step the active windows take the new
measurements, the fullest window whose covariance is usable gives the
estimate, the empty window is restarted about it with Speyer's
initialisation (include/cauchy_util.hpp:23-113) and processes the last
measurement, and the full window is reset.

Batching: ``n_mgr`` independent window managers advance in lock-step, so the
windows in the same slot of every manager are always in the same phase; each
slot is one batched estimator handle (``BatchedCauchyEstimator``), i.e. one
GPU launch sequence per slot and measurement instead of one per window.

The estimator backend is pluggable: ``backend="gpu"`` (default) or an object
with the same batch interface (the tests drive an oracle-backed twin).
"""
from __future__ import annotations

import numpy as np

COV_UNSTABLE = 2   # ERROR_COVARIANCE_UNSTABLE_CURRENT_STEP_FINAL_MSMT bit
COV_DNE = 8        # ERROR_COVARIANCE_AT_CURRENT_STEP_DNE bit
COV_EIGENVALUE_TOLERANCE = -1e-5


def speyers_window_init(x1_hat, Var, H, gamma, z1, var_boost=None):
    """Restart statistics (A0, p0, b0) of a window about an estimate
    (include/cauchy_util.hpp:23-113): A0 rows are the eigenvectors of
    Var + Var H^T H Var / s with s = gamma^2 + (z1 - H x1)^2, b0 = x1 - Var H^T
    (z1 - H x1)/s and p0_i = lambda_i |v_i . H| gamma / (s + H Var H^T).
    Eigen-pairs come from numpy (the reference uses tred2/tqli); the initial
    characteristic function does not depend on their order or signs."""
    x1_hat = np.asarray(x1_hat, dtype=np.float64).reshape(-1)
    n = x1_hat.size
    Var = np.array(Var, dtype=np.float64).reshape(n, n)
    H = np.asarray(H, dtype=np.float64).reshape(n)
    if var_boost is not None:
        Var[np.diag_indices(n)] += np.asarray(var_boost, dtype=np.float64)
    ev = np.linalg.eigvalsh(0.5 * (Var + Var.T))
    if np.any(ev < COV_EIGENVALUE_TOLERANCE):
        Var[np.diag_indices(n)] += COV_EIGENVALUE_TOLERANCE - ev.min()
    VH = Var @ H
    Hx = float(H @ x1_hat)
    scale = gamma * gamma + (z1 - Hx) ** 2
    A0m = Var + np.outer(VH, VH) / scale
    lam, V = np.linalg.eigh(0.5 * (A0m + A0m.T))
    b0 = x1_hat - VH * ((z1 - Hx) / scale)
    hv = V.T @ H
    scale3 = (scale + float(H @ VH)) / gamma
    p0 = lam / scale3 * np.abs(hv)
    return V.T.copy(), p0, b0


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
        self.est.reset()

    def reinit(self, i, A0, p0, b0):
        self.est.reinitialize_start_statistics(A0, p0, b0, i)

    def set_master_step(self, ms):
        self.est.set_master_step(ms)

    def post_mu_terms(self):
        return self.est.post_mu_terms()

    def close(self):
        self.est.close()


class SlidingWindowManager:
    """n_mgr independent sliding-window estimators of W windows each.

    A0, p0, b0: (n_mgr, d, d), (n_mgr, d), (n_mgr, d) initial statistics.
    step(msmts (n_mgr, p), Phi (n_mgr, d, d), Gamma (n_mgr, d, pncc),
         beta (n_mgr, pncc), H (n_mgr, p, d), gamma (n_mgr, p))
    returns the best windows' (xhat, Phat, window index, error code) per manager.
    """

    def __init__(self, num_windows, A0, p0, b0, d, pncc, p, cmcc=0, slot_factory=None):
        assert num_windows >= 2
        self.W = int(num_windows)
        self.d, self.pncc, self.p, self.cmcc = int(d), int(pncc), int(p), int(cmcc)
        A0 = np.asarray(A0, dtype=np.float64)
        self.n_mgr = A0.shape[0]
        make = slot_factory or (lambda *a: _GpuSlot(*a))
        self.slots = [make(A0, np.asarray(p0, dtype=np.float64), np.asarray(b0, dtype=np.float64), self.W, self.d,
                           self.cmcc, self.pncc, self.p) for _ in range(self.W)]
        self.win_counts = np.zeros(self.W, dtype=np.int64)
        self.step_idx = 0
        # per slot, the measurement models of its last step (for restarts)
        self._last = [None] * self.W
        self.post_mu_terms = 0
        self.history = []

    def _step_slot(self, w, msmts, Phi, Gamma, beta, H, gamma):
        errs = None
        for j in range(self.p):
            errs = self.slots[w].step(msmts[:, j], Phi, Gamma, beta, H[:, j, :], gamma[:, j])
        self._last[w] = (msmts, H, gamma)
        return errs

    def _best_windows(self):
        """_best_window_est (cauchy_estimator.py:1181-1219) per manager: the
        fullest window whose covariance is usable; ties go to the higher slot."""
        best = np.zeros(self.n_mgr, dtype=np.int64)
        if self.step_idx == 0:
            return best
        for m in range(self.n_mgr):
            cands = []
            for w in range(self.W):
                if self.win_counts[w] > 0:
                    err = self.slots[w].errors(m)
                    if not ((err & COV_UNSTABLE) or (err & COV_DNE)):
                        cands.append((w, self.win_counts[w]))
            if not cands:
                raise RuntimeError("no window is available without an error code (manager %d)" % m)
            best[m] = list(reversed(sorted(cands, key=lambda x: x[1])))[0][0]
        return best

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
        best = self._best_windows()
        out = []
        for m in range(self.n_mgr):
            mo = self.slots[best[m]].moments(m)
            out.append((mo["mean"].real.copy(), mo["cov"].real.copy(), int(best[m]),
                        self.slots[best[m]].errors(m)))
        if self.step_idx > 0:
            # restart the empty window about each manager's best window with the
            # last measurement of this step (reset_about_estimator, msmt_idx = p-1)
            j = self.p - 1
            slot = self.slots[min_idx]
            for m in range(self.n_mgr):
                xh, Ph = out[m][0], out[m][1]
                A0, p0, b0 = speyers_window_init(xh, Ph, H[m, j], gamma[m, j], msmts[m, j])
                slot.reinit(m, A0, p0, b0)
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
        return out

    def total_post_mu_terms(self):
        """Terms present after every MU of every window since construction."""
        return self.post_mu_terms + sum(s.post_mu_terms() for s in self.slots)

    def close(self):
        for s in self.slots:
            s.close()
