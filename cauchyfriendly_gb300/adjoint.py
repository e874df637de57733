"""Gradients of the accumulated log-likelihood of an MCE run.

``AdjointRun`` records one estimator's run through the GPU step path
(mce_adjoint_* in libmce_gb300.so) and returns the gradient of
sum_k w_k Re(fz_k) with respect to (beta, gamma, p0, Phi, Gamma, H), holding
the enumerated cell structure fixed; fz_k = 1/(2 pi G_SCALE_FACTOR_k)
(include/cauchy_estimator.hpp:340-357) is the normaliser of update k.
Because every g-table is rescaled by 1/(2 pi Re fz_k) after update k and the
rest of the computation is linear in the tables, sum_k log Re fz_k over a run
is log Re of the unscaled last fz, so its gradient is one seed,
w_K = 1/Re fz_K, on the last update (``loglik_weights``).

``MCELogLikelihood`` exposes it as a torch.autograd.Function over float64
tensors: forward runs the estimator and returns sum_k log fz_k, backward the
hand-written adjoint.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

PARAM_NAMES = ("beta", "gamma", "p0", "Phi", "Gamma", "H")


def loglik_weights(fz):
    """Seeds of sum_k log Re fz_k: 1/Re fz on the last update, 0 elsewhere."""
    w = np.zeros(len(fz))
    w[-1] = 1.0 / fz[-1]
    return w


class AdjointRun:
    """One estimator (LTI model, no controls) of d states, pncc process-noise
    columns and p measurements per step, run for `steps` steps from
    (A0, p0, b0).  root_point / b_pert are the constants the reference draws
    with rand() (see oracle.draw_reference_constants / mce_draw_reference_constants)."""

    def __init__(self, d, pncc, p, steps, A0, p0, b0, root_point, b_pert):
        self._L = _lib.load()
        self.d, self.pncc, self.p, self.steps = int(d), int(pncc), int(p), int(steps)
        f = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))
        self.A0, self.b0 = f(A0), f(b0)
        self.root_point, self.b_pert = f(root_point), f(b_pert)
        st = ctypes.c_int(0)
        self._h = self._L.mce_adjoint_create(self.d, self.pncc, self.p, self.steps, _lib.dp(self.A0),
                                             _lib.dp(f(p0)), _lib.dp(self.b0), _lib.dp(self.root_point),
                                             _lib.dp(self.b_pert), ctypes.byref(st))
        if not self._h:
            raise _lib.MceError("mce_adjoint_create failed (%d): %s" % (st.value, _lib.last_error()))
        self.fz = None

    def forward(self, msmts, Phi, Gamma, beta, H, gamma, p0=None):
        """Runs and records every update; returns Re fz of each.  p0 (or None:
        the constructor's) is the initial scale vector of this run.  Phi is
        (d, d), or (steps, d, d) for a time-varying model (the gradient's Phi
        is then that of a perturbation common to every step's Phi)."""
        f = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))
        if p0 is not None:
            self._recreate(f(p0))
        ltv = np.asarray(Phi).ndim == 3
        self._model = [f(x) for x in (msmts, Phi, Gamma, beta, H, gamma)]
        fz = np.zeros(self.steps * self.p)
        fn = self._L.mce_adjoint_forward_ltv if ltv else self._L.mce_adjoint_forward
        _lib.check(fn(self._h, *[_lib.dp(x) for x in self._model], _lib.dp(fz)), "mce_adjoint_forward")
        self.fz = fz
        return fz

    def _recreate(self, p0):
        self._L.mce_adjoint_destroy(self._h)
        st = ctypes.c_int(0)
        self._h = self._L.mce_adjoint_create(self.d, self.pncc, self.p, self.steps, _lib.dp(self.A0), _lib.dp(p0),
                                             _lib.dp(self.b0), _lib.dp(self.root_point), _lib.dp(self.b_pert),
                                             ctypes.byref(st))
        if not self._h:
            raise _lib.MceError("mce_adjoint_create failed (%d): %s" % (st.value, _lib.last_error()))

    def backward(self, w):
        """Gradient of sum_k w_k Re fz_k as a dict of arrays shaped like the
        parameters (beta (pncc,), gamma (p,), p0 (d,), Phi (d, d),
        Gamma (d, pncc), H (p, d))."""
        w = np.ascontiguousarray(np.asarray(w, dtype=np.float64).reshape(-1))
        n = self._L.mce_adjoint_num_params(self._h)
        g = np.zeros(n)
        _lib.check(self._L.mce_adjoint_backward(self._h, _lib.dp(w), _lib.dp(g)), "mce_adjoint_backward")
        d, pncc, p = self.d, self.pncc, self.p
        shapes = ((pncc,), (p,), (d,), (d, d), (d, pncc), (p, d))
        out, k = {}, 0
        for name, sh in zip(PARAM_NAMES, shapes):
            sz = int(np.prod(sh))
            out[name] = g[k:k + sz].reshape(sh)
            k += sz
        return out

    def check(self):
        """(largest relative difference of the recorded g-tables, of the
        recorded Re fz) from the GPU run."""
        a, b = ctypes.c_double(), ctypes.c_double()
        _lib.check(self._L.mce_adjoint_check(self._h, ctypes.byref(a), ctypes.byref(b)), "mce_adjoint_check")
        return a.value, b.value

    def timing(self):
        """Wall ms so far: step path, forward tape, table reverse, record chain."""
        t = np.zeros(4)
        _lib.check(self._L.mce_adjoint_timing(self._h, _lib.dp(t)), "mce_adjoint_timing")
        return t

    def close(self):
        if getattr(self, "_h", None):
            self._L.mce_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AdjointBatch:
    """Adjoint runs of d states, pncc process-noise columns and p
    measurements per step, stepped together: run r has steps[r] steps from
    (A0[r], p0[r], b0[r]) with its own rand() constants (root_point[r],
    b_pert[r]); one LTI model for all, or (forward with per-run Phi
    sequences) a time-varying model per run.  first_sub = p - 1 makes every
    run a window restarted with the last measurement of its first step.  One
    batched handle steps every run (mce_adjoint_batch_*), and the runs'
    records and reverses spread over the host's cores; each run's gradient is
    the one an AdjointRun of its own gives."""

    def __init__(self, d, pncc, p, steps, A0, p0, b0, root_point, b_pert, first_sub=0):
        self._L = _lib.load()
        self.d, self.pncc, self.p = int(d), int(pncc), int(p)
        self.first_sub = int(first_sub)
        self.steps = np.ascontiguousarray(np.asarray(steps, dtype=np.int32).reshape(-1))
        self.n = len(self.steps)
        f = lambda a, *sh: np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(self.n, *sh))
        A0, p0, b0, rp = f(A0, d, d), f(p0, d), f(b0, d), f(root_point, d)
        bp = np.ascontiguousarray(np.asarray(b_pert, dtype=np.float64).reshape(self.n, -1))
        st = ctypes.c_int(0)
        self._h = self._L.mce_adjoint_batch_create(
            self.n, self.d, self.pncc, self.p, self.steps.ctypes.data_as(_lib._ip), _lib.dp(A0), _lib.dp(p0),
            _lib.dp(b0), _lib.dp(rp), _lib.dp(bp), bp.shape[1], ctypes.byref(st))
        if not self._h:
            raise _lib.MceError("mce_adjoint_batch_create failed (%d): %s" % (st.value, _lib.last_error()))
        self.max_steps = int(self.steps.max())
        if self.first_sub:
            _lib.check(self._L.mce_adjoint_batch_set_first_sub(self._h, self.first_sub),
                       "mce_adjoint_batch_set_first_sub")

    def updates(self, r):
        """Updates of run r: steps[r] * p less the first measurement index."""
        return int(self.steps[r]) * self.p - self.first_sub

    def forward(self, msmts, Phi, Gamma, beta, H, gamma):
        """msmts: run r's measurements (steps[r]*p values) for every r.  Phi:
        one (d, d) matrix for every run, or for a time-varying model run r's
        Phi of each of its steps (a list of (steps[r], d, d) arrays).
        Returns Re fz of every update of every run (a list of arrays)."""
        stride = self.max_steps * self.p
        M = np.zeros((self.n, stride))
        for r, m in enumerate(msmts):
            m = np.asarray(m, dtype=np.float64).reshape(-1)
            M[r, :len(m)] = m
        f = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))
        fz = np.zeros((self.n, stride))
        ltv = isinstance(Phi, (list, tuple)) or np.asarray(Phi).ndim == 3
        if ltv:
            # each run its own Phi sequence, Gamma and H (one of each given
            # for all runs is repeated)
            d, n = self.d, self.n
            Ph = np.zeros((n, self.max_steps, d, d))
            for r, q in enumerate(Phi):
                q = np.asarray(q, dtype=np.float64).reshape(-1, d, d)
                Ph[r, :len(q)] = q
                Ph[r, len(q):] = q[-1]
            per = lambda x, sz: (np.stack([np.asarray(v, dtype=np.float64).reshape(-1) for v in x])
                                 if isinstance(x, (list, tuple)) else
                                 np.tile(np.asarray(x, dtype=np.float64).reshape(1, -1), (n, 1)))
            Gamma = per(Gamma, d * self.pncc)
            H = per(H, self.p * d)
            fn, Phi = self._L.mce_adjoint_batch_forward_ltv, Ph
        else:
            fn = self._L.mce_adjoint_batch_forward
        _lib.check(fn(self._h, _lib.dp(M), self.max_steps, *[_lib.dp(f(x)) for x in (Phi, Gamma, beta, H, gamma)],
                      _lib.dp(fz)), "mce_adjoint_batch_forward")
        return [fz[r, :self.updates(r)].copy() for r in range(self.n)]

    def backward(self, ws):
        """ws: run r's seeds (steps[r]*p values) for every r.  Returns a list
        of gradient dicts shaped as AdjointRun.backward's."""
        stride = self.max_steps * self.p
        Wt = np.zeros((self.n, stride))
        for r, w in enumerate(ws):
            w = np.asarray(w, dtype=np.float64).reshape(-1)
            Wt[r, :len(w)] = w
        N = self._L.mce_adjoint_batch_num_params(self._h)
        g = np.zeros((self.n, N))
        _lib.check(self._L.mce_adjoint_batch_backward(self._h, _lib.dp(Wt), self.max_steps, _lib.dp(g)),
                   "mce_adjoint_batch_backward")
        d, pncc, p = self.d, self.pncc, self.p
        shapes = ((pncc,), (p,), (d,), (d, d), (d, pncc), (p, d))
        outs = []
        for r in range(self.n):
            out, k = {}, 0
            for name, sh in zip(PARAM_NAMES, shapes):
                sz = int(np.prod(sh))
                out[name] = g[r, k:k + sz].reshape(sh)
                k += sz
            outs.append(out)
        return outs

    def check(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        _lib.check(self._L.mce_adjoint_batch_check(self._h, ctypes.byref(a), ctypes.byref(b)),
                   "mce_adjoint_batch_check")
        return a.value, b.value

    def timing(self):
        """Wall ms: batched step path, forward records, reverse; and the
        runs' summed record-chain ms."""
        t = np.zeros(4)
        _lib.check(self._L.mce_adjoint_batch_timing(self._h, _lib.dp(t)), "mce_adjoint_batch_timing")
        return t

    def close(self):
        if getattr(self, "_h", None):
            self._L.mce_adjoint_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _make_function():
    import torch

    class MCELogLikelihood(torch.autograd.Function):
        """sum_k log fz_k of one estimator's run as a differentiable function
        of (beta, gamma, p0, Phi, Gamma, H), float64 tensors; `run` is an
        AdjointRun and `msmts` the measurement history (steps, p).  The
        backward pass is the library's adjoint (mce_adjoint_backward)."""

        @staticmethod
        def forward(ctx, beta, gamma, p0, Phi, Gamma, H, run, msmts):
            np_ = lambda t: t.detach().cpu().numpy().astype(np.float64)
            fz = run.forward(msmts, np_(Phi), np_(Gamma), np_(beta), np_(H), np_(gamma), p0=np_(p0))
            ctx.run = run
            ctx.w = loglik_weights(fz)
            ctx.like = [beta, gamma, p0, Phi, Gamma, H]
            return torch.tensor(float(np.sum(np.log(fz))), dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            g = ctx.run.backward(ctx.w)
            outs = []
            for name, like in zip(PARAM_NAMES, ctx.like):
                outs.append(gout * torch.as_tensor(g[name].reshape(like.shape), dtype=like.dtype,
                                                   device=like.device))
            return (*outs, None, None)

    return MCELogLikelihood


def windowed_log_likelihood(prob, W, root_point, b_pert, p0=None, beta=None, gamma=None, Phi=None, Gamma=None,
                            H=None, starts=None, best=None, with_grad=True):
    """Sliding-window log-likelihood sum_k log fz_k of a one-measurement LTI
    problem, fz_k the normaliser of the window chosen at step k
    (PySlidingWindowManager's best window, cauchy_estimator.py:1181-1216),
    and its gradient with respect to (beta, gamma, p0, Phi, Gamma, H) with the
    window-boundary checkpoints held fixed: every window life is recomputed
    from its start statistics (the initial ones for the first life of window
    0, Speyer's restart about the best window for the others) as one run of
    an AdjointBatch, and gets the seeds +1/Re fz on each update at which it is the
    chosen window and -1/Re fz on the update before it (log fz_u =
    log Re U_u - log Re U_(u-1), U the unscaled normaliser).  p0 enters only
    the first life.

    prob: a problem dict (workloads); root_point (W, d) / b_pert (W, stride)
    the windows' constants.  The parameters default to prob's.  starts/best
    (from a first call, returned in the result) hold the checkpoints fixed for
    finite differences.  Returns a dict: loglik, grad (dict), starts, best."""
    from .windows import SlidingWindowManager
    d, pncc, p = prob["d"], prob["pncc"], prob["p"]
    if p != 1:
        raise ValueError("windowed_log_likelihood supports one measurement per step")
    P = {"beta": prob["beta"] if beta is None else beta, "gamma": prob["gamma"] if gamma is None else gamma,
         "p0": prob["p0"] if p0 is None else p0, "Phi": prob["Phi"] if Phi is None else Phi,
         "Gamma": prob["Gamma"] if Gamma is None else Gamma, "H": prob["H"] if H is None else H}
    P = {k: np.asarray(v, dtype=np.float64) for k, v in P.items()}
    steps = prob["msmts"].shape[0]
    rp = np.asarray(root_point, dtype=np.float64)
    bp = np.asarray(b_pert, dtype=np.float64)
    if starts is None:
        mgr = SlidingWindowManager(W, prob["A0"][None], P["p0"][None], prob["b0"][None], d, pncc, p,
                                   root_point=rp[:, None, :], b_pert=bp[:, None, :])
        best = []
        for k in range(steps):
            out = mgr.step(prob["msmts"][k][None], P["Phi"][None], P["Gamma"].reshape(1, d, pncc),
                           P["beta"][None], P["H"].reshape(1, p, d), P["gamma"][None])
            best.append(out[0][2])
        starts = [{"slot": s["slot"], "step": s["step"], "A0": np.asarray(s["A0"])[0], "p0": np.asarray(s["p0"])[0],
                   "b0": np.asarray(s["b0"])[0]} for s in mgr.starts]
        mgr.close()
    # every window life is one run of a batch: one batched step per update,
    # the records and reverses spread over the host's cores
    lens = [min(W, steps - st["step"]) for st in starts]
    batch = AdjointBatch(d, pncc, p, lens, [st["A0"] for st in starts],
                         [P["p0"] if li == 0 else st["p0"] for li, st in enumerate(starts)],
                         [st["b0"] for st in starts], [rp[st["slot"]] for st in starts],
                         [bp[st["slot"]] for st in starts])
    try:
        fzs = batch.forward([prob["msmts"][st["step"]:st["step"] + n].reshape(-1) for st, n in zip(starts, lens)],
                            P["Phi"], P["Gamma"], P["beta"], P["H"], P["gamma"])
        Ls, ws = [], []
        for st, n, fz in zip(starts, lens, fzs):
            s0 = st["step"]
            w = np.zeros(n)
            Ll = 0.0
            for u in range(n):
                if best[s0 + u] == st["slot"]:
                    Ll += float(np.log(fz[u]))
                    w[u] += 1.0 / fz[u]
                    if u >= 1:
                        w[u - 1] -= 1.0 / fz[u - 1]
            Ls.append(Ll)
            ws.append(w)
        gs = batch.backward(ws) if with_grad else [None] * len(starts)
        timing = batch.timing()
    finally:
        batch.close()
    results = [(Ll, g if np.any(w != 0) else None, None) for Ll, g, w in zip(Ls, gs, ws)]
    L = 0.0
    grad = {k: np.zeros_like(v) for k, v in P.items()}
    for li, (Ll, g, _) in enumerate(results):
        L += Ll
        if g is not None:
            for k in grad:
                if k == "p0" and li > 0:
                    continue
                grad[k] += g[k].reshape(grad[k].shape)
    return {"loglik": L, "grad": grad, "starts": starts, "best": best, "timing_ms": timing}


def windowed_log_likelihood_batch(probs, W, root_point, b_pert, beta, gamma, p0, steps=None, checkpoints=None,
                                  with_grad=True, no_window="raise"):
    """Sliding-window log-likelihood of n estimators that share the scales
    (beta, gamma, p0) and have each their own model (probs[i]: Phi (d, d) or
    per step (steps, d, d), Gamma, H), measurements (steps, p) and step count
    steps[i] (at most its measurement count): the sum over estimators, over
    their steps k < steps[i] and the p updates of step k, of log fz of the
    update in the window chosen at step k (PySlidingWindowManager's best
    window), and its gradient with respect to beta, gamma and p0 with the
    window-boundary checkpoints held fixed.  One window manager runs all n
    estimators (to their longest step count); every window life of every
    estimator is recomputed from its checkpoint in two AdjointBatch sets, the
    first lives (from the initial statistics, where p0 enters) and the
    restarted ones (which begin with the last measurement of their first
    step).  The seeds are windowed_log_likelihood's, per update.

    checkpoints: (starts, best) from a first call, to hold them fixed.
    no_window: the manager's rule for a step where every window has an error
    code (SlidingWindowManager: "raise" as the reference, or "fullest").
    Returns a dict: loglik, grad (beta, gamma, p0), checkpoints, timing_ms,
    no_window_steps."""
    from .windows import SlidingWindowManager
    n = len(probs)
    d, pncc, p = probs[0]["d"], probs[0]["pncc"], probs[0]["p"]
    beta = np.asarray(beta, dtype=np.float64).reshape(pncc)
    gamma = np.asarray(gamma, dtype=np.float64).reshape(p)
    p0 = np.asarray(p0, dtype=np.float64).reshape(d)
    steps = [int(q["msmts"].shape[0]) for q in probs] if steps is None else [int(k) for k in steps]
    K = max(steps)
    rp = np.asarray(root_point, dtype=np.float64)
    bp = np.asarray(b_pert, dtype=np.float64)
    phi = lambda q, k: np.asarray(q["Phi"] if np.asarray(q["Phi"]).ndim == 2 else q["Phi"][k], dtype=np.float64)
    if checkpoints is None:
        mgr = SlidingWindowManager(W, np.stack([q["A0"] for q in probs]), np.tile(p0, (n, 1)),
                                   np.stack([q["b0"] for q in probs]), d, pncc, p,
                                   root_point=np.repeat(rp[:, None, :], n, axis=1),
                                   b_pert=np.repeat(bp[:, None, :], n, axis=1), no_window=no_window)
        best = []
        try:
            for k in range(K):
                out = mgr.step(np.stack([q["msmts"][k] for q in probs]), np.stack([phi(q, k) for q in probs]),
                               np.stack([np.asarray(q["Gamma"]).reshape(d, pncc) for q in probs]),
                               np.tile(beta, (n, 1)), np.stack([np.asarray(q["H"]).reshape(p, d) for q in probs]),
                               np.tile(gamma, (n, 1)))
                best.append([o[2] for o in out])
            starts = [{"slot": s_["slot"], "step": s_["step"], "A0": np.asarray(s_["A0"]), "p0": np.asarray(s_["p0"]),
                       "b0": np.asarray(s_["b0"])} for s_ in mgr.starts]
            no_window_steps = mgr.no_window_steps
        finally:
            mgr.close()
    else:
        starts, best = checkpoints
        no_window_steps = 0
    L = 0.0
    grad = {"beta": np.zeros(pncc), "gamma": np.zeros(p), "p0": np.zeros(d)}
    timing = np.zeros(4)
    for first in (True, False):
        # the runs: (estimator, life) with the life's first step before the
        # estimator's step count
        runs = []
        for li, st in enumerate(starts):
            if (li == 0) != first:
                continue
            for i in range(n):
                if st["step"] < steps[i]:
                    runs.append((i, li, min(W, steps[i] - st["step"])))
        if not runs:
            continue
        fs = 0 if first else p - 1
        A0 = [starts[li]["A0"][i] for i, li, _ in runs]
        P0 = [p0 if first else starts[li]["p0"][i] for i, li, _ in runs]
        B0 = [starts[li]["b0"][i] for i, li, _ in runs]
        batch = AdjointBatch(d, pncc, p, [m for _, _, m in runs], A0, P0, B0,
                             [rp[starts[li]["slot"]] for _, li, _ in runs],
                             [bp[starts[li]["slot"]] for _, li, _ in runs], first_sub=fs)
        try:
            ms, Ph, Gs, Hs = [], [], [], []
            for i, li, m in runs:
                s0 = starts[li]["step"]
                z = np.asarray(probs[i]["msmts"][s0:s0 + m], dtype=np.float64).reshape(-1)[fs:]
                ms.append(z)
                Ph.append(np.stack([phi(probs[i], s0 + k) for k in range(m)]))
                Gs.append(probs[i]["Gamma"])
                Hs.append(probs[i]["H"])
            fzs = batch.forward(ms, Ph, Gs, beta, Hs, gamma)
            ws = []
            for (i, li, m), fz in zip(runs, fzs):
                s0, slot = starts[li]["step"], starts[li]["slot"]
                w = np.zeros(len(fz))
                for u in range(len(fz)):
                    k = s0 + (u + fs) // p
                    if best[k][i] == slot:
                        L += float(np.log(fz[u]))
                        w[u] += 1.0 / fz[u]
                        if u >= 1:
                            w[u - 1] -= 1.0 / fz[u - 1]
                ws.append(w)
            if with_grad:
                for g in batch.backward(ws):
                    grad["beta"] += g["beta"]
                    grad["gamma"] += g["gamma"]
                    if first:
                        grad["p0"] += g["p0"]
            timing += batch.timing()
        finally:
            batch.close()
    return {"loglik": L, "grad": grad, "checkpoints": (starts, best), "timing_ms": timing,
            "no_window_steps": no_window_steps}


_FN = None


def mce_log_likelihood(beta, gamma, p0, Phi, Gamma, H, run, msmts):
    """sum_k log fz_k of `run` (an AdjointRun) over `msmts`, differentiable in
    the six parameter tensors (torch.autograd.Function)."""
    global _FN
    if _FN is None:
        _FN = _make_function()
    return _FN.apply(beta, gamma, p0, Phi, Gamma, H, run, msmts)
