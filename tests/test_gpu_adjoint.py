"""The adjoint of the accumulated log-likelihood (cauchyfriendly_gb300.adjoint,
mce_adjoint_* in the library) on the GPU:

* the recorded tape describes the GPU run: every kept g-table and every Re fz
  recomputed from it agree with the run's within 1e-12;
* the gradient of sum_k log fz_k with respect to (beta, gamma, p0, Phi,
  Gamma, H) agrees with central finite differences of the REFERENCE's own
  log-likelihood (tests/golden/adj_*.npz, made by the unmodified reference)
  and with central finite differences of the GPU forward run;
* the torch.autograd.Function returns the same value and gradient.

Finite differences carry their own error (the fixtures keep a second set at a
quarter of the step to show it), so the gradients are compared within 1e-4
relative per entry, with a floor of 1e-6 of the largest entry.
"""
import os

import numpy as np
import pytest

from tests import golden_cases as G

pytestmark = pytest.mark.gpu

NAMES = ("beta", "gamma", "p0", "Phi", "Gamma", "H")


def _need_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _load(name):
    return np.load(os.path.join(G.GOLDEN, name + ".npz"))


def _run(z):
    from cauchyfriendly_gb300.adjoint import AdjointRun
    return AdjointRun(int(z["d"]), int(z["pncc"]), int(z["p"]), int(z["steps"]), z["A0"], z["p0"], z["b0"],
                      z["root_point"], z["b_pert"])


def _flat(g):
    return np.concatenate([np.asarray(g[n]).reshape(-1) for n in NAMES])


def _params(z):
    return {n: np.asarray(z[n], dtype=np.float64) for n in NAMES}


def _loglik(run, z, P):
    fz = run.forward(z["msmts"].reshape(-1), P["Phi"], P["Gamma"], P["beta"], P["H"], P["gamma"], p0=P["p0"])
    return float(np.sum(np.log(fz))), fz


def _close(a, b, rtol=1e-4, floor=1e-6):
    a = np.asarray(a); b = np.asarray(b)
    tol = rtol * np.abs(b) + floor * np.max(np.abs(b))
    return np.all(np.abs(a - b) <= tol), np.max(np.abs(a - b) / (np.abs(b) + floor * np.max(np.abs(b))))


@pytest.mark.parametrize("name", ["adj_four_state", "adj_five_state_two_msmt"])
def test_adjoint_matches_reference_finite_differences(name):
    _need_gpu()
    from cauchyfriendly_gb300.adjoint import loglik_weights
    z = _load(name)
    run = _run(z)
    P = _params(z)
    L, fz = _loglik(run, z, P)
    # the GPU run's log-likelihood is the reference's
    assert abs(L - float(z["loglik"])) <= 1e-9 * abs(float(z["loglik"])), (L, float(z["loglik"]))
    te, fe = run.check()
    assert te <= 1e-12 and fe <= 1e-12, (te, fe)
    g = _flat(run.backward(loglik_weights(fz)))
    ok, err = _close(g, z["fd_grad"])
    assert ok, (err, g, z["fd_grad"])
    run.close()


def test_adjoint_matches_gpu_finite_differences():
    """Central differences of the GPU forward run itself, on a second seed
    of the four-state problem and a seed other than the loglik one."""
    _need_gpu()
    import oracle
    from cauchyfriendly_gb300 import workloads as W
    from cauchyfriendly_gb300.adjoint import loglik_weights
    prob = W.four_state_lti(seed=9, steps=5)
    rp, bp = oracle.draw_reference_constants(77, 4, oracle.max_shape_of(prob))
    z = dict(prob)
    z["root_point"], z["b_pert"] = rp, bp
    run = _run(z)
    P = _params(z)
    L, fz = _loglik(run, z, P)
    g = run.backward(loglik_weights(fz))
    fd = {}
    for n in NAMES:
        a = P[n]
        fd[n] = np.zeros_like(a)
        for idx in np.ndindex(a.shape):
            h = 1e-6 * max(abs(a[idx]), 1e-3)
            Pp = {k: v.copy() for k, v in P.items()}
            Pm = {k: v.copy() for k, v in P.items()}
            Pp[n][idx] += h
            Pm[n][idx] -= h
            fd[n][idx] = (_loglik(run, z, Pp)[0] - _loglik(run, z, Pm)[0]) / (2 * h)
    ok, err = _close(_flat(g), _flat(fd))
    assert ok, err
    run.close()


def test_torch_function_gives_the_adjoint_gradient():
    _need_gpu()
    import torch
    from cauchyfriendly_gb300.adjoint import loglik_weights, mce_log_likelihood
    z = _load("adj_four_state")
    run = _run(z)
    ts = [torch.tensor(np.asarray(z[n], dtype=np.float64), requires_grad=True) for n in NAMES]
    L = mce_log_likelihood(*ts, run, z["msmts"].reshape(-1))
    assert abs(float(L) - float(z["loglik"])) <= 1e-9 * abs(float(z["loglik"]))
    grads = torch.autograd.grad(L, ts)
    run2 = _run(z)
    P = _params(z)
    _, fz = _loglik(run2, z, P)
    want = run2.backward(loglik_weights(fz))
    for n, gt in zip(NAMES, grads):
        assert np.allclose(gt.numpy(), want[n], rtol=1e-12, atol=1e-14), n
    run.close()
    run2.close()


def test_windowed_gradient_with_fixed_checkpoints():
    """The sliding-window log-likelihood (4-state LTI, window 4, 10 steps;
    each step's fz from the chosen window) and its gradient with the
    window-boundary checkpoints held fixed: against central differences of the
    same objective recomputed from the same checkpoints, on a subset of the
    parameters (beta, gamma, a p0 entry, Phi, Gamma and H entries)."""
    _need_gpu()
    import oracle
    from cauchyfriendly_gb300 import workloads as W
    from cauchyfriendly_gb300.adjoint import windowed_log_likelihood
    prob = W.four_state_lti(seed=4, steps=10)
    Wn = 4
    ms = oracle.max_shape_of({"steps": Wn, "d": 4, "pncc": 1})
    cs = [oracle.draw_reference_constants(60 + w, 4, ms) for w in range(Wn)]
    rp = np.stack([c[0] for c in cs])
    bp = np.stack([c[1] for c in cs])
    res = windowed_log_likelihood(prob, Wn, rp, bp)
    assert len(res["starts"]) == 10 and np.isfinite(res["loglik"])
    picks = [("beta", (0,)), ("gamma", (0,)), ("p0", (1,)), ("Phi", (2, 1)), ("Gamma", (3, 0)), ("H", (0, 2))]
    for name, idx in picks:
        base = np.asarray(prob[name], dtype=np.float64)
        h = 1e-6 * max(abs(base[idx]), 1e-3)
        vals = []
        for sgn in (1, -1):
            a = base.copy()
            a[idx] += sgn * h
            r = windowed_log_likelihood(prob, Wn, rp, bp, starts=res["starts"], best=res["best"], with_grad=False,
                                        **{name: a})
            vals.append(r["loglik"])
        fd = (vals[0] - vals[1]) / (2 * h)
        g = res["grad"][name][idx]
        assert abs(g - fd) <= 1e-4 * abs(fd) + 1e-7, (name, idx, g, fd)


def test_batch_runs_match_their_own_runs():
    """AdjointBatch (one batched handle for every run, the records and
    reverses on several host threads) against an AdjointRun per run: the
    window lives of a 4-state window-4 problem (runs of 1 to 4 steps, each
    from its own start statistics and constants).  Re fz is the same doubles
    (the batched step path is the single one); the gradients agree within
    1e-12 (the reverse's atomic sums may add in another order)."""
    _need_gpu()
    import oracle
    from cauchyfriendly_gb300 import workloads as W
    from cauchyfriendly_gb300.adjoint import AdjointBatch, AdjointRun, loglik_weights, windowed_log_likelihood
    prob = W.four_state_lti(seed=4, steps=10)
    Wn = 4
    ms = oracle.max_shape_of({"steps": Wn, "d": 4, "pncc": 1})
    cs = [oracle.draw_reference_constants(60 + w, 4, ms) for w in range(Wn)]
    rp = np.stack([c[0] for c in cs])
    bp = np.stack([c[1] for c in cs])
    starts = windowed_log_likelihood(prob, Wn, rp, bp, with_grad=False)["starts"]
    lens = [min(Wn, 10 - st["step"]) for st in starts]
    msm = [prob["msmts"][st["step"]:st["step"] + n].reshape(-1) for st, n in zip(starts, lens)]
    P = _params(prob)
    model = (P["Phi"], P["Gamma"], P["beta"], P["H"], P["gamma"])
    batch = AdjointBatch(4, 1, 1, lens, [st["A0"] for st in starts], [st["p0"] for st in starts],
                         [st["b0"] for st in starts], [rp[st["slot"]] for st in starts],
                         [bp[st["slot"]] for st in starts])
    fzb = batch.forward(msm, *model)
    te, fe = batch.check()
    assert te <= 1e-12 and fe <= 1e-12, (te, fe)
    ws = [loglik_weights(f) for f in fzb]
    ws[1] = np.zeros_like(ws[1])  # a run without seeds gets a zero gradient
    gb = batch.backward(ws)
    for r, st in enumerate(starts):
        run = AdjointRun(4, 1, 1, lens[r], st["A0"], st["p0"], st["b0"], rp[st["slot"]], bp[st["slot"]])
        fz = run.forward(msm[r], *model)
        assert np.array_equal(fz, fzb[r]), (r, fz, fzb[r])
        if r == 1:
            assert np.all(_flat(gb[r]) == 0.0)
        else:
            g = _flat(run.backward(ws[r]))
            assert np.allclose(_flat(gb[r]), g, rtol=1e-12, atol=1e-12 * np.max(np.abs(g))), r
        run.close()
    batch.close()


def test_adjoint_of_records_above_sixteen_rows():
    """A 3-state run with seven process-noise columns over 3 steps (records
    of 17 hyperplanes, 684 terms: the record chain's 32-row instantiation)
    against central differences of the GPU forward run."""
    _need_gpu()
    import oracle
    from cauchyfriendly_gb300 import workloads as W
    from cauchyfriendly_gb300.adjoint import loglik_weights
    prob = W.many_gamma(3, 7, 3, seed=1)
    assert oracle.max_shape_of(prob) > 16
    rp, bp = oracle.draw_reference_constants(78, 3, oracle.max_shape_of(prob))
    z = dict(prob)
    z["root_point"], z["b_pert"] = rp, bp
    run = _run(z)
    P = _params(z)
    L, fz = _loglik(run, z, P)
    assert np.isfinite(L)
    te, fe = run.check()
    assert te <= 1e-12 and fe <= 1e-12, (te, fe)
    g = run.backward(loglik_weights(fz))
    fd = {}
    for n in NAMES:
        a = P[n]
        fd[n] = np.zeros_like(a)
        for idx in np.ndindex(a.shape):
            h = 1e-6 * max(abs(a[idx]), 1e-3)
            Pp = {k: v.copy() for k, v in P.items()}
            Pm = {k: v.copy() for k, v in P.items()}
            Pp[n][idx] += h
            Pm[n][idx] -= h
            fd[n][idx] = (_loglik(run, z, Pp)[0] - _loglik(run, z, Pm)[0]) / (2 * h)
    ok, err = _close(_flat(g), _flat(fd))
    assert ok, err
    run.close()


def test_batched_windowed_gradient_of_time_varying_models():
    """windowed_log_likelihood_batch: two 3-state LTV estimators (two
    process-noise columns, two measurements per step, each its own model and
    step count), window 2, sharing (beta, gamma, p0): the gradient with the
    window checkpoints held fixed against central differences of the same
    objective, on every shared scale."""
    _need_gpu()
    import oracle
    from cauchyfriendly_gb300 import workloads as W
    from cauchyfriendly_gb300.adjoint import windowed_log_likelihood_batch
    probs = [W.ltv_windows(3, seed=s, steps=6) for s in (21, 22)]
    Wn = 2
    ms = oracle.max_shape_of({"steps": Wn, "d": 3, "pncc": 2})
    cs = [oracle.draw_reference_constants(90 + w, 3, ms) for w in range(Wn)]
    rp = np.stack([c[0] for c in cs])
    bp = np.stack([c[1] for c in cs])
    beta, gamma, p0 = probs[0]["beta"], probs[0]["gamma"], probs[0]["p0"]
    res = windowed_log_likelihood_batch(probs, Wn, rp, bp, beta, gamma, p0, steps=[6, 5])
    assert np.isfinite(res["loglik"])
    scales = {"beta": beta, "gamma": gamma, "p0": p0}
    for name, base in scales.items():
        for idx in range(len(base)):
            h = 1e-6 * max(abs(base[idx]), 1e-3)
            vals = []
            for sgn in (1, -1):
                sc = {k: np.array(v, dtype=np.float64) for k, v in scales.items()}
                sc[name][idx] += sgn * h
                r = windowed_log_likelihood_batch(probs, Wn, rp, bp, sc["beta"], sc["gamma"], sc["p0"], steps=[6, 5],
                                                  checkpoints=res["checkpoints"], with_grad=False)
                vals.append(r["loglik"])
            fd = (vals[0] - vals[1]) / (2 * h)
            g = res["grad"][name][idx]
            assert abs(g - fd) <= 1e-4 * abs(fd) + 1e-6, (name, idx, g, fd)


def test_adjoint_of_a_time_varying_model():
    """AdjointRun with a Phi per step (a 3-state LTV model, two process-noise
    columns, two measurements per step, 3 steps): the gradient with respect
    to (beta, gamma, p0, a perturbation common to every step's Phi, Gamma,
    H) against central differences of the GPU forward run."""
    _need_gpu()
    import oracle
    from cauchyfriendly_gb300 import workloads as W
    from cauchyfriendly_gb300.adjoint import loglik_weights
    prob = W.ltv_windows(3, seed=31, steps=3)
    assert prob["Phi"].ndim == 3
    rp, bp = oracle.draw_reference_constants(79, 3, oracle.max_shape_of(prob))
    z = dict(prob)
    z["root_point"], z["b_pert"] = rp, bp
    run = _run(z)
    P = _params(z)
    L, fz = _loglik(run, z, P)
    te, fe = run.check()
    assert te <= 1e-12 and fe <= 1e-12, (te, fe)
    g = run.backward(loglik_weights(fz))
    assert g["Phi"].shape == (3, 3)
    fd = {}
    for n in NAMES:
        a = P[n]
        shape = a.shape[1:] if n == "Phi" else a.shape
        fd[n] = np.zeros(shape)
        for idx in np.ndindex(shape):
            ref = a[(0,) + idx] if n == "Phi" else a[idx]
            h = 1e-6 * max(abs(ref), 1e-3)
            vals = []
            for sgn in (1, -1):
                Q = {k: v.copy() for k, v in P.items()}
                if n == "Phi":
                    Q[n][(slice(None),) + idx] += sgn * h  # every step's Phi
                else:
                    Q[n][idx] += sgn * h
                vals.append(_loglik(run, z, Q)[0])
            fd[n][idx] = (vals[0] - vals[1]) / (2 * h)
    ok, err = _close(_flat(g), _flat(fd))
    assert ok, err
    run.close()
