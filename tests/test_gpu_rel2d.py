"""Relative-then-transformed 2-D system of two estimators on the GPU
(mce_rel2d_create / mce_rel2d_grid) against the reference's own results
(tests/golden/rel2d_*.npz) and against the oracle on pairs of a random batch:
pair and approximated-out counts exact, relative moments and pdf values within
REL_TOL."""
import numpy as np
import pytest

import oracle
from tests import golden_cases as G

pytestmark = pytest.mark.gpu


def _need_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cauchyfriendly_gb300 import BatchedCauchyEstimator, CauchyEstimator, RelativeSystem2D, _lib
    return BatchedCauchyEstimator, CauchyEstimator, RelativeSystem2D, _lib


def _stepped_gpu(CE, prob, consts, updates):
    rp, bp = consts
    est = CE(prob["A0"], prob["p0"], prob["b0"], prob["steps"], prob["d"], prob["cmcc"], prob["pncc"], prob["p"],
             root_point=rp, b_pert=bp)
    n = 0
    for k in range(prob["steps"]):
        for s in range(prob["p"]):
            if n < updates:
                Phi = prob["Phi"] if prob["Phi"].ndim == 2 else prob["Phi"][k]
                est.step(prob["msmts"][k, s], Phi, prob["Gamma"], prob["beta"], prob["H"][s], prob["gamma"][s])
                n += 1
    return est


@pytest.mark.parametrize("name", G.rel2d_names())
def test_gpu_rel2d_matches_reference(name):
    _, CE, Rel, _ = _need_gpu()
    pp, pc, sp, sc, updates, case = G.load_rel2d(name)
    P, S = _stepped_gpu(CE, pp, pc, updates), _stepped_gpu(CE, sp, sc, updates)
    rs = Rel(P, S, case["Trel"], full_solve=bool(case["full"]), get_relative_moments=True, with_term_approx=True,
             term_approx_eps=case["eps"], bar_nu_full=case["bar_nu_full"])
    assert rs.pairs == case["pairs"]
    assert rs.approxed_out == case["approxed_out"]
    m = rs.moments
    assert G.relerr([m["fz"]], [case["fz"]]) <= G.REL_TOL
    assert G.relerr(m["mean"], case["mean"]) <= G.REL_TOL
    assert G.relerr(m["cov"], case["cov"]) <= G.REL_TOL
    # the reference offsets its grid by its own relative mean
    g, mu = case["grid"], case["mean"].real
    X, Y, Z, nx, ny = rs.grid(g[0] + mu[0], g[1] + mu[0], g[2], g[3] + mu[1], g[4] + mu[1], g[5])
    assert nx * ny == case["z"].size
    assert np.array_equal(X, case["x"]) and np.array_equal(Y, case["y"])
    assert G.relerr(Z, case["z"]) <= G.REL_TOL, G.relerr(Z, case["z"])
    rs.close()
    assert P.device_errors() == 0 and S.device_errors() == 0
    P.close()
    S.close()


def test_gpu_rel2d_batch_pairs_match_oracle():
    """Pairs of estimators of one batch (several thousand to ~10^5 pairs, so
    the moment and grid sums run in chunks), half and full solve, against the
    oracle; then the refusal after the last update."""
    BCE, _, Rel, _lib = _need_gpu()
    from cauchyfriendly_gb300 import workloads as W
    probs = W.batched_three_state(6, seed=21, steps_lo=7, steps_hi=8)
    n = len(probs)
    consts = [oracle.draw_reference_constants(700 + i, 3, oracle.max_shape_of(q)) for i, q in enumerate(probs)]
    steps = np.array([q["steps"] for q in probs], np.int32)
    ms = oracle.max_shape_of({"steps": int(steps.max()), "d": 3, "pncc": 1})
    bp = np.zeros((n, ms))
    for i, c in enumerate(consts):
        bp[i, :len(c[1])] = c[1]
    bat = BCE(np.stack([q["A0"] for q in probs]), np.stack([q["p0"] for q in probs]),
              np.stack([q["b0"] for q in probs]), steps, 3, 0, 1, 1, np.stack([c[0] for c in consts]), bp)
    orcs = [oracle.Oracle(q, *c) for q, c in zip(probs, consts)]
    Phi = np.stack([q["Phi"] for q in probs])
    Gam = np.stack([q["Gamma"] for q in probs])
    beta = np.stack([q["beta"] for q in probs])
    H = np.stack([q["H"][0] for q in probs])
    gam = np.stack([q["gamma"][0] for q in probs])
    for k in range(5):
        bat.step(np.array([q["msmts"][k, 0] for q in probs]), Phi, Gam, beta, H, gam, shared_model=False)
        for o in orcs:
            o.step(k, 0)
    T = np.array([[1.0, 0.2, 0.0], [0.0, 1.0, -0.4]])
    nu = np.array([0.31, -0.52, 0.77])
    checked = 0
    for (ip, is_), full in (((0, 1), False), ((2, 3), True), ((4, 5), False)):
        rs = Rel((bat, ip), (bat, is_), T, full_solve=full, with_term_approx=True, term_approx_eps=1e-8,
                 bar_nu_full=nu)
        ref = oracle.oracle_rel2d(orcs[ip], orcs[is_], T, nu, (-1.5, 1.5, 0.125), (-1.0, 1.0, 0.125),
                                  full_solve=full)
        assert rs.pairs == ref["pairs"] == bat.num_terms(ip) * bat.num_terms(is_)
        assert rs.approxed_out == ref["approxed_out"]
        for k in ("fz", "mean", "cov"):
            assert G.relerr(np.atleast_1d(rs.moments[k]), np.atleast_1d(ref[k])) <= G.REL_TOL, k
        mu = ref["mean"].real
        X, Y, Z, nx, ny = rs.grid(-1.5 + mu[0], 1.5 + mu[0], 0.125, -1.0 + mu[1], 1.0 + mu[1], 0.125)
        assert np.array_equal(X, ref["x"]) and np.array_equal(Y, ref["y"])
        assert G.relerr(Z, ref["z"]) <= G.REL_TOL, G.relerr(Z, ref["z"])
        checked += rs.pairs
        rs.close()
    assert checked > 3000
    # to the last update: refused there (its g-tables are skipped)
    for k in range(5, int(steps.max())):
        bat.step(np.array([q["msmts"][min(k, q["steps"] - 1), 0] for q in probs]), Phi, Gam, beta, H, gam,
                 shared_model=False)
    with pytest.raises(_lib.MceError):
        Rel((bat, 0), (bat, 1), T, bar_nu_full=nu)
    bat.close()


def test_gpu_rel2d_pycauchy_entry_point():
    """pycauchy_single_step_eval_2d_rsys_cpdf returns the reference's 9-tuple,
    equal to RelativeSystem2D with the same rand() draw of bar_nu_full."""
    _need_gpu()
    import ctypes
    from cauchyfriendly_gb300 import RelativeSystem2D
    from cauchyfriendly_gb300 import pycauchy as pc
    from cauchyfriendly_gb300 import workloads as W
    from cauchyfriendly_gb300.estimator import draw_rel_bar_nu
    probs = [W.three_state_lti(seed=s, steps=6) for s in (0, 1)]
    hs = []
    for q in probs:
        hs.append(pc.pycauchy_initialize_lti(q["steps"], q["A0"].reshape(-1), q["p0"], q["b0"], q["Phi"].reshape(-1),
                                             q["Gamma"].reshape(-1), np.zeros(0), q["beta"], q["H"].reshape(-1),
                                             q["gamma"], 0, 0, False))
    for k in range(3):
        for h, q in zip(hs, probs):
            pc.pycauchy_single_step_ltiv(h, np.array([q["msmts"][k, 0]]), np.zeros(0))
    T = np.array([1.0, 0.0, 0.0, 0.0, 1.0, 0.0])
    nu = draw_rel_bar_nu(3, seed=1234)
    rs = RelativeSystem2D(hs[0].est, hs[1].est, T.reshape(2, 3), with_term_approx=True, term_approx_eps=1e-8,
                          bar_nu_full=nu)
    mu = rs.moments["mean"].real
    X, Y, Z, nx, ny = rs.grid(-1.0 + mu[0], 1.0 + mu[0], 0.25, -1.0 + mu[1], 1.0 + mu[1], 0.25)
    rs.close()
    ctypes.CDLL(None).srand(1234)
    fz, xhat, Phat, cfz, cx, cP, pts, gx, gy = pc.pycauchy_single_step_eval_2d_rsys_cpdf(
        T, hs[1], hs[0], 1e-8, -1.0, 1.0, 0.25, -1.0, 1.0, 0.25)
    assert fz.shape == (1,) and xhat.shape == (2,) and Phat.shape == (4,) and cP.shape == (4,)
    assert (gx, gy) == (nx, ny) == (9, 9)
    assert np.array_equal(xhat, mu) and np.array_equal(cx, rs.moments["mean"].imag)
    assert np.array_equal(pts[0::3], X) and np.array_equal(pts[1::3], Y) and np.array_equal(pts[2::3], Z)
    for h in hs:
        pc.pycauchy_single_step_shutdown(h)
