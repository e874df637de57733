"""Marginal 1-D pdf on the GPU (mce_cpdf_1d_grid) against the reference's own
grids (tests/golden/cpdf1d_*.npz) and against the oracle on a random batch:
grid points exact, values within REL_TOL, on the first (exact at its first
point, caching) and the second (cached) call for every state."""
import numpy as np
import pytest

import oracle
from tests import golden_cases as G

pytestmark = pytest.mark.gpu


def _need_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cauchyfriendly_gb300 import BatchedCauchyEstimator, CauchyEstimator, _lib
    return BatchedCauchyEstimator, CauchyEstimator, _lib


def _updates(prob):
    return [(k, s) for k in range(prob["steps"]) for s in range(prob["p"])]


@pytest.mark.parametrize("name", G.cpdf_names())
def test_gpu_cpdf_matches_reference_grids(name):
    _, CE, _ = _need_gpu()
    prob, (rp, bp), updates, bar_nu, grids = G.load_cpdf(name)
    est = CE(prob["A0"], prob["p0"], prob["b0"], prob["steps"], prob["d"], prob["cmcc"], prob["pncc"], prob["p"],
             root_point=rp, b_pert=bp)
    for k, s in _updates(prob)[:updates]:
        Phi = prob["Phi"] if prob["Phi"].ndim == 2 else prob["Phi"][k]
        est.step(prob["msmts"][k, s], Phi, prob["Gamma"], prob["beta"], prob["H"][s], prob["gamma"][s])
    for marg, call, (lo, hi, res), x, y in grids:
        xg, yg = est.cpdf_1d_grid(0, marg, lo, hi, res, bar_nu)
        assert np.array_equal(xg, x), (marg, call)
        assert G.relerr(yg, y) <= G.REL_TOL, (marg, call, G.relerr(yg, y))
    assert est.device_errors() == 0
    est.close()


def test_gpu_cpdf_batch_matches_oracle_and_refuses_last_step():
    BCE, _, _lib = _need_gpu()
    from cauchyfriendly_gb300 import workloads as W
    probs = W.batched_three_state(16, seed=9, steps_lo=5, steps_hi=6)
    n = len(probs)
    consts = [oracle.draw_reference_constants(500 + i, 3, oracle.max_shape_of(q)) for i, q in enumerate(probs)]
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
    nu = np.array([0.3, 1.1, 1.7])
    for k in range(4):
        bat.step(np.array([q["msmts"][k, 0] for q in probs]), Phi, Gam, beta, H, gam, shared_model=False)
        for o in orcs:
            o.step(k, 0)
    for e in range(n):
        for marg in (0, 2):
            for _ in range(2):
                xg, yg = bat.cpdf_1d_grid(e, marg, -1.5, 1.5, 0.05, nu)
                xo, yo = orcs[e].cpdf_1d_grid(marg, nu, -1.5, 1.5, 0.05)
                assert np.array_equal(xg, xo)
                assert G.relerr(yg, yo) <= G.REL_TOL, (e, marg, G.relerr(yg, yo))
    # run every estimator to its last update: the pdf is refused there
    last = int(steps.max())
    for k in range(4, last):
        bat.step(np.array([q["msmts"][min(k, q["steps"] - 1), 0] for q in probs]), Phi, Gam, beta, H, gam,
                 shared_model=False)
    with pytest.raises(_lib.MceError):
        bat.cpdf_1d_grid(0, 0, -1.0, 1.0, 0.1, nu)
    assert bat.device_errors() == 0
    for o in orcs:
        o.close()
    bat.close()


@pytest.mark.parametrize("name", G.cpdf2d_names())
def test_gpu_cpdf2d_matches_reference_grids(name):
    """mce_cpdf_2d_grid against the reference's 2-D grids.  The GPU's sines,
    cosines and arctangents are CUDA's, the reference's glibc's: the values
    agree within REL_TOL, the grid points exactly."""
    _, CE, _ = _need_gpu()
    prob, (rp, bp), updates, bar_nu, grids = G.load_cpdf2d(name)
    est = CE(prob["A0"], prob["p0"], prob["b0"], prob["steps"], prob["d"], prob["cmcc"], prob["pncc"], prob["p"],
             root_point=rp, b_pert=bp)
    for k, s in _updates(prob)[:updates]:
        Phi = prob["Phi"] if prob["Phi"].ndim == 2 else prob["Phi"][k]
        est.step(prob["msmts"][k, s], Phi, prob["Gamma"], prob["beta"], prob["H"][s], prob["gamma"][s])
    for i1, i2, call, gx, gy, x, y, z in grids:
        xg, yg, zg = est.cpdf_2d_grid(0, i1, i2, gx, gy, bar_nu, reset_cache=(call == 1))
        assert np.array_equal(xg, x) and np.array_equal(yg, y), (i1, i2, call)
        assert G.relerr(zg, z) <= G.REL_TOL, (i1, i2, call, G.relerr(zg, z))
    assert est.device_errors() == 0
    est.close()


def _stepped_gpu(CE, prob, rp, bp, updates):
    est = CE(prob["A0"], prob["p0"], prob["b0"], prob["steps"], prob["d"], prob["cmcc"], prob["pncc"], prob["p"],
             root_point=rp, b_pert=bp)
    for k, s in _updates(prob)[:updates]:
        Phi = prob["Phi"] if prob["Phi"].ndim == 2 else prob["Phi"][k]
        est.step(prob["msmts"][k, s], Phi, prob["Gamma"], prob["beta"], prob["H"][s], prob["gamma"][s])
    return est


@pytest.mark.parametrize("name", G.cpdfnd_names())
def test_gpu_nd_pdf_matches_reference(name):
    """mce_cpdf_nd at all of a fixture's points in one call against the
    reference's PointWiseNDimCauchyCPDF::evaluate_cpdf (tests/golden/
    cpdfnd_*.npz, values from 1e-16 to 35): within 1e-9 relative wherever the
    pdf is above 1e-3 of its largest value, within 1e-12 of that largest
    value below.  The reference adds the g-tables of lowered terms whose
    arrangements agree within REDUCTION_EPS (1e-8) and lowers the sum once;
    the GPU lowers every (point, term) pair, and the oracle doing the same
    differs from the reference by up to 3e-12 relative above 1e-3 of the peak
    and 2.2e-14 of the peak below (the gap the floor covers)."""
    _, CE, _ = _need_gpu()
    prob, (rp, bp), updates, X, F = G.load_cpdfnd(name)
    est = _stepped_gpu(CE, prob, rp, bp, updates)
    got = est.cpdf_nd(X)
    assert G.relerr(got, F, floor=1e-3) <= G.REL_TOL, (name, G.relerr(got, F, floor=1e-3))
    # one point at a time gives the same values
    one = np.array([est.cpdf_nd(x)[0] for x in X[:3]])
    assert G.bitwise_equal(one, got[:3])
    assert est.device_errors() == 0
    est.close()


@pytest.mark.parametrize("name", G.cpdfmarg_names())
def test_gpu_marginal_pdf_matches_reference(name):
    """mce_cpdf_marginal for every subset of the states short of all of them
    (one call per subset, all its points at once) against the reference's
    PointWiseNDimCauchyCPDF::evaluate_marginal_cpdf (tests/golden/
    cpdfmarg_*.npz), each case at the nu_bar the reference drew: within 1e-9
    relative, with a floor of 1e-3 of the fixture's largest value (the GPU
    lowers every (point, term) pair without the reference's term reduction
    between the lowerings, as mce_cpdf_nd does).  A nu_bar other than the
    reference's gives the same values within the same tolerance."""
    _, CE, _ = _need_gpu()
    prob, (rp, bp), updates, cases = G.load_cpdfmarg(name)
    est = _stepped_gpu(CE, prob, rp, bp, updates)
    want = np.array([f for _, _, _, f in cases])
    got = np.zeros(len(cases), dtype=complex)
    other = np.zeros(len(cases), dtype=complex)
    groups = {}
    for i, (idx, xm, nu, _) in enumerate(cases):
        groups.setdefault((tuple(idx), tuple(nu)), []).append(i)
    for (idx, nu), rows in groups.items():
        X = np.array([cases[i][1] for i in rows])
        got[rows] = est.cpdf_marginal(X, list(idx), nu_bar=np.array(nu))
        other[rows] = est.cpdf_marginal(X, list(idx))
    assert G.relerr(got, want, floor=1e-3) <= G.REL_TOL, (name, G.relerr(got, want, floor=1e-3))
    assert G.relerr(other, want, floor=1e-3) <= G.REL_TOL, (name, G.relerr(other, want, floor=1e-3))
    with pytest.raises(Exception):
        est.cpdf_marginal(np.zeros((1, 2)), [1, 0])  # indices must ascend
    with pytest.raises(Exception):
        est.cpdf_marginal(np.zeros((1, prob["d"])), list(range(prob["d"])))  # fewer than d states
    assert est.device_errors() == 0
    est.close()


def test_gpu_nd_pdf_against_oracle_on_larger_estimators():
    """Larger term sets than the fixtures (a 4-state estimator after 6 updates,
    a 5-state two-measurement one after 5, a 3-state one after 8): the GPU
    at 64 points each out to 10 standard deviations in one call, against the
    oracle with the reference's term reduction at 8 of them (two per scale)
    and the oracle lowering every child apart as the GPU does at 2 (it is
    slow), both within 1e-9 relative above 1e-3 of the largest value and
    1e-12 of it below (the values are sums of 10^4-10^6 terms as large as the
    peak: an order of summation moves a far-tail value of 1e-15 by a few
    1e-14); and the status of the calls the reference refuses."""
    _, CE, _lib = _need_gpu()
    from cauchyfriendly_gb300 import workloads as W
    cases = [(W.four_state_lti(seed=11, steps=7), 6), (W.five_state_two_msmt(seed=12, steps=4), 5),
             (W.many_gamma(3, 1, 9, seed=13), 8)]
    for prob, updates in cases:
        rp, bp = oracle.draw_reference_constants(21, prob["d"], oracle.max_shape_of(prob))
        est = _stepped_gpu(CE, prob, rp, bp, updates)
        orc = oracle.Oracle(prob, rp, bp)
        for k, s in _updates(prob)[:updates]:
            orc.step(k, s)
        if orc.errors():
            est.close()
            orc.close()
            continue
        mo = orc.moments()
        mu = mo["mean"].real
        sd = np.sqrt(np.abs(np.diag(mo["cov"].real)))
        rng = np.random.Generator(np.random.PCG64(3))
        X = mu + sd * rng.standard_normal((64, prob["d"])) * np.repeat([0.5, 1.5, 4.0, 10.0], 16)[:, None]
        got = est.cpdf_nd(X)
        peak = float(np.max(np.abs(got)))
        pick = [0, 1, 16, 17, 32, 33, 48, 49]
        want = np.array([orc.cpdf_nd(X[i]) for i in pick])
        apart = np.array([orc.cpdf_nd(X[i], reduce=False) for i in pick[:2]])
        close = lambda a, b: np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-3 * peak))
        assert close(got[pick], want) <= G.REL_TOL, (prob["d"], updates, est.num_terms(), close(got[pick], want))
        assert close(got[pick[:2]], apart) <= G.REL_TOL, (prob["d"], close(got[pick[:2]], apart))
        est.close()
        orc.close()
    # a handle with room for 21 hyperplanes: its terms of at most 9 rows after
    # 4 steps are evaluated (against the oracle, lowering every pair apart),
    # its terms of 17 rows after 8 steps are refused
    prob = W.many_gamma(3, 2, 10, seed=14)
    rp, bp = oracle.draw_reference_constants(23, 3, oracle.max_shape_of(prob))
    est = CE(prob["A0"], prob["p0"], prob["b0"], 10, 3, 0, 2, 1, root_point=rp, b_pert=bp)
    orc = oracle.Oracle(prob, rp, bp)
    for k in range(4):
        est.step(prob["msmts"][k, 0], prob["Phi"], prob["Gamma"], prob["beta"], prob["H"][0], prob["gamma"][0])
        orc.step(k, 0)
    mu = orc.moments()["mean"].real
    X = mu + np.array([[0.0, 0.0, 0.0], [0.3, -0.2, 0.1], [-1.0, 0.5, 2.0]])
    got = est.cpdf_nd(X)
    want = np.array([orc.cpdf_nd(x, reduce=False) for x in X])
    assert G.relerr(got, want, floor=1e-3) <= G.REL_TOL, G.relerr(got, want, floor=1e-3)
    orc.close()
    for k in range(4, 8):
        est.step(prob["msmts"][k, 0], prob["Phi"], prob["Gamma"], prob["beta"], prob["H"][0], prob["gamma"][0])
    with pytest.raises(_lib.MceError, match="16 hyperplanes"):
        est.cpdf_nd(np.zeros(3))
    est.close()
    # before the first step and after the last one
    prob = W.four_state_lti(seed=1, steps=2)
    rp, bp = oracle.draw_reference_constants(22, 4, oracle.max_shape_of(prob))
    est = CE(prob["A0"], prob["p0"], prob["b0"], 2, 4, 0, 1, 1, root_point=rp, b_pert=bp)
    with pytest.raises(_lib.MceError):
        est.cpdf_nd(np.zeros(4))
    for k in range(2):
        est.step(prob["msmts"][k, 0], prob["Phi"], prob["Gamma"], prob["beta"], prob["H"][0], prob["gamma"][0])
    with pytest.raises(_lib.MceError):
        est.cpdf_nd(np.zeros(4))
    est.close()
