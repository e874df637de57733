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
