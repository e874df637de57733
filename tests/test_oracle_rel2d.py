"""The oracle's relative-then-transformed 2-D system of two estimators
(get_marg2d_relative_and_transformed_cpdf and
grid_eval_marg2d_relative_and_transformed_cpdf, include/cauchy_prediction.hpp)
against the reference's own results in tests/golden/rel2d_*.npz: pair and
approximated-out counts and grid points exact, relative moments and pdf values
within REL_TOL."""
import numpy as np
import pytest

import oracle
from tests import golden_cases as G


def _stepped(prob, consts, updates):
    est = oracle.Oracle(prob, *consts)
    n = 0
    for k in range(prob["steps"]):
        for s in range(prob["p"]):
            if n < updates:
                est.step(k, s)
                n += 1
    return est


@pytest.mark.parametrize("name", G.rel2d_names())
def test_oracle_rel2d_matches_reference(name):
    pp, pc, sp, sc, updates, case = G.load_rel2d(name)
    P, S = _stepped(pp, pc, updates), _stepped(sp, sc, updates)
    g = case["grid"]
    out = oracle.oracle_rel2d(P, S, case["Trel"], case["bar_nu_full"], g[:3], g[3:], full_solve=bool(case["full"]),
                              term_approx_eps=case["eps"])
    assert out["pairs"] == case["pairs"] == P.num_terms() * S.num_terms()
    assert out["approxed_out"] == case["approxed_out"]
    assert G.relerr([out["fz"]], [case["fz"]]) <= G.REL_TOL
    assert G.relerr(out["mean"], case["mean"]) <= G.REL_TOL
    assert G.relerr(out["cov"], case["cov"]) <= G.REL_TOL
    assert np.array_equal(out["x"], case["x"]) and np.array_equal(out["y"], case["y"])
    assert G.relerr(out["z"], case["z"]) <= G.REL_TOL, G.relerr(out["z"], case["z"])
    P.close()
    S.close()


def test_oracle_rel2d_refuses_before_the_first_and_at_the_last_step():
    from cauchyfriendly_gb300 import workloads as W
    prob = W.three_state_lti(seed=0, steps=2)
    consts = oracle.draw_reference_constants(5, 3, oracle.max_shape_of(prob))
    P, S = _stepped(prob, consts, 0), _stepped(prob, consts, 1)
    T = np.eye(3)[:2]
    with pytest.raises(RuntimeError):
        oracle.oracle_rel2d(P, S, T, np.zeros(3), (-1, 1, 0.5), (-1, 1, 0.5))
    P.step(0)
    S.step(1)
    with pytest.raises(RuntimeError):
        oracle.oracle_rel2d(P, S, T, np.zeros(3), (-1, 1, 0.5), (-1, 1, 0.5))
    P.close()
    S.close()
