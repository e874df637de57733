"""The oracle's marginal 1-D pdf (PointWiseNDimCauchyCPDF::
evaluate_1D_marginal_cpdf and CauchyCPDFGridDispatcher1D, include/cpdf_ndim.hpp)
against the reference's own grids in tests/golden/cpdf1d_*.npz: grid points
exact, pdf values within REL_TOL, on the first (exact, caching) and second
(cached) call for every state."""
import numpy as np
import pytest

import oracle
from tests import golden_cases as G


def _stepped_oracle(prob, consts, updates):
    est = oracle.Oracle(prob, *consts)
    n = 0
    for k in range(prob["steps"]):
        for s in range(prob["p"]):
            if n < updates:
                est.step(k, s)
                n += 1
    return est


@pytest.mark.parametrize("name", G.cpdf_names())
def test_oracle_cpdf_matches_reference_grids(name):
    prob, consts, updates, bar_nu, grids = G.load_cpdf(name)
    est = _stepped_oracle(prob, consts, updates)
    for marg, call, (lo, hi, res), x, y in grids:
        xo, yo = est.cpdf_1d_grid(marg, bar_nu, lo, hi, res)
        assert np.array_equal(xo, x), (marg, call)
        assert G.relerr(yo, y) <= G.REL_TOL, (marg, call, G.relerr(yo, y))
    est.close()


def test_oracle_cpdf_refuses_the_last_step():
    from cauchyfriendly_gb300 import workloads as W
    prob = W.three_state_lti(seed=0, steps=3)
    est = _stepped_oracle(prob, oracle.draw_reference_constants(5, 3, oracle.max_shape_of(prob)), 3)
    with pytest.raises(RuntimeError):
        est.cpdf_1d_grid(0, np.ones(3), -1.0, 1.0, 0.1)
    est.close()


@pytest.mark.parametrize("name", G.cpdf2d_names())
def test_oracle_cpdf2d_matches_reference_grids(name):
    """PointWiseNDimCauchyCPDF::evaluate_2D_marginal_cpdf through
    CauchyCPDFGridDispatcher2D: every state pair's three grid calls (caching,
    cached then reset, exact again)."""
    prob, consts, updates, bar_nu, grids = G.load_cpdf2d(name)
    est = _stepped_oracle(prob, consts, updates)
    for i1, i2, call, gx, gy, x, y, z in grids:
        xo, yo, zo = est.cpdf_2d_grid(i1, i2, bar_nu, gx, gy, reset_cache=(call == 1))
        assert np.array_equal(xo, x) and np.array_equal(yo, y), (i1, i2, call)
        assert G.relerr(zo, z) <= G.REL_TOL, (i1, i2, call, G.relerr(zo, z))
    est.close()


@pytest.mark.parametrize("name", G.cpdfnd_names())
def test_oracle_nd_pdf_matches_reference_bitwise(name):
    """The oracle's N-D pdf (PointWiseNDimCauchyCPDF::evaluate_cpdf, with the
    reference's lowering, term reduction and g-tables) gives the reference's
    values bit for bit (tests/golden/cpdfnd_*.npz)."""
    prob, consts, updates, X, F = G.load_cpdfnd(name)
    est = _stepped_oracle(prob, consts, updates)
    got = np.array([est.cpdf_nd(x) for x in X])
    est.close()
    assert G.bitwise_equal(got, F), (name, G.relerr(got, F))


@pytest.mark.parametrize("name", G.cpdfmarg_names())
def test_oracle_marginal_pdf_matches_reference_bitwise(name):
    """The oracle's marginal pdf of every subset of the states
    (PointWiseNDimCauchyCPDF::evaluate_marginal_cpdf: columns reordered, the
    kept states lowered out, the rest looked up at nu_bar) gives the
    reference's values bit for bit (tests/golden/cpdfmarg_*.npz)."""
    prob, consts, updates, cases = G.load_cpdfmarg(name)
    est = _stepped_oracle(prob, consts, updates)
    got = np.array([est.cpdf_marginal(xm, idx, nu) for idx, xm, nu, _ in cases])
    want = np.array([f for _, _, _, f in cases])
    est.close()
    assert G.bitwise_equal(got, want), (name, G.relerr(got, want))


def test_oracle_nd_pdf_refuses_before_the_first_step():
    from cauchyfriendly_gb300 import workloads as W
    prob = W.four_state_lti(seed=0, steps=3)
    est = oracle.Oracle(prob, *oracle.draw_reference_constants(5, 4, oracle.max_shape_of(prob)))
    with pytest.raises(RuntimeError):
        est.cpdf_nd(np.zeros(4))
    est.close()
