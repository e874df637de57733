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
