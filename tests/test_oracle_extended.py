"""The oracle's extended-mode helpers (finalize_extended_moments,
deterministic_time_prop, shift_cf_by_bias; include/cauchy_estimator.hpp:
1312-1394) against the reference through the fixed op sequences recorded in
tests/golden/ext_*.npz: term counts and error bits exact, moments and x_bar
within REL_TOL after every op."""
import pytest

import oracle
from tests import golden_cases as G


@pytest.mark.parametrize("name", G.ext_names())
def test_oracle_extended_ops_match_reference(name):
    prob, consts, want = G.load_ext(name)
    est = oracle.Oracle(prob, *consts)
    got = G.run_extended(est, prob, G.extended_ops(prob))
    est.close()
    G.compare_extended(got, want)
