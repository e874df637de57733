"""The pycauchy drop-in (cauchyfriendly_gb300/pycauchy.py) through the C ABI:
same call sequence and 13-tuple as the reference's SWIG functions
(pycauchy.hpp:295-543), checked against the oracle's reported moments."""
import ctypes as ct

import numpy as np
import pytest

import oracle
from tests import golden_cases as G

pytestmark = pytest.mark.gpu


def _need_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_lti_single_step_tuple_matches_oracle():
    _need_gpu()
    from cauchyfriendly_gb300 import pycauchy, workloads as W
    prob = W.three_state_lti(seed=2, steps=7)
    d = prob["d"]
    # pycauchy draws the constants with rand() like the reference; seed libc first
    rp, bp = oracle.draw_reference_constants(5, d, oracle.max_shape_of(prob))
    ct.CDLL(None).srand(5)  # the estimator's constructor draws the same constants next
    h = pycauchy.pycauchy_initialize_lti(prob["steps"], prob["A0"].reshape(-1), prob["p0"], prob["b0"],
                                         prob["Phi"].reshape(-1), prob["Gamma"].reshape(-1), np.array([]),
                                         prob["beta"], prob["H"].reshape(-1), prob["gamma"], 0.0, 0, False)
    orc = oracle.Oracle(prob, rp, bp)
    for k in range(prob["steps"]):
        out = pycauchy.pycauchy_single_step_ltiv(h, prob["msmts"][k], np.array([]))
        assert len(out) == 13
        fz, xhat, Phat, cfz, cx, cP, err = out[6:]
        e2 = orc.step(k, 0)
        mo = orc.moments()
        assert int(err[0]) == e2
        assert abs(fz[0] - mo["fz"].real) <= 1e-9 * max(1.0, abs(mo["fz"].real))
        assert G.relerr(xhat, mo["mean"].real) <= 1e-9 or np.allclose(xhat, mo["mean"].real, atol=1e-12)
        assert G.relerr(Phat, mo["cov"].real.reshape(-1)) <= 1e-9
        assert pycauchy.pycauchy_single_step_get_number_of_terms(h) == orc.num_terms()
    pycauchy.pycauchy_single_step_shutdown(h)
    orc.close()


def test_ltv_callback_updates_dynamics():
    _need_gpu()
    from cauchyfriendly_gb300 import pycauchy, workloads as W
    base = W.three_state_lti(seed=4, steps=6)
    d = 3
    # time-varying Phi_k = Phi * (1 + 0.01 k) applied through the callback
    phis = [base["Phi"] * (1.0 + 0.01 * k) for k in range(base["steps"])]
    state = {"k": 0}

    def cb(duc_ptr):
        duc = duc_ptr.contents
        k = state["k"]
        for i in range(d * d):
            duc.Phi[i] = float(phis[k].reshape(-1)[i])
        state["k"] += 1

    f = pycauchy._CALLBACK(cb)
    fptr = ct.cast(f, ct.c_void_p).value
    rp, bp = oracle.draw_reference_constants(9, d, oracle.max_shape_of(base))
    ct.CDLL(None).srand(9)
    h = pycauchy.pycauchy_initialize_ltv(base["steps"], base["A0"].reshape(-1), base["p0"], base["b0"],
                                         base["Phi"].reshape(-1), base["Gamma"].reshape(-1), np.array([]),
                                         base["beta"], base["H"].reshape(-1), base["gamma"], fptr, 0.0, 0, False)
    prob = dict(base)
    prob["Phi"] = np.stack(phis)
    orc = oracle.Oracle(prob, rp, bp)
    for k in range(base["steps"]):
        out = pycauchy.pycauchy_single_step_ltiv(h, base["msmts"][k], np.array([]))
        assert np.allclose(out[0], phis[k].reshape(-1))
        orc.step(k, 0)
        mo = orc.moments()
        assert abs(out[6][0] - mo["fz"].real) <= 1e-9 * max(1.0, abs(mo["fz"].real))
        assert pycauchy.pycauchy_single_step_get_number_of_terms(h) == orc.num_terms()
    pycauchy.pycauchy_single_step_shutdown(h)
    orc.close()
