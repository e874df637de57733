"""The reference's own Python API over the drop-in.

scripts/swig/cauchy/cauchy_estimator.py (the reference's Python layer, from
the unmodified copy the oracle build keeps in oracle/_ref/src) is imported
with ``pycauchy`` bound to cauchyfriendly_gb300.pycauchy, so every call it
makes lands on the GPU library.  Its PyCauchyEstimator and
PySlidingWindowManager then replay the fixtures that the same Python code
made over the reference's C++ (tests/golden/make_windows_golden.py): equal
window choices, error bits, step and term counts, estimates within 1e-9
element-wise.  Skipped where the copy is absent."""
import ctypes as ct
import os

import numpy as np
import pytest

import oracle
from tests import golden_cases as G

pytestmark = pytest.mark.gpu


def _api():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cauchyfriendly_gb300 import pycauchy
    ce = oracle.reference_python_api(pycauchy)
    if ce is None:
        pytest.skip("no copy of the reference's Python API")
    return ce


@pytest.fixture(autouse=True)
def _serial_reference_draws():
    """The fixtures come from a serial build of the reference (NUM_CPUS = 1):
    each estimator it makes advances rand() by one b_pert draw, which decides
    the constants of every window after the first."""
    from cauchyfriendly_gb300 import _lib
    lib = _lib.load()
    old = lib.mce_set_reference_num_cpus(1)
    yield
    lib.mce_set_reference_num_cpus(old)


def _load(name):
    return np.load(os.path.join(G.GOLDEN, name + ".npz"))


def _srand(seed):
    ct.CDLL(None).srand(ct.c_uint(int(seed)))


@pytest.mark.parametrize("name", ["win_py_four_state", "win_py_five_state_two_msmt"])
def test_reference_py_window_manager_runs_on_drop_in(name):
    """PySlidingWindowManager (cauchy_estimator.py:1092-1335) over the
    drop-in: Speyer restarts through pycauchy_speyers_window_init /
    pycauchy_single_step_reset, window choice by the reference's own Python."""
    ce = _api()
    z = _load(name)
    W, steps = int(z["W"]), int(z["steps"])
    _srand(z["srand_seed"])
    mgr = ce.PySlidingWindowManager("lti", W, swm_debug_print=False, win_debug_print=False)
    mgr.initialize_lti(z["A0"], z["p0"], z["b0"], z["Phi"], None, z["Gamma"], z["beta"], z["H"], z["gamma"])
    for k in range(steps):
        xhat, Phat, wx, wP = mgr.step(z["msmts"][k], None)
        pre = "s%d_" % k
        mi = mgr.moment_info
        assert int(mi["win_idx"][-1]) == int(z[pre + "win_idx"]), k
        assert int(mi["err_code"][-1]) == int(z[pre + "err_code"]), k
        assert np.array_equal(mgr.win_counts, z[pre + "win_counts"]), k
        nts = [e.get_num_CF_terms() for e in mgr.cauchyEsts]
        assert nts == list(z[pre + "nt"]), (k, nts, list(z[pre + "nt"]))
        assert G.relerr(xhat, z[pre + "xhat"]) <= G.REL_TOL, (k, "xhat")
        assert G.relerr(Phat, z[pre + "Phat"]) <= G.REL_TOL, (k, "Phat")
        assert G.relerr(wx, z[pre + "wavg_xhat"]) <= G.REL_TOL, (k, "wavg xhat")
        assert G.relerr(wP, z[pre + "wavg_Phat"]) <= G.REL_TOL, (k, "wavg Phat")
        assert G.relerr([mi["fz"][-1]], [float(z[pre + "fz"])]) <= G.REL_TOL, (k, "fz")
    mgr.shutdown()


def test_reference_py_estimator_runs_on_drop_in():
    """PyCauchyEstimator (cauchy_estimator.py, lti mode) over the drop-in,
    against the reference's run of the same script (the fixture's first
    search-axis ordering, the default one)."""
    ce = _api()
    z = _load("tr_ordering_three_state")
    steps = int(z["steps"])
    _srand(z["srand_seed"])
    est = ce.PyCauchyEstimator("lti", steps, False)
    est.initialize_lti(z["A0"], z["p0"], z["b0"], z["Phi"], None, z["Gamma"], z["beta"], z["H"], z["gamma"])
    for k in range(steps):
        est.step(z["msmts"][k], None)
        pre = "o0_s%d_" % k
        assert est.get_num_CF_terms() == int(z[pre + "nt"]), k
        assert np.array_equal(est._err_code, z[pre + "err"]), k
        assert G.relerr(est._x, z[pre + "x"]) <= G.REL_TOL, (k, "x")
        assert G.relerr(est._P, z[pre + "P"]) <= G.REL_TOL, (k, "P")
        assert G.relerr(est._fz, z[pre + "fz"]) <= G.REL_TOL, (k, "fz")
    est.shutdown()


def test_reference_py_nonlin_window_manager_runs_on_drop_in():
    """PySlidingWindowManager in "nonlin" mode over the drop-in: its windows
    run pycauchy_initialize_nonlin / pycauchy_single_step_nonlin and restart
    about x_bar through pycauchy_get_reinitialization_statistics and
    pycauchy_single_step_reset, on the callbacks of
    workloads.nonlin_callbacks."""
    ce = _api()
    from cauchyfriendly_gb300 import workloads as W
    z = _load("win_py_nonlin_three_state")
    Wn, steps = int(z["W"]), int(z["steps"])
    dyn, msmt, ext = W.nonlin_callbacks()
    _srand(z["srand_seed"])
    mgr = ce.PySlidingWindowManager("nonlin", Wn, swm_debug_print=False, win_debug_print=False)
    mgr.initialize_nonlin(z["x0"], z["A0"], z["p0"], z["b0"], z["beta"], z["gamma"], dyn, msmt, ext, 0, W.NONLIN_DT,
                          0)
    for k in range(steps):
        xhat, Phat, wx, wP = mgr.step(z["msmts"][k], None)
        pre = "s%d_" % k
        mi = mgr.moment_info
        assert int(mi["win_idx"][-1]) == int(z[pre + "win_idx"]), k
        assert int(mi["err_code"][-1]) == int(z[pre + "err_code"]), k
        assert np.array_equal(mgr.win_counts, z[pre + "win_counts"]), k
        nts = [e.get_num_CF_terms() for e in mgr.cauchyEsts]
        assert nts == list(z[pre + "nt"]), (k, nts, list(z[pre + "nt"]))
        assert G.relerr(xhat, z[pre + "xhat"]) <= G.REL_TOL, (k, "xhat")
        assert G.relerr(Phat, z[pre + "Phat"]) <= G.REL_TOL, (k, "Phat")
        assert G.relerr(wx, z[pre + "wavg_xhat"]) <= G.REL_TOL, (k, "wavg xhat")
        assert G.relerr(wP, z[pre + "wavg_Phat"]) <= G.REL_TOL, (k, "wavg Phat")
        assert G.relerr([mi["fz"][-1]], [float(z[pre + "fz"])]) <= G.REL_TOL, (k, "fz")
    mgr.shutdown()
