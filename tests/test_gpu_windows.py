"""Sliding-window estimation on the GPU against the same window logic driving
oracle estimators: per step the chosen window, its error bits and term
counts must agree exactly, the estimates within 1e-9 relative."""
import numpy as np
import pytest

import oracle
from tests import golden_cases as G

pytestmark = pytest.mark.gpu


def _need_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _managers(make_prob, n_mgr, W, steps):
    probs = [make_prob(seed) for seed in range(n_mgr)]
    for p in probs:
        p["steps"] = steps
    return probs


def _run(probs, W, backend):
    from cauchyfriendly_gb300 import windows
    d, pncc, p = probs[0]["d"], probs[0]["pncc"], probs[0]["p"]
    n = len(probs)
    A0 = np.stack([q["A0"] for q in probs])
    p0 = np.stack([q["p0"] for q in probs])
    b0 = np.stack([q["b0"] for q in probs])
    ms = oracle.max_shape_of({"steps": W, "d": d, "pncc": pncc})
    consts = [oracle.draw_reference_constants(50 + m, d, ms) for m in range(n)]
    rp = np.stack([c[0] for c in consts])
    bp = np.stack([c[1] for c in consts])
    if backend == "gpu":
        factory = lambda *a: windows._GpuSlot(*a, root_point=rp, b_pert=bp)
    else:
        factory = lambda A0_, p0_, b0_, steps_, d_, cmcc_, pncc_, p_: oracle.OracleSlot(
            A0_, p0_, b0_, steps_, d_, cmcc_, pncc_, p_, consts)
    mgr = windows.SlidingWindowManager(W, A0, p0, b0, d, pncc, p, slot_factory=factory)
    Phi = np.stack([q["Phi"] for q in probs])
    Gam = np.stack([q["Gamma"] for q in probs])
    beta = np.stack([q["beta"] for q in probs])
    H = np.stack([q["H"] for q in probs])
    gam = np.stack([q["gamma"] for q in probs])
    recs = []
    for k in range(probs[0]["steps"]):
        z = np.stack([q["msmts"][k] for q in probs])
        out = mgr.step(z, Phi, Gam, beta, H, gam)
        nts = [[mgr.slots[w].num_terms(m) for m in range(n)] for w in range(W)]
        recs.append((out, nts, mgr.win_counts.copy()))
    total = mgr.total_post_mu_terms()
    mgr.close()
    return recs, total


@pytest.mark.parametrize("case", ["four_state", "five_state_two_msmt"])
def test_windows_gpu_matches_oracle_windows(case):
    _need_gpu()
    from cauchyfriendly_gb300 import workloads as W
    if case == "four_state":
        probs = _managers(lambda s: W.four_state_lti(seed=s, steps=10), 3, 4, 10)
        Wn = 4
    else:
        probs = _managers(lambda s: W.five_state_two_msmt(seed=s, steps=6), 2, 3, 6)
        Wn = 3
    got, total_got = _run(probs, Wn, "gpu")
    want, total_want = _run(probs, Wn, "oracle")
    assert total_got == total_want
    for k, ((og, ng, cg), (ow, nw, cw)) in enumerate(zip(got, want)):
        assert np.array_equal(cg, cw)
        assert ng == nw, (k, ng, nw)
        for m, (a, b) in enumerate(zip(og, ow)):
            assert a[2] == b[2] and a[3] == b[3], (k, m, a[2:], b[2:])
            assert G.relerr(a[0], b[0]) <= 1e-9, (k, m, "xhat")
            assert G.relerr(a[1], b[1]) <= 1e-9, (k, m, "Phat")


# ---- pinned to the reference's own window managers -------------------------

def _load_win(name):
    import os
    return np.load(os.path.join(G.GOLDEN, name + ".npz"))


def _tile(a, n):
    a = np.asarray(a, dtype=np.float64)
    return np.stack([a] * n)


@pytest.mark.parametrize("name", ["win_py_four_state", "win_py_five_state_two_msmt"])
def test_python_window_manager_matches_reference(name):
    """windows.SlidingWindowManager against the reference's own
    PySlidingWindowManager (cauchy_estimator.py:1092-1335, run unmodified on
    the reference's C++ to make the fixture): per step the chosen window, its
    error bits, every window's step count and term count exactly; the estimate,
    fz and the weighted-average estimate within 1e-9 element-wise.  Two
    managers of the same problem run side by side in each window slot's batch,
    with each window's own rand() constants."""
    _need_gpu()
    from cauchyfriendly_gb300 import windows
    z = _load_win(name)
    d, pncc, p, Wn, steps = int(z["d"]), int(z["pncc"]), int(z["p"]), int(z["W"]), int(z["steps"])
    nm = 2
    rp = np.stack([z["root_point"]] * nm, axis=1)
    bp = np.stack([z["b_pert"]] * nm, axis=1)
    mgr = windows.SlidingWindowManager(Wn, _tile(z["A0"], nm), _tile(z["p0"], nm), _tile(z["b0"], nm), d, pncc, p,
                                       root_point=rp, b_pert=bp)
    Phi, Gam, beta = _tile(z["Phi"], nm), _tile(z["Gamma"], nm), _tile(z["beta"], nm)
    H, gam = _tile(z["H"], nm), _tile(z["gamma"], nm)
    for k in range(steps):
        out = mgr.step(_tile(z["msmts"][k], nm), Phi, Gam, beta, H, gam)
        pre = "s%d_" % k
        assert np.array_equal(mgr.win_counts, z[pre + "win_counts"]), (k, mgr.win_counts, z[pre + "win_counts"])
        for m in range(nm):
            xh, Ph, wi, err = out[m]
            assert wi == int(z[pre + "win_idx"]) and err == int(z[pre + "err_code"]), (k, m, wi, err)
            nts = [mgr.slots[w].num_terms(m) for w in range(Wn)]
            assert nts == list(z[pre + "nt"]), (k, m, nts, list(z[pre + "nt"]))
            assert G.relerr(xh, z[pre + "xhat"]) <= G.REL_TOL, (k, m, "xhat", G.relerr(xh, z[pre + "xhat"]))
            assert G.relerr(Ph, z[pre + "Phat"]) <= G.REL_TOL, (k, m, "Phat", G.relerr(Ph, z[pre + "Phat"]))
            last = mgr.last[m]
            assert G.relerr([last["fz"]], [float(z[pre + "fz"])]) <= G.REL_TOL, (k, m, "fz")
            assert G.relerr(last["wavg_xhat"], z[pre + "wavg_xhat"]) <= G.REL_TOL, (k, m, "wavg x")
            assert G.relerr(last["wavg_Phat"], z[pre + "wavg_Phat"]) <= G.REL_TOL, (k, m, "wavg P")
    mgr.close()


def _ltv_table_callback(table):
    import ctypes as ct
    from cauchyfriendly_gb300.pycauchy import C_CauchyDynamicsUpdateContainer

    def cb(duc_ptr):
        duc = duc_ptr.contents
        k = min(max(int(duc.step), 0), table.shape[0] - 1)
        flat = table[k].reshape(-1)
        for i in range(duc.n * duc.n):
            duc.Phi[i] = float(flat[i])
    return ct.CFUNCTYPE(None, ct.POINTER(C_CauchyDynamicsUpdateContainer))(cb)


@pytest.mark.parametrize("name", ["win_cpp_four_state", "win_cpp_five_state_ltv"])
def test_cpp_window_manager_matches_reference(name):
    """The drop-in pycauchy_initialize_lti/ltv_window_manager + pycauchy_step
    (the library's C++ mce_swm_*) against the reference's C++
    SlidingWindowManager with its forked windows (include/cauchy_windows.hpp,
    driven through the reference's pycauchy.hpp): per step the pycauchy_step
    8-tuple -- window index and error bits exactly, fz and the estimate within
    1e-9.  The LTV case calls a dynamics callback that sets Phi_k by the
    container's step.  rand() is seeded as the fixture was, so the windows'
    root point and b_pert are the reference's."""
    _need_gpu()
    import ctypes as ct
    from cauchyfriendly_gb300 import pycauchy
    z = _load_win(name)
    steps, Wn = int(z["steps"]), int(z["W"])
    f = lambda a: np.asarray(a, dtype=np.float64).reshape(-1)
    empty = np.array([], dtype=np.float64)
    Phi0 = z["Phi"] if z["Phi"].ndim == 2 else z["Phi"][0]
    ct.CDLL(None).srand(ct.c_uint(int(z["srand_seed"])))
    cb = None
    if int(z["ltv"]):
        cb = _ltv_table_callback(np.asarray(z["Phi"]))
        pycauchy.pycauchy_initialize_ltv_window_manager(Wn, steps, f(z["A0"]), f(z["p0"]), f(z["b0"]), f(Phi0),
                                                        f(z["Gamma"]), empty, f(z["beta"]), f(z["H"]), f(z["gamma"]),
                                                        ct.cast(cb, ct.c_void_p).value, False, False, False, None,
                                                        0.1, 0, empty)
    else:
        pycauchy.pycauchy_initialize_lti_window_manager(Wn, steps, f(z["A0"]), f(z["p0"]), f(z["b0"]), f(Phi0),
                                                        f(z["Gamma"]), empty, f(z["beta"]), f(z["H"]), f(z["gamma"]),
                                                        False, False, False, None, 0.0, 0, empty)
    try:
        for k in range(steps):
            fz, x, P, cfz, cx, cP, wi, err = pycauchy.pycauchy_step(f(z["msmts"][k]), empty)
            pre = "s%d_" % k
            assert wi == int(z[pre + "win_idx"]) and err == int(z[pre + "err_code"]), (k, wi, err)
            assert G.relerr([fz], [float(z[pre + "fz"])]) <= G.REL_TOL, (k, "fz")
            assert G.relerr(x, z[pre + "xhat"]) <= G.REL_TOL, (k, "xhat", G.relerr(x, z[pre + "xhat"]))
            assert G.relerr(P, z[pre + "Phat"]) <= G.REL_TOL, (k, "Phat", G.relerr(P, z[pre + "Phat"]))
    finally:
        pycauchy.pycauchy_shutdown()


def test_cpp_window_manager_batched_managers_match_reference():
    """Three managers of the fixture's LTI problem in one CppSlidingWindowManager
    (one batched handle per window slot): every manager reproduces the
    reference's C++ manager, with its windows' constants given explicitly."""
    _need_gpu()
    import oracle
    from cauchyfriendly_gb300 import windows
    z = _load_win("win_cpp_four_state")
    steps, Wn, d = int(z["steps"]), int(z["W"]), int(z["d"])
    nm = 3
    ms = (Wn - 1) * int(z["pncc"]) + d
    rp, bp = oracle.draw_reference_constants(int(z["srand_seed"]), d, ms)
    mgr = windows.CppSlidingWindowManager(Wn, steps, _tile(z["A0"], nm), _tile(z["p0"], nm), _tile(z["b0"], nm),
                                          _tile(z["Phi"], nm), _tile(z["Gamma"], nm), None, _tile(z["beta"], nm),
                                          _tile(z["H"], nm), _tile(z["gamma"], nm), root_point=_tile(rp, nm),
                                          b_pert=_tile(bp, nm))
    for k in range(steps):
        out = mgr.step(_tile(z["msmts"][k], nm))
        pre = "s%d_" % k
        for m in range(nm):
            fz, x, P, cfz, cx, cP, wi, err = out[m]
            assert wi == int(z[pre + "win_idx"]) and err == int(z[pre + "err_code"]), (k, m)
            assert G.relerr(x, z[pre + "xhat"]) <= G.REL_TOL and G.relerr(P.reshape(-1), z[pre + "Phat"]) <= G.REL_TOL
    assert mgr.total_post_mu_terms() > 0
    mgr.close()


def test_drop_in_ignores_search_axis_ordering_like_the_reference():
    """The drop-in pycauchy single-estimator path, with the search-axis
    ordering set to the fixture's second ordering, against the reference run
    under that ordering (tests/golden/tr_ordering_three_state.npz): the same
    term counts and error bits, estimates within 1e-9."""
    _need_gpu()
    import ctypes as ct
    from cauchyfriendly_gb300 import pycauchy
    z = _load_win("tr_ordering_three_state")
    order = list(z["orderings"][1])
    assert pycauchy.pycauchy_set_tr_search_idxs_ordering(np.array(order + list(range(len(order), 12)))) == 0
    ct.CDLL(None).srand(ct.c_uint(int(z["srand_seed"])))
    h = pycauchy.pycauchy_initialize_lti(int(z["steps"]), z["A0"], z["p0"], z["b0"], z["Phi"], z["Gamma"],
                                         np.array([]), z["beta"], z["H"], z["gamma"], 0.0, 0, False)
    for k in range(int(z["steps"])):
        out = pycauchy.pycauchy_single_step_ltiv(h, z["msmts"][k], np.array([]))
        pre = "o1_s%d_" % k
        assert pycauchy.pycauchy_single_step_get_number_of_terms(h) == int(z[pre + "nt"]), k
        assert np.array_equal(out[12], z[pre + "err"]), k
        assert G.relerr(out[7], z[pre + "x"]) <= G.REL_TOL, (k, "x")
        assert G.relerr(out[8], z[pre + "P"]) <= G.REL_TOL, (k, "P")
    pycauchy.pycauchy_single_step_shutdown(h)


def test_cpp_window_manager_nonlin_matches_reference():
    """The C++ manager in extended mode (pycauchy_initialize_nonlin_window_manager
    + pycauchy_step) against the reference's own extended-mode manager
    (include/cauchy_windows.hpp with is_extended, forked window processes
    running the same callbacks, tests/golden/win_cpp_nonlin_three_state.npz):
    per step the chosen window and its error bits exactly, fz, estimate and
    covariance within 1e-9 element-wise."""
    _need_gpu()
    import ctypes as ct
    from cauchyfriendly_gb300 import pycauchy
    from cauchyfriendly_gb300 import workloads as W
    z = _load_win("win_cpp_nonlin_three_state")
    dyn, msmt, ext = W.nonlin_callbacks()
    C = pycauchy.C_CauchyDynamicsUpdateContainer
    keep = (ct.CFUNCTYPE(None, ct.POINTER(C))(dyn), ct.CFUNCTYPE(None, ct.POINTER(C), ct.POINTER(ct.c_double))(msmt),
            ct.CFUNCTYPE(None, ct.POINTER(C))(ext))
    ptr = lambda c: ct.cast(c, ct.c_void_p).value
    ct.CDLL(None).srand(ct.c_uint(int(z["srand_seed"])))
    pycauchy.pycauchy_initialize_nonlin_window_manager(int(z["W"]), int(z["steps"]), z["x0"], z["A0"], z["p0"],
                                                       z["b0"], z["beta"], z["gamma"], ptr(keep[0]), ptr(keep[1]),
                                                       ptr(keep[2]), 0, False, False, False, None, W.NONLIN_DT, 0,
                                                       np.array([]))
    try:
        for k in range(int(z["steps"])):
            fz, x, P, cfz, cx, cP, wi, err = pycauchy.pycauchy_step(z["msmts"][k], np.array([]))
            pre = "s%d_" % k
            assert wi == int(z[pre + "win_idx"]) and err == int(z[pre + "err_code"]), (k, wi, err)
            assert G.relerr([fz], [float(z[pre + "fz"])]) <= G.REL_TOL, (k, "fz")
            assert G.relerr(x, z[pre + "xhat"]) <= G.REL_TOL, (k, "xhat", x, z[pre + "xhat"])
            assert G.relerr(P, z[pre + "Phat"]) <= G.REL_TOL, (k, "Phat")
    finally:
        pycauchy.pycauchy_shutdown()
    del keep
