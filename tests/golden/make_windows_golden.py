"""Generates the window-manager fixtures (win_*.npz, speyer_kats.npz,
tr_ordering_*.npz) from the REFERENCE itself.

The reference's own Python API, scripts/swig/cauchy/cauchy_estimator.py, is
imported UNMODIFIED with ``pycauchy`` bound to oracle/ref_pycauchy.py (the
reference's scripts/swig/cauchy/pycauchy.hpp compiled as is, serial build) and
a stand-in for matplotlib (plotting is not used).  It then runs:

* ``PySlidingWindowManager`` (cauchy_estimator.py:1092-1335, in-process
  windows with Speyer restarts): per step the chosen window, its estimate,
  error bits, fz, the weighted-average estimate, and every window's term
  count and step count (win_py_*.npz);
* ``pycauchy_initialize_*_window_manager`` + ``pycauchy_step`` (the C++
  SlidingWindowManager of include/cauchy_windows.hpp, forked window
  processes): per step the 8-tuple pycauchy_step returns (win_cpp_*.npz), LTI
  and LTV (a dynamics callback that sets Phi_k from a table by the
  container's step);
* ``pycauchy_speyers_window_init`` on random estimates, some with a covariance
  that needs the eigenvalue boost (speyer_kats.npz);
* ``PyCauchyEstimator`` under two term-reduction search-axis orderings
  (``pycauchy_set_tr_search_idxs_ordering``, tr_ordering_*.npz);
* both managers in extended (nonlinear) mode on the problem and callbacks of
  workloads.nonlin_three_state / nonlin_callbacks (win_py_nonlin_*.npz,
  win_cpp_nonlin_*.npz).

Each window fixture also stores the root point and b_pert every window's
estimator drew from rand() (srand(seed) before the manager is made).

Needs the reference sources:  python tests/golden/make_windows_golden.py
"""
import ctypes as ct
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from cauchyfriendly_gb300 import workloads as W  # noqa: E402


def _reference_api():
    oracle.build()
    from oracle import ref_pycauchy
    sys.modules["pycauchy"] = ref_pycauchy
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", plt)
    sys.path.insert(0, os.path.join(oracle.REFERENCE_ROOT, "scripts", "swig", "cauchy"))
    import cauchy_estimator as ce
    return ce, ref_pycauchy


def _model(prob):
    return dict(A0=prob["A0"], p0=prob["p0"], b0=prob["b0"], Phi=prob["Phi"] if prob["Phi"].ndim == 2 else prob["Phi"][0],
                B=None, Gamma=prob["Gamma"], beta=prob["beta"], H=prob["H"], gamma=prob["gamma"])


def _problem_arrays(prob):
    return {k: prob[k] for k in ("Phi", "Gamma", "beta", "H", "gamma", "A0", "p0", "b0", "msmts", "d", "pncc", "p")}


def py_manager(name, prob, W_, steps, seed):
    ce, rp = _reference_api()
    rp.srand(seed)
    m = _model(prob)
    mgr = ce.PySlidingWindowManager("lti", W_, swm_debug_print=False, win_debug_print=False)
    mgr.initialize_lti(m["A0"], m["p0"], m["b0"], m["Phi"], m["B"], m["Gamma"], m["beta"], m["H"], m["gamma"])
    consts = [rp.get_constants(e.py_handle) for e in mgr.cauchyEsts]
    arr = _problem_arrays(prob)
    arr.update(W=W_, steps=steps, srand_seed=seed, root_point=np.stack([c[0] for c in consts]),
               b_pert=np.stack([c[1] for c in consts]))
    for k in range(steps):
        xhat, Phat, wx, wP = mgr.step(prob["msmts"][k], None)
        pre = "s%d_" % k
        mi = mgr.moment_info
        arr[pre + "xhat"] = np.asarray(xhat)
        arr[pre + "Phat"] = np.asarray(Phat)
        arr[pre + "wavg_xhat"] = np.asarray(wx)
        arr[pre + "wavg_Phat"] = np.asarray(wP)
        arr[pre + "win_idx"] = int(mi["win_idx"][-1])
        arr[pre + "err_code"] = int(mi["err_code"][-1])
        arr[pre + "fz"] = float(mi["fz"][-1])
        arr[pre + "cerr"] = np.array([mi["cerr_fz"][-1], mi["cerr_x"][-1], mi["cerr_P"][-1]], dtype=np.float64)
        arr[pre + "win_counts"] = mgr.win_counts.copy()
        arr[pre + "nt"] = np.array([e.get_num_CF_terms() for e in mgr.cauchyEsts], dtype=np.int64)
    mgr.shutdown()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arr)
    print(name, "done")


_PHI_TABLE = None


def _ltv_callback(duc_ptr):
    """Dynamics callback of the LTV fixtures: Phi_k from the problem's table,
    k = the container's step (clamped)."""
    duc = duc_ptr.contents
    n = duc.n
    k = min(max(int(duc.step), 0), _PHI_TABLE.shape[0] - 1)
    flat = _PHI_TABLE[k].reshape(-1)
    for i in range(n * n):
        duc.Phi[i] = float(flat[i])


def cpp_manager(name, prob, W_, steps, seed, ltv=False):
    global _PHI_TABLE
    ce, rp = _reference_api()
    rp.srand(seed)
    m = _model(prob)
    arr = _problem_arrays(prob)
    arr.update(W=W_, steps=steps, srand_seed=seed, ltv=int(ltv))
    f = lambda a: np.asarray(a, dtype=np.float64).reshape(-1)
    empty = np.array([], dtype=np.float64)
    keep = None
    if ltv:
        _PHI_TABLE = np.asarray(prob["Phi"], dtype=np.float64)
        cb = ct.CFUNCTYPE(None, ct.POINTER(ce.C_CauchyDynamicsUpdateContainer))(_ltv_callback)
        keep = cb
        rp.pycauchy_initialize_ltv_window_manager(W_, steps, f(m["A0"]), f(m["p0"]), f(m["b0"]), f(m["Phi"]),
                                                  f(m["Gamma"]), empty, f(m["beta"]), f(m["H"]), f(m["gamma"]),
                                                  ct.cast(cb, ct.c_void_p).value, False, False, False, None, 0.1, 0,
                                                  empty)
    else:
        rp.pycauchy_initialize_lti_window_manager(W_, steps, f(m["A0"]), f(m["p0"]), f(m["b0"]), f(m["Phi"]),
                                                  f(m["Gamma"]), empty, f(m["beta"]), f(m["H"]), f(m["gamma"]),
                                                  False, False, False, None, 0.0, 0, empty)
    for k in range(steps):
        fz, x, P, cfz, cx, cP, wi, err = rp.pycauchy_step(f(prob["msmts"][k]), empty)
        pre = "s%d_" % k
        arr[pre + "fz"] = fz
        arr[pre + "xhat"] = x
        arr[pre + "Phat"] = P
        arr[pre + "cerr"] = np.array([cfz, cx, cP])
        arr[pre + "win_idx"] = wi
        arr[pre + "err_code"] = err
    rp.pycauchy_shutdown()
    del keep
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arr)
    print(name, "done")


def _nonlin_arrays(prob):
    return {k: prob[k] for k in ("x0", "A0", "p0", "b0", "beta", "gamma", "Gamma", "msmts", "d", "pncc", "p")}


def py_nonlin_manager(name, prob, W_, steps, seed):
    """PySlidingWindowManager in "nonlin" mode (PyCauchyEstimator windows on
    pycauchy_initialize_nonlin / pycauchy_single_step_nonlin, restarts with
    x_bar) over the problem's callbacks (workloads.nonlin_callbacks)."""
    ce, rp = _reference_api()
    rp.srand(seed)
    dyn, msmt, ext = W.nonlin_callbacks()
    mgr = ce.PySlidingWindowManager("nonlin", W_, swm_debug_print=False, win_debug_print=False)
    mgr.initialize_nonlin(prob["x0"], prob["A0"], prob["p0"], prob["b0"], prob["beta"], prob["gamma"], dyn, msmt, ext,
                          0, W.NONLIN_DT, 0)
    consts = [rp.get_constants(e.py_handle) for e in mgr.cauchyEsts]
    arr = _nonlin_arrays(prob)
    arr.update(W=W_, steps=steps, srand_seed=seed, root_point=np.stack([c[0] for c in consts]),
               b_pert=np.stack([c[1] for c in consts]))
    for k in range(steps):
        xhat, Phat, wx, wP = mgr.step(prob["msmts"][k], None)
        pre = "s%d_" % k
        mi = mgr.moment_info
        arr[pre + "xhat"] = np.asarray(xhat)
        arr[pre + "Phat"] = np.asarray(Phat)
        arr[pre + "wavg_xhat"] = np.asarray(wx)
        arr[pre + "wavg_Phat"] = np.asarray(wP)
        arr[pre + "win_idx"] = int(mi["win_idx"][-1])
        arr[pre + "err_code"] = int(mi["err_code"][-1])
        arr[pre + "fz"] = float(mi["fz"][-1])
        arr[pre + "win_counts"] = mgr.win_counts.copy()
        arr[pre + "nt"] = np.array([e.get_num_CF_terms() for e in mgr.cauchyEsts], dtype=np.int64)
    mgr.shutdown()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arr)
    print(name, "done")


def cpp_nonlin_manager(name, prob, W_, steps, seed):
    """pycauchy_initialize_nonlin_window_manager + pycauchy_step: the C++
    SlidingWindowManager in extended mode (forked window processes running
    the problem's callbacks)."""
    ce, rp = _reference_api()
    rp.srand(seed)
    arr = _nonlin_arrays(prob)
    arr.update(W=W_, steps=steps, srand_seed=seed)
    f = lambda a: np.asarray(a, dtype=np.float64).reshape(-1)
    empty = np.array([], dtype=np.float64)
    dyn, msmt, ext = W.nonlin_callbacks()
    t1 = ct.CFUNCTYPE(None, ct.POINTER(ce.C_CauchyDynamicsUpdateContainer))
    t2 = ct.CFUNCTYPE(None, ct.POINTER(ce.C_CauchyDynamicsUpdateContainer), ct.POINTER(ct.c_double))
    keep = (t1(dyn), t2(msmt), t1(ext))
    ptr = lambda c: ct.cast(c, ct.c_void_p).value
    rp.pycauchy_initialize_nonlin_window_manager(W_, steps, f(prob["x0"]), f(prob["A0"]), f(prob["p0"]),
                                                 f(prob["b0"]), f(prob["beta"]), f(prob["gamma"]), ptr(keep[0]),
                                                 ptr(keep[1]), ptr(keep[2]), 0, False, False, False, None,
                                                 W.NONLIN_DT, 0, empty)
    for k in range(steps):
        fz, x, P, cfz, cx, cP, wi, err = rp.pycauchy_step(f(prob["msmts"][k]), empty)
        pre = "s%d_" % k
        arr[pre + "fz"] = fz
        arr[pre + "xhat"] = x
        arr[pre + "Phat"] = P
        arr[pre + "cerr"] = np.array([cfz, cx, cP])
        arr[pre + "win_idx"] = wi
        arr[pre + "err_code"] = err
    rp.pycauchy_shutdown()
    del keep
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arr)
    print(name, "done")


def speyer_kats():
    _, rp = _reference_api()
    rng = np.random.Generator(np.random.PCG64(77))
    arr = {}
    i = 0
    for n in (2, 3, 4, 5, 6, 7):
        for kind in range(4):
            M = rng.standard_normal((n, n))
            P = M @ M.T * 0.1 + 0.01 * np.eye(n)
            if kind == 3:
                # an indefinite covariance: the restart boosts its diagonal
                w, V = np.linalg.eigh(P)
                w[0] = -1e-3
                P = (V * w) @ V.T
            x = rng.standard_normal(n)
            H = rng.standard_normal(n)
            g = float(np.exp(rng.uniform(np.log(0.02), np.log(0.5))))
            z = float(H @ x + rng.standard_cauchy() * g)
            A0, p0, b0 = rp.pycauchy_speyers_window_init(x, P.reshape(-1), H, g, z)
            pre = "k%d_" % i
            arr.update({pre + "x": x, pre + "P": P, pre + "H": H, pre + "gamma": g, pre + "z": z,
                        pre + "A0": A0.reshape(n, n), pre + "p0": p0, pre + "b0": b0})
            i += 1
    arr["count"] = i
    np.savez_compressed(os.path.join(HERE, "speyer_kats.npz"), **arr)
    print("speyer_kats done")


def tr_ordering(name, prob, seed, orderings):
    ce, rp = _reference_api()
    arr = _problem_arrays(prob)
    arr["steps"] = prob["steps"]
    arr["srand_seed"] = seed
    arr["orderings"] = np.array(orderings, dtype=np.int32)
    m = _model(prob)
    for oi, order in enumerate(orderings):
        rp.pycauchy_set_tr_search_idxs_ordering(np.array(list(order) + list(range(len(order), 12)), np.int32))
        rp.srand(seed)
        est = ce.PyCauchyEstimator("lti", prob["steps"], False)
        est.initialize_lti(m["A0"], m["p0"], m["b0"], m["Phi"], m["B"], m["Gamma"], m["beta"], m["H"], m["gamma"])
        if oi == 0:
            r, b = rp.get_constants(est.py_handle)
            arr["root_point"], arr["b_pert"] = r, b
        for k in range(prob["steps"]):
            est.step(prob["msmts"][k], None)
            pre = "o%d_s%d_" % (oi, k)
            arr[pre + "x"] = est._x.copy()
            arr[pre + "P"] = est._P.copy()
            arr[pre + "fz"] = est._fz.copy()
            arr[pre + "err"] = est._err_code.copy()
            arr[pre + "nt"] = est.get_num_CF_terms()
        est.shutdown()
    rp.pycauchy_set_tr_search_idxs_ordering(np.arange(12, dtype=np.int32))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arr)
    print(name, "done")


if __name__ == "__main__":
    what = sys.argv[1:] or ["py", "cpp", "speyer", "order", "nonlin"]
    if "py" in what:
        py_manager("win_py_four_state", W.four_state_lti(seed=0, steps=12), 4, 12, 21)
        py_manager("win_py_five_state_two_msmt", W.five_state_two_msmt(seed=1, steps=7), 3, 7, 22)
    if "cpp" in what:
        cpp_manager("win_cpp_four_state", W.four_state_lti(seed=2, steps=12), 4, 12, 23)
        cpp_manager("win_cpp_five_state_ltv", W.five_state_ltv_windows(seed=3, steps=7), 3, 7, 24, ltv=True)
    if "speyer" in what:
        speyer_kats()
    if "nonlin" in what:
        py_nonlin_manager("win_py_nonlin_three_state", W.nonlin_three_state(seed=8, steps=10), 3, 10, 26)
        cpp_nonlin_manager("win_cpp_nonlin_three_state", W.nonlin_three_state(seed=9, steps=10), 3, 10, 27)
    if "order" in what:
        tr_ordering("tr_ordering_three_state", W.three_state_lti(seed=7, steps=9), 25, [(0, 1, 2), (2, 0, 1)])
