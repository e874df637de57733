"""Host logic of the sliding-window manager (cauchyfriendly_gb300.windows) on
CPU: Speyer's restart statistics and the window bookkeeping, driven by
oracle estimators (no GPU)."""
import os

import numpy as np
import pytest

import oracle
from cauchyfriendly_gb300 import windows, workloads as W
from tests import golden_cases as G


def test_speyer_restart_matches_reference_kats():
    """The library's C++ Speyer restart (mce_speyers_window_init, host code:
    no GPU needed) against the reference's pycauchy_speyers_window_init on 24
    random estimates of 2-7 states, 6 of them with an indefinite covariance
    that the restart boosts first (tests/golden/speyer_kats.npz): the same
    doubles -- eigenvector order and signs included."""
    z = np.load(os.path.join(G.GOLDEN, "speyer_kats.npz"))
    boosted = 0
    for i in range(int(z["count"])):
        pre = "k%d_" % i
        A0, p0, b0 = windows.speyers_window_init(z[pre + "x"], z[pre + "P"], z[pre + "H"], float(z[pre + "gamma"]),
                                                 float(z[pre + "z"]))
        assert np.array_equal(A0, z[pre + "A0"]), (i, G.relerr(A0, z[pre + "A0"]))
        assert np.array_equal(p0, z[pre + "p0"]), (i, G.relerr(p0, z[pre + "p0"]))
        assert np.array_equal(b0, z[pre + "b0"]), (i, G.relerr(b0, z[pre + "b0"]))
        boosted += np.linalg.eigvalsh(z[pre + "P"]).min() < -1e-5
    assert boosted == 6
    # the drop-in module returns them flattened, as the SWIG module does
    from cauchyfriendly_gb300 import pycauchy
    a, p, b = pycauchy.pycauchy_speyers_window_init(z["k0_x"], z["k0_P"].reshape(-1), z["k0_H"],
                                                    float(z["k0_gamma"]), float(z["k0_z"]))
    assert np.array_equal(a, z["k0_A0"].reshape(-1)) and np.array_equal(p, z["k0_p0"])


def test_sym_eig_is_an_eigen_decomposition():
    rng = np.random.default_rng(3)
    for n in (1, 2, 5, 8):
        M = rng.standard_normal((n, n))
        S = M + M.T
        w, V = windows.sym_eig(S)
        assert np.allclose(S @ V, V * w, atol=1e-12)
        assert np.allclose(V.T @ V, np.eye(n), atol=1e-12)
        assert np.allclose(np.sort(w), np.linalg.eigvalsh(S), atol=1e-12)


def test_reference_results_do_not_depend_on_search_axis_ordering():
    """The reference itself under two term-reduction search-axis orderings
    (pycauchy_set_tr_search_idxs_ordering) gives the same doubles at every
    update (tests/golden/tr_ordering_three_state.npz), which is why the
    drop-in accepts the ordering with no effect."""
    z = np.load(os.path.join(G.GOLDEN, "tr_ordering_three_state.npz"))
    assert len(z["orderings"]) == 2 and not np.array_equal(z["orderings"][0], z["orderings"][1])
    for k in range(int(z["steps"])):
        for q in ("x", "P", "fz", "err", "nt"):
            assert np.array_equal(z["o0_s%d_%s" % (k, q)], z["o1_s%d_%s" % (k, q)]), (k, q)
    assert int(z["o0_s%d_nt" % (int(z["steps"]) - 1)]) > 1000


def test_speyer_restart_statistics():
    rng = np.random.default_rng(0)
    n = 4
    M = rng.standard_normal((n, n))
    P = M @ M.T + 0.1 * np.eye(n)
    x = rng.standard_normal(n)
    H = rng.standard_normal(n)
    A0, p0, b0 = windows.speyers_window_init(x, P, H, 0.2, 0.7)
    assert np.allclose(A0 @ A0.T, np.eye(n), atol=1e-12)
    assert np.all(p0 > 0) and np.all(np.isfinite(b0))
    # b0 is the Kalman-like update of x toward the measurement
    s = 0.2 ** 2 + (0.7 - H @ x) ** 2
    assert np.allclose(b0, x - P @ H * (0.7 - H @ x) / s)


def test_window_bookkeeping_with_oracle_estimators():
    oracle.build(with_reference=False)
    Wn, steps, n = 3, 8, 2
    probs = [W.four_state_lti(seed=s, steps=steps) for s in range(n)]
    d = 4
    ms = oracle.max_shape_of({"steps": Wn, "d": d, "pncc": 1})
    consts = [oracle.draw_reference_constants(7 + m, d, ms) for m in range(n)]
    factory = lambda A0_, p0_, b0_, st_, d_, cm_, pn_, p_: oracle.OracleSlot(A0_, p0_, b0_, st_, d_, cm_, pn_, p_,
                                                                             consts)
    mgr = windows.SlidingWindowManager(Wn, np.stack([p["A0"] for p in probs]), np.stack([p["p0"] for p in probs]),
                                       np.stack([p["b0"] for p in probs]), d, 1, 1, slot_factory=factory)
    seen_counts = []
    for k in range(steps):
        out = mgr.step(np.stack([p["msmts"][k] for p in probs]), np.stack([p["Phi"] for p in probs]),
                       np.stack([p["Gamma"] for p in probs]), np.stack([p["beta"] for p in probs]),
                       np.stack([p["H"] for p in probs]), np.stack([p["gamma"] for p in probs]))
        assert len(out) == n
        for xh, Ph, w, err in out:
            assert 0 <= w < Wn and xh.shape == (d,) and Ph.shape == (d, d)
        seen_counts.append(mgr.win_counts.copy())
    # after warm-up the counts cycle through {0, 1, ..., W-1} (one window restarts each step)
    for c in seen_counts[Wn:]:
        assert sorted(c.tolist()) == list(range(Wn))
    mgr.close()


def test_window_manager_without_a_usable_window():
    """A step at which every window of a manager carries a covariance error
    code: the manager raises, as the reference exits
    (cauchy_estimator.py:1181-1216), unless built with no_window="fullest",
    which takes the fullest window and counts the step.  The slots are
    oracle estimators whose error codes are forced on from the third step."""
    oracle.build(with_reference=False)
    Wn, steps, n, d = 3, 6, 1, 4
    probs = [W.four_state_lti(seed=s, steps=steps) for s in range(n)]
    ms = oracle.max_shape_of({"steps": Wn, "d": d, "pncc": 1})
    consts = [oracle.draw_reference_constants(7 + m, d, ms) for m in range(n)]

    class Forced(oracle.OracleSlot):
        step_no = [0]

        def errors(self, i):
            return (windows.COV_UNSTABLE if self.step_no[0] >= 3 else 0) | super().errors(i)

    def run(rule):
        Forced.step_no[0] = 0
        factory = lambda A0_, p0_, b0_, st_, d_, cm_, pn_, p_: Forced(A0_, p0_, b0_, st_, d_, cm_, pn_, p_, consts)
        mgr = windows.SlidingWindowManager(Wn, np.stack([p["A0"] for p in probs]), np.stack([p["p0"] for p in probs]),
                                           np.stack([p["b0"] for p in probs]), d, 1, 1, slot_factory=factory,
                                           no_window=rule)
        try:
            for k in range(steps):
                Forced.step_no[0] = k
                counts = mgr.win_counts.copy()
                out = mgr.step(np.stack([p["msmts"][k] for p in probs]), np.stack([p["Phi"] for p in probs]),
                               np.stack([p["Gamma"] for p in probs]), np.stack([p["beta"] for p in probs]),
                               np.stack([p["H"] for p in probs]), np.stack([p["gamma"] for p in probs]))
                if k >= 3:
                    # the fullest window of the step (each stepped window's count grew by one)
                    assert counts[out[0][2]] == max(counts)
            return mgr.no_window_steps
        finally:
            mgr.close()

    with pytest.raises(RuntimeError):
        run("raise")
    assert run("fullest") == steps - 3
