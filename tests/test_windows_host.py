"""Host logic of the sliding-window manager (cauchyfriendly_gb300.windows) on
CPU: Speyer's restart statistics and the window bookkeeping, driven by
oracle estimators (no GPU)."""
import numpy as np

import oracle
from cauchyfriendly_gb300 import windows, workloads as W


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
