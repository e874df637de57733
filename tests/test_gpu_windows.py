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
