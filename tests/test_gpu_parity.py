"""Parity of the GPU path (through the C ABI) with the reference.

* golden fixtures made by the reference itself: integer structure (term
  counts, terms per shape, error bits, g-table keys) bit-exact; fz, mean,
  covariance and g values within 1e-9 relative (REL_TOL in golden_cases);
* larger seeded problems against the oracle (oracle/mce_oracle.cpp), the
  batched path against per-estimator oracle runs.
"""
import numpy as np
import pytest

import oracle
from tests import golden_cases as G

pytestmark = pytest.mark.gpu


def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cauchyfriendly_gb300 import BatchedCauchyEstimator, CauchyEstimator
    return CauchyEstimator, BatchedCauchyEstimator


class _GpuAdapter:
    """Gives a GPU CauchyEstimator the stepping interface oracle.run uses."""

    def __init__(self, prob, root_point, b_pert):
        CE, _ = _gpu()
        self.prob = prob
        self.est = CE(prob["A0"], prob["p0"], prob["b0"], prob["steps"], prob["d"], prob["cmcc"], prob["pncc"],
                      prob["p"], print_basic_info=prob.get("print_basic_info", False), root_point=root_point,
                      b_pert=b_pert)

    def step(self, k, sub=0):
        pr = self.prob
        Phi = pr["Phi"] if pr["Phi"].ndim == 2 else pr["Phi"][k]
        return self.est.step(pr["msmts"][k, sub], Phi, pr["Gamma"], pr["beta"], pr["H"][sub], pr["gamma"][sub])

    def moments(self):
        return self.est.moments()

    def num_terms(self):
        return self.est.num_terms()

    def terms_per_shape(self):
        return self.est.terms_per_shape()

    def dump_terms(self, max_shape):
        return self.est.dump_terms(0, max_shape)

    def close(self):
        self.est.close()


@pytest.mark.parametrize("name", G.names())
def test_gpu_matches_reference_golden(name):
    prob, (rp, bp), want = G.load(name)
    est = _GpuAdapter(prob, rp, bp)
    got = oracle.run(est, prob, record_terms_upto=10**9)
    assert est.est.device_errors() == 0
    est.close()
    G.compare_records(got, want)


@pytest.mark.parametrize("name", G.names())
def test_gpu_bit_identical_to_reference_golden(name):
    """The step records are the reference's doubles exactly: raw and reported
    fz, mean, covariance, G_SCALE_FACTOR and every dumped term's A, p, b and
    g values, not merely within 1e-9 (the kernels keep the reference's
    operation order, are built without contraction into fused multiply-adds,
    and divide complex numbers by Smith's method as the host runtime does)."""
    prob, (rp, bp), want = G.load(name)
    est = _GpuAdapter(prob, rp, bp)
    got = oracle.run(est, prob, record_terms_upto=10**9)
    est.close()
    bad = G.bitwise_mismatches(got, want)
    assert not bad, bad[:10]


def _batch_run_compare(probs, consts, check_terms=False):
    _, BCE = _gpu()
    n = len(probs)
    d = probs[0]["d"]
    steps = np.array([p["steps"] for p in probs], np.int32)
    A0 = np.stack([p["A0"] for p in probs])
    p0 = np.stack([p["p0"] for p in probs])
    b0 = np.stack([p["b0"] for p in probs])
    ms = oracle.max_shape_of({"steps": int(steps.max()), "d": d, "pncc": probs[0]["pncc"]})
    rp = np.stack([c[0] for c in consts])
    bp = np.zeros((n, ms))
    for i, c in enumerate(consts):
        bp[i, :len(c[1])] = c[1]
    bat = BCE(A0, p0, b0, steps, d, probs[0]["cmcc"], probs[0]["pncc"], probs[0]["p"], rp, bp)
    maxs = int(steps.max())
    msm = np.zeros((n, maxs, probs[0]["p"]))
    for i, p in enumerate(probs):
        msm[i, :p["steps"]] = p["msmts"]
    Phi = np.stack([p["Phi"] for p in probs])
    Gam = np.stack([p["Gamma"] for p in probs])
    beta = np.stack([p["beta"] for p in probs])
    H = np.stack([p["H"] for p in probs])
    gam = np.stack([p["gamma"] for p in probs])
    # step by step so per-estimator term dumps can be compared too
    recs = [[] for _ in range(n)]
    for k in range(maxs):
        for s in range(probs[0]["p"]):
            bat.step(msm[:, k, s], Phi, Gam, beta, H[:, s, :], gam[:, s], shared_model=False)
            for i, p in enumerate(probs):
                if k < p["steps"]:
                    r = bat.moments(i)
                    r["err"] = bat.errors(i)
                    r["Nt"] = bat.num_terms(i)
                    r["tps"] = bat.terms_per_shape(i)
                    if check_terms and k < p["steps"] - 1:
                        r["terms"] = bat.dump_terms(i, oracle.max_shape_of(p))
                    recs[i].append(r)
    assert bat.device_errors() == 0
    total = bat.post_mu_terms()
    bat.close()
    return recs, total


def test_batched_matches_golden_per_estimator():
    names = [n for n in G.names() if n.startswith("batched_three_state")]
    loaded = [G.load(n) for n in names]
    probs = [l[0] for l in loaded]
    consts = [l[1] for l in loaded]
    recs, _ = _batch_run_compare(probs, consts, check_terms=True)
    for (prob, _, want), got in zip(loaded, recs):
        G.compare_records(got, want)


def _oracle_records(prob, rp, bp, terms_upto=0):
    est = oracle.Oracle(prob, rp, bp)
    r = oracle.run(est, prob, terms_upto)
    n = est.post_mu_terms()
    est.close()
    return r, n


def test_batched_random_three_state_against_oracle():
    from cauchyfriendly_gb300 import workloads as W
    probs = W.batched_three_state(48, seed=11, steps_lo=4, steps_hi=8)
    consts = [oracle.draw_reference_constants(100 + i, 3, oracle.max_shape_of(p)) for i, p in enumerate(probs)]
    recs, total = _batch_run_compare(probs, consts)
    want_total = 0
    for prob, c, got in zip(probs, consts, recs):
        want, n = _oracle_records(prob, *c)
        want_total += n
        G.compare_records(got, want, check_terms=False)
    assert total == want_total


def test_full_size_bench_batch_sampled_against_oracle():
    """The bench's batch at its full size (4096 3-state LTI estimators, steps
    U{4..9}, 5% outliers at 100x, seed 0, the bench's reference constants):
    the whole batch on the GPU, every 16th estimator against the oracle at
    every step (moments, Nt, terms per shape, error bits)."""
    import bench
    from cauchyfriendly_gb300 import workloads as W
    probs = W.batched_three_state(4096, seed=0)
    rp, bp = bench.constants(probs, 0)
    consts = [(rp[i], bp[i, :oracle.max_shape_of(p)]) for i, p in enumerate(probs)]
    recs, total = _batch_run_compare(probs, consts)
    assert total > 5e7  # the bench's 53.5 M post-MU terms per pass
    for i in range(0, len(probs), 16):
        want, _ = _oracle_records(probs[i], *consts[i])
        G.compare_records(recs[i], want, check_terms=False)


def test_batched_tables_against_oracle_with_promoted_roots():
    """Every term's g-table against the oracle for a batch in which many
    reduction groups lose their root to the term approximation and promote a
    member (the promoted-root flat pass takes the members left after it)."""
    from cauchyfriendly_gb300 import workloads as W
    probs = W.batched_three_state(32, seed=4, steps_lo=6, steps_hi=8)
    consts = [oracle.draw_reference_constants(300 + i, 3, oracle.max_shape_of(p)) for i, p in enumerate(probs)]
    recs, _ = _batch_run_compare(probs, consts, check_terms=True)
    for prob, c, got in zip(probs, consts, recs):
        want, _ = _oracle_records(prob, *c, terms_upto=10**9)
        G.compare_records(got, want, check_terms=True)


def test_batched_print_basic_info_on_some_estimators():
    """print_basic_info set on every other estimator of a batch: those report
    the post-reduction moments (compute_moments(false)), the others fz = 1."""
    _, BCE = _gpu()
    from cauchyfriendly_gb300 import workloads as W
    probs = W.batched_three_state(8, seed=6, steps_lo=5, steps_hi=7)
    consts = [oracle.draw_reference_constants(400 + i, 3, oracle.max_shape_of(p)) for i, p in enumerate(probs)]
    n = len(probs)
    steps = np.array([p["steps"] for p in probs], np.int32)
    ms = oracle.max_shape_of({"steps": int(steps.max()), "d": 3, "pncc": 1})
    bp = np.zeros((n, ms))
    for i, c in enumerate(consts):
        bp[i, :len(c[1])] = c[1]
    bat = BCE(np.stack([p["A0"] for p in probs]), np.stack([p["p0"] for p in probs]),
              np.stack([p["b0"] for p in probs]), steps, 3, 0, 1, 1, np.stack([c[0] for c in consts]), bp)
    orcs = []
    for i, (p, c) in enumerate(zip(probs, consts)):
        o = oracle.Oracle(p, *c)
        if i % 2 == 0:
            bat.set_print_basic_info(True, i)
            o.set_print_basic_info(True)
        orcs.append(o)
    Phi = np.stack([p["Phi"] for p in probs])
    Gam = np.stack([p["Gamma"] for p in probs])
    beta = np.stack([p["beta"] for p in probs])
    H = np.stack([p["H"][0] for p in probs])
    gam = np.stack([p["gamma"][0] for p in probs])
    for k in range(int(steps.max())):
        bat.step(np.array([p["msmts"][min(k, p["steps"] - 1), 0] for p in probs]), Phi, Gam, beta, H, gam,
                 shared_model=False)
        for i, (p, o) in enumerate(zip(probs, orcs)):
            if k >= p["steps"]:
                continue
            o.step(k, 0)
            got, want = bat.moments(i), o.moments()
            for key in ("fz", "mean", "cov"):
                assert G.relerr(np.atleast_1d(got[key]), np.atleast_1d(want[key])) <= G.REL_TOL, (i, k, key)
            assert abs(got["gscale"] - want["gscale"]) <= G.REL_TOL * abs(want["gscale"]), (i, k)
            if i % 2 and k < p["steps"] - 1:
                assert got["fz"] == 1
    assert bat.device_errors() == 0
    bat.close()
    for o in orcs:
        o.close()


@pytest.mark.parametrize("steps", [10])
def test_three_state_longer_against_oracle(steps):
    from cauchyfriendly_gb300 import workloads as W
    prob = W.three_state_lti(seed=5, steps=steps)
    rp, bp = oracle.draw_reference_constants(3, 3, oracle.max_shape_of(prob))
    est = _GpuAdapter(prob, rp, bp)
    got = oracle.run(est, prob, 0)
    est.close()
    want, _ = _oracle_records(prob, rp, bp)
    G.compare_records(got, want, check_terms=False)


def test_stepping_past_the_last_step_returns_status():
    CE, _ = _gpu()
    from cauchyfriendly_gb300 import _lib, workloads as W
    prob = W.three_state_lti(seed=1, steps=3)
    est = CE(prob["A0"], prob["p0"], prob["b0"], prob["steps"], 3, 0, 1, 1)
    for k in range(3):
        est.step(prob["msmts"][k, 0], prob["Phi"], prob["Gamma"], prob["beta"], prob["H"][0], prob["gamma"][0])
    # the reference calls exit(1) here (cauchy_estimator.hpp:1220-1225)
    with pytest.raises(_lib.MceError):
        est.step(0.0, prob["Phi"], prob["Gamma"], prob["beta"], prob["H"][0], prob["gamma"][0])
    # reset makes it usable again, with the same results
    est.reset()
    est.step(prob["msmts"][0, 0], prob["Phi"], prob["Gamma"], prob["beta"], prob["H"][0], prob["gamma"][0])
    assert est.num_terms() >= 1
    assert est.device_errors() == 0
    est.close()


def test_autotuned_block_sizes_keep_results_bit_identical():
    """The block-size autotuner only changes launch shapes: with the tuner
    off, on every pass while it tunes (measurement launches in flight) and on
    the tuned sizes, a batch gives the same doubles at every update; every
    settled key holds one of the candidate sizes."""
    _, BCE = _gpu()
    from cauchyfriendly_gb300 import autotune_configure, autotune_table
    from cauchyfriendly_gb300 import workloads as W
    import bench
    probs = W.batched_three_state(1024, seed=5, steps_lo=6, steps_hi=9)
    rp, bp = bench.constants(probs, 5)
    B = bench.batch_arrays(probs)
    est = BCE(B["A0"], B["p0"], B["b0"], B["steps"], 3, 0, 1, 1, rp, bp)

    def one_pass():
        est.reset()
        return est.run(B["msmts"], B["Phi"], B["Gamma"], B["beta"], B["H"], B["gamma"], shared_model=False)

    try:
        autotune_configure(False)
        fixed = one_pass()
        assert autotune_table() == []
        autotune_configure(True)
        sizes = []
        for _ in range(16):
            out = one_pass()
            for k in ("fz", "mean", "cov", "err", "nt"):
                assert np.array_equal(out[k], fixed[k]), (len(sizes), k)
            sizes.append(len(autotune_table()))
            if len(sizes) >= 3 and sizes[-1] == sizes[-2] == sizes[-3] and sizes[-1] > 0:
                break
        table = autotune_table()
        tuned = one_pass()
    finally:
        autotune_configure(True)
        est.close()
    for k in ("fz", "mean", "cov", "err", "nt"):
        assert np.array_equal(tuned[k], fixed[k]), k
    assert table and all(r["block"] in (64, 128, 256, 512) for r in table), (sizes, table)
    # launches of 2^15 items or more are tuned: the per-(term, cell) evaluation always has them
    assert "gtable_eval" in {r["kernel"] for r in table}, table


def test_trim_memory_between_reset_and_step():
    """mce_trim_memory frees the term-sized buffers after a reset (not after a
    step), and the next run allocates them again with the same results."""
    _, BCE = _gpu()
    from cauchyfriendly_gb300 import workloads as W
    import bench
    probs = W.batched_three_state(64, seed=6, steps_lo=5, steps_hi=7)
    rp, bp = bench.constants(probs, 6)
    B = bench.batch_arrays(probs)
    est = BCE(B["A0"], B["p0"], B["b0"], B["steps"], 3, 0, 1, 1, rp, bp)
    run = lambda: est.run(B["msmts"], B["Phi"], B["Gamma"], B["beta"], B["H"], B["gamma"], shared_model=False)
    first = run()
    assert est._lib.mce_trim_memory(est._h, 0) == -1  # MCE_ERR_ARG: after a step
    est.reset()
    assert est.trim_memory(1 << 40) == 0  # below the threshold: kept
    assert est.trim_memory() > 0
    assert est.trim_memory() == 0
    second = run()
    est.close()
    for k in ("fz", "mean", "cov", "err", "nt"):
        assert np.array_equal(first[k], second[k]), k


@pytest.mark.parametrize("mode", ["batched", "persistent", "graph"])
def test_term_reduction_round_modes_keep_results_bit_identical(mode):
    """MCE_FTR_ROUNDS picks how the term reduction's rounds after the first
    run: queued in batches (the host reading the worklist length once per
    batch), in one persistent cooperative launch over the device worklists,
    or as a device-side WHILE loop in a CUDA graph.  Under each, the golden
    fixtures stay bit-identical and a random batch matches the oracle (a
    subprocess: the switch is read once per process)."""
    _gpu()
    import os
    import subprocess
    import sys
    env = dict(os.environ, MCE_FTR_ROUNDS=mode)
    env.pop("MCE_FTR_PERSISTENT", None)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-m", "pytest", os.path.join(root, "tests", "test_gpu_parity.py"), "-q",
                        "-p", "no:cacheprovider", "-k", "(bit_identical or random_three_state) and not round_modes"],
                       cwd=root, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert " passed" in r.stdout


def test_seven_state_ltv_window_against_oracle():
    """The 7-state LTV model of the batched 7-state sliding-window
    configuration (two measurements per step): a window-8 estimator (room for
    (8-1)*2+7 = 21 hyperplanes per term, above the shared-memory bitmap
    limit) through its first 6 updates (3 steps, about 10,800 terms) against
    the oracle on the same host: integer structure exact, moments within
    1e-9.  (The sixth update holds a g value within an ulp of the term
    approximation's threshold, where the host's hypot decides: 10,810 terms
    with x86-64 glibc, 10,811 with aarch64 glibc.)"""
    from cauchyfriendly_gb300 import workloads as W
    prob = W.seven_state_ltv_windows(seed=0, steps=8)
    rp, bp = oracle.draw_reference_constants(500, 7, oracle.max_shape_of(prob))
    gpu = _GpuAdapter(prob, rp, bp)
    orc = oracle.Oracle(prob, rp, bp)
    got, want = [], []
    for k in range(3):
        for s in range(2):
            for est, out in ((gpu, got), (orc, want)):
                err = est.step(k, s)
                rec = est.moments()
                rec["err"] = int(err)
                rec["Nt"] = est.num_terms()
                rec["tps"] = est.terms_per_shape()
                out.append(rec)
    gpu.close()
    orc.close()
    assert [r["Nt"] for r in want][:5] == [8, 36, 192, 678, 3308]
    G.compare_records(got, want, check_terms=False)
