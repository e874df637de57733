#!/usr/bin/env python
"""Benchmark of the GB300 MCE step path.

Workload: the batched plain-MCE configuration -- 4096 independent 3-state LTI
estimators (random stable Phi with eigenvalue moduli in [0.8, 1.0],
Gamma=[0,0,1]^T, H=[1,0,0], beta/gamma/p0 log-uniform in [0.02, 0.5], step
counts uniform in 4..9, Cauchy measurement histories with 5% outliers at
100x), seeded synthetic data.  One bench step = one pass of the whole batch
through every measurement update.

metric: MCE terms updated per second = sum over updates of the terms present
after each measurement update (the reference's "Total Terms after MU(C)"
counter) / time.

  value   device time (CUDA events on the library's stream, summed over the
          updates of the pass; inputs are per-update scalars already on the
          host-side engine, the term state lives in HBM)
  e2e     the same through the public C ABI call mce_batch_run with host
          measurement buffers, wall clock around the call

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Other workloads (--workload, one JSON line each; see their functions):
  windows5  the 5-state LTV sliding-window configuration (window 6, two
            measurements per step) for --window-steps steps
  adjoint   one gradient of the 4-state window-7 sliding-window
            log-likelihood against the manager's forward run, with the
            reference's central-difference gradient as the CPU baseline
  mle       Adam on the shared log-scales of 64 LTV sliding-window
            estimators over batched adjoint gradients
  window7   one window of the 7-state LTV model as far as its tables fit
  rel2d     the relative-system 2-D pdf of two 5-state estimators
  cpdfnd    the N-D conditional pdf of a 4-state estimator at many points
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MCE terms updated/sec (1 GB300, FP64) at rel err <=1e-9; batched/adjoint vs plain"
UNIT = "terms/s"
WORKLOAD = "batched plain MCE: 4096 x 3-state LTI, steps U{4..9}, 5% outliers at 100x"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--no-autotune", action="store_true", help="fixed block sizes (no block-size autotuner)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n-est", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU time of the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the one-estimator-per-handle comparison")
    ap.add_argument("--plain-stride", type=int, default=16)
    ap.add_argument("--adjoint-steps", type=int, default=100)
    ap.add_argument("--workload", default="batched3",
                    choices=["batched3", "windows5", "rel2d", "adjoint", "cpdfnd", "window7", "mle"],
                    help="batched3: the batched 3-state configuration (default); windows5: the sliding-window "
                         "5-state LTV configuration for --window-steps steps; rel2d: the relative 2-D system of "
                         "two 5-state estimators; cpdfnd: the N-D conditional pdf of a 4-state estimator at "
                         "--nd-points points; window7: one window of the 7-state LTV model (window 8, two "
                         "measurements per step) as far as its g-tables stay below --max-cells cells; mle: "
                         "maximum-likelihood tuning of the shared scales of --mle-estimators LTV sliding-window "
                         "estimators of --mle-states states (window --mle-window) with Adam on batched adjoint "
                         "gradients")
    ap.add_argument("--nd-points", type=int, default=256)
    ap.add_argument("--window-steps", type=int, default=12)
    ap.add_argument("--rel-updates", type=int, default=6, help="rel2d: updates of both estimators (6: 12.2 M pairs)")
    ap.add_argument("--max-cells", type=float, default=4e8,
                    help="window7: stop before an update whose g-table cells, projected by the largest growth "
                         "seen so far, would pass this")
    ap.add_argument("--cpu-updates", type=int, default=6, help="window7: updates the CPU baseline runs")
    ap.add_argument("--mle-estimators", type=int, default=64)
    ap.add_argument("--mle-states", type=int, default=3)
    ap.add_argument("--mle-window", type=int, default=3)
    ap.add_argument("--mle-iters", type=int, default=4, help="mle: Adam iterations (the configuration's is 50)")
    return ap.parse_args()


def batch_arrays(probs):
    n = len(probs)
    d = probs[0]["d"]
    steps = np.array([p["steps"] for p in probs], np.int32)
    maxs = int(steps.max())
    msm = np.zeros((n, maxs, 1))
    for i, p in enumerate(probs):
        msm[i, :p["steps"]] = p["msmts"]
    return {
        "steps": steps, "A0": np.stack([p["A0"] for p in probs]), "p0": np.stack([p["p0"] for p in probs]),
        "b0": np.stack([p["b0"] for p in probs]), "Phi": np.stack([p["Phi"] for p in probs]),
        "Gamma": np.stack([p["Gamma"] for p in probs]), "beta": np.stack([p["beta"] for p in probs]),
        "H": np.stack([p["H"] for p in probs]), "gamma": np.stack([p["gamma"] for p in probs]), "msmts": msm, "d": d,
    }


def constants(probs, seed):
    import ctypes
    from cauchyfriendly_gb300 import _lib, max_shape
    lib = _lib.load()
    ms = max(max_shape(p["steps"], p["d"], p["pncc"]) for p in probs)
    rp = np.zeros((len(probs), probs[0]["d"]))
    bp = np.zeros((len(probs), ms))
    dp = ctypes.POINTER(ctypes.c_double)
    for i, p in enumerate(probs):
        m = max_shape(p["steps"], p["d"], p["pncc"])
        r = np.zeros(p["d"])
        b = np.zeros(m)
        lib.mce_draw_reference_constants(seed * 100003 + i, p["d"], m, 8, r.ctypes.data_as(dp), b.ctypes.data_as(dp))
        rp[i] = r
        bp[i, :m] = b
    return rp, bp


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-i", "0", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_figures():
    """Figures bench.py takes from the committed ncu summaries: lines
    'bench: <name> <group> <value>' in profiles/*.md (DRAM traffic per
    algorithmic byte and FP64-pipe activity of a kernel group)."""
    out = {}
    pdir = os.path.join(ROOT, "profiles")
    try:
        names = sorted(os.listdir(pdir))
    except OSError:
        return out
    for fn in names:
        if not fn.endswith(".md"):
            continue
        for ln in open(os.path.join(pdir, fn)):
            if ln.startswith("bench: "):
                f = ln.split()
                if len(f) == 4:
                    out[(f[1], f[2])] = float(f[3])
    return out


def combine_ranks(dev_ms, wall_s, terms, device):
    """Whole-job figures of a replicas run (one independent batch per rank, no
    data-path collective): the slowest rank's device and wall times per pass
    and the terms all ranks processed.  A single process returns its own."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return dev_ms, wall_s, terms
    t = torch.tensor([dev_ms, wall_s], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([float(terms)], device=device, dtype=torch.float64)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(t[0]), float(t[1]), int(round(float(n[0])))


def _cpu_pass_fn(probs, consts, seeds, threads):
    """A function timing one pass of the CPU implementation over a list of
    estimator indices: the reference's own C++ (oracle/_ref, built on this
    host from the reference's headers) in a process pool when it is built,
    else the oracle port on a thread pool.  Returns (fn, kind, closer)."""
    import oracle
    oracle.build(with_reference=True)
    if oracle.reference_available():
        pool = oracle.ReferencePool(probs, seeds, threads)
        return pool.run, "reference", pool.close

    def port(idx):
        return oracle.run_oracle_batch([probs[i] for i in idx], [consts[i] for i in idx], threads)[1]
    return port, "port", lambda: None


def _post_mu_terms(probs, consts, idx, threads):
    import oracle
    oracle.build(with_reference=False)
    return oracle.run_oracle_batch([probs[i] for i in idx], [consts[i] for i in idx], threads)[0]


def cpu_sample(probs, consts, seeds, target_seconds):
    """Bounded sample of the same workload for the CPU baseline: every k-th
    estimator, k chosen so one pass needs about target_seconds, on all host
    cores."""
    threads = os.cpu_count() or 1
    fn, kind, close = _cpu_pass_fn(probs, consts, seeds, threads)
    try:
        k = 64
        t = fn(list(range(0, len(probs), k)))
        if t < target_seconds * 0.3:
            k = max(1, int(k * t / (target_seconds * 0.5)))
        idx = list(range(0, len(probs), k))
        t = fn(idx)
    finally:
        close()
    n = _post_mu_terms(probs, consts, idx, threads)
    return {"value": n / t, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": "every %d-th estimator of the batch (%d estimators, %d post-MU terms, %.1f s)"
                      % (k, len(idx), n, t)}


def run_reference(args):
    """Reference arm: the reference's own C++ (oracle/_ref, compiled on this
    host from the reference's headers; serial build, one process per host
    core, one estimator per task) stepping the whole batch of the gb300 arm
    -- the same 4096 estimators, measurement histories and rand()-drawn
    constants -- once per step.  Falls back to the oracle port on all host
    threads where the reference is not built."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from cauchyfriendly_gb300 import workloads as W
    import oracle
    probs = W.batched_three_state(args.n_est, seed=args.seed)
    seeds = [args.seed * 100003 + i for i in range(len(probs))]
    consts = [oracle.draw_reference_constants(s, p["d"], oracle.max_shape_of(p)) for s, p in zip(seeds, probs)]
    threads = os.cpu_count() or 1
    fn, kind, close = _cpu_pass_fn(probs, consts, seeds, threads)
    idx = list(range(len(probs)))
    try:
        for _ in range(args.warmup):
            fn(idx)
        tot_t = 0.0
        for _ in range(args.steps):
            tot_t += fn(idx)
    finally:
        close()
    # terms present after each MU of the batch (the GPU path and the reference agree exactly)
    n_terms = _post_mu_terms(probs, consts, idx, threads)
    v = n_terms * args.steps / tot_t
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "n_estimators": args.n_est, "seed": args.seed,
                                            "terms_per_step": n_terms},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": "the whole batch per step (%d estimators, %d post-MU terms); %s" %
                                       (len(probs), n_terms,
                                        "the reference's C++, serial build, %d processes" % threads
                                        if kind == "reference" else "oracle port, %d threads" % threads)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def plain_sample(probs, consts, stride):
    """The plain path the metric compares against: one estimator per handle
    (mce_create / mce_step, one launch sequence per estimator and update), on
    every stride-th estimator of the batch.  Returns post-MU terms, device
    seconds and wall seconds of the steps (handle creation excluded)."""
    from cauchyfriendly_gb300 import CauchyEstimator
    import torch
    terms = 0
    dev = wall = 0.0
    for i in range(0, len(probs), stride):
        p = probs[i]
        ms = (p["steps"] - 1) * p["pncc"] + p["d"]
        est = CauchyEstimator(p["A0"], p["p0"], p["b0"], p["steps"], p["d"], 0, p["pncc"], p["p"],
                              root_point=consts[0][i], b_pert=consts[1][i][:ms])
        d0 = est._lib.mce_device_time_ms(est._h)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(p["steps"]):
            est.step(p["msmts"][k, 0], p["Phi"], p["Gamma"], p["beta"], p["H"][0], p["gamma"][0])
        torch.cuda.synchronize()
        wall += time.perf_counter() - t0
        dev += (est._lib.mce_device_time_ms(est._h) - d0) / 1e3
        terms += int(est._lib.mce_post_mu_terms(est._h))
        est.close()
    return terms, dev, wall


def run_windows5(args):
    """Sliding-window 5-state LTV MCE (window 6, 2 measurements per step),
    run for --window-steps steps; terms/s over the device time of all window
    updates (value) and the wall clock of the manager steps (e2e)."""
    import torch
    from cauchyfriendly_gb300 import windows, workloads as W
    torch.cuda.set_device(0)
    prob = W.five_state_ltv_windows(seed=args.seed, steps=args.window_steps)
    Wn = 6
    A0, p0, b0 = prob["A0"][None], prob["p0"][None], prob["b0"][None]

    import ctypes
    from cauchyfriendly_gb300 import _lib
    lib = _lib.load()
    groups = [lib.mce_kernel_group_name(k).decode() for k in range(lib.mce_num_kernel_groups())]
    kms = {g: 0.0 for g in groups}

    def one_pass():
        mgr = windows.SlidingWindowManager(Wn, A0, p0, b0, 5, 2, 2)
        for s in mgr.slots:
            lib.mce_set_profiling(s.est._h, 1)
            lib.mce_clear_profile(s.est._h)
        t0 = time.perf_counter()
        dev0 = [lib.mce_device_time_ms(s.est._h) for s in mgr.slots]
        for k in range(prob["steps"]):
            mgr.step(prob["msmts"][k][None], prob["Phi"][k][None], prob["Gamma"][None], prob["beta"][None],
                     prob["H"][None], prob["gamma"][None])
        wall = time.perf_counter() - t0
        dev = sum(lib.mce_device_time_ms(s.est._h) for s in mgr.slots) - sum(dev0)
        terms = mgr.total_post_mu_terms()
        per = {}
        for k, g in enumerate(groups):
            tot = 0.0
            for s in mgr.slots:
                ms, nl, ab, af = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double(), ctypes.c_double()
                lib.mce_kernel_group_stats(s.est._h, k, ctypes.byref(ms), ctypes.byref(nl), ctypes.byref(ab),
                                           ctypes.byref(af))
                tot += ms.value
            per[g] = tot
        mgr.close()
        return terms, dev / 1e3, wall, per

    for _ in range(max(0, args.warmup - 2)):
        one_pass()
    tot_terms = tot_dev = tot_wall = 0.0
    for _ in range(args.steps):
        n, dv, wl, per = one_pass()
        tot_terms += n
        tot_dev += dv
        tot_wall += wl
        for g in groups:
            kms[g] += per[g]
    ksum = sum(kms.values()) or 1.0
    line = {"metric": METRIC, "value": tot_terms / tot_dev, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot_dev / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "sliding-window 5-state LTV MCE, window 6, 2 msmts/step, %d steps"
                                   % args.window_steps, "terms_per_step": tot_terms / args.steps},
            "e2e": {"value": tot_terms / tot_wall, "unit": UNIT, "wall_s_per_step": tot_wall / args.steps},
            "kernel_time_share": {g: round(kms[g] / ksum, 4) for g in groups},
            "kernel_ms_per_step": {g: round(kms[g] / args.steps, 3) for g in groups}}
    print(json.dumps(line), flush=True)



def _adjoint_ref_forward(job):
    """One forward run of the adjoint workload's sliding-window problem
    through the reference's own PySlidingWindowManager
    (scripts/swig/cauchy/cauchy_estimator.py, the unmodified copy in
    oracle/_ref) over its C++ (oracle/_ref, serial build); seconds, or None
    where the copy is absent."""
    seed, steps, Wn = job
    # the reference's manager prints as it shuts windows down: keep it off
    # this process's stdout, which the bench's one JSON line shares
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    sys.stdout = open(os.devnull, "w")
    import oracle
    from oracle import ref_pycauchy
    from cauchyfriendly_gb300 import workloads as W
    ce = oracle.reference_python_api(ref_pycauchy)
    if ce is None:
        return None
    prob = W.four_state_lti(seed=seed, steps=steps)
    t0 = time.perf_counter()
    mgr = ce.PySlidingWindowManager("lti", Wn, swm_debug_print=False, win_debug_print=False)
    mgr.initialize_lti(prob["A0"], prob["p0"], prob["b0"], prob["Phi"], None, prob["Gamma"], prob["beta"],
                       prob["H"], prob["gamma"])
    for k in range(steps):
        mgr.step(prob["msmts"][k], None)
    mgr.shutdown()
    return time.perf_counter() - t0


def run_adjoint(args):
    """Adjoint workload (the 4-state LTI sliding-window configuration: Phi
    random with spectral radius 0.95, Gamma 4x1 and H 1x4 N(0,1), beta 0.1,
    gamma 0.2, window 7, 100 steps): one gradient = the sliding-window
    log-likelihood sum_k log fz_k and its gradient with respect to (beta,
    gamma, p0, Phi, Gamma, H) with the window checkpoints held fixed
    (cauchyfriendly_gb300.adjoint.windowed_log_likelihood: the manager run,
    every window life recomputed from its checkpoint, the reverse pass).
    value: gradients/s (wall clock of the public call); forward_s: the same
    manager run alone; the ratio is the gradient's cost in forward runs."""
    import torch
    from cauchyfriendly_gb300 import windows, workloads as W
    from cauchyfriendly_gb300.adjoint import windowed_log_likelihood
    import oracle
    torch.cuda.set_device(0)
    steps = args.adjoint_steps
    prob = W.four_state_lti(seed=args.seed, steps=steps)
    Wn = 7
    ms = (Wn - 1) * 1 + 4
    cs = [oracle.draw_reference_constants(1000 + w, 4, ms) for w in range(Wn)]
    rp = np.stack([c[0] for c in cs])
    bp = np.stack([c[1] for c in cs])

    def forward():
        t0 = time.perf_counter()
        mgr = windows.SlidingWindowManager(Wn, prob["A0"][None], prob["p0"][None], prob["b0"][None], 4, 1, 1,
                                           root_point=rp[:, None, :], b_pert=bp[:, None, :])
        for k in range(steps):
            mgr.step(prob["msmts"][k][None], prob["Phi"][None], prob["Gamma"][None], prob["beta"][None],
                     prob["H"][None], prob["gamma"][None])
        terms = mgr.total_post_mu_terms()
        mgr.close()
        return time.perf_counter() - t0, terms

    def gradient():
        t0 = time.perf_counter()
        r = windowed_log_likelihood(prob, Wn, rp, bp)
        return time.perf_counter() - t0, r

    for _ in range(max(1, args.warmup - 2)):
        forward()
        gradient()
    fw, gw, terms, r = 0.0, 0.0, 0, None
    for _ in range(args.steps):
        t, terms = forward()
        fw += t
        t, r = gradient()
        gw += t
    fw /= args.steps
    gw /= args.steps
    line = {"metric": "MCE log-likelihood gradients/s (1 GB300, FP64; sliding window, checkpointed adjoint)",
            "value": 1.0 / gw, "unit": "gradients/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * gw, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "4-state LTI sliding-window MCE, window 7, %d steps, 1 msmt/step" % steps,
                       "params": 30, "window_lives": len(r["starts"]), "terms_per_forward": terms},
            "forward_s": fw, "gradient_s": gw, "gradient_over_forward": gw / fw,
            "gradient_ms_split": {k: round(float(v) / 1.0, 1) for k, v in
                                  zip(("step_path", "forward_tape", "table_reverse", "record_chain"),
                                      r["timing_ms"])},
            "loglik": r["loglik"], "grad_norm": float(np.sqrt(sum(float(np.sum(v ** 2)) for v in r["grad"].values())))}
    if not args.no_cpu_baseline:
        # The reference has no derivatives: its gradient is central
        # differences of its own forward run, 2 x 30 runs.  One run per host
        # core, all at once; the gradient's time is 60 runs at that rate.
        import multiprocessing as mp
        cores = os.cpu_count() or 1
        t0 = time.perf_counter()
        with mp.get_context("spawn").Pool(cores) as pool:
            ts = pool.map(_adjoint_ref_forward, [(args.seed, steps, Wn)] * cores)
        wall = time.perf_counter() - t0
        if all(t is not None for t in ts):
            runs_per_s = cores / wall
            line["cpu_baseline"] = {"value": runs_per_s / 60.0, "unit": "gradients/s", "cores": cores,
                                    "kind": "reference",
                                    "sample": "the reference's PySlidingWindowManager forward run (serial C++), one "
                                              "per core at once (%.1f s wall, %.1f s per run); a gradient = 2 x 30 "
                                              "runs (central differences)" % (wall, max(ts))}
    print(json.dumps(line), flush=True)


def run_rel2d(args):
    """Relative-then-transformed 2-D system (rel = secondary - primary through
    Trel = rows e0, e2) of two 5-state estimators with two measurements per
    step, after 6 updates each (3,076 x 3,962 = 12.2 M term pairs): one
    evaluation = the pair cache with term approximation (eps 1e-8), the
    relative moments and a 17 x 17 pdf grid around the relative mean.
    value: pairs/s over the device time of the three phases (CUDA events on
    the object's stream; the kept-pair compaction counts with the moments);
    e2e: pairs/s over the wall clock of the public calls
    (RelativeSystem2D(...) + grid())."""
    import ctypes
    import torch
    from cauchyfriendly_gb300 import CauchyEstimator, RelativeSystem2D, _lib, workloads as W
    torch.cuda.set_device(0)
    lib = _lib.load()
    probs = [W.five_state_two_msmt(seed=s, steps=4) for s in (0, 1)]
    updates = args.rel_updates
    ests, consts = [], []
    for i, q in enumerate(probs):
        ms = (q["steps"] - 1) * q["pncc"] + q["d"]
        rp, bp = np.zeros(q["d"]), np.zeros(ms)
        P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        lib.mce_draw_reference_constants(40 + i, q["d"], ms, 1, P(rp), P(bp))
        consts.append((rp, bp))
        est = CauchyEstimator(q["A0"], q["p0"], q["b0"], q["steps"], q["d"], q["cmcc"], q["pncc"], q["p"],
                              root_point=rp, b_pert=bp)
        n = 0
        for k in range(q["steps"]):
            for sub in range(q["p"]):
                if n < updates:
                    est.step(q["msmts"][k, sub], q["Phi"][k] if q["Phi"].ndim == 3 else q["Phi"], q["Gamma"],
                             q["beta"], q["H"][sub], q["gamma"][sub])
                    n += 1
        ests.append(est)
    T = np.zeros((2, 5))
    T[0, 0] = T[1, 2] = 1.0
    nu = np.array([0.3, -0.2, 0.5, -0.7, 0.1])

    def grid_of(mom):
        mu = mom["mean"].real
        sd = np.sqrt(np.abs(np.diag(mom["cov"].real)))
        sd = np.where(np.isfinite(sd) & (sd > 1e-6), sd, 1.0)
        return (mu[0] - 3 * sd[0], mu[0] + 3 * sd[0], 6 * sd[0] / 16), (mu[1] - 3 * sd[1], mu[1] + 3 * sd[1],
                                                                        6 * sd[1] / 16)

    def one():
        t0 = time.perf_counter()
        rs = RelativeSystem2D(ests[0], ests[1], T, with_term_approx=True, term_approx_eps=1e-8, bar_nu_full=nu)
        gx, gy = grid_of(rs.moments)
        X, Y, Z, nx, ny = rs.grid(*gx, *gy)
        wall = time.perf_counter() - t0
        out = (rs.pairs, rs.terms, rs.device_ms(), wall, nx * ny, rs.launch_count())
        rs.close()
        return out

    for _ in range(args.warmup):
        one()
    torch.cuda.synchronize()
    clk = ClockSampler()
    clk.start()
    tot = {"pairs": 0.0, "moments": 0.0, "grid": 0.0}
    walls, pairs, kept, npts, launches = 0.0, 0, 0, 0, 0
    for _ in range(args.steps):
        pairs, kept, dm, wl, npts, nl = one()
        launches += nl
        walls += wl
        for k in tot:
            tot[k] += dm[k]
    torch.cuda.synchronize()
    clocks = clk.stop()
    dev_s = sum(tot.values()) / 1e3 / args.steps
    wall_s = walls / args.steps
    # algorithmic work: per pair the two terms read (A, p, b), a cache row of
    # (mp + ms) cells written (6 doubles a cell + 5) with its kept flag and
    # moment row; per grid point and kept term, 56 FP64 flops a cell
    tps = [e.terms_per_shape(0).astype(np.float64) for e in ests]
    mp = np.arange(len(tps[0]))
    msh = np.arange(len(tps[1]))
    Np, Ns = tps[0].sum(), tps[1].sum()
    rd = lambda m: 8.0 * (m * 5 + m + 5)
    pair_bytes = Ns * float((tps[0] * rd(mp)).sum()) + Np * float((tps[1] * rd(msh)).sum())
    cells_sum = Ns * float((tps[0] * mp).sum()) + Np * float((tps[1] * msh).sum())
    pair_bytes += 8.0 * (6 * cells_sum + 5 * pairs) + (4 + 112) * pairs
    mean_cells = cells_sum / max(1, pairs)
    grid_flops = 56.0 * npts * kept * mean_cells
    peak, peak_kind = measured_peaks()
    ms_pairs, ms_grid = tot["pairs"] / args.steps, tot["grid"] / args.steps
    top = "grid" if ms_grid >= ms_pairs else "pairs"
    roofline = {"bound": "hbm", "kernel": "k_rel2d_points" if top == "grid" else "k_rel2d_pairs",
                "achieved": (pair_bytes / (ms_pairs / 1e3) if top == "pairs" else
                             8.0 * kept * (6 * mean_cells + 5) / (ms_grid / 1e3)) / 1e9,
                "peak": peak, "unit": "GB/s", "peak_source": peak_kind, "traffic": None,
                "note": "FP64-bound: the grid kernel reads the pair cache from L2 once per point block; the FP64 "
                        "pipe is its limit (see fp64)",
                "fp64": {"algorithmic_tflops": grid_flops / (ms_grid / 1e3) / 1e12 if ms_grid > 0 else 0.0,
                         "nominal_peak_tflops": 1.25}}
    roofline["frac"] = roofline["achieved"] / peak
    line = {"metric": "relative-system 2-D term pairs/s (cache + moments + 17x17 pdf grid, FP64)",
            "value": pairs / dev_s, "unit": "pairs/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dev_s * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "relative 2-D system of two 5-state, 2-measurement estimators after %d updates "
                                   "(Trel rows e0, e2)" % updates, "pairs": int(pairs), "kept_terms": int(kept),
                       "grid_points": int(npts), "l2": "the pair cache (several GB) exceeds L2"},
            "e2e": {"value": pairs / wall_s, "unit": "pairs/s", "h2d_bytes_per_step": int(8 * (10 + 5 + 2 * npts)),
                    "d2h_bytes_per_step": int(8 * (14 + npts) + 4 * pairs), "wall_s_per_step": wall_s},
            "gpu_launches": launches,
            "device_ms_per_step": {k: round(v / args.steps, 3) for k, v in tot.items()},
            "roofline": roofline, "clocks": clocks}
    if not args.no_cpu_baseline:
        import oracle
        oracle.build(with_reference=False)
        # calibrate a per-process sample on one core, then run one process per
        # host core, each on its own share of the pairs (offset i modulo the
        # stride), as the reference spreads the pairs over NUM_CPUS threads
        t1 = _rel2d_cpu_share((probs, consts, updates, T, nu, 512, 0))[1]
        cores = os.cpu_count() or 1
        stride = int(max(cores, 512 * t1 / max(args.cpu_seconds, 1e-3)))
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(cores) as pool:
            t0 = time.perf_counter()
            res = pool.map(_rel2d_cpu_share, [(probs, consts, updates, T, nu, stride, i) for i in range(cores)])
            wall = time.perf_counter() - t0
        done = sum(r[0] for r in res)
        slowest = max(r[1] for r in res)
        line["cpu_baseline"] = {"value": done / slowest, "unit": "pairs/s", "cores": cores, "kind": "port",
                                "sample": "%d processes, each every %d-th pair of the same evaluation (cache, "
                                          "moments, 17x17 grid) at its own offset: %d pairs, slowest share %.1f s "
                                          "(%.1f s with process start)" % (cores, stride, done, slowest, wall)}
    for e in ests:
        e.close()
    print(json.dumps(line), flush=True)


def _nd_problem():
    from cauchyfriendly_gb300 import workloads as W
    return W.four_state_lti(seed=11, steps=7), 6


def _nd_points(mo, d, n):
    mu = mo["mean"].real
    sd = np.sqrt(np.abs(np.diag(mo["cov"].real)))
    rng = np.random.Generator(np.random.PCG64(3))
    return mu + sd * rng.standard_normal((n, d)) * np.resize([0.5, 1.5, 4.0], n)[:, None]


def _nd_cpu_share(job):
    """One process's share of the N-D pdf baseline: the reference's own
    estimator (oracle/_ref, serial build) stepped like the GPU's, then
    PointWiseNDimCauchyCPDF::evaluate_cpdf at its points; (points, seconds)."""
    import oracle
    seed, X = job
    prob, updates = _nd_problem()
    ref = oracle.Reference(prob, seed=seed)
    n = 0
    for k in range(prob["steps"]):
        for s in range(prob["p"]):
            if n < updates:
                ref.step(k, s)
                n += 1
    t0 = time.perf_counter()
    for x in X:
        ref.cpdf_nd(x)
    t1 = time.perf_counter() - t0
    ref.close()
    return len(X), t1


def run_cpdfnd(args):
    """The N-D conditional pdf (PointWiseNDimCauchyCPDF::evaluate_cpdf) of a
    4-state LTI estimator after 6 updates (3,428 terms) at --nd-points points
    around its mean (0.5, 1.5 and 4 standard deviations) per step, through
    mce_cpdf_nd (one call, host points in, host values out): points/s over
    the wall clock of the call (value and e2e; the call synchronises between
    its lowering levels).  CPU baseline: the reference's own evaluate_cpdf,
    one process per host core, each on its share of a point sample."""
    import torch
    import oracle
    from cauchyfriendly_gb300 import CauchyEstimator
    torch.cuda.set_device(0)
    prob, updates = _nd_problem()
    ref = oracle.Reference(prob, seed=77) if os.path.exists(os.path.join(oracle.REF_OUT, "libmce_ref_serial.so")) \
        else None
    if ref is not None:
        rp, bp = ref.constants()
        ref.close()
    else:
        rp, bp = oracle.draw_reference_constants(77, prob["d"], oracle.max_shape_of(prob))
    est = CauchyEstimator(prob["A0"], prob["p0"], prob["b0"], prob["steps"], prob["d"], 0, prob["pncc"], prob["p"],
                          root_point=rp, b_pert=bp)
    n = 0
    for k in range(prob["steps"]):
        for s in range(prob["p"]):
            if n < updates:
                est.step(prob["msmts"][k, s], prob["Phi"], prob["Gamma"], prob["beta"], prob["H"][s],
                         prob["gamma"][s])
                n += 1
    X = _nd_points(est.moments(), prob["d"], args.nd_points)
    for _ in range(args.warmup):
        est.cpdf_nd(X)
    torch.cuda.synchronize()
    clk = ClockSampler()
    clk.start()
    l0 = int(est._lib.mce_launch_count(est._h))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        est.cpdf_nd(X)
    wall = (time.perf_counter() - t0) / args.steps
    launches = int(est._lib.mce_launch_count(est._h)) - l0
    clocks = clk.stop()
    line = {"metric": "N-D conditional pdf points/s (FP64, PointWiseNDimCauchyCPDF::evaluate_cpdf)",
            "value": len(X) / wall, "unit": "points/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": wall * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "4-state LTI estimator after 6 updates (%d terms), %d points at 0.5/1.5/4 "
                                   "standard deviations" % (est.num_terms(), len(X))},
            "e2e": {"value": len(X) / wall, "unit": "points/s", "h2d_bytes_per_step": int(X.nbytes),
                    "d2h_bytes_per_step": int(16 * len(X)), "wall_s_per_step": wall},
            "gpu_launches": launches, "clocks": clocks,
            "note": "value and e2e are both the wall clock of mce_cpdf_nd (it reads sizes back between levels)"}
    if not args.no_cpu_baseline and ref is not None:
        import multiprocessing as mp
        cores = os.cpu_count() or 1
        # about cpu_seconds of work: 0.5 s a point on one core
        per = max(1, int(args.cpu_seconds / 0.5))
        Xs = _nd_points(est.moments(), prob["d"], per * cores)
        with mp.get_context("spawn").Pool(cores) as pool:
            res = pool.map(_nd_cpu_share, [(77, Xs[i * per:(i + 1) * per]) for i in range(cores)])
        done = sum(r[0] for r in res)
        slowest = max(r[1] for r in res)
        line["cpu_baseline"] = {"value": done / slowest, "unit": "points/s", "cores": cores, "kind": "reference",
                                "sample": "%d processes, %d points each (the same estimator and point "
                                          "distribution), slowest %.1f s" % (cores, per, slowest)}
    est.close()
    print(json.dumps(line), flush=True)


def _rel2d_cpu_share(job):
    """One process's share of the relative-system CPU baseline: the oracle's
    two estimators stepped as the GPU ones, then every stride-th pair from
    offset; returns (pairs, seconds of the evaluation)."""
    import oracle
    probs, consts, updates, T, nu, stride, offset = job
    orcs = []
    for q, c in zip(probs, consts):
        o = oracle.Oracle(q, *c)
        n = 0
        for k in range(q["steps"]):
            for sub in range(q["p"]):
                if n < updates:
                    o.step(k, sub)
                    n += 1
        orcs.append(o)
    t0 = time.perf_counter()
    r = oracle.oracle_rel2d(orcs[0], orcs[1], T, nu, (-1.0, 1.0, 0.125), (-1.0, 1.0, 0.125), pair_stride=stride,
                            pair_offset=offset)
    t1 = time.perf_counter() - t0
    for o in orcs:
        o.close()
    return r["pairs"], t1


def run_window7(args):
    """One window of the 7-state LTV model of the batched 7-state
    sliding-window configuration (workloads.seven_state_ltv_windows: Gamma
    7x2, H 2x7, two measurements per step; a window of 8 steps is 16
    updates, up to (8-1)*2+7 = 21 hyperplanes per term), one estimator from
    the initial statistics, update by update while the g-tables fit: the run
    stops before an update whose cells, projected with the largest growth
    factor seen so far, would pass --max-cells.  Reports per update the
    terms, g-table cells and device ms, and the memory the next updates would
    need.  value: post-MU terms / device time over the updates run;
    cpu_baseline: the reference's C++ (serial build; the oracle port where it
    is not built) over the first --cpu-updates updates, with the GPU's terms/s
    on the same updates beside it."""
    import ctypes
    import torch
    import oracle
    from cauchyfriendly_gb300 import CauchyEstimator, _lib
    from cauchyfriendly_gb300 import workloads as W
    torch.cuda.set_device(0)
    lib = _lib.load()
    Wn = 8
    prob = W.seven_state_ltv_windows(seed=args.seed, steps=Wn)
    ms = oracle.max_shape_of(prob)
    have_ref = os.path.exists(os.path.join(oracle.REF_OUT, "libmce_ref_serial.so"))
    if have_ref:
        ref = oracle.Reference(prob, seed=500)
        rp, bp = ref.constants()
        ref.close()
    else:
        rp, bp = oracle.draw_reference_constants(500, prob["d"], ms)

    def gpu_run():
        est = CauchyEstimator(prob["A0"], prob["p0"], prob["b0"], Wn, 7, 0, 2, 2, root_point=rp, b_pert=bp)
        rows, prev_cells, growth = [], None, 1.0
        stop = None
        for k in range(Wn):
            for j in range(2):
                if prev_cells is not None and prev_cells * growth > args.max_cells:
                    stop = "next update projected at %.3g cells (growth %.1fx) > --max-cells %.3g" % (
                        prev_cells * growth, growth, args.max_cells)
                    break
                pm0 = est.post_mu_terms()
                est.step(prob["msmts"][k, j], prob["Phi"][k], prob["Gamma"], prob["beta"], prob["H"][j],
                         prob["gamma"][j])
                cells = int(lib.mce_total_cells(est._h, 0))
                rows.append({"update": 2 * k + j, "terms": int(est.num_terms()),
                             "post_mu_terms": int(est.post_mu_terms() - pm0), "cells": cells,
                             "device_ms": round(float(est.last_step_ms()), 3), "errors": int(est.errors())})
                if prev_cells:
                    growth = max(growth, cells / prev_cells)
                prev_cells = cells
            if stop:
                break
        est.close()
        return rows, stop, growth

    for _ in range(max(0, args.warmup - 2)):
        gpu_run()
    rows, stop, growth = gpu_run()
    terms = sum(r["post_mu_terms"] for r in rows)
    dev_s = sum(r["device_ms"] for r in rows) / 1e3
    # the memory the rest of the window would take (16 bytes per g-table cell;
    # the terms' records are small beside it), each update grown by the last
    # growth factor of its kind: a step's first update (time propagation adds
    # the Gamma hyperplanes) or its second (measurement update only)
    kind_growth = {}
    for r0, r1 in zip(rows, rows[1:]):
        if r0["cells"] > 0:
            kind_growth[r1["update"] % 2] = r1["cells"] / r0["cells"]
    proj, c = [], rows[-1]["cells"]
    for u in range(len(rows), 2 * Wn):
        c *= kind_growth.get(u % 2, growth)
        proj.append({"update": u, "cells": float("%.3g" % c), "table_gb": float("%.3g" % (16 * c / 1e9))})
    line = {"metric": METRIC, "value": terms / dev_s, "unit": UNIT, "n_gpus": 1, "steps": 1,
            "warmup": args.warmup, "ms_per_step": 1e3 * dev_s, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "one window of the 7-state LTV model (window 8, 2 msmts/step, up to 21 "
                                   "hyperplanes per term), updates 0..%d" % (len(rows) - 1),
                       "max_cells": args.max_cells},
            "updates": rows, "stopped": stop,
            "growth_per_update_kind": {"first_of_step": kind_growth.get(0), "second_of_step": kind_growth.get(1)},
            "projected_rest_of_window": proj}
    if not args.no_cpu_baseline:
        nu = min(args.cpu_updates, len(rows))
        if have_ref:
            cpu = oracle.Reference(prob, seed=500)
            kind = "reference"
        else:
            cpu = oracle.Oracle(prob, rp, bp)
            kind = "port"
        t0 = time.perf_counter()
        n = 0
        for k in range(Wn):
            for j in range(2):
                if n < nu:
                    cpu.step(k, j)
                    n += 1
        t_cpu = time.perf_counter() - t0
        cpu.close()
        sub_terms = sum(r["post_mu_terms"] for r in rows[:nu])
        sub_dev = sum(r["device_ms"] for r in rows[:nu]) / 1e3
        line["cpu_baseline"] = {"value": sub_terms / t_cpu, "unit": UNIT, "cores": 1, "kind": kind,
                                "sample": "updates 0..%d of the window, serial (%d post-MU terms, %.1f s)"
                                          % (nu - 1, sub_terms, t_cpu),
                                "gpu_same_updates": sub_terms / sub_dev}
    print(json.dumps(line), flush=True)


def run_mle(args):
    """Maximum-likelihood tuning of log(beta), log(gamma) and log(p0) shared
    by --mle-estimators LTV sliding-window estimators of --mle-states states
    (workloads.ltv_windows, seeds 0..n-1, each its own model and
    measurements; Gamma d x 2, H 2 x d, two measurements per step), step
    counts uniform in 100..150, window --mle-window, with Adam (lr 0.05) on
    the gradient of the summed sliding-window log-likelihood
    (adjoint.windowed_log_likelihood_batch: one window manager for all
    estimators, every window life recomputed in batched adjoint runs),
    starting from the generating scales times 3.  This is the batched 7-state
    configuration's pipeline; at 7 states a window short enough to
    recompute (at most 3 steps, 6 measurements) leaves the windows without a
    covariance (the manager finds no usable window and stops, as the
    reference's does), and a window of 8 does not fit in the GPU's memory
    (--workload window7), so it runs at --mle-states.  Short windows meet
    steps where every window of a manager has an error code (the reference
    exits there); the manager takes the fullest window then and counts the
    steps (no_window_steps per iteration).  value: gradients/s (each
    gradient covers every estimator); the log-likelihood and scales per
    iteration."""
    import torch
    from cauchyfriendly_gb300 import workloads as W
    from cauchyfriendly_gb300.adjoint import windowed_log_likelihood_batch
    import oracle
    torch.cuda.set_device(0)
    n, Wn, dd = args.mle_estimators, args.mle_window, args.mle_states
    rng = np.random.Generator(np.random.PCG64(args.seed + 7))
    steps = [int(k) for k in rng.integers(100, 151, size=n)]
    probs = [W.ltv_windows(dd, seed=args.seed + i, steps=150) for i in range(n)]
    ms = oracle.max_shape_of({"steps": Wn, "d": dd, "pncc": 2})
    cs = [oracle.draw_reference_constants(700 + w, dd, ms) for w in range(Wn)]
    rp = np.stack([c[0] for c in cs])
    bp = np.stack([c[1] for c in cs])
    true = {"beta": probs[0]["beta"], "gamma": probs[0]["gamma"], "p0": probs[0]["p0"]}
    theta = {k: torch.tensor(np.log(3.0 * np.asarray(v)), dtype=torch.float64, requires_grad=True)
             for k, v in true.items()}
    opt = torch.optim.Adam(list(theta.values()), lr=0.05)
    hist, tg = [], []
    stopped = None
    for it in range(args.mle_iters):
        sc = {k: np.exp(v.detach().numpy()) for k, v in theta.items()}
        t0 = time.perf_counter()
        try:
            r = windowed_log_likelihood_batch(probs, Wn, rp, bp, sc["beta"], sc["gamma"], sc["p0"], steps=steps,
                                              no_window="fullest")
        except RuntimeError as e:
            stopped = "iteration %d: %s" % (it, e)
            break
        tg.append(time.perf_counter() - t0)
        opt.zero_grad()
        for k, v in theta.items():
            # maximise the log-likelihood: minimise its negative; d/dlog s = s d/ds
            v.grad = torch.as_tensor(-sc[k] * r["grad"][k], dtype=torch.float64)
        opt.step()
        hist.append({"iter": it, "loglik": r["loglik"], "seconds": round(tg[-1], 3),
                     "no_window_steps": int(r["no_window_steps"]),
                     "beta": [float(x) for x in sc["beta"]], "gamma": [float(x) for x in sc["gamma"]],
                     "p0_mean": float(np.mean(sc["p0"]))})
        print(json.dumps(hist[-1]), file=sys.stderr, flush=True)
    timed = tg[1:] if len(tg) > 1 else tg
    g_s = float(np.mean(timed)) if timed else float("nan")
    line = {"metric": "MCE log-likelihood gradients/s (1 GB300, FP64; batched sliding-window adjoint)",
            "value": 1.0 / g_s, "unit": "gradients/s", "n_gpus": 1, "steps": len(timed), "warmup": len(tg) - len(timed),
            "ms_per_step": 1e3 * g_s, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "%d x %d-state LTV sliding-window MCE, window %d, 2 msmts/step, steps U{100..150}, "
                                   "Adam on log(beta, gamma, p0)" % (n, dd, Wn),
                       "estimators": n, "states": dd, "window": Wn, "iterations": args.mle_iters,
                       "estimator_steps": int(sum(steps))},
            "iterations": hist, "stopped": stopped,
            "true_scales": {k: [float(x) for x in np.asarray(v).reshape(-1)] for k, v in true.items()}}
    print(json.dumps(line), flush=True)


def autotune_summary(table, passes, off):
    """The autotuner's settled block sizes per kernel as {log2 items: block}."""
    if off:
        return {"enabled": False}
    blocks = {}
    for r in table:
        blocks.setdefault(r["kernel"], {})[str(r["log2_items"])] = r["block"]
    return {"enabled": True, "settled_keys": len(table), "tuning_passes": passes, "blocks": blocks}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "windows5":
        run_windows5(args)
        return
    if args.workload == "rel2d":
        run_rel2d(args)
        return
    if args.workload == "adjoint":
        run_adjoint(args)
        return
    if args.workload == "cpdfnd":
        run_cpdfnd(args)
        return
    if args.workload == "window7":
        run_window7(args)
        return
    if args.workload == "mle":
        run_mle(args)
        return
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from cauchyfriendly_gb300 import BatchedCauchyEstimator, workloads as W
    from cauchyfriendly_gb300 import _lib
    # each rank runs its own replica of the batch (independent estimators shard trivially)
    probs = W.batched_three_state(args.n_est, seed=args.seed + rank)
    consts = constants(probs, args.seed + rank)
    B = batch_arrays(probs)
    est = BatchedCauchyEstimator(B["A0"], B["p0"], B["b0"], B["steps"], 3, 0, 1, 1, consts[0], consts[1])
    lib = _lib.load()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def one_pass():
        est.reset()
        t0 = time.perf_counter()
        est.run(B["msmts"], B["Phi"], B["Gamma"], B["beta"], B["H"], B["gamma"], shared_model=False, outputs=False)
        return time.perf_counter() - t0

    # algorithmic bytes / flops per kernel group: one untimed pass
    lib.mce_set_profiling(est._h, 2)
    lib.mce_clear_profile(est._h)
    one_pass()
    groups = [lib.mce_kernel_group_name(k).decode() for k in range(lib.mce_num_kernel_groups())]
    import ctypes
    alg = {}
    for k, g in enumerate(groups):
        ms, nl, ab, af = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double(), ctypes.c_double()
        lib.mce_kernel_group_stats(est._h, k, ctypes.byref(ms), ctypes.byref(nl), ctypes.byref(ab), ctypes.byref(af))
        alg[g] = (ab.value, af.value)
    lib.mce_set_profiling(est._h, 1)
    from cauchyfriendly_gb300 import autotune_configure, autotune_table
    tuning_passes = 0
    if args.no_autotune:
        autotune_configure(False)
    else:
        # untimed passes until the block-size autotuner settles every key it has seen
        prev, stable = -1, 0
        while tuning_passes < 16 and stable < 2:
            one_pass()
            tuning_passes += 1
            n = len(autotune_table())
            stable = stable + 1 if n == prev else 0
            prev = n
    for _ in range(max(0, args.warmup - 1)):
        one_pass()
    terms_per_pass = est.post_mu_terms()
    lib.mce_clear_profile(est._h)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler()
    clk.start()
    walls = []
    dev_ms_total = 0.0
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        before = lib.mce_device_time_ms(est._h)
        walls.append(one_pass())
        dev_ms_total += lib.mce_device_time_ms(est._h) - before
    torch.cuda.synchronize()
    clocks = clk.stop()
    launches = int(lib.mce_launch_count(est._h))
    kstats = {}
    for k, g in enumerate(groups):
        ms, nl, ab, af = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double(), ctypes.c_double()
        lib.mce_kernel_group_stats(est._h, k, ctypes.byref(ms), ctypes.byref(nl), ctypes.byref(ab), ctypes.byref(af))
        kstats[g] = (ms.value, nl.value)
    dev_ms = dev_ms_total / args.steps
    wall_s = sum(walls) / args.steps
    host_ms = {k: lib.mce_host_time_ms(est._h, i) / args.steps for i, k in enumerate(("step", "pack", "checks"))}
    dev_ms, wall_s, total_terms = combine_ranks(dev_ms, wall_s, terms_per_pass, "cuda")
    value = total_terms / (dev_ms / 1e3)
    e2e = total_terms / wall_s
    # roofline of the dominant kernel group (largest device time)
    top = max((g for g in kstats if g != "wait"), key=lambda g: kstats[g][0])
    top_ms, top_launches = kstats[top]
    ab, af = alg.get(top, (0.0, 0.0))
    secs = top_ms / 1e3 / args.steps  # per pass
    peak, peak_kind = measured_peaks()
    achieved = ab / secs / 1e9 if secs > 0 else 0.0
    figs = profile_figures()
    tr = figs.get(("traffic_bytes_per_alg_byte", top))
    per_launch = ab / max(1, top_launches / args.steps)
    roofline = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": tr * per_launch if tr else None,
                "alg_bytes_per_launch": per_launch,
                "launches_per_pass": top_launches / args.steps,
                "note": "FP64-bound: the FP64 pipe, not HBM, limits this kernel (see fp64)",
                "fp64": {"algorithmic_tflops": af / secs / 1e12 if secs > 0 else 0.0, "nominal_peak_tflops": 1.25,
                         "pipe_active_pct_ncu": figs.get(("fp64_pipe_active_pct", top)),
                         "frac_pipe": (figs[("fp64_pipe_active_pct", top)] / 100.0
                                       if ("fp64_pipe_active_pct", top) in figs else None),
                         "peak_source": "nominal GB300 FP64; pipe activity (the fraction of SM cycles the FP64 "
                                        "pipe is busy, the roof these kernels meet) from the committed ncu capture"}}
    alg_per_pass = {g: {"bytes": alg[g][0], "flops": alg[g][1]} for g in alg}
    share = {g: round(kstats[g][0] / max(1e-9, sum(v[0] for v in kstats.values())), 4) for g in kstats}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "n_estimators": args.n_est, "seed": args.seed,
                   "terms_per_step": terms_per_pass, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "256 MiB buffer written between passes; term state per pass is several GB"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(B["msmts"].nbytes + B["Phi"].nbytes
                                                                       + B["Gamma"].nbytes + B["beta"].nbytes
                                                                       + B["H"].nbytes + B["gamma"].nbytes),
                "d2h_bytes_per_step": int(B["steps"].sum() * (2 + 2 * 3 + 2 * 9) * 8), "wall_s_per_step": wall_s},
        "gpu_launches": launches,
        "host_ms_per_step": {k: round(v, 3) for k, v in host_ms.items()},
        "kernel_time_share": share,
        "kernel_ms_per_step": {g: round(kstats[g][0] / args.steps, 3) for g in kstats},
        "alg_per_pass": alg_per_pass,
        "roofline": roofline,
        "clocks": clocks,
        "autotune": autotune_summary(autotune_table(), tuning_passes, args.no_autotune),
    }
    if rank == 0 and not args.no_plain:
        # batched vs plain: the same estimators one handle at a time
        pt, pdev, pwall = plain_sample(probs, consts, args.plain_stride)
        line["plain"] = {"workload": "every %d-th estimator of the batch, one handle each (mce_create/mce_step)"
                                     % args.plain_stride, "terms": pt, "value_device": pt / pdev,
                         "value_wall": pt / pwall, "unit": UNIT}
        line["batched_over_plain"] = {"device": value / (pt / pdev), "wall": e2e / (pt / pwall)}
    if rank == 0 and not args.no_cpu_baseline:
        seeds = [args.seed * 100003 + i for i in range(len(probs))]
        line["cpu_baseline"] = cpu_sample(probs, list(zip(consts[0], consts[1])), seeds, args.cpu_seconds)
    est.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
