"""Generates the golden fixtures in this folder from the REFERENCE itself.

Runs the reference estimator (natsnyder1/CauchyFriendly, compiled from its own
headers by oracle/ref_harness.cpp, serial build) on seeded synthetic problems
and records, after every measurement update: the error bitmask, the term count,
terms per shape, the reported and raw moments, G_SCALE_FACTOR, and (for small
steps) every term's shape, A, p, b and sorted g-table.

It also records the reference's marginal 1-D pdf grids (cpdf1d_*.npz) after
a few updates of some of the same problems, the moments through a fixed
sequence of updates and extended-mode calls (ext_*.npz), and the
relative-then-transformed 2-D system of two estimators (rel2d_*.npz).

Needs the reference sources (only present where the fixtures are made):
    python tests/golden/make_golden.py          # everything
    python tests/golden/make_golden.py --cpdf   # the pdf fixtures only
    python tests/golden/make_golden.py --ext    # the extended-mode fixtures only
    python tests/golden/make_golden.py --rel    # the relative-system fixtures only
    python tests/golden/make_golden.py --postftr  # print_basic_info fixtures only
    python tests/golden/make_golden.py --wide   # terms above 16 hyperplanes only
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from cauchyfriendly_gb300 import workloads as W  # noqa: E402

TERM_DUMP_CAP = 700


def cases():
    out = [
        ("three_state_lti", W.three_state_lti(seed=0, steps=8), 1),
        ("two_state_lti", W.two_state_lti(seed=0, steps=8), 2),
        ("four_state_lti", W.four_state_lti(seed=0, steps=5), 3),
        ("five_state_two_msmt", W.five_state_two_msmt(seed=0, steps=3), 4),
    ]
    for i, p in enumerate(W.batched_three_state(6, seed=3, steps_lo=4, steps_hi=7)):
        out.append(("batched_three_state_%d" % i, p, 10 + i))
    return out


def pack(name, prob, seed, print_basic_info=False):
    """Step records of the reference; with print_basic_info the constructor
    flag is set, so the reported moments after every table build are the
    post-FTR ones of compute_moments(false) (the reference also prints its
    progress on stdout)."""
    ref = oracle.Reference(prob, seed=seed)
    rp, bp = ref.constants()
    if print_basic_info:
        ref.set_print_basic_info(True)
    recs = oracle.run(ref, prob, record_terms_upto=TERM_DUMP_CAP)
    ref.close()
    arr = {
        "d": prob["d"], "pncc": prob["pncc"], "cmcc": prob["cmcc"], "p": prob["p"], "steps": prob["steps"],
        "Phi": prob["Phi"], "Gamma": prob["Gamma"], "beta": prob["beta"], "H": prob["H"],
        "gamma": prob["gamma"], "A0": prob["A0"], "p0": prob["p0"], "b0": prob["b0"],
        "msmts": prob["msmts"], "srand_seed": seed, "root_point": rp, "b_pert": bp,
        "n_updates": len(recs), "print_basic_info": int(bool(print_basic_info)),
    }
    for i, r in enumerate(recs):
        pre = "u%d_" % i
        arr[pre + "err"] = r["err"]
        arr[pre + "Nt"] = r["Nt"]
        arr[pre + "tps"] = r["tps"]
        for k in ("fz", "raw_fz", "mean", "raw_mean", "cov", "raw_cov"):
            arr[pre + k] = np.asarray(r[k])
        arr[pre + "gscale"] = r["gscale"]
        if "terms" in r:
            for k, v in r["terms"].items():
                arr[pre + "T_" + k] = v
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arr)
    return len(recs)


def post_ftr_cases():
    """Problems run with print_basic_info (post-FTR moments reported)."""
    return [
        ("postftr_three_state_lti", W.three_state_lti(seed=0, steps=8), 1),
        ("postftr_five_state_two_msmt", W.five_state_two_msmt(seed=0, steps=3), 4),
        ("postftr_batched_three_state", W.batched_three_state(1, seed=7, steps_lo=7, steps_hi=8)[0], 17),
    ]


def cpdf_cases():
    """(name, problem, srand seed, updates before the pdf, srand seed of the pdf object)."""
    return [
        ("cpdf1d_three_state_lti", W.three_state_lti(seed=0, steps=8), 1, 5, 77),
        ("cpdf1d_two_state_lti", W.two_state_lti(seed=0, steps=8), 2, 6, 78),
        ("cpdf1d_four_state_lti", W.four_state_lti(seed=0, steps=5), 3, 4, 79),
        ("cpdf1d_five_state_two_msmt", W.five_state_two_msmt(seed=0, steps=3), 4, 3, 80),
        ("cpdf1d_batched_three_state_0", W.batched_three_state(6, seed=3, steps_lo=4, steps_hi=7)[0], 10, 3, 81),
    ]


def pack_cpdf(name, prob, seed, updates, cpdf_seed):
    """The reference's marginal 1-D pdf grids (CauchyCPDFGridDispatcher1D)
    after `updates` measurement updates: for every state, two grid calls (the
    first exact at its first point and caching, the second from the cache)."""
    import ctypes
    ref = oracle.Reference(prob, seed=seed)
    rp, bp = ref.constants()
    n = 0
    for k in range(prob["steps"]):
        for s in range(prob["p"]):
            if n < updates:
                ref.step(k, s)
                n += 1
    mo = ref.moments()
    ctypes.CDLL(None).srand(cpdf_seed)
    arr = {
        "d": prob["d"], "pncc": prob["pncc"], "cmcc": prob["cmcc"], "p": prob["p"], "steps": prob["steps"],
        "Phi": prob["Phi"], "Gamma": prob["Gamma"], "beta": prob["beta"], "H": prob["H"],
        "gamma": prob["gamma"], "A0": prob["A0"], "p0": prob["p0"], "b0": prob["b0"],
        "msmts": prob["msmts"], "srand_seed": seed, "root_point": rp, "b_pert": bp, "updates": updates,
    }
    for marg in range(prob["d"]):
        mu = float(mo["raw_mean"].real[marg])
        sd = float(np.sqrt(abs(mo["raw_cov"].real[marg, marg])))
        if not np.isfinite(mu):
            mu = 0.0
        if not (np.isfinite(sd) and sd > 1e-6):
            sd = 1.0
        lo, hi, res = mu - 4 * sd, mu + 4 * sd, 8 * sd / 50
        for call in range(2):
            x, y, nu = ref.cpdf_1d_grid(marg, lo, hi, res)
            pre = "m%d_c%d_" % (marg, call)
            arr[pre + "grid"] = np.array([lo, hi, res])
            arr[pre + "x"] = x
            arr[pre + "y"] = y
        arr["bar_nu"] = nu
    ref.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arr)


def pack_cpdf2d(name, prob, seed, updates, cpdf_seed):
    """The reference's marginal 2-D pdf grids (CauchyCPDFGridDispatcher2D)
    after `updates` updates, for the state pairs (0, 1) and (0, d-1): three
    grid calls each (caching, cached with a reset after, exact again)."""
    import ctypes
    ref = oracle.Reference(prob, seed=seed)
    rp, bp = ref.constants()
    n = 0
    for k in range(prob["steps"]):
        for s in range(prob["p"]):
            if n < updates:
                ref.step(k, s)
                n += 1
    mo = ref.moments()
    ctypes.CDLL(None).srand(cpdf_seed)
    d = prob["d"]
    arr = {
        "d": d, "pncc": prob["pncc"], "cmcc": prob["cmcc"], "p": prob["p"], "steps": prob["steps"],
        "Phi": prob["Phi"], "Gamma": prob["Gamma"], "beta": prob["beta"], "H": prob["H"],
        "gamma": prob["gamma"], "A0": prob["A0"], "p0": prob["p0"], "b0": prob["b0"],
        "msmts": prob["msmts"], "srand_seed": seed, "root_point": rp, "b_pert": bp, "updates": updates,
    }
    pairs = sorted({(0, 1), (0, d - 1)})
    arr["pairs"] = np.array(pairs)
    mu = mo["raw_mean"].real
    sd = np.sqrt(np.abs(np.diag(mo["raw_cov"].real)))
    sd = np.where(np.isfinite(sd) & (sd > 1e-6), sd, 1.0)
    mu = np.where(np.isfinite(mu), mu, 0.0)
    for pi, (i1, i2) in enumerate(pairs):
        gx = (mu[i1] - 3 * sd[i1], mu[i1] + 3 * sd[i1], 6 * sd[i1] / 16)
        gy = (mu[i2] - 3 * sd[i2], mu[i2] + 3 * sd[i2], 6 * sd[i2] / 16)
        for call in range(3):
            x, y, z, nu = ref.cpdf_2d_grid(i1, i2, gx, gy, reset_cache=(call == 1))
            pre = "p%d_c%d_" % (pi, call)
            arr[pre + "grid"] = np.array(list(gx) + list(gy))
            arr[pre + "x"], arr[pre + "y"], arr[pre + "z"] = x, y, z
        arr["bar_nu"] = nu
    ref.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arr)


def cpdf2d_cases():
    return [
        ("cpdf2d_three_state_lti", W.three_state_lti(seed=0, steps=8), 1, 5, 91),
        ("cpdf2d_two_state_lti", W.two_state_lti(seed=0, steps=8), 2, 5, 92),
        ("cpdf2d_four_state_lti", W.four_state_lti(seed=0, steps=5), 3, 4, 93),
        ("cpdf2d_five_state_two_msmt", W.five_state_two_msmt(seed=0, steps=3), 4, 3, 94),
    ]


def ext_cases():
    return [
        ("ext_three_state_lti", W.three_state_lti(seed=0, steps=6), 1),
        ("ext_two_state_lti", W.two_state_lti(seed=0, steps=6), 2),
        ("ext_five_state_two_msmt", W.five_state_two_msmt(seed=0, steps=3), 4),
    ]


def pack_ext(name, prob, seed):
    """The reference through a fixed sequence of updates and extended-mode
    calls (finalize_extended_moments, deterministic_time_prop,
    shift_cf_by_bias; the sequence is tests.golden_cases.extended_ops)."""
    from tests import golden_cases as G
    ref = oracle.Reference(prob, seed=seed)
    rp, bp = ref.constants()
    recs = G.run_extended(ref, prob, G.extended_ops(prob))
    ref.close()
    arr = {
        "d": prob["d"], "pncc": prob["pncc"], "cmcc": prob["cmcc"], "p": prob["p"], "steps": prob["steps"],
        "Phi": prob["Phi"], "Gamma": prob["Gamma"], "beta": prob["beta"], "H": prob["H"],
        "gamma": prob["gamma"], "A0": prob["A0"], "p0": prob["p0"], "b0": prob["b0"],
        "msmts": prob["msmts"], "srand_seed": seed, "root_point": rp, "b_pert": bp, "n_ops": len(recs),
    }
    for i, r in enumerate(recs):
        for k, v in r.items():
            arr["r%d_%s" % (i, k)] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arr)


def rel2d_cases():
    """(name, problem family, primary/secondary workload seeds, srand seeds,
    updates, Trel rows, full solve, bar_nu seed)"""
    return [
        ("rel2d_three_state_lti", W.three_state_lti, (0, 1), (1, 5), 4, [[1, 0, 0], [0, 1, 0]], False, 71),
        ("rel2d_two_state_lti_full", W.two_state_lti, (0, 1), (2, 6), 5, [[1, 0], [0, 1]], True, 72),
        ("rel2d_four_state_lti", W.four_state_lti, (0, 1), (3, 7), 3, [[1, 0, 0.5, 0], [0, 1, 0, -0.25]], False,
         73),
        ("rel2d_five_state_two_msmt", W.five_state_two_msmt, (0, 1), (4, 8), 2,
         [[1, 0, 0, 0, 0], [0, 0, 1, 0, 0]], False, 74),
    ]


def _prob_arrays(prefix, prob, seed, rp, bp):
    out = {}
    for k in ("d", "pncc", "cmcc", "p", "steps", "Phi", "Gamma", "beta", "H", "gamma", "A0", "p0", "b0", "msmts"):
        out[prefix + k] = prob[k]
    out[prefix + "srand_seed"] = seed
    out[prefix + "root_point"] = rp
    out[prefix + "b_pert"] = bp
    return out


def pack_rel2d(name, family, wseeds, seeds, updates, trel, full, bar_seed):
    """The reference's relative-then-transformed system of two estimators of
    the same family (get_marg2d_relative_and_transformed_cpdf, single-thread
    term order) after `updates` updates of both: the relative moments, the
    pair counts and the pdf grid centred on the relative mean, as
    pycauchy_single_step_eval_2d_rsys_cpdf evaluates it (term approximation
    on, eps 1e-8)."""
    probs = [family(seed=ws, steps=6) for ws in wseeds]
    refs, arr = [], {"updates": updates, "Trel": np.array(trel, dtype=float), "full": int(full),
                     "bar_seed": bar_seed, "eps": 1e-8}
    for pre, prob, seed in zip(("P_", "S_"), probs, seeds):
        ref = oracle.Reference(prob, seed=seed)
        rp, bp = ref.constants()
        arr.update(_prob_arrays(pre, prob, seed, rp, bp))
        n = 0
        for k in range(prob["steps"]):
            for s in range(prob["p"]):
                if n < updates:
                    ref.step(k, s)
                    n += 1
        refs.append(ref)
    # a first call on a wide grid gives the relative covariance for the grid
    wide = oracle.reference_rel2d(refs[0], refs[1], arr["Trel"], bar_seed, (-1.0, 1.0, 1.0), (-1.0, 1.0, 1.0),
                                  full_solve=full)
    sd = np.sqrt(np.abs(np.diag(wide["cov"].real)))
    sd = np.where(np.isfinite(sd) & (sd > 1e-6), sd, 1.0)
    gx, gy = (-3 * sd[0], 3 * sd[0], 6 * sd[0] / 16), (-3 * sd[1], 3 * sd[1], 6 * sd[1] / 16)
    out = oracle.reference_rel2d(refs[0], refs[1], arr["Trel"], bar_seed, gx, gy, full_solve=full)
    arr["grid"] = np.array(list(gx) + list(gy))
    arr["bar_nu_full"] = out["bar_nu_full"]
    arr["fz"] = np.array([out["fz"].real, out["fz"].imag])
    arr["mean"] = out["mean"]
    arr["cov"] = out["cov"]
    arr["pairs"] = out["pairs"]
    arr["approxed_out"] = out["approxed_out"]
    arr["x"], arr["y"], arr["z"] = out["x"], out["y"], out["z"]
    for r in refs:
        r.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arr)


def wide_cases():
    """Terms above 16 hyperplanes (the cell bitmaps leave shared memory):
    three Gamma columns (3 states, up to 21 rows; 4 states, up to 19) and
    four (2 states, up to 22)."""
    return [
        ("wide_three_state_21", W.many_gamma(3, 3, 7, seed=5), 41),
        ("wide_two_state_22", W.many_gamma(2, 4, 6, seed=6), 42),
        ("wide_four_state_19", W.many_gamma(4, 3, 6, seed=7), 43),
    ]


def main():
    oracle.build()
    only = [a[2:] for a in sys.argv[1:] if a.startswith("--")]
    if not only or "wide" in only:
        for name, prob, seed in wide_cases():
            n = pack(name, prob, seed)
            print("wrote %s.npz (%d updates)" % (name, n))
    if not only:
        for name, prob, seed in cases():
            n = pack(name, prob, seed)
            print("wrote %s.npz (%d updates)" % (name, n))
    if not only or "postftr" in only:
        for name, prob, seed in post_ftr_cases():
            n = pack(name, prob, seed, print_basic_info=True)
            print("wrote %s.npz (%d updates)" % (name, n), file=sys.stderr)
    if not only or "cpdf" in only:
        for name, prob, seed, updates, cseed in cpdf_cases():
            pack_cpdf(name, prob, seed, updates, cseed)
            print("wrote %s.npz" % name)
    if not only or "cpdf" in only:
        for name, prob, seed, updates, cseed in cpdf2d_cases():
            pack_cpdf2d(name, prob, seed, updates, cseed)
            print("wrote %s.npz" % name)
    if not only or "ext" in only:
        for name, prob, seed in ext_cases():
            pack_ext(name, prob, seed)
            print("wrote %s.npz" % name)
    if not only or "rel" in only:
        for c in rel2d_cases():
            pack_rel2d(*c)
            print("wrote %s.npz" % c[0])


if __name__ == "__main__":
    main()
