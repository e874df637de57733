"""Loads the golden fixtures (made by tests/golden/make_golden.py from the
reference itself) and compares estimator records against them."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# fz, mean and covariance tolerance, element by element (relerr); integer
# structure is compared exactly.
REL_TOL = 1e-9


def names():
    """The step-record fixtures (the marginal pdf ones are cpdf_names())."""
    return sorted(n for n in (os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
                  if not n.startswith(("cpdf1d_", "cpdf2d_", "cpdfnd_", "cpdfmarg_", "ext_", "rel2d_", "win_", "speyer_",
                                       "tr_ordering_", "adj_")))


def cpdf_names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "cpdf1d_*.npz")))


def load_cpdf(name):
    """(problem, (root_point, b_pert), updates, bar_nu, [(marg, call, (lo, hi, res), x, y)])"""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    prob = {k: z[k] for k in ("Phi", "Gamma", "beta", "H", "gamma", "A0", "p0", "b0", "msmts")}
    for k in ("d", "pncc", "cmcc", "p", "steps"):
        prob[k] = int(z[k])
    prob["B"] = None
    grids = []
    for marg in range(prob["d"]):
        for call in range(2):
            pre = "m%d_c%d_" % (marg, call)
            grids.append((marg, call, tuple(float(v) for v in z[pre + "grid"]), z[pre + "x"], z[pre + "y"]))
    return prob, (z["root_point"], z["b_pert"]), int(z["updates"]), z["bar_nu"], grids


def cpdfnd_names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "cpdfnd_*.npz")))


def load_cpdfnd(name):
    """(problem, (root_point, b_pert), updates, points [n][d], complex values)"""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    prob = {k: z[k] for k in ("Phi", "Gamma", "beta", "H", "gamma", "A0", "p0", "b0", "msmts")}
    for k in ("d", "pncc", "cmcc", "p", "steps"):
        prob[k] = int(z[k])
    prob["B"] = None
    return prob, (z["root_point"], z["b_pert"]), int(z["updates"]), z["x"], z["f"]


def cpdfmarg_names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "cpdfmarg_*.npz")))


def load_cpdfmarg(name):
    """(problem, (root_point, b_pert), updates, [(idx, xm, nu_bar, complex value)])"""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    prob = {k: z[k] for k in ("Phi", "Gamma", "beta", "H", "gamma", "A0", "p0", "b0", "msmts")}
    for k in ("d", "pncc", "cmcc", "p", "steps"):
        prob[k] = int(z[k])
    prob["B"] = None
    d = prob["d"]
    cases = []
    for idx, xm, nu, f in zip(z["idx"], z["xm"], z["nu_bar"], z["f"]):
        nm = int(np.sum(idx >= 0))
        cases.append((idx[:nm].astype(np.int32), xm[:nm], nu[:d - nm], complex(f)))
    return prob, (z["root_point"], z["b_pert"]), int(z["updates"]), cases


def rel2d_names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "rel2d_*.npz")))


def load_rel2d(name):
    """(primary problem, primary (root_point, b_pert), secondary problem, its
    constants, updates, case dict: Trel, full, eps, grid, bar_nu_full and the
    reference's fz, mean, cov, pairs, approxed_out, x, y, z)"""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    out = []
    for pre in ("P_", "S_"):
        prob = {k: z[pre + k] for k in ("Phi", "Gamma", "beta", "H", "gamma", "A0", "p0", "b0", "msmts")}
        for k in ("d", "pncc", "cmcc", "p", "steps"):
            prob[k] = int(z[pre + k])
        prob["B"] = None
        out += [prob, (z[pre + "root_point"], z[pre + "b_pert"])]
    case = {k: z[k] for k in ("Trel", "grid", "bar_nu_full", "mean", "cov", "x", "y", "z")}
    case["fz"] = complex(z["fz"][0], z["fz"][1])
    for k in ("full", "pairs", "approxed_out"):
        case[k] = int(z[k])
    case["eps"] = float(z["eps"])
    return out[0], out[1], out[2], out[3], int(z["updates"]), case

def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    prob = {k: z[k] for k in ("Phi", "Gamma", "beta", "H", "gamma", "A0", "p0", "b0", "msmts")}
    for k in ("d", "pncc", "cmcc", "p", "steps"):
        prob[k] = int(z[k])
    prob["B"] = None
    prob["print_basic_info"] = bool(int(z["print_basic_info"])) if "print_basic_info" in z else False
    recs = []
    for i in range(int(z["n_updates"])):
        pre = "u%d_" % i
        r = {k: z[pre + k] for k in ("err", "Nt", "tps", "fz", "raw_fz", "mean", "raw_mean", "cov", "raw_cov",
                                      "gscale")}
        r["err"] = int(r["err"]); r["Nt"] = int(r["Nt"])
        if (pre + "T_shape") in z:
            r["terms"] = {k: z[pre + "T_" + k] for k in ("shape", "A", "p", "b", "cells", "keys", "g")}
        recs.append(r)
    return prob, (z["root_point"], z["b_pert"]), recs


ABS_FLOOR = 1e-12


def relerr(a, b, floor=ABS_FLOOR):
    """Largest element-wise relative error of a against the reference b:
    max_i |a_i - b_i| / max(|b_i|, floor * max_j |b_j|).  The floor only
    covers entries that are structurally zero up to rounding (a covariance
    entry of a decoupled state, a pdf value far in the tail); every other
    entry is held to the tolerance on its own magnitude."""
    a = np.asarray(a); b = np.asarray(b)
    if a.size == 0 and b.size == 0:
        return 0.0
    mag = np.abs(b)
    den = np.maximum(mag, max(floor * float(np.max(mag)), 1e-300))
    return float(np.max(np.abs(a - b) / den))


def bitwise_equal(a, b):
    """True when a and b hold the same doubles element by element (complex
    parts included; +0 and -0 count as equal, so do two NaNs)."""
    a = np.asarray(a); b = np.asarray(b)
    return a.shape == b.shape and bool(np.array_equal(a, b, equal_nan=True))


def compare_records(got, want, rel_tol=REL_TOL, check_terms=True, first_raw_from_reported=True):
    """Asserts a run's per-update records equal the golden ones: exact term
    counts, shapes, error bits and g-table keys; moments within rel_tol."""
    assert len(got) == len(want), (len(got), len(want))
    for i, (g, w) in enumerate(zip(got, want)):
        ctx = "update %d" % i
        assert g["Nt"] == w["Nt"], (ctx, "Nt", g["Nt"], w["Nt"])
        assert np.array_equal(np.asarray(g["tps"])[:len(w["tps"])], w["tps"]), (ctx, "terms per shape")
        assert g["err"] == w["err"], (ctx, "error bits", g["err"], w["err"])
        # update 0 never reaches the numeric check, so the raw copy is the reported one
        if i == 0:
            pairs = (("fz", "fz"), ("mean", "mean"), ("cov", "cov"))
        else:
            pairs = (("raw_fz", "raw_fz"), ("raw_mean", "raw_mean"), ("raw_cov", "raw_cov"), ("fz", "fz"),
                     ("mean", "mean"), ("cov", "cov"))
        for a, b in pairs:
            assert relerr(g[a], w[b]) <= rel_tol, (ctx, a, relerr(g[a], w[b]))
        assert abs(g["gscale"] - float(w["gscale"])) <= rel_tol * abs(float(w["gscale"])), (ctx, "gscale")
        if check_terms and "terms" in w:
            gt, wt = g["terms"], w["terms"]
            assert np.array_equal(gt["shape"], wt["shape"]), (ctx, "term shapes")
            assert np.array_equal(gt["cells"], wt["cells"]), (ctx, "cell counts")
            assert np.array_equal(gt["keys"], wt["keys"]), (ctx, "g-table keys")
            for k in ("A", "p", "b"):
                assert relerr(gt[k], wt[k]) <= 1e-12, (ctx, k, relerr(gt[k], wt[k]))
            assert relerr(gt["g"], wt["g"]) <= rel_tol, (ctx, "g values", relerr(gt["g"], wt["g"]))


def bitwise_mismatches(got, want):
    """Names of the floating-point quantities of a run's per-update records
    that are not bit-identical to the golden ones (raw and reported moments,
    G_SCALE_FACTOR, every dumped term's A, p, b and g values)."""
    bad = []
    for i, (g, w) in enumerate(zip(got, want)):
        keys = ("fz", "mean", "cov") if i == 0 else ("raw_fz", "raw_mean", "raw_cov", "fz", "mean", "cov")
        for k in keys:
            if not bitwise_equal(np.asarray(g[k], np.complex128).ravel(), np.asarray(w[k], np.complex128).ravel()):
                bad.append((i, k, relerr(g[k], w[k])))
        if float(g["gscale"]) != float(w["gscale"]):
            bad.append((i, "gscale", abs(g["gscale"] / float(w["gscale"]) - 1)))
        if "terms" in w and "terms" in g:
            for k in ("A", "p", "b", "g"):
                a = np.asarray(g["terms"][k]).ravel(); b = np.asarray(w["terms"][k]).ravel()
                if not bitwise_equal(a.astype(b.dtype), b):
                    bad.append((i, "term " + k, relerr(a, b)))
    return bad


def extended_ops(prob):
    """A fixed sequence of updates and extended-mode calls for a problem:
    ("step", k, s), ("finalize", x_bar), ("dtp", Phi), ("bias", b)."""
    d = prob["d"]
    rng = np.random.Generator(np.random.PCG64(1234 + d))
    ups = [(k, s) for k in range(prob["steps"]) for s in range(prob["p"])]
    ops = []
    for i, (k, s) in enumerate(ups):
        ops.append(("step", k, s))
        if i == len(ups) - 1:
            ops.append(("finalize", 0.1 * rng.standard_normal(d)))  # after the final MU: mean only
            break
        if i % 3 == 0:
            ops.append(("finalize", 0.1 * rng.standard_normal(d)))
        elif i % 3 == 1:
            M = np.eye(d) + 0.05 * rng.standard_normal((d, d))
            ops.append(("dtp", M))
            ops.append(("bias", 0.05 * rng.standard_normal(d)))
    return ops


def run_extended(est, prob, ops):
    """Applies ops to an estimator with step(k, s), finalize_extended_moments,
    deterministic_time_prop, shift_cf_by_bias and the read-outs; one record
    per op (moments, Nt, error bits, and x_bar after a finalize)."""
    recs = []
    for op in ops:
        r = {}
        if op[0] == "step":
            r["err"] = int(est.step(op[1], op[2]))
        elif op[0] == "finalize":
            r["xbar"] = np.asarray(est.finalize_extended_moments(op[1]))
        elif op[0] == "dtp":
            est.deterministic_time_prop(op[1])
        elif op[0] == "bias":
            est.shift_cf_by_bias(op[1])
        r.update(est.moments())
        r["Nt"] = est.num_terms()
        recs.append(r)
    return recs


def compare_extended(got, want, rel_tol=REL_TOL):
    """Records of run_extended: exact term counts and error bits, moments and
    x_bar within rel_tol.  The raw (pre-check) moments exist from the second
    update on: the first update never reaches the numeric check."""
    assert len(got) == len(want)
    steps = 0
    for i, (g, w) in enumerate(zip(got, want)):
        steps += "err" in w
        assert g["Nt"] == w["Nt"], (i, g["Nt"], w["Nt"])
        if "err" in w:
            assert g["err"] == w["err"], (i, "err")
        if "xbar" in w:
            assert relerr(g["xbar"], w["xbar"]) <= rel_tol, (i, "xbar")
        keys = ("fz", "mean", "cov") + (("raw_fz", "raw_mean", "raw_cov") if steps >= 2 else ())
        for k in keys:
            assert relerr(g[k], w[k]) <= rel_tol, (i, k, relerr(g[k], w[k]))


def ext_names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "ext_*.npz")))


def load_ext(name):
    """(problem, (root_point, b_pert), records) of an extended-mode fixture."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    prob = {k: z[k] for k in ("Phi", "Gamma", "beta", "H", "gamma", "A0", "p0", "b0", "msmts")}
    for k in ("d", "pncc", "cmcc", "p", "steps"):
        prob[k] = int(z[k])
    prob["B"] = None
    recs = []
    for i in range(int(z["n_ops"])):
        pre = "r%d_" % i
        r = {k[len(pre):]: z[k] for k in z.files if k.startswith(pre)}
        r["Nt"] = int(r["Nt"])
        if "err" in r:
            r["err"] = int(r["err"])
        recs.append(r)
    return prob, (z["root_point"], z["b_pert"]), recs


def cpdf2d_names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "cpdf2d_*.npz")))


def load_cpdf2d(name):
    """(problem, (root_point, b_pert), updates, bar_nu,
    [(i1, i2, call, gx, gy, x, y, z)]); call 1 resets the cache afterwards."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    prob = {k: z[k] for k in ("Phi", "Gamma", "beta", "H", "gamma", "A0", "p0", "b0", "msmts")}
    for k in ("d", "pncc", "cmcc", "p", "steps"):
        prob[k] = int(z[k])
    prob["B"] = None
    grids = []
    for pi, (i1, i2) in enumerate(z["pairs"]):
        for call in range(3):
            pre = "p%d_c%d_" % (pi, call)
            g = [float(v) for v in z[pre + "grid"]]
            grids.append((int(i1), int(i2), call, tuple(g[:3]), tuple(g[3:]), z[pre + "x"], z[pre + "y"],
                          z[pre + "z"]))
    return prob, (z["root_point"], z["b_pert"]), int(z["updates"]), z["bar_nu"], grids
