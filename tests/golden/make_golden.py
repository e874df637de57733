"""Generates the golden fixtures in this folder from the REFERENCE itself.

Runs the reference estimator (natsnyder1/CauchyFriendly, compiled from its own
headers by oracle/ref_harness.cpp, serial build) on seeded synthetic problems
and records, after every measurement update: the error bitmask, the term count,
terms per shape, the reported and raw moments, G_SCALE_FACTOR, and (for small
steps) every term's shape, A, p, b and sorted g-table.

Needs the reference sources (only present where the fixtures are made):
    python tests/golden/make_golden.py
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


def pack(name, prob, seed):
    ref = oracle.Reference(prob, seed=seed)
    rp, bp = ref.constants()
    recs = oracle.run(ref, prob, record_terms_upto=TERM_DUMP_CAP)
    ref.close()
    arr = {
        "d": prob["d"], "pncc": prob["pncc"], "cmcc": prob["cmcc"], "p": prob["p"], "steps": prob["steps"],
        "Phi": prob["Phi"], "Gamma": prob["Gamma"], "beta": prob["beta"], "H": prob["H"],
        "gamma": prob["gamma"], "A0": prob["A0"], "p0": prob["p0"], "b0": prob["b0"],
        "msmts": prob["msmts"], "srand_seed": seed, "root_point": rp, "b_pert": bp,
        "n_updates": len(recs),
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


def main():
    oracle.build()
    for name, prob, seed in cases():
        n = pack(name, prob, seed)
        print("wrote %s.npz (%d updates)" % (name, n))


if __name__ == "__main__":
    main()
