"""Generates the marginal pdf fixtures (cpdfmarg_*.npz) from the REFERENCE
itself: PointWiseNDimCauchyCPDF::evaluate_marginal_cpdf
(include/cpdf_ndim.hpp:918-1230) called through oracle/ref_harness.cpp on an
estimator stepped by the reference (serial build), for every subset of the
states short of all of them, at points around the marginal's mean.

The function draws its nu_bar from rand(); the harness seeds rand() before
each call and returns the nu_bar it drew, kept with each value.  Each fixture
holds the problem arrays, the constructor's rand() constants, the number of
updates and, per case, the state indices (padded with -1), the point (padded
with 0), nu_bar (padded with 0) and the complex value.

Needs the reference sources:  python tests/golden/make_cpdfmarg_golden.py
"""
import itertools
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from cauchyfriendly_gb300 import workloads as W  # noqa: E402


def pack(name, prob, seed, updates, per_subset):
    ref = oracle.Reference(prob, seed=seed)
    rp, bp = ref.constants()
    n = 0
    for k in range(prob["steps"]):
        for s in range(prob["p"]):
            if n < updates:
                ref.step(k, s)
                n += 1
    mo = ref.moments()
    d = prob["d"]
    mu = np.asarray(mo["mean"].real)
    sd = np.sqrt(np.abs(np.diag(mo["cov"].real)))
    sd = np.where(np.isfinite(sd) & (sd > 1e-6), sd, 1.0)
    rng = np.random.Generator(np.random.PCG64(seed))
    idx_l, x_l, nu_l, f_l = [], [], [], []
    call = 0
    for nm in range(1, d):
        for idx in itertools.combinations(range(d), nm):
            idx = list(idx)
            for q in range(per_subset):
                scale = 0.5 if q % 2 == 0 else 2.5
                xm = mu[idx] + sd[idx] * rng.standard_normal(nm) * scale
                v, nb = ref.cpdf_marginal(xm, idx, 1000 + call)
                call += 1
                idx_l.append(idx + [-1] * (d - nm))
                x_l.append(list(xm) + [0.0] * (d - nm))
                nu_l.append(list(nb) + [0.0] * (d - len(nb)))
                f_l.append(v)
    arr = {
        "d": d, "pncc": prob["pncc"], "cmcc": prob["cmcc"], "p": prob["p"], "steps": prob["steps"],
        "Phi": prob["Phi"], "Gamma": prob["Gamma"], "beta": prob["beta"], "H": prob["H"],
        "gamma": prob["gamma"], "A0": prob["A0"], "p0": prob["p0"], "b0": prob["b0"],
        "msmts": prob["msmts"], "srand_seed": seed, "root_point": rp, "b_pert": bp, "updates": updates,
        "idx": np.array(idx_l, dtype=np.int32), "xm": np.array(x_l), "nu_bar": np.array(nu_l),
        "f": np.array(f_l), "Nt": ref.num_terms(),
    }
    ref.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arr)
    print(name, "terms", arr["Nt"], "cases", len(f_l), "|f| range", float(np.min(np.abs(f_l))),
          float(np.max(np.abs(f_l))))


if __name__ == "__main__":
    oracle.build()
    pack("cpdfmarg_three_state", W.many_gamma(3, 1, 7, seed=5), 92, 6, 3)
    pack("cpdfmarg_four_state", W.four_state_lti(seed=2, steps=6), 93, 4, 2)
    pack("cpdfmarg_five_state_two_msmt", W.five_state_two_msmt(seed=3, steps=4), 94, 4, 1)
