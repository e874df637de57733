"""Generates the N-D conditional pdf fixtures (cpdfnd_*.npz) from the
REFERENCE itself: PointWiseNDimCauchyCPDF::evaluate_cpdf
(include/cpdf_ndim.hpp:677-904) called through oracle/ref_harness.cpp on an
estimator stepped by the reference (serial build), at points around its mean
(a grid for two states, as the reference's own test_2d_cpdf evaluates one;
seeded random points in the tails and the bulk otherwise).

Each fixture holds the problem arrays, the rand() constants the reference
drew (srand(seed) before the constructor), the number of updates, the points
and the complex values.

Needs the reference sources:  python tests/golden/make_cpdfnd_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from cauchyfriendly_gb300 import workloads as W  # noqa: E402


def points_for(mo, d, n, seed, grid=False):
    mu = np.asarray(mo["mean"].real, dtype=np.float64)
    sd = np.sqrt(np.abs(np.diag(mo["cov"].real)))
    sd = np.where(np.isfinite(sd) & (sd > 1e-6), sd, 1.0)
    if grid:
        g = np.linspace(-3.0, 3.0, 9)
        return np.array([[mu[0] + a * sd[0], mu[1] + b * sd[1]] for a in g for b in g])
    rng = np.random.Generator(np.random.PCG64(seed))
    scales = np.concatenate([np.full(n // 2, 0.7), np.full(n - n // 2, 3.0)])
    return mu + sd * rng.standard_normal((n, d)) * scales[:, None]


def pack(name, prob, seed, updates, npts, grid=False):
    ref = oracle.Reference(prob, seed=seed)
    rp, bp = ref.constants()
    n = 0
    errs = []
    for k in range(prob["steps"]):
        for s in range(prob["p"]):
            if n < updates:
                errs.append(int(ref.step(k, s)))
                n += 1
    assert errs[-1] == 0, (name, errs)
    mo = ref.moments()
    X = points_for(mo, prob["d"], npts, seed, grid)
    vals = np.array([ref.cpdf_nd(x) for x in X])
    arr = {
        "d": prob["d"], "pncc": prob["pncc"], "cmcc": prob["cmcc"], "p": prob["p"], "steps": prob["steps"],
        "Phi": prob["Phi"], "Gamma": prob["Gamma"], "beta": prob["beta"], "H": prob["H"],
        "gamma": prob["gamma"], "A0": prob["A0"], "p0": prob["p0"], "b0": prob["b0"],
        "msmts": prob["msmts"], "srand_seed": seed, "root_point": rp, "b_pert": bp, "updates": updates,
        "x": X, "f": vals, "Nt": ref.num_terms(),
    }
    ref.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arr)
    print(name, "terms", arr["Nt"], "points", len(X), "f range", float(np.min(np.abs(vals))),
          float(np.max(np.abs(vals))))


if __name__ == "__main__":
    oracle.build()
    pack("cpdfnd_two_state", W.two_state_lti(seed=4, steps=8), 91, 6, 81, grid=True)
    pack("cpdfnd_three_state", W.many_gamma(3, 1, 7, seed=5), 92, 6, 24)
    pack("cpdfnd_four_state", W.four_state_lti(seed=2, steps=6), 93, 4, 24)
    pack("cpdfnd_five_state_two_msmt", W.five_state_two_msmt(seed=3, steps=4), 94, 4, 16)
