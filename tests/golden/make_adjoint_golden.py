"""Generates the adjoint fixtures (adj_*.npz) from the REFERENCE itself:
central finite differences of the reference's accumulated log-likelihood
sum_k log fz_k, fz_k = 1/(2 pi G_SCALE_FACTOR_k) read after every
CauchyEstimator::step (include/cauchy_estimator.hpp:340-357), with respect to
every entry of (beta, gamma, p0, Phi, Gamma, H), for seeded LTI problems run
by the unmodified reference (oracle/ref_harness.cpp, serial build).

Step: h_i = 1e-6 max(|theta_i|, 1e-3); the fixture also keeps the gradient at
h/4 so that a test can see the differences' own truncation error.

Needs the reference sources:  python tests/golden/make_adjoint_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from cauchyfriendly_gb300 import workloads as W  # noqa: E402

NAMES = ("beta", "gamma", "p0", "Phi", "Gamma", "H")


def flat(prob):
    return np.concatenate([np.asarray(prob[k], dtype=np.float64).reshape(-1) for k in NAMES])


def unflat(prob, th):
    q = dict(prob)
    k = 0
    for n in NAMES:
        sh = np.asarray(prob[n]).shape
        sz = int(np.prod(sh))
        q[n] = th[k:k + sz].reshape(sh).copy()
        k += sz
    return q


def loglik(prob, seed):
    ref = oracle.Reference(prob, seed=seed)
    s = 0.0
    for k in range(prob["steps"]):
        for j in range(prob["p"]):
            ref.step(k, j)
            s += np.log(1.0 / (2 * np.pi * ref.moments()["gscale"]))
    ref.close()
    return s


def make(name, prob, seed):
    oracle.build()
    th = flat(prob)
    base = loglik(prob, seed)
    grads = []
    for frac in (1.0, 0.25):
        g = np.zeros_like(th)
        for i in range(th.size):
            h = 1e-6 * max(abs(th[i]), 1e-3) * frac
            tp, tm = th.copy(), th.copy()
            tp[i] += h
            tm[i] -= h
            g[i] = (loglik(unflat(prob, tp), seed) - loglik(unflat(prob, tm), seed)) / (2 * h)
        grads.append(g)
    ref = oracle.Reference(prob, seed=seed)
    rp, bp = ref.constants()
    ref.close()
    arr = {k: prob[k] for k in ("Phi", "Gamma", "beta", "H", "gamma", "A0", "p0", "b0", "msmts", "d", "pncc", "p",
                                "steps")}
    arr.update(srand_seed=seed, root_point=rp, b_pert=bp, loglik=base, fd_grad=grads[0], fd_grad_quarter=grads[1])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arr)
    print(name, "loglik", base, "max |g|", np.abs(grads[0]).max(),
          "h vs h/4", np.max(np.abs(grads[0] - grads[1]) / (np.abs(grads[0]) + 1e-8)))


if __name__ == "__main__":
    make("adj_four_state", W.four_state_lti(seed=3, steps=6), 31)
    make("adj_five_state_two_msmt", W.five_state_two_msmt(seed=2, steps=3), 32)
