"""Seeded synthetic estimation problems.

The reference publishes no dataset for this path; its demos feed fixed or
simulated measurement sequences into ``CauchyEstimator::step``
(src/cauchy_estimator.cpp:57-433).  These generators build linear systems of
the documented shapes and simulate Cauchy-noise measurement histories with
numpy's PCG64 so every consumer (tests, bench, the CPU baseline) sees the same
inputs for a given seed.

A problem is a plain dict:
  d, pncc, cmcc, p       state dim, process-noise columns, control columns,
                         scalar measurements per step
  Phi (d,d)  Gamma (d,pncc)  beta (pncc,)  H (p,d)  gamma (p,)
  B (d,cmcc) or None
  A0 (d,d)  p0 (d,)  b0 (d,)
  steps                  estimation steps (the reference's ``steps`` argument)
  msmts (steps, p)       measurement history; row k is fed at step k
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "simulate", "three_state_lti", "random_stable", "batched_three_state",
    "four_state_lti", "two_state_lti", "five_state_two_msmt", "nonlin_three_state", "nonlin_callbacks",
]


def _cauchy(rng, scale, size=None):
    return rng.standard_cauchy(size) * scale


def simulate(prob, rng, outlier_frac=0.0, outlier_scale=1.0):
    """Simulates x_{k+1} = Phi x_k + Gamma w_k, z_k = H x_k + v_k with Cauchy w, v.

    The first measurement is taken at the initial state, matching the
    reference's first step, which is a measurement update only
    (include/cauchy_estimator.hpp:1179).
    """
    d, p, pncc = prob["d"], prob["p"], prob["pncc"]
    Phi, Gamma, H = prob["Phi"], prob["Gamma"], prob["H"]
    beta, gamma = np.asarray(prob["beta"]), np.asarray(prob["gamma"])
    A0, p0, b0 = prob["A0"], prob["p0"], prob["b0"]
    # initial state: b0 + A0^{-1} (Cauchy(p0)) -- scales act along the rows of A0
    x = b0 + np.linalg.solve(A0, _cauchy(rng, p0, d))
    zs = np.zeros((prob["steps"], p))
    for k in range(prob["steps"]):
        if k > 0:
            w = _cauchy(rng, beta, pncc)
            x = Phi @ x + Gamma @ w
        v = _cauchy(rng, gamma, p)
        if outlier_frac > 0:
            mask = rng.random(p) < outlier_frac
            v = np.where(mask, v * outlier_scale, v)
        zs[k] = H @ x + v
    return zs


def _base(d, pncc, p, Phi, Gamma, beta, H, gamma, p0, steps):
    return {
        "d": d, "pncc": pncc, "cmcc": 0, "p": p,
        "Phi": np.asarray(Phi, dtype=np.float64).reshape(d, d),
        "Gamma": np.asarray(Gamma, dtype=np.float64).reshape(d, pncc),
        "beta": np.asarray(beta, dtype=np.float64).reshape(pncc),
        "H": np.asarray(H, dtype=np.float64).reshape(p, d),
        "gamma": np.asarray(gamma, dtype=np.float64).reshape(p),
        "B": None,
        "A0": np.eye(d), "p0": np.asarray(p0, dtype=np.float64).reshape(d),
        "b0": np.zeros(d), "steps": int(steps),
    }


def three_state_lti(seed=0, steps=8):
    """Plain 3-state LTI problem: Phi=[[1,.1,0],[0,1,.1],[0,0,.95]],
    Gamma=[0,0,1]^T, H=[1,0,0], beta=0.1, gamma=0.2, p0=[.1,.08,.05]."""
    prob = _base(3, 1, 1,
                 [[1.0, 0.1, 0.0], [0.0, 1.0, 0.1], [0.0, 0.0, 0.95]],
                 [0.0, 0.0, 1.0], [0.1], [1.0, 0.0, 0.0], [0.2], [0.1, 0.08, 0.05], steps)
    prob["msmts"] = simulate(prob, np.random.Generator(np.random.PCG64(seed)))
    return prob


def random_stable(rng, d, rho_lo, rho_hi):
    """Random real matrix with eigenvalue moduli uniform in [rho_lo, rho_hi]:
    a block-diagonal real-Schur-like matrix (2x2 rotation-scale blocks plus a
    1x1 block for odd d) under a random orthogonal similarity."""
    blocks = np.zeros((d, d))
    i = 0
    while i < d:
        r = rng.uniform(rho_lo, rho_hi)
        if i + 1 < d and rng.random() < 0.5:
            th = rng.uniform(0.05, np.pi - 0.05)
            c, s = np.cos(th), np.sin(th)
            blocks[i:i + 2, i:i + 2] = r * np.array([[c, -s], [s, c]])
            i += 2
        else:
            blocks[i, i] = r * (1.0 if rng.random() < 0.8 else -1.0)
            i += 1
    Q, R = np.linalg.qr(rng.standard_normal((d, d)))
    Q = Q * np.sign(np.diag(R))
    return Q @ blocks @ Q.T


def _log_uniform(rng, lo, hi, size=None):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size))


def batched_three_state(n, seed=0, steps_lo=4, steps_hi=9, outlier_frac=0.05, outlier_scale=100.0):
    """Batch of independent 3-state LTI estimators: random stable Phi with
    eigenvalue moduli in [0.8, 1.0], Gamma=[0,0,1]^T, H=[1,0,0], beta, gamma
    and p0 log-uniform in [0.02, 0.5], steps uniform in [steps_lo, steps_hi],
    measurement histories with 5% impulsive outliers at 100x scale."""
    rng = np.random.Generator(np.random.PCG64(seed))
    probs = []
    for _ in range(n):
        Phi = random_stable(rng, 3, 0.8, 1.0)
        beta = _log_uniform(rng, 0.02, 0.5, 1)
        gamma = _log_uniform(rng, 0.02, 0.5, 1)
        p0 = _log_uniform(rng, 0.02, 0.5, 3)
        steps = int(rng.integers(steps_lo, steps_hi + 1))
        prob = _base(3, 1, 1, Phi, [0.0, 0.0, 1.0], beta, [1.0, 0.0, 0.0], gamma, p0, steps)
        prob["msmts"] = simulate(prob, rng, outlier_frac, outlier_scale)
        probs.append(prob)
    return probs


def four_state_lti(seed=0, steps=7):
    """4-state LTI problem: Phi random with spectral radius 0.95, Gamma 4x1 and
    H 1x4 with N(0,1) entries, beta=0.1, gamma=0.2."""
    rng = np.random.Generator(np.random.PCG64(seed))
    M = rng.standard_normal((4, 4))
    Phi = 0.95 * M / np.max(np.abs(np.linalg.eigvals(M)))
    Gamma = rng.standard_normal((4, 1))
    H = rng.standard_normal((1, 4))
    prob = _base(4, 1, 1, Phi, Gamma, [0.1], H, [0.2], [0.1, 0.1, 0.1, 0.1], steps)
    prob["msmts"] = simulate(prob, rng)
    return prob


def two_state_lti(seed=0, steps=10):
    """2-state LTI problem with a non-trivial H.Gamma (well-defined moments)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    Phi = random_stable(rng, 2, 0.85, 1.0)
    prob = _base(2, 1, 1, Phi, [1.0, 0.3], [0.1], [1.0, 1.0], [0.2], [0.1, 0.05], steps)
    prob["msmts"] = simulate(prob, rng)
    return prob


def five_state_two_msmt(seed=0, steps=3):
    """5-state problem with two process-noise columns and two scalar
    measurements per step (Phi = expm(0.1 A), A ~ N(0, 0.3^2))."""
    from scipy.linalg import expm
    rng = np.random.Generator(np.random.PCG64(seed))
    Phi = expm(0.1 * rng.normal(0.0, 0.3, (5, 5)))
    Gamma = 0.1 * rng.standard_normal((5, 2))
    H = rng.standard_normal((2, 5))
    prob = _base(5, 2, 2, Phi, Gamma, [0.05, 0.05], H, [0.1, 0.1], 0.1 * np.ones(5), steps)
    prob["msmts"] = simulate(prob, rng)
    return prob


def five_state_ltv_windows(seed=0, steps=200, dt=0.1, outlier_frac=0.02, outlier_scale=50.0):
    """Sliding-window 5-state LTV problem: Phi_k = expm(A_k dt) with A_k a
    seeded N(0, 0.3^2) 5x5 matrix plus a slow sinusoidal drift of amplitude
    0.05 in each entry, Gamma 5x2 = 0.1 N(0,1), H 2x5 = N(0,1), beta = gamma =
    [0.05, 0.05] / [0.1, 0.1], p0 = 0.1, two measurements per step, 2% of the
    noise samples replaced by outliers at 50x.  Phi has shape (steps, 5, 5)."""
    return ltv_windows(5, seed, steps, dt, outlier_frac, outlier_scale)


def seven_state_ltv_windows(seed=0, steps=150, dt=0.1, outlier_frac=0.02, outlier_scale=50.0):
    """The 7-state version of five_state_ltv_windows (Gamma 7x2, H 2x7), the
    model of the batched 7-state sliding-window estimators (window 8)."""
    return ltv_windows(7, seed, steps, dt, outlier_frac, outlier_scale)


def ltv_windows(d, seed=0, steps=200, dt=0.1, outlier_frac=0.02, outlier_scale=50.0):
    """d-state LTV problem with two process-noise columns and two
    measurements per step, seeded as five_state_ltv_windows describes."""
    from scipy.linalg import expm
    rng = np.random.Generator(np.random.PCG64(seed))
    A = rng.normal(0.0, 0.3, (d, d))
    ph = rng.uniform(0, 2 * np.pi, (d, d))
    Phis = np.stack([expm(dt * (A + 0.05 * np.sin(0.05 * k + ph))) for k in range(steps)])
    Gamma = 0.1 * rng.standard_normal((d, 2))
    H = rng.standard_normal((2, d))
    prob = _base(d, 2, 2, Phis[0], Gamma, [0.05, 0.05], H, [0.1, 0.1], 0.1 * np.ones(d), steps)
    prob["Phi"] = Phis
    # simulate with the time-varying Phi
    x = np.linalg.solve(prob["A0"], _cauchy(rng, prob["p0"], d))
    zs = np.zeros((steps, 2))
    for k in range(steps):
        if k > 0:
            w = _cauchy(rng, prob["beta"], 2)
            x = Phis[k] @ x + Gamma @ w
        v = _cauchy(rng, prob["gamma"], 2)
        v = np.where(rng.random(2) < outlier_frac, v * outlier_scale, v)
        zs[k] = H @ x + v
    prob["msmts"] = zs
    return prob


def many_gamma(d, pncc, steps, seed=0):
    """LTI problem whose terms grow pncc hyperplanes per step (pncc process-noise
    columns, Gamma 0.3 N(0,1)): up to (steps-1)*pncc + d hyperplanes, the
    shapes above the shared-memory bitmap limit.  Phi random stable
    (eigenvalue moduli in [0.8, 0.95]), H N(0,1), beta 0.05, gamma 0.2,
    p0 0.1."""
    rng = np.random.Generator(np.random.PCG64(seed))
    Phi = random_stable(rng, d, 0.8, 0.95)
    Gamma = 0.3 * rng.standard_normal((d, pncc))
    H = rng.standard_normal((1, d))
    prob = _base(d, pncc, 1, Phi, Gamma, [0.05] * pncc, H, [0.2], [0.1] * d, steps)
    prob["msmts"] = simulate(prob, rng)
    return prob


# -- a nonlinear (extended-mode) problem ---------------------------------------
# x = (angle, rate, drive); dt = 0.1
#   f(x) = (x0 + dt x1, x1 + dt (-0.5 sin x0 - 0.2 x1 + x2), 0.9 x2) + Gamma w,
#   Gamma = (0.05, 0.1, 1)
#   h(x) = (x0 + sqrt(1 + x0^2) - 1, x1 + 0.2 sin x2) + v
NONLIN_DT = 0.1
NONLIN_GAMMA = np.array([[0.05], [0.1], [1.0]])
NONLIN_BETA = np.array([0.1])
NONLIN_MSMT_GAMMA = np.array([0.2, 0.15])


def nonlin_f(x):
    dt = NONLIN_DT
    return np.array([x[0] + dt * x[1], x[1] + dt * (-0.5 * np.sin(x[0]) - 0.2 * x[1] + x[2]), 0.9 * x[2]])


def nonlin_F(x):
    """Jacobian of nonlin_f."""
    dt = NONLIN_DT
    return np.array([[1.0, dt, 0.0], [-0.5 * dt * np.cos(x[0]), 1.0 - 0.2 * dt, dt], [0.0, 0.0, 0.9]])


def nonlin_h(x):
    return np.array([x[0] + np.sqrt(1.0 + x[0] * x[0]) - 1.0, x[1] + 0.2 * np.sin(x[2])])


def nonlin_Hj(x):
    """Jacobian of nonlin_h."""
    return np.array([[1.0 + x[0] / np.sqrt(1.0 + x[0] * x[0]), 0.0, 0.0], [0.0, 1.0, 0.2 * np.cos(x[2])]])


def nonlin_three_state(seed=0, steps=10):
    """The extended-mode problem above: x_bar_0 = (0.3, -0.2, 0.1), A0 = I,
    p0 = (0.1, 0.08, 0.05), b0 = 0, beta = 0.1, gamma = (0.2, 0.15); the
    truth starts at x_bar_0 plus Cauchy(p0) noise."""
    rng = np.random.Generator(np.random.PCG64(seed))
    x0 = np.array([0.3, -0.2, 0.1])
    prob = {"d": 3, "pncc": 1, "cmcc": 0, "p": 2, "steps": steps, "x0": x0, "A0": np.eye(3),
            "p0": np.array([0.1, 0.08, 0.05]), "b0": np.zeros(3), "beta": NONLIN_BETA.copy(),
            "gamma": NONLIN_MSMT_GAMMA.copy(), "Gamma": NONLIN_GAMMA.copy()}
    x = x0 + _cauchy(rng, prob["p0"], 3)
    zs = np.zeros((steps, 2))
    for k in range(steps):
        if k > 0:
            x = nonlin_f(x) + NONLIN_GAMMA[:, 0] * _cauchy(rng, NONLIN_BETA[0])
        zs[k] = nonlin_h(x) + _cauchy(rng, NONLIN_MSMT_GAMMA, 2)
    prob["msmts"] = zs
    return prob


def nonlin_callbacks():
    """The problem's three extended-mode callbacks as Python functions over a
    pointer to the dynamics container (ctypes; any Structure with the
    reference's CauchyDynamicsUpdateContainer field names):
    dynamics (x <- f(x), Phi = F(x), Gamma, beta, is_xbar_set_for_ece),
    measurement model (zbar = h(x)) and extended update (H = dh/dx, gamma)."""

    def dyn(duc_ptr):
        c = duc_ptr.contents
        x = np.array([c.x[i] for i in range(3)])
        F = nonlin_F(x).reshape(-1)
        xn = nonlin_f(x)
        for i in range(3):
            c.x[i] = float(xn[i])
        for i in range(9):
            c.Phi[i] = float(F[i])
        for i in range(3):
            c.Gamma[i] = float(NONLIN_GAMMA[i, 0])
        c.beta[0] = float(NONLIN_BETA[0])
        c.is_xbar_set_for_ece = True

    def msmt(duc_ptr, zbar_ptr):
        c = duc_ptr.contents
        z = nonlin_h(np.array([c.x[i] for i in range(3)]))
        zbar_ptr[0], zbar_ptr[1] = float(z[0]), float(z[1])

    def ext(duc_ptr):
        c = duc_ptr.contents
        H = nonlin_Hj(np.array([c.x[i] for i in range(3)])).reshape(-1)
        for i in range(6):
            c.H[i] = float(H[i])
        c.gamma[0], c.gamma[1] = float(NONLIN_MSMT_GAMMA[0]), float(NONLIN_MSMT_GAMMA[1])

    return dyn, msmt, ext
