"""mce_batch_step_noalloc (no counterpart in the reference) against
mce_batch_step, both called through the C ABI.

The same batch stepped through either entry point must give the same term
counts, terms per shape and error bits, and moments within 1e-9 relative
(REL_TOL); several calls of the no-allocation step follow each other, and a
second pass after a reset runs on a static scratch array that still holds the
first pass's contents.  Collected last so it also runs after every other test
in the same process.
"""
import ctypes

import numpy as np
import pytest

import oracle
from tests import golden_cases as G

pytestmark = pytest.mark.gpu

MCE_ERR_NOMEM = -6


def _need_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cauchyfriendly_gb300 import BatchedCauchyEstimator, _lib
    return BatchedCauchyEstimator, _lib


def _p(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


class _Batch:
    """One batched handle over `probs`, stepped through either entry point."""

    def __init__(self, probs, consts):
        BCE, self.lib = _need_gpu()
        n = len(probs)
        self.probs = probs
        steps = np.array([q["steps"] for q in probs], np.int32)
        ms = oracle.max_shape_of({"steps": int(steps.max()), "d": probs[0]["d"], "pncc": probs[0]["pncc"]})
        rp = np.stack([c[0] for c in consts])
        bp = np.zeros((n, ms))
        for i, c in enumerate(consts):
            bp[i, :len(c[1])] = c[1]
        q0 = probs[0]
        self.est = BCE(np.stack([q["A0"] for q in probs]), np.stack([q["p0"] for q in probs]),
                       np.stack([q["b0"] for q in probs]), steps, q0["d"], q0["cmcc"], q0["pncc"], q0["p"], rp, bp)
        self.max_steps = int(steps.max())
        self.p = q0["p"]
        self.z = np.zeros((n, self.max_steps, self.p))
        for i, q in enumerate(probs):
            self.z[i, :q["steps"]] = q["msmts"]
        self.Phi = np.ascontiguousarray(np.stack([q["Phi"] for q in probs]))
        self.Gam = np.ascontiguousarray(np.stack([q["Gamma"] for q in probs]))
        self.beta = np.ascontiguousarray(np.stack([q["beta"] for q in probs]))
        self.H = np.stack([q["H"] for q in probs])
        self.gam = np.stack([q["gamma"] for q in probs])

    def updates(self):
        return [(k, s) for k in range(self.max_steps) for s in range(self.p)]

    def call(self, fn_name, k, s):
        """One update of every estimator through the named C entry point;
        returns (status, error bits)."""
        n = len(self.probs)
        z = np.ascontiguousarray(self.z[:, k, s])
        H = np.ascontiguousarray(self.H[:, s, :])
        g = np.ascontiguousarray(self.gam[:, s])
        err = np.zeros(n, np.int32)
        fn = getattr(self.lib.load(), fn_name)
        rc = fn(self.est._h, _p(z), _p(self.Phi), _p(self.Gam), _p(self.beta), _p(H), _p(g), None, None, 0,
                _p(err, ctypes.c_int))
        return rc, err

    def record(self, k):
        out = []
        for i, q in enumerate(self.probs):
            if k < q["steps"]:
                r = self.est.moments(i)
                r["err"] = self.est.errors(i)
                r["Nt"] = self.est.num_terms(i)
                r["tps"] = self.est.terms_per_shape(i)
                out.append(r)
            else:
                out.append(None)
        return out

    def run(self, fn_name):
        recs = []
        for k, s in self.updates():
            rc, err = self.call(fn_name, k, s)
            assert rc == 0, (fn_name, k, s, rc, self.lib.load().mce_last_error())
            recs.append((err.copy(), self.record(k)))
        return recs

    def close(self):
        self.est.close()


def _compare(got, want):
    assert len(got) == len(want)
    for u, ((eg, rg), (ew, rw)) in enumerate(zip(got, want)):
        assert np.array_equal(eg, ew), u
        for i, (a, b) in enumerate(zip(rg, rw)):
            assert (a is None) == (b is None)
            if a is None:
                continue
            assert a["err"] == b["err"] and a["Nt"] == b["Nt"], (u, i)
            assert np.array_equal(a["tps"], b["tps"]), (u, i)
            for key in ("fz", "mean", "cov", "raw_fz", "raw_mean", "raw_cov", "gscale"):
                assert G.relerr(a[key], b[key]) <= G.REL_TOL, (u, i, key)


def _three_state_batch():
    from cauchyfriendly_gb300 import workloads as W
    probs = W.batched_three_state(40, seed=21, steps_lo=4, steps_hi=8)
    consts = [oracle.draw_reference_constants(300 + i, 3, oracle.max_shape_of(q)) for i, q in enumerate(probs)]
    return probs, consts


def _five_state_batch():
    # 5 states, two measurements per step, up to 11 hyperplanes: each warp
    # needs 386 half-cells (6 KB) of g-table scratch, so the static array
    # holds 5,433 warps where the allocating path launches 9,728, and the
    # later updates have more roots than that
    from cauchyfriendly_gb300 import workloads as W
    probs = [W.five_state_two_msmt(seed=s, steps=4) for s in range(3)]
    consts = [oracle.draw_reference_constants(400 + i, 5, oracle.max_shape_of(q)) for i, q in enumerate(probs)]
    return probs, consts


@pytest.mark.parametrize("make", [_three_state_batch, _five_state_batch], ids=["three_state", "five_state"])
def test_noalloc_step_matches_allocating_step(make):
    _need_gpu()
    probs, consts = make()
    ref = _Batch(probs, consts)
    want = ref.run("mce_batch_step")
    ref.close()
    if make is _five_state_batch:
        # the case is meant to cover the clamped launch: some table build has
        # more roots (post-reduction terms) than the static array has warp slots
        roots = [sum(r["Nt"] for r in recs if r is not None) for _, recs in want[:-1]]
        assert max(roots) > 5433, roots

    b = _Batch(probs, consts)
    # a fresh handle holds no term buffers yet: the first step needs memory
    # and the no-allocation entry point refuses it
    rc, _ = b.call("mce_batch_step_noalloc", 0, 0)
    assert rc == MCE_ERR_NOMEM
    assert b"may not allocate" in b.lib.load().mce_last_error()
    b.est.reset()
    # the allocating step sizes the handle's buffers for this history
    b.run("mce_batch_step")
    b.est.reset()
    got = b.run("mce_batch_step_noalloc")
    _compare(got, want)
    # again, on a scratch array that keeps the previous calls' contents
    b.est.reset()
    got2 = b.run("mce_batch_step_noalloc")
    _compare(got2, want)
    assert b.est.device_errors() == 0
    b.close()

