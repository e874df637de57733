"""Extended-mode helpers on the GPU (mce_finalize_extended_moments,
mce_deterministic_time_prop, mce_shift_cf_by_bias) against the reference's
recorded op sequences (tests/golden/ext_*.npz)."""
import pytest

from tests import golden_cases as G

pytestmark = pytest.mark.gpu


class _Gpu:
    """A GPU CauchyEstimator with the interface run_extended drives."""

    def __init__(self, prob, rp, bp):
        torch = pytest.importorskip("torch")
        if not torch.cuda.is_available():
            pytest.skip("no CUDA device")
        from cauchyfriendly_gb300 import CauchyEstimator
        self.prob = prob
        self.est = CauchyEstimator(prob["A0"], prob["p0"], prob["b0"], prob["steps"], prob["d"], prob["cmcc"],
                                   prob["pncc"], prob["p"], root_point=rp, b_pert=bp)

    def step(self, k, s):
        pr = self.prob
        Phi = pr["Phi"] if pr["Phi"].ndim == 2 else pr["Phi"][k]
        return self.est.step(pr["msmts"][k, s], Phi, pr["Gamma"], pr["beta"], pr["H"][s], pr["gamma"][s])

    def finalize_extended_moments(self, x):
        return self.est.finalize_extended_moments(x)

    def deterministic_time_prop(self, Phi):
        self.est.deterministic_time_prop(Phi)

    def shift_cf_by_bias(self, b):
        self.est.shift_cf_by_bias(b)

    def moments(self):
        return self.est.moments()

    def num_terms(self):
        return self.est.num_terms()


@pytest.mark.parametrize("name", G.ext_names())
def test_gpu_extended_ops_match_reference(name):
    prob, (rp, bp), want = G.load_ext(name)
    g = _Gpu(prob, rp, bp)
    got = G.run_extended(g, prob, G.extended_ops(prob))
    assert g.est.device_errors() == 0
    g.est.close()
    G.compare_extended(got, want)
