"""The Gaussian likelihoods of polarimetry on the GPU (through the C ABI)
against the reference's own values."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gl():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import xpsi_gb300
    xpsi_gb300.lib()
    from xpsi_gb300.likelihoods import (_gaussian_likelihood_given_background_IQU as gb,
                                        _gaussian_likelihood_QnUn as qn)
    return gb, qn


def test_gaussian_given_background_vs_reference(gl, golden):
    gb, _ = gl
    f, z = golden("config1"), golden("gaussian")
    ll, expec = gb.gaussian_likelihood_given_background(
        float(z["exposure"]), f["phase_edges"], z["counts"], z["errors"], (f["folded"][:40],),
        (f["comp_phases"],), np.array([0.2]), z["bkg"])
    np.testing.assert_allclose(expec, z["expec"], rtol=1e-12, atol=0)
    assert abs(ll - float(z["loglike"])) <= 1e-7


def test_gaussian_QnUn_vs_reference(gl, golden):
    _, qn = gl
    z = golden("gaussian")
    ll, star = qn.gaussian_likelihood_QnUn(golden("config1")["phase_edges"], z["qn"],
                                          z["qn_err"], z["star"])
    np.testing.assert_array_equal(star, z["star"])
    assert abs(ll - float(z["loglike_qn"])) <= 1e-7


def test_gaussian_many_rows(gl):
    """More rows than the kernel keeps per lane (> 256): the same value as
    the sequential sum to rounding."""
    from oracle import oracle as O
    _, qn = gl
    rng = np.random.default_rng(4)
    d = rng.normal(0, 1, (700, 12))
    e = rng.uniform(0.5, 1.5, (700, 12))
    s = rng.normal(0, 1, 12)
    ll, _ = qn.gaussian_likelihood_QnUn(np.linspace(0, 1, 13), d, e, s)
    ref = O.gaussian_loglike(s, d, e)
    assert abs(ll - ref) <= 1e-12 * abs(ref)
