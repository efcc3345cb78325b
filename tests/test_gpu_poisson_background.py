"""The known-background Poisson likelihood
(_poisson_likelihood_given_background.pyx:14-113) through the drop-in
against the reference on config1's signal and data
(tests/golden/poisson_given_background.npz): expected counts within 1e-12,
log L within 1e-7 absolute, with and without the data-factorial constants;
zero-count channels with nothing expected add nothing; a channel with counts
but nothing expected draws the reference's penalty, -1e90 (0.1 + 0.9 U) per
such bin from numpy's generator (the reference's own penalty branch needs
numpy < 2 to run, so it is checked against that formula here)."""
import numpy as np
import pytest

from conftest import load_golden
from xpsi_gb300.likelihoods._poisson_likelihood_given_background import (
    poisson_likelihood_given_background as plgb)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _args(f, reg, counts, bg):
    return (float(f["exposure"]), f["phase_edges"], counts, [reg], [f["comp_phases"]],
            f["shifts"], bg)


def test_poisson_given_background_vs_reference(cuda):
    f = load_golden("poisson_given_background")
    ll, ex = plgb(*_args(f, f["registered"], f["counts"], f["background"]))
    np.testing.assert_allclose(ex, f["expec"], rtol=1e-12, atol=0)
    assert abs(ll - float(f["ll_nopre"])) <= 1e-7
    ll2, _ = plgb(*_args(f, f["registered"], f["counts"], f["background"]), f["precomp"])
    assert abs(ll2 - float(f["ll_pre"])) <= 1e-7


def test_zero_channels_and_penalty(cuda):
    f = load_golden("poisson_given_background")
    r0, c0, b0 = f["registered"].copy(), f["counts"].copy(), f["background"].copy()
    r0[:3] = c0[:3] = b0[:3] = 0.0
    ll, ex = plgb(*_args(f, r0, c0, b0), f["precomp"])
    assert np.all(ex[:3] == 0.0)
    np.testing.assert_allclose(ex, f["expec_zero"], rtol=1e-12, atol=0)
    assert abs(ll - float(f["ll_zero"])) <= 1e-7
    r1, b1 = f["registered"].copy(), f["background"].copy()
    r1[0] = b1[0] = 0.0
    n_pen = int(np.count_nonzero(f["counts"][0] > 0))
    assert n_pen > 0
    np.random.seed(11)
    ll, _ = plgb(*_args(f, r1, f["counts"], b1), f["precomp"])
    np.random.seed(11)
    pen = sum(-1.0e90 * (0.1 + 0.9 * np.random.rand(1))[0] for _ in range(n_pen))
    assert ll == pytest.approx(pen, rel=1e-12)
    assert -1.0e90 * n_pen <= ll <= -0.1e90 * n_pen
