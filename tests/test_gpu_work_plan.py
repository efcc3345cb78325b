"""The integrator's device work plan: the same batch cut into very different
numbers of chunks (target_ctas 1, 3, 50 and the default) gives the same
fluxes to round-off -- every parallel is integrated exactly once whatever the
cut -- including a star near the photon sphere, whose parallels carry
several images and so the heaviest chunks."""
import numpy as np
import pytest

from batch_cases import small_num4d
from conftest import row_rel
from xpsi_gb300 import batch as BT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_chunk_counts_agree(cuda):
    m, params = small_num4d(V=5)
    params = params.copy()
    # vector 0: radius 1.02 x the photon sphere's (3 r_g), so its rays wind
    # round the star and its parallels hold several images
    r_g_km = params[0, 0] * 0.5 * 2.95325024
    params[0, 1] = 3.06 * r_g_km
    P = BT.prepare(m, params)
    out = {}
    for tc in (0, 1, 3, 50):
        ev = BT.BatchEvaluator(m)
        ev.target_ctas = tc
        B = ev.upload(P)
        ev.run(B)
        cuda.cuda.synchronize()
        out[tc] = (B["flux"].cpu().numpy(), ev.statuses(B), B["loglike"].cpu().numpy())
    f0, s0, l0 = out[0]
    assert np.abs(f0).max() > 0
    for tc in (1, 3, 50):
        f, st, ll = out[tc]
        np.testing.assert_array_equal(st, s0)
        for i in range(f0.shape[0]):
            assert row_rel(f[i], f0[i]) <= 1e-12, (tc, i)
        ok = s0 == 0
        assert np.max(np.abs(ll[ok] - l0[ok])) <= 1e-9
