"""The sampler adapter on the GPU: a sampler's points in its own column
order give the batched path's log-likelihoods of the same vectors."""
import numpy as np
import pytest

from xpsi_gb300 import batch as BT
from xpsi_gb300 import synthetic as SY
from xpsi_gb300.sampler import BatchedLikelihood

pytestmark = pytest.mark.gpu


def test_batched_likelihood_matches_evaluator():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    model = SY.config2_model()
    params = SY.config3_vectors(6, seed=7)
    ours = BT.param_names(model)
    names = list(reversed([n for n in ours if n != "distance"]))
    like = BatchedLikelihood(model, names, fixed={"distance": 1.0}, max_batch=4)
    pts = np.stack([params[:, ours.index(n)] for n in names], axis=1)
    ll = like(pts)
    ref, st = BT.BatchEvaluator(model).loglikelihood(params)
    ok = st == 0
    np.testing.assert_allclose(ll[ok], ref[ok], rtol=0, atol=1e-7)
    assert like.calls == 1 and like.points == 6
