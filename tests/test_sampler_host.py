"""The sampler adapter's host logic (column mapping, fixed parameters,
chunking, early-exit values) with a stand-in evaluator; CPU only."""
import numpy as np
import pytest

from xpsi_gb300 import batch as BT
from xpsi_gb300 import synthetic as SY
from xpsi_gb300.sampler import BatchedLikelihood


@pytest.fixture(scope="module")
def model():
    return SY.config2_model()


class FakeEvaluator:
    """log L = sum of the parameter vector; status 5 when the first entry < 0."""

    def __init__(self):
        self.batches = []

    def loglikelihood(self, params):
        self.batches.append(params.shape[0])
        st = np.where(params[:, 0] < 0, 5, 0).astype(np.int32)
        return params.sum(axis=1), st


def test_columns_fixed_and_chunks(model):
    ours = BT.param_names(model)
    names = list(reversed([n for n in ours if n != "distance"]))
    fake = FakeEvaluator()
    like = BatchedLikelihood(model, names, fixed={"distance": 2.5}, max_batch=4,
                             evaluator=fake)
    rng = np.random.default_rng(1)
    pts = rng.uniform(0.1, 1.0, (10, len(names)))
    ll = like(pts)
    assert fake.batches == [4, 4, 2]
    np.testing.assert_allclose(ll, pts.sum(axis=1) + 2.5)
    full = like.full_vectors(pts)
    for j, n in enumerate(ours):
        if n == "distance":
            assert np.all(full[:, j] == 2.5)
        else:
            np.testing.assert_array_equal(full[:, j], pts[:, names.index(n)])


def test_exit_value_and_errors(model):
    ours = BT.param_names(model)
    like = BatchedLikelihood(model, None, fixed={"distance": 1.0}, exit_value="-inf",
                             evaluator=FakeEvaluator())
    pts = np.ones((3, like.ndim))
    assert like.names[0] == "mass"  # the fake evaluator flags a negative first entry
    pts[1, 0] = -1.0
    ll = like(pts)
    assert ll[1] == -np.inf and np.all(np.isfinite(ll[[0, 2]]))
    with pytest.raises(KeyError):
        BatchedLikelihood(model, ["mass", "nonsense"], evaluator=FakeEvaluator())
    with pytest.raises(KeyError):
        BatchedLikelihood(model, ours[1:], evaluator=FakeEvaluator())  # mass neither
    with pytest.raises(ValueError):
        like(np.ones((2, like.ndim + 1)))
