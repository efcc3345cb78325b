"""The batched GPU path (many parameter vectors per launch) against the CPU
oracle run vector by vector on the same packed inputs."""
import numpy as np
import pytest

from batch_cases import small_blackbody, small_num4d
from conftest import row_rel
from oracle import pipeline as OP
from xpsi_gb300 import batch as BT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("builder", [small_num4d, small_blackbody])
def test_batch_loglike_vs_oracle(cuda, builder):
    m, params = builder()
    P = BT.prepare(m, params)
    ref, ref_st, stages = OP.loglike(m, P, return_stages=True)
    ev = BT.BatchEvaluator(m)
    B = ev.upload(P)
    ev.run(B)
    cuda.cuda.synchronize()
    st = ev.statuses(B)
    ll = B["loglike"].cpu().numpy()
    np.testing.assert_array_equal(st, ref_st)
    ok = st == 0
    assert ok.any()
    assert np.max(np.abs(ll[ok] - ref[ok])) <= 1e-7
    flux = B["flux"].cpu().numpy()
    k = 0
    for v in range(P.V):
        if ref_st[v]:
            continue
        for h in range(P.H):
            assert row_rel(flux[v * P.H + h], stages[k]["flux"]) <= 1e-9
            k += 1


def test_batch_vector_independence(cuda):
    """A vector's result does not depend on what else is in the batch (the
    parallels of a mesh may be summed in different chunkings, so the check
    is to round-off, 1e-12 relative)."""
    m, params = small_num4d(V=4)
    ev = BT.BatchEvaluator(m)
    ll_all, _ = ev.loglikelihood(params)
    ll_one, _ = ev.loglikelihood(params[2:3])
    assert abs(ll_all[2] - ll_one[0]) <= 1e-12 * abs(ll_one[0])


def test_pipelined_equals_sequential(cuda):
    """Batches evaluated two at a time on separate streams give exactly the
    sequential results, in order."""
    m, params = small_num4d(V=4)
    ev = BT.BatchEvaluator(m)
    batches = [params[:2], params[2:], params[1:3]]
    seq = [ev.loglikelihood(b) for b in batches]
    pipe = list(ev.loglikelihood_pipelined(batches, depth=2))
    assert len(pipe) == len(seq)
    for (a, sa), (b, sb) in zip(seq, pipe):
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(sa, sb)
