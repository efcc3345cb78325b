"""The allocation-free likelihood entry point, xgpu_likelihood_batch_static.

It serves callers that cannot allocate device memory when they evaluate the
likelihood (a host whose framework owns all device memory through its own
pool, or code held to a fixed memory budget): they pass device inputs and
outputs, and the per-channel scratch lives in a fixed array inside the
library.  Here it is called twice in a row through the C ABI and must agree
with xgpu_likelihood_batch, which takes caller-provided scratch, to the
log-likelihood tolerance of the other tests (1e-7 absolute).  This file is
collected last so that a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LOGL_ATOL = 1e-7


def _data(torch, f, n_vec):
    dev = torch.device("cuda", 0)
    t = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    reg = f["registered"]
    K, N_P = reg.shape
    B = f["counts"].shape[1]
    keep = dict(
        phase_edges=t(f["phase_edges"]), comp_phases=t(f["comp_phases"]),
        counts=t(np.asarray(f["counts"], np.float64)), precomp=t(f["precomp"]),
        support=t(f["support"]),
        signals=t(np.array(np.broadcast_to(reg, (n_vec, 1, K, N_P)))),
        shifts=t(np.zeros((n_vec, 1)) + f["shifts"][0]),
        allow_negative=t(np.zeros(1), torch.int32),
        chan_ll=torch.empty((n_vec, K), dtype=torch.float64, device=dev),
        chan_flag=torch.empty((n_vec, K), dtype=torch.int32, device=dev),
        loglike=torch.empty(n_vec, dtype=torch.float64, device=dev),
        status=torch.empty(n_vec, dtype=torch.int32, device=dev))
    from xpsi_gb300._native import LikelihoodBatchData
    d = LikelihoodBatchData()
    d.n_vec, d.K, d.B, d.H, d.N_P = n_vec, K, B, 1, N_P
    d.exposure, d.epsabs, d.epsrel = float(f["exposure"]), 0.0, 1e-8
    d.epsilon, d.sigmas, d.llzero, d.slim = 1e-3, 10.0, -1e90, 20.0
    for k in ("phase_edges", "comp_phases", "counts", "precomp", "support", "signals",
              "shifts", "allow_negative", "chan_ll", "chan_flag", "loglike", "status"):
        setattr(d, k, keep[k].data_ptr())
    d.background = d.star = d.mcl_bg = d.mcl_bg_support = None
    return d, keep


def test_static_scratch_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conftest import load_golden
    from xpsi_gb300._native import lib
    f = load_golden("examples_fast")
    L = lib()
    stream = torch.cuda.current_stream().cuda_stream
    d, keep = _data(torch, f, n_vec=3)
    assert L.xgpu_likelihood_batch(C.byref(d), stream) == 0
    torch.cuda.synchronize()
    ref = keep["loglike"].cpu().numpy().copy()
    ref_st = keep["status"].cpu().numpy().copy()
    assert abs(ref[0] - float(f["logL"])) <= LOGL_ATOL
    for _ in range(2):
        keep["loglike"].fill_(0.0)
        keep["status"].fill_(-1)
        assert L.xgpu_likelihood_batch_static(C.byref(d), stream) == 0
        torch.cuda.synchronize()
        np.testing.assert_allclose(keep["loglike"].cpu().numpy(), ref, rtol=0, atol=LOGL_ATOL)
        np.testing.assert_array_equal(keep["status"].cpu().numpy(), ref_st)


def test_static_scratch_rejects_oversize():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conftest import load_golden
    from xpsi_gb300._native import lib
    f = load_golden("examples_fast")
    d, keep = _data(torch, f, n_vec=1)
    d.n_vec = 349525 // d.K + 1  # one evaluation more than the array holds
    assert lib().xgpu_likelihood_batch_static(C.byref(d), None) == -3
