"""The tensor-core fold (tcgen05, 3xTF32 split products, FP32 accumulation)
against the FP64-class (double-float) fold on the same inputs: FP32-class agreement, 1e-6 of
each output row's largest value, on shapes that exercise the padding of
every tile dimension (channels, columns across signals, input intervals)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-6


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch

SHAPES = [(130, 32, 128, 1), (1500, 128, 128, 3), (300, 64, 64, 5), (257, 100, 50, 7)]


@pytest.mark.parametrize("K,q,N,batch", SHAPES)
def test_fold_tc_matches_fp64(cuda, K, q, N, batch):
    from xpsi_gb300._native import lib, check
    torch = cuda
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(K + q + N + batch)
    M = torch.tensor(rng.uniform(0, 1, (K, q)) * 10 ** rng.uniform(-3, 3, (K, 1)), device=dev)
    X = torch.tensor(rng.uniform(0, 1, (batch, q, N)), device=dev)
    ref = torch.empty((batch, K, N), dtype=torch.float64, device=dev)
    out = torch.full((batch, K, N), np.nan, dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream().cuda_stream
    L = lib()
    check(L.xgpu_fold_batch(batch, K, q, N, M.data_ptr(), q, X.data_ptr(), ref.data_ptr(), st))
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    check(L.xgpu_fold_batch_tc(batch, K, q, N, M.data_ptr(), q, X.data_ptr(), out.data_ptr(),
                               status.data_ptr(), st))
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    a, r = out.cpu().numpy(), ref.cpu().numpy()
    assert np.isfinite(a).all()
    rel = np.max(np.abs(a - r) / np.max(np.abs(r), axis=2, keepdims=True))
    assert rel <= TOL


def test_fold_tc_timeout_path_reports_status(cuda):
    """The failure path without a fault: a tile whose producer issues no
    copies lets both bounded waits run out; the kernel reports status 2,
    frees its tensor memory and returns, and the context stays usable (a
    regular fold afterwards is correct)."""
    import ctypes
    from xpsi_gb300._native import lib, check
    st = ctypes.c_int32(-1)
    check(lib().xgpu_fold_tc_timeout_selftest(ctypes.byref(st)))
    assert st.value == 2
    test_fold_tc_matches_fp64(cuda, 300, 64, 64, 1)
