"""The batched response fold (xgpu_fold_batch: power-of-two scaled
double-float products and sums) against an FP64 product on the host.

Bar: each output within 1e-12 of the sum of its terms' magnitudes
(|M| @ |X|; the median within 3e-14), where a plain FP64 sum carries ~1e-16
of it.  The float exponent range bounds what the scaling can carry: an
operand more than ~2^-186 below the largest of its matrix row or input column
is held at the float's subnormal spacing, so the bar adds q 2^-190 of (row
maximum x column maximum) -- 1e-55 of the largest product, far below any
count rate the likelihood can resolve.  The wide-range case hits that floor
on purpose: matrix rows whose scales differ by 60 decades with Gaussian
tails, columns with exponential tails down to 1e-300, subnormal and zero
entries, a zero row and a zero column, negative values; then a row stride
larger than q, tile padding in every dimension, and an empty batch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _fold(torch, M, X, ld=None):
    from xpsi_gb300._native import lib, check
    dev = torch.device("cuda", 0)
    K, q = M.shape
    batch, _, N = X.shape
    ld = ld or q
    Mp = np.zeros((K, ld))
    Mp[:, :q] = M
    Mp[:, q:] = np.nan  # columns past q must not be read
    dM = torch.tensor(Mp, device=dev)
    dX = torch.tensor(X, device=dev)
    out = torch.full((batch, K, N), np.nan, dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream().cuda_stream
    check(lib().xgpu_fold_batch(batch, K, q, N, dM.data_ptr(), ld, dX.data_ptr(),
                                out.data_ptr(), st))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _check(M, X, got, floor=True):
    q = M.shape[1]
    ref = np.einsum("kq,bqn->bkn", M, X)
    mag = np.einsum("kq,bqn->bkn", np.abs(M), np.abs(X))
    rowmax = np.abs(M).max(axis=1)[None, :, None]
    colmax = np.abs(X).max(axis=1)[:, None, :]
    bound = TOL * mag + (q * 2.0 ** -190 * rowmax * colmax if floor else 0.0)
    err = np.abs(got - ref)
    assert np.isfinite(got).all()
    assert np.all(err <= bound)
    # the median over outputs clear of the floor
    clear = mag > 1e-40 * rowmax * colmax
    assert clear.sum() >= 0.05 * clear.size
    assert np.median(err[clear] / mag[clear]) <= 3e-14


@pytest.mark.parametrize("K,q,N,batch", [(1500, 128, 128, 2), (97, 29, 13, 3), (65, 16, 64, 1),
                                         (3, 300, 70, 2)])
def test_fold_wide_range(cuda, K, q, N, batch):
    rng = np.random.default_rng(7 * K + q)
    # rows: Gaussian redistribution around a channel energy, row scales over 60 decades
    e = np.linspace(0, 1, q)
    c = rng.uniform(0, 1, (K, 1))
    M = np.exp(-0.5 * ((e[None, :] - c) / 0.03) ** 2) * 10 ** rng.uniform(-30, 30, (K, 1))
    M[rng.uniform(size=M.shape) < 0.05] = 0.0
    M[0] = 0.0
    # columns: exponential spectra with column scales over 40 decades and tails to 1e-300
    X = np.exp(-rng.uniform(5, 700, (batch, 1, N)) * e[None, :, None])
    X *= 10 ** rng.uniform(-20, 20, (batch, 1, N))
    X[:, :, 0] = 0.0
    X[0, q // 2, 1 % N] = 5e-324  # subnormal
    X[-1, :, -1] *= np.where(rng.uniform(size=q) < 0.3, -1.0, 1.0)
    got = _fold(cuda, M, X)
    _check(M, X, got)
    assert np.all(got[:, 0, :] == 0) and np.all(got[:, :, 0] == 0)  # zero row, zero column


def test_fold_ordinary_range(cuda):
    """Rows within 1e-21 and columns within 1e-13 of their maxima: the bar
    holds with no floor."""
    rng = np.random.default_rng(11)
    K, q, N = 1500, 128, 128
    e = np.linspace(0, 1, q)
    c = rng.uniform(0, 1, (K, 1))
    M = np.exp(-0.5 * ((e[None, :] - c) / 0.1) ** 2) * 10 ** rng.uniform(-30, 30, (K, 1))
    X = np.exp(-rng.uniform(5, 30, (2, 1, N)) * e[None, :, None])
    X *= 10 ** rng.uniform(-20, 20, (2, 1, N))
    _check(M, X, _fold(cuda, M, X), floor=False)


def test_fold_row_stride(cuda):
    rng = np.random.default_rng(3)
    M = rng.uniform(-1, 1, (200, 50))
    X = rng.uniform(0, 1, (2, 50, 40))
    _check(M, X, _fold(cuda, M, X, ld=64))


def test_fold_empty_batch(cuda):
    """batch 0 launches nothing and succeeds."""
    from xpsi_gb300._native import lib, check
    torch = cuda
    st = torch.cuda.current_stream().cuda_stream
    M = torch.ones((4, 4), dtype=torch.float64, device="cuda")
    check(lib().xgpu_fold_batch(0, 4, 4, 4, M.data_ptr(), 4, 0, 0, st))
