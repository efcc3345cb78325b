"""The instrument-response fold of Instrument.__call__ (xpsi/Instrument.py:163-197)."""
import numpy as np

from ._arr import f64, ptr
from ._native import check, lib


def fold(matrix, signal, irange=None, orange=None):
    """matrix[orange, irange] @ signal on the GPU (FP64).

    irange/orange are (start, stop) pairs as in Instrument.__call__; None
    means the full axis.
    """
    M = f64(matrix)
    if orange is not None:
        M = M[orange[0]:orange[1]]
    if irange is not None:
        M = M[:, irange[0]:irange[1]]
    M = f64(M)
    S = f64(signal)
    K, q = M.shape
    if S.shape[0] != q:
        raise ValueError("signal rows must match the matrix input intervals")
    out = np.empty((K, S.shape[1]))
    check(lib().xgpu_response_fold(K, q, S.shape[1], ptr(M), q, ptr(S), ptr(out)))
    return out


def gpu_instrument_call(self, signal, irange, orange):
    """A replacement for Instrument.__call__ that folds on the GPU and keeps
    the reference's caching of the registered signal (Instrument.py:192-197)."""
    self._cached_signal = fold(self.matrix, signal, irange, orange)
    return self._cached_signal
