"""Drop-in for xpsi.likelihoods._poisson_likelihood_given_background
(xpsi/likelihoods/_poisson_likelihood_given_background.pyx:14-113), on the
GPU: the expected counts (star components plus the known background) and
the Poisson log-likelihood are formed by the library; the reference's
randomised penalty for bins with no expected but some observed counts is
drawn here, one numpy.random.rand(1) per bin as the reference draws it."""
import numpy as np

from .._arr import f64, ptr
from .._interp import require_default_interpolants
from .._native import Component, check, lib
from ..tools.synthesise import _allow_negative


def poisson_likelihood_given_background(exposure_time, phases, counts, components,
                                        component_phases, phase_shifts, background,
                                        neg_sum_ln_data_factorial=None, allow_negative=False):
    """(log L, expected counts [K, B]) as the reference returns them."""
    require_default_interpolants(phase=True, energy=False)
    ph = f64(phases)
    comps = [f64(c) for c in components]
    cph = [f64(c) for c in component_phases]
    H = len(comps)
    if H == 0 or len(cph) != H:
        raise ValueError("one phase array per component is needed")
    K = comps[0].shape[0]
    B = ph.size - 1
    d = f64(counts)
    if d.shape != (K, B):
        raise ValueError("counts must be [channels, phase intervals]")
    sh = f64(phase_shifts).reshape(-1)
    if sh.size != H:
        raise ValueError("one phase shift per component is needed")
    arr = (Component * H)()
    for h, (c, p) in enumerate(zip(comps, cph)):
        if c.ndim != 2 or c.shape[0] != K or c.shape[1] != p.size:
            raise ValueError("component %d must be [channels, phases]" % h)
        arr[h] = Component(c.ctypes.data, p.ctypes.data, c.shape[1], c.shape[1], float(sh[h]))
    bg = f64(background)
    if bg.shape != (K, B):
        raise ValueError("background must be [channels, phase intervals]")
    pre = f64(neg_sum_ln_data_factorial) if neg_sum_ln_data_factorial is not None else None
    if pre is not None and pre.size != K:
        raise ValueError("neg_sum_ln_data_factorial must have one entry per channel")
    an = _allow_negative(allow_negative, H)
    expec = np.empty((K, B))
    ll = np.zeros(1)
    pen = np.zeros(1, dtype=np.int64)
    check(lib().xgpu_poisson_likelihood_given_background(
        float(exposure_time), B, ptr(ph), K, ptr(d), H, arr, ptr(bg), ptr(pre), ptr(an),
        ptr(expec), ptr(ll), ptr(pen)))
    LOGLIKE = float(ll[0])
    for _ in range(int(pen[0])):
        LOGLIKE += -1.0e90 * (0.1 + 0.9 * np.random.rand(1))[0]
    return (LOGLIKE, np.asarray(expec, order="C", dtype=np.double))
