"""Drop-in for xpsi.likelihoods.default_background_marginalisation
(xpsi/likelihoods/default_background_marginalisation.pyx:38-734)."""
import ctypes as C

import numpy as np

from .._arr import f64, i32, ptr
from .._interp import require_default_interpolants
from .._native import check, lib

XGPU_SLIM_CUT = 5
XGPU_QUAD_FAIL = 4


def precomputation(data):
    """Negative sum over phase bins of log-factorials of the counts, per channel."""
    d = i32(data)
    out = np.zeros(d.shape[0])
    check(lib().xgpu_precomputation(d.shape[0], d.shape[1], ptr(d), ptr(out)))
    return out


def eval_marginal_likelihood(exposure_time, phases, counts, components, component_phases,
                             phase_shifts, neg_sum_ln_data_factorial, support,
                             workspace_intervals, epsabs, epsrel, epsilon, sigmas, llzero,
                             allow_negative=False, slim=20.0, background=None):
    """Expected counts and the background-marginalised Poisson log-likelihood.

    Returns (logL, STAR[K, B], MCL_BACKGROUND[K], MCL_BACKGROUND_GIVEN_SUPPORT[K])
    like the reference, and raises TypeError on an invalid support as it does
    (:596-603).  When the reference would return a random value near llzero
    (slim cut, vanished integral) so does this, drawn from a hash of the
    channel index instead of numpy's global generator.
    """
    require_default_interpolants(phase=True, energy=False)
    ph = f64(phases)
    cnt = f64(counts)
    comps = [f64(c) for c in components]
    cph = [f64(c) for c in component_phases]
    H = len(comps)
    K, B = cnt.shape
    sup = f64(support)
    if sup.shape[0] != K:
        raise TypeError('The number of energy channels in the background support does not '
                        'match to that of the data.')
    for i in range(sup.shape[0]):
        if sup[i, 1] == 0:
            raise TypeError('Background upper limit cannot be set to 0.')
        if sup[i, 1] > 0 and sup[i, 1] - sup[i, 0] < 0:
            raise TypeError('Background upper limit must be higher than the lower limit.')
    if isinstance(allow_negative, bool):
        an = np.full(H, int(allow_negative), dtype=np.int32)
    else:
        if len(allow_negative) != H:
            raise ValueError('Number of allow_negative declarations does not match the '
                             'number of components..')
        an = i32([int(x) for x in allow_negative])
    cptr = (C.c_void_p * H)(*[c.ctypes.data for c in comps])
    pptr = (C.c_void_p * H)(*[c.ctypes.data for c in cph])
    nph = (C.c_size_t * H)(*[c.shape[1] for c in comps])
    sh = f64(phase_shifts)
    pre = f64(neg_sum_ln_data_factorial)
    bg = f64(background) if background is not None else None
    STAR = np.zeros((K, B))
    mb = np.zeros(K)
    mbs = np.zeros(K)
    ll = C.c_double(0.0)
    check(lib().xgpu_eval_marginal_likelihood(
        float(exposure_time), B, ptr(ph), K, ptr(cnt), H, C.cast(cptr, C.c_void_p),
        C.cast(nph, C.c_void_p), C.cast(pptr, C.c_void_p), ptr(sh), ptr(pre), ptr(sup),
        float(epsabs), float(epsrel), float(epsilon), float(sigmas), float(llzero), ptr(an),
        float(slim), ptr(bg), C.byref(ll), ptr(STAR), ptr(mb), ptr(mbs)))
    return (ll.value, STAR, mb, mbs)
