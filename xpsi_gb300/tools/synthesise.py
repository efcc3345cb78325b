"""Drop-ins for xpsi.tools.synthesise (xpsi/tools/synthesise.pyx:35-276):
expected counts on the GPU (compute_expected_counts.pyx:200-276) and their
Poisson realisations drawn on the GPU.

The realisations follow the Poisson law as the reference's gsl_ran_poisson
draws do, from a counter-based generator (Philox4x32-10) keyed by gsl_seed:
the same seed gives the same data, but not the numbers of GSL's stream."""
import time

import numpy as np

from .._arr import f64, ptr
from .._interp import require_default_interpolants
from .._native import Component, check, lib


def _allow_negative(allow_negative, H):
    if isinstance(allow_negative, (bool, np.bool_, int)):
        return np.full(H, int(bool(allow_negative)), dtype=np.int32)
    a = np.asarray([int(bool(x)) for x in allow_negative], dtype=np.int32)
    if a.size != H:
        raise ValueError("allow_negative needs one entry per component")
    return a


def compute_expected_counts(exposure_time, phases, components, component_phases,
                            phase_shifts, background, allow_negative=False):
    """[K, B] expected counts: exposure x (the components' bin-integrated
    count rates, clamped at zero, + the background count rates [K, B])."""
    require_default_interpolants(phase=True, energy=False)
    ph = f64(phases)
    comps = [f64(c) for c in components]
    cph = [f64(c) for c in component_phases]
    H = len(comps)
    if H == 0 or len(cph) != H:
        raise ValueError("one phase array per component is needed")
    K = comps[0].shape[0]
    B = ph.size - 1
    sh = f64(phase_shifts).reshape(-1)
    if sh.size != H:
        raise ValueError("one phase shift per component is needed")
    arr = (Component * H)()
    for h, (c, p) in enumerate(zip(comps, cph)):
        if c.ndim != 2 or c.shape[0] != K or c.shape[1] != p.size:
            raise ValueError("component %d must be [channels, phases]" % h)
        arr[h] = Component(c.ctypes.data, p.ctypes.data, c.shape[1], c.shape[1], float(sh[h]))
    bg = f64(background) if background is not None else None
    if bg is not None and bg.shape != (K, B):
        raise ValueError("background must be [channels, phase intervals]")
    an = _allow_negative(allow_negative, H)
    out = np.empty((K, B))
    check(lib().xgpu_compute_expected_counts(float(exposure_time), B, ptr(ph), K, H, arr,
                                             ptr(bg), ptr(an), ptr(out)))
    return out


def poisson(mean, seed, offset=0):
    """Poisson realisations of `mean` (any shape) keyed by (seed, element)."""
    m = f64(mean)
    out = np.empty_like(m)
    rc = check(lib().xgpu_poisson(m.size, ptr(m), int(seed) & (2 ** 64 - 1),
                                  int(offset), ptr(out)))
    if rc == 1:
        raise RuntimeError("a Poisson draw hit the rejection loop's bound")
    return out


def _seed(gsl_seed):
    return int(gsl_seed) if gsl_seed is not None else int(time.time())


def synthesise_exposure(exposure_time, phases, components, component_phases, phase_shifts,
                        expected_background_counts, background, allow_negative=False,
                        gsl_seed=None):
    """(EXPEC [K, B], SYNTHETIC [K, B], SCALE_BACKGROUND) as the reference
    returns them (synthesise.pyx:35-140)."""
    bkg = f64(background)
    BACKGROUND = 0.0
    for v in bkg.ravel():
        BACKGROUND += float(v)
    SCALE_BACKGROUND = 0.0 if BACKGROUND == 0.0 else expected_background_counts / BACKGROUND
    rate = bkg * SCALE_BACKGROUND / exposure_time
    EXPEC = compute_expected_counts(exposure_time, phases, components, component_phases,
                                    phase_shifts, rate, allow_negative)
    SYNTHETIC = poisson(EXPEC, _seed(gsl_seed))
    return (EXPEC, SYNTHETIC, SCALE_BACKGROUND)


def synthesise_given_total_count_number(phases, expected_star_counts, components,
                                        component_phases, phase_shifts,
                                        expected_background_counts, background,
                                        allow_negative=False, gsl_seed=None):
    """(EXPEC, SYNTHETIC, SCALE_STAR, SCALE_BACKGROUND / SCALE_STAR) as the
    reference returns them (synthesise.pyx:143-276)."""
    bkg = f64(background)
    STAR = compute_expected_counts(1e5, phases, components, component_phases, phase_shifts,
                                   np.zeros_like(bkg), allow_negative)
    STAR_total = 0.0
    BACKGROUND = 0.0
    for s_, b_ in zip(STAR.ravel(), bkg.ravel()):
        STAR_total += float(s_)
        BACKGROUND += float(b_)
    SCALE_STAR = expected_star_counts / STAR_total
    SCALE_BACKGROUND = 0.0 if BACKGROUND == 0.0 else expected_background_counts / BACKGROUND
    EXPEC = STAR * SCALE_STAR + bkg * SCALE_BACKGROUND
    SYNTHETIC = poisson(EXPEC, _seed(gsl_seed))
    return (EXPEC, SYNTHETIC, SCALE_STAR, SCALE_BACKGROUND / SCALE_STAR)
