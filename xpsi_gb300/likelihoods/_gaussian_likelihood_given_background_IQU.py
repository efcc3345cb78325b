"""Drop-in for xpsi.likelihoods._gaussian_likelihood_given_background_IQU
(xpsi/likelihoods/_gaussian_likelihood_given_background_IQU.pyx:10-80): the
expected counts (compute_expected_counts) and the Gaussian likelihood, both
on the GPU."""
import numpy as np

from .._arr import f64, ptr
from .._native import check, lib
from ..tools.synthesise import compute_expected_counts


def gaussian_likelihood_given_background(exposure_time, phases, counts, errors, components,
                                         component_phases, phase_shifts, background,
                                         allow_negative=False):
    """(log L, EXPEC [channels, bins]) as the reference returns them."""
    EXPEC = compute_expected_counts(exposure_time, phases, components, component_phases,
                                    phase_shifts, background, allow_negative)
    d = f64(counts)
    e = f64(errors)
    if d.shape != EXPEC.shape or e.shape != EXPEC.shape:
        raise ValueError("counts and errors must be [channels, phase intervals]")
    out = np.zeros(1)
    check(lib().xgpu_gaussian_loglike(d.shape[0], d.shape[1], ptr(EXPEC), d.shape[1], ptr(d),
                                      ptr(e), ptr(out)))
    return (float(out[0]), EXPEC)
