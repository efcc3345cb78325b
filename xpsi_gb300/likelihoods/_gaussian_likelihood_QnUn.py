"""Drop-in for xpsi.likelihoods._gaussian_likelihood_QnUn
(xpsi/likelihoods/_gaussian_likelihood_QnUn.pyx:9-38), on the GPU."""
import numpy as np

from .._arr import f64, ptr
from .._native import check, lib


def gaussian_likelihood_QnUn(phases, counts, errors, star):
    """(log L, star): the Gaussian likelihood of normalised Stokes data
    counts[rows, bins] with errors against the model star[bins]."""
    d = f64(counts)
    e = f64(errors)
    s = f64(star).reshape(-1)
    if d.ndim != 2 or e.shape != d.shape or s.size != d.shape[1]:
        raise ValueError("counts and errors must be [rows, bins] and star [bins]")
    out = np.zeros(1)
    check(lib().xgpu_gaussian_loglike(d.shape[0], d.shape[1], ptr(s), 0, ptr(d), ptr(e),
                                      ptr(out)))
    return (float(out[0]), np.asarray(s, order="C", dtype=np.double))
