"""Drop-in for xpsi.cellmesh.rays.compute_rays (xpsi/cellmesh/rays.pyx:249-390)."""
import numpy as np

from .._arr import f64, ptr
from .._native import check, lib


def compute_rays(N_T, N_u, r_s, r_s_over_R, maxAlpha, N_R):
    """Compute ray properties in the Schwarzschild spacetime on the GPU.

    Same arguments and returns as the reference: (terminate, deflection,
    cos_alpha, lag, maxDeflection), tables [N_u, N_R].  ``maxAlpha`` is
    clamped in place (rays.pyx:317-318); ``N_T`` (OpenMP threads) is
    accepted and ignored.
    """
    N_u = int(N_u)
    N_R = int(N_R)
    u = f64(r_s_over_R)
    if not (isinstance(maxAlpha, np.ndarray) and maxAlpha.dtype == np.float64
            and maxAlpha.flags.c_contiguous):
        raise ValueError("maxAlpha must be a C-contiguous float64 array")
    if u.shape[0] != N_u or maxAlpha.shape[0] != N_u:
        raise ValueError("r_s_over_R and maxAlpha need N_u elements")
    D = np.empty((N_u, N_R))
    CA = np.empty((N_u, N_R))
    L = np.empty((N_u, N_R))
    MD = np.empty(N_u)
    t = check(lib().xgpu_compute_rays(N_u, float(r_s), ptr(u), ptr(maxAlpha), N_R, ptr(D),
                                      ptr(CA), ptr(L), ptr(MD)))
    return (t, D, CA, L, MD)
