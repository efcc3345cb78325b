"""Drop-in for xpsi.cellmesh.integrator_for_time_invariance.integrate
(xpsi/cellmesh/integrator_for_time_invariance.pyx:59-338): the spectrum of
the photosphere elsewhere, integrated on the GPU."""
import ctypes as C

import numpy as np

from .._arr import f64, ptr
from .._native import Atmos4D, check, lib

SUCCESS = 0
ERROR = 1


def integrate(numThreads, R, omega, r_s, inclination, sqrt_numPix, cellArea,
              radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams, numRays,
              deflection, cos_alpha, maxDeflection, cos_gammaArray, energies, atmosphere,
              atm_ext, image_order_limit=None, *args):
    """Returns (0, flux[N_E]) or (1, None) exactly as the reference does.
    Supported: blackbody (atm_ext 1) and numerical 4-D (2) atmospheres; the
    user extension (3) raises NotImplementedError rather than silently
    computing something else."""
    ext = int(atm_ext)
    if ext not in (1, 2):
        raise NotImplementedError("elsewhere atmosphere extension %d is not on the GPU path"
                                  % ext)
    S = int(sqrt_numPix)
    par = f64(srcCellParams)
    if par.ndim != 3 or par.shape[:2] != (S, S):
        raise ValueError("srcCellParams must be [sqrt_numPix, sqrt_numPix, n_params]")
    E = f64(energies)
    N_R = int(numRays)
    arrs = [f64(radialCoords_of_parallels), f64(r_s_over_r), f64(theta), f64(phi),
            f64(deflection), f64(cos_alpha), f64(maxDeflection), f64(cos_gammaArray)]
    if arrs[4].shape != (S, N_R) or arrs[5].shape != (S, N_R):
        raise ValueError("ray tables must be [sqrt_numPix, numRays]")
    atmos = None
    keep = ()
    if ext == 2:
        if not atmosphere:
            raise ValueError("numerical atmosphere data were not preloaded")
        keep = tuple(f64(a) for a in atmosphere[:5])
        atmos = Atmos4D(*(k.ctypes.data for k in keep), keep[0].size, keep[1].size,
                        keep[2].size, keep[3].size, None)
    flux = np.empty(E.size)
    st = check(lib().xgpu_integrate_time_invariant(
        float(R), float(omega), float(r_s), float(inclination), S, float(cellArea),
        ptr(arrs[0]), ptr(arrs[1]), ptr(arrs[2]), ptr(arrs[3]), ptr(par), par.shape[2], N_R,
        ptr(arrs[4]), ptr(arrs[5]), ptr(arrs[6]), ptr(arrs[7]), E.size, ptr(E), ext,
        None if atmos is None else C.byref(atmos),
        int(image_order_limit) if image_order_limit is not None else 0, ptr(flux)))
    del keep
    if st != 0:
        return (ERROR, None)
    return (SUCCESS, flux)
