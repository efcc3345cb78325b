"""Drop-in for xpsi.cellmesh.integrator_for_azimuthal_invariance_split.integrate
(xpsi/cellmesh/integrator_for_azimuthal_invariance_split.pyx:74-103), the
integrator of a uniform hot region whose atmosphere is split
(HotRegion(split=True), HotRegion.py:557-561)."""
import ctypes as C

import numpy as np

from .._arr import f64, i32, ptr
from .._interp import require_default_interpolants
from .._native import check, lib
from ._tables import table5d

SUCCESS = 0
ERROR = 1


def integrate(numThreads, R, omega, r_s, inclination, cellArea,
              radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams,
              CELL_RADIATES, correction_srcCellParams, numRays, deflection, cos_alpha,
              lag, maxDeflection, cos_gammaArray, energies, leaves, phases,
              hot_atmosphere, elsewhere_atmosphere, hot_atm_ext, else_atm_ext, beam_opt,
              image_order_limit=None, R_in=1e6):
    """Integrate over the image of a star with a split hot atmosphere (GPU).

    hot_atmosphere is the preloaded tuple (t_e, t_bb, tau, mu, E grids,
    intensity) of hot_Num5D_split.pyx:77-220; the table is reduced to
    (mu, E) at the first cell's (t_e, t_bb, tau) (:270-275) and evaluated at
    E / Z in electron rest energies (:457-471); hot_atm_ext is ignored, as the
    reference ignores it.  Returns (0, flux[N_E, N_P]) or (1, None).
    Supported: beam_opt 0, no disk (R_in >= 1e6), with or without the
    correction for a blackbody elsewhere (else_atm_ext 1); other options
    raise NotImplementedError.
    """
    require_default_interpolants(phase=True, energy=False)
    corr = None
    if correction_srcCellParams is not None:
        if int(else_atm_ext) != 1:
            raise NotImplementedError("the GPU path corrects for a blackbody elsewhere only")
        corr = f64(correction_srcCellParams)
        if corr.ndim != 3 or corr.shape[:2] != f64(cellArea).shape:
            raise ValueError("correction_srcCellParams must be [rows, cells, n_params]")
    if int(beam_opt) != 0:
        raise NotImplementedError("beaming options 1-3 are not on the GPU path")
    if R_in < 1e6:
        raise NotImplementedError("disk occultation is not on the GPU path")
    A = f64(cellArea)
    S0, S1 = A.shape
    par = f64(srcCellParams)
    if par.ndim != 3 or par.shape[2] < 3:
        raise ValueError("srcCellParams must be [rows, cells, >= 3] (t_e, t_bb, tau)")
    rad = i32(CELL_RADIATES)
    E = f64(energies)
    Lv = f64(leaves)
    P = f64(phases)
    arrs = [f64(radialCoords_of_parallels), f64(r_s_over_r), f64(theta), f64(phi),
            f64(deflection), f64(cos_alpha), f64(lag), f64(maxDeflection),
            f64(cos_gammaArray)]
    N_R = int(numRays)
    if arrs[4].shape != (S0, N_R):
        raise ValueError("ray tables must be [rows, numRays]")
    atmos, keep = table5d(hot_atmosphere)
    flux = np.empty((E.size, P.size))
    st = check(lib().xgpu_integrate_split(
        float(R), float(omega), float(r_s), float(inclination), S0, S1, ptr(A),
        ptr(arrs[0]), ptr(arrs[1]), ptr(arrs[2]), ptr(arrs[3]), ptr(par), par.shape[2],
        ptr(rad), ptr(corr), corr.shape[2] if corr is not None else 0, N_R, ptr(arrs[4]),
        ptr(arrs[5]), ptr(arrs[6]), ptr(arrs[7]), ptr(arrs[8]), E.size, ptr(E), Lv.size,
        ptr(Lv), P.size, ptr(P), C.byref(atmos),
        int(else_atm_ext) if corr is not None else 0,
        int(image_order_limit) if image_order_limit is not None else 0, ptr(flux)))
    del keep
    if st != 0:
        return (ERROR, None)
    return (SUCCESS, flux)
