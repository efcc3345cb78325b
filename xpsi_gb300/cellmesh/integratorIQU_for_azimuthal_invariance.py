"""Drop-in for xpsi.cellmesh.integratorIQU_for_azimuthal_invariance.integrate
(xpsi/cellmesh/integratorIQU_for_azimuthal_invariance.pyx:68-743), the
Stokes I, Q, U integrator of HotRegion.integrate_stokes, on the GPU."""
import ctypes as C

import numpy as np

from .._arr import f64, i32, ptr
from .._interp import require_default_interpolants
from .._native import check, lib
from . import integrator_for_azimuthal_invariance as _az
from ._tables import same_grids, table2d

SUCCESS = 0
ERROR = 1


def integrate(numThreads, R, omega, r_s, inclination, cellArea,
              radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams,
              CELL_RADIATES, correction_srcCellParams, numRays, deflection, cos_alpha,
              lag, maxDeflection, cos_gammaArray, energies, leaves, phases,
              hot_atmosphere_I, hot_atmosphere_Q, elsewhere_atmosphere, hot_atm_ext,
              else_atm_ext, beam_opt, image_order_limit=None, R_in=1e6):
    """Returns (0, flux_I, flux_Q, flux_U) or (1, None) as the reference does.

    Atmospheres: the burst blackbody (hot_atm_ext 3, hot_BB_burst.pyx,
    polarised), Pol_Num2D (4, hot_Num2D.pyx: hot_atmosphere_I and _Q are the
    (mu, log10 E, values) tables), the blackbody (1) and the numerical 4-D
    table (2), for which the reference's Q is zero and I is the azimuthal
    integrator's.  beam_opt 0, no disk, and the correction for a blackbody
    elsewhere; other options raise NotImplementedError."""
    require_default_interpolants(phase=True, energy=False)
    ext = int(hot_atm_ext)
    if int(beam_opt) != 0:
        raise NotImplementedError("beaming options 1-3 are not on the GPU path")
    if R_in < 1e6:
        raise NotImplementedError("disk occultation is not on the GPU path")
    if ext == 2:
        out = _az.integrate(numThreads, R, omega, r_s, inclination, cellArea,
                            radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams,
                            CELL_RADIATES, correction_srcCellParams, numRays, deflection,
                            cos_alpha, lag, maxDeflection, cos_gammaArray, energies, leaves,
                            phases, hot_atmosphere_I, elsewhere_atmosphere, ext, else_atm_ext,
                            beam_opt, image_order_limit, R_in)
        if out[0] != SUCCESS:
            return (ERROR, None)
        return (SUCCESS, out[1], np.zeros_like(out[1]), np.zeros_like(out[1]))
    if ext not in (1, 3, 4):
        raise NotImplementedError("hot atmosphere extension %d is not on the GPU Stokes path"
                                  % ext)
    A = f64(cellArea)
    S0, S1 = A.shape
    corr = None
    if correction_srcCellParams is not None:
        if int(else_atm_ext) != 1:
            raise NotImplementedError("the GPU path corrects for a blackbody elsewhere only")
        corr = f64(correction_srcCellParams)
        if corr.ndim != 3 or corr.shape[:2] != (S0, S1):
            raise ValueError("correction_srcCellParams must be [rows, cells, n_params]")
    par = f64(srcCellParams)
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
    aI = aQ = None
    keep = ()
    if ext == 4:
        if not same_grids(hot_atmosphere_I, hot_atmosphere_Q, (0, 1)):
            raise NotImplementedError("I and Q tables on different grids")
        aI, kI = table2d(hot_atmosphere_I, "hot_atmosphere_I")
        aQ, kQ = table2d(hot_atmosphere_Q, "hot_atmosphere_Q")
        keep = kI + kQ
    fI, fQ, fU = (np.empty((E.size, P.size)) for _ in range(3))
    st = check(lib().xgpu_integrate_stokes(
        float(R), float(omega), float(r_s), float(inclination), S0, S1, ptr(A),
        ptr(arrs[0]), ptr(arrs[1]), ptr(arrs[2]), ptr(arrs[3]), ptr(par), par.shape[2],
        ptr(rad), ptr(corr), corr.shape[2] if corr is not None else 0, N_R, ptr(arrs[4]),
        ptr(arrs[5]), ptr(arrs[6]), ptr(arrs[7]), ptr(arrs[8]), E.size, ptr(E), Lv.size,
        ptr(Lv), P.size, ptr(P), ext, C.byref(aI) if aI is not None else None,
        C.byref(aQ) if aQ is not None else None, int(else_atm_ext) if corr is not None else 0,
        int(image_order_limit) if image_order_limit is not None else 0, ptr(fI), ptr(fQ),
        ptr(fU)))
    del keep
    if st != 0:
        return (ERROR, None)
    return (SUCCESS, fI, fQ, fU)
