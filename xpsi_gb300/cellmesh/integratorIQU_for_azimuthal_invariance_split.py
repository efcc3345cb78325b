"""Drop-in for xpsi.cellmesh.integratorIQU_for_azimuthal_invariance_split.integrate
(xpsi/cellmesh/integratorIQU_for_azimuthal_invariance_split.pyx:75-758), the
Stokes integrator of a split hot region (HotRegion(split=True),
HotRegion.py:557-561), on the GPU."""
import ctypes as C

import numpy as np

from .._arr import f64, i32, ptr
from .._interp import require_default_interpolants
from .._native import check, lib
from ._tables import same_grids, table5d

SUCCESS = 0
ERROR = 1


def integrate(numThreads, R, omega, r_s, inclination, cellArea,
              radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams,
              CELL_RADIATES, correction_srcCellParams, numRays, deflection, cos_alpha,
              lag, maxDeflection, cos_gammaArray, energies, leaves, phases,
              hot_atmosphere_I, hot_atmosphere_Q, elsewhere_atmosphere, hot_atm_ext,
              else_atm_ext, beam_opt, image_order_limit=None, R_in=1e6):
    """Returns (0, flux_I, flux_Q, flux_U) or (1, None) as the reference does.

    hot_atmosphere_I and hot_atmosphere_Q are split tables (t_e, t_bb, tau,
    mu, E grids, values) with the same mu and E grids; each is reduced to
    (mu, E) at the first cell's (t_e, t_bb, tau) (:310-322); I (clipped at
    0) and Q are evaluated at E / Z in electron rest energies (:515-530).
    hot_atm_ext is ignored, as the reference ignores it.  beam_opt 0, no
    disk, and the correction for a blackbody elsewhere; other options raise
    NotImplementedError."""
    require_default_interpolants(phase=True, energy=False)
    if int(beam_opt) != 0:
        raise NotImplementedError("beaming options 1-3 are not on the GPU path")
    if R_in < 1e6:
        raise NotImplementedError("disk occultation is not on the GPU path")
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
    if par.ndim != 3 or par.shape[2] < 3:
        raise ValueError("srcCellParams must be [rows, cells, >= 3] (t_e, t_bb, tau)")
    aI, kI = table5d(hot_atmosphere_I, "hot_atmosphere_I")
    aQ, kQ = table5d(hot_atmosphere_Q, "hot_atmosphere_Q")
    if not same_grids(kI, kQ, (3, 4)):
        raise NotImplementedError("I and Q split tables on different (mu, E) grids")
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
    fI, fQ, fU = (np.empty((E.size, P.size)) for _ in range(3))
    st = check(lib().xgpu_integrate_split_stokes(
        float(R), float(omega), float(r_s), float(inclination), S0, S1, ptr(A),
        ptr(arrs[0]), ptr(arrs[1]), ptr(arrs[2]), ptr(arrs[3]), ptr(par), par.shape[2],
        ptr(rad), ptr(corr), corr.shape[2] if corr is not None else 0, N_R, ptr(arrs[4]),
        ptr(arrs[5]), ptr(arrs[6]), ptr(arrs[7]), ptr(arrs[8]), E.size, ptr(E), Lv.size,
        ptr(Lv), P.size, ptr(P), C.byref(aI), C.byref(aQ),
        int(else_atm_ext) if corr is not None else 0,
        int(image_order_limit) if image_order_limit is not None else 0, ptr(fI), ptr(fQ),
        ptr(fU)))
    del kI, kQ
    if st != 0:
        return (ERROR, None)
    return (SUCCESS, fI, fQ, fU)
