"""Drop-in for xpsi.cellmesh.integrator_for_azimuthal_invariance.integrate
(xpsi/cellmesh/integrator_for_azimuthal_invariance.pyx:70-665)."""
import ctypes as C

import numpy as np

from .._arr import f64, i32, ptr
from .._interp import require_default_interpolants
from .._native import Atmos4D, check, lib
from ._tables import table2d

SUCCESS = 0
ERROR = 1


def integrate(numThreads, R, omega, r_s, inclination, cellArea,
              radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams,
              CELL_RADIATES, correction_srcCellParams, numRays, deflection, cos_alpha,
              lag, maxDeflection, cos_gammaArray, energies, leaves, phases,
              hot_atmosphere, elsewhere_atmosphere, hot_atm_ext, else_atm_ext, beam_opt,
              image_order_limit=None, R_in=1e6):
    """Integrate over the image of a star on a distant observer's sky (GPU).

    Returns (0, flux[N_E, N_P]) or (1, None) exactly as the reference does.
    Supported: blackbody (hot_atm_ext 1), numerical 4-D (2), the burst
    blackbody's intensity (3) and Pol_Num2D's intensity table (4,
    hot_atmosphere = (mu, log10 E, I)) hot atmospheres with no disk
    (R_in >= 1e6), with or without the correction for a blackbody elsewhere
    (else_atm_ext 1).  beam_opt 0-3 as the reference's (hot_wrapper.pyx:
    153-199): options 1-3 read (abb, bbb, cbb, dbb, nimu) from
    srcCellParams[..., 2:7]; option 3 takes hot_atm_ext 1 or 2.  Other
    options raise NotImplementedError rather than silently computing
    something else.
    """
    require_default_interpolants(phase=True, energy=False)
    corr = None
    if correction_srcCellParams is not None:
        if int(else_atm_ext) != 1:
            raise NotImplementedError("the GPU path corrects for a blackbody elsewhere only")
        corr = f64(correction_srcCellParams)
        if corr.ndim != 3 or corr.shape[:2] != f64(cellArea).shape:
            raise ValueError("correction_srcCellParams must be [rows, cells, n_params]")
    beam = int(beam_opt)
    if beam not in (0, 1, 2, 3):
        raise ValueError("beam_opt must be 0, 1, 2 or 3")
    if beam == 3 and int(hot_atm_ext) not in (1, 2):
        raise NotImplementedError("beam_opt 3 is on the GPU path for hot_atm_ext 1 and 2")
    if beam and f64(srcCellParams).shape[-1] < 7:
        raise ValueError("beaming options read srcCellParams[..., 2:7] (abb, bbb, cbb, dbb, "
                         "nimu)")
    if R_in < 1e6:
        raise NotImplementedError("disk occultation is not on the GPU path")
    atm = int(hot_atm_ext)
    if atm not in (1, 2, 3, 4):
        raise NotImplementedError("hot atmosphere extension %d is not on the GPU path" % atm)
    A = f64(cellArea)
    S0, S1 = A.shape
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
    atmos = None
    keep = ()
    if atm == 4:
        atmos, keep = table2d(hot_atmosphere)
    if atm == 2:
        if not hot_atmosphere:
            raise ValueError("numerical atmosphere data were not preloaded")
        keep = tuple(f64(a) for a in hot_atmosphere[:5])
        atmos = Atmos4D(*(k.ctypes.data for k in keep), keep[0].size, keep[1].size,
                        keep[2].size, keep[3].size, None)
    flux = np.empty((E.size, P.size))
    st = check(lib().xgpu_integrate(
        float(R), float(omega), float(r_s), float(inclination), S0, S1, ptr(A),
        ptr(arrs[0]), ptr(arrs[1]), ptr(arrs[2]), ptr(arrs[3]), ptr(par), par.shape[2],
        ptr(rad), ptr(corr), corr.shape[2] if corr is not None else 0, N_R, ptr(arrs[4]),
        ptr(arrs[5]), ptr(arrs[6]), ptr(arrs[7]), ptr(arrs[8]), E.size, ptr(E), Lv.size,
        ptr(Lv), P.size, ptr(P), atm, C.byref(atmos) if atmos is not None else None,
        int(else_atm_ext) if corr is not None else 0,
        int(image_order_limit) if image_order_limit is not None else 0, beam, ptr(flux)))
    del keep
    if st != 0:
        return (ERROR, None)
    return (SUCCESS, flux)
