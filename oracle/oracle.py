"""ctypes front-end of the CPU oracle (oracle/xpsi_oracle.c + gslsub).

TEST INFRASTRUCTURE.  The functions below mirror the reference's module-level
callables (same argument meaning, numpy in / numpy out) so tests read like
the reference's own: they are the checker for the CUDA path and the timed CPU
baseline, never the product.
"""
import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SOURCES = [os.path.join(HERE, "xpsi_oracle.c"),
           os.path.join(HERE, "xpsi_oracle_mesh.c"),
           os.path.join(HERE, "gslsub", "gslsub.c")]

_lock = threading.Lock()
_lib = None


def build(force=False):
    """Compile the oracle shared library (gcc, OpenMP, no FMA contraction)."""
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SOURCES + [
        os.path.join(HERE, "gslsub", "include", "gslsub.h"),
        os.path.join(HERE, "gslsub", "include", "gk_nodes.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O3", "-fPIC", "-shared", "-fopenmp",
                           "-ffp-contract=off", "-std=c11", "-D_GNU_SOURCE",
                           "-I", os.path.join(HERE, "gslsub", "include"),
                           *SOURCES, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


class Atmos4D(C.Structure):
    _fields_ = [("logT", C.c_void_p), ("logg", C.c_void_p), ("mu", C.c_void_p),
                ("logE", C.c_void_p), ("I", C.c_void_p),
                ("nT", C.c_size_t), ("ng", C.c_size_t), ("nmu", C.c_size_t),
                ("nE", C.c_size_t), ("Q", C.c_void_p)]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB)
            P = C.c_void_p
            L.xo_compute_rays.restype = C.c_int
            L.xo_compute_rays.argtypes = [C.c_int, C.c_size_t, C.c_double, P, P,
                                          C.c_size_t, P, P, P, P]
            L.xo_integrate.restype = C.c_int
            L.xo_integrate.argtypes = [
                C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                C.c_size_t, C.c_size_t, P, P, P, P, P, P, C.c_size_t, P, P, C.c_size_t,
                C.c_size_t, P, P, P, P, P, C.c_size_t, P, C.c_size_t, P,
                C.c_size_t, P, C.c_int, P, C.c_int, P, P, P]
            L.xo_integrate_split.restype = C.c_int
            L.xo_integrate_split.argtypes = list(L.xo_integrate.argtypes)[:-6] + [P, C.c_int, P]
            L.xo_pol_angle.restype = C.c_double
            L.xo_pol_angle.argtypes = [C.c_double] * 17
            L.xo_phase_interpolator.restype = None
            L.xo_phase_interpolator.argtypes = [C.c_size_t, P, C.c_size_t, P, C.c_size_t, P,
                                                C.c_double, C.c_int, P]
            L.xo_energy_interpolator.restype = None
            L.xo_energy_interpolator.argtypes = [C.c_size_t, C.c_size_t, P, P, C.c_size_t, P, P]
            L.xo_integrate_split_iqu.restype = C.c_int
            L.xo_integrate_split_iqu.argtypes = (list(L.xo_integrate.argtypes)[:-6] +
                                                 [P, P, C.c_int, P, P, P])
            L.xo_integrate_general.restype = C.c_int
            L.xo_integrate_general.argtypes = list(L.xo_integrate.argtypes)
            L.xo_integrate_time_invariant.restype = C.c_int
            L.xo_integrate_time_invariant.argtypes = [
                C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                C.c_size_t, C.c_double, P, P, P, P, P, C.c_size_t, C.c_size_t,
                P, P, P, P, C.c_size_t, P, C.c_int, P, C.c_int, P]
            L.xo_energy_integrator.restype = None
            L.xo_energy_integrator.argtypes = [C.c_int, C.c_size_t, C.c_size_t, P,
                                               P, C.c_size_t, P, P]
            L.xo_precomputation.restype = None
            L.xo_precomputation.argtypes = [C.c_size_t, C.c_size_t, P, P]
            L.xo_eval_marginal_likelihood.restype = C.c_int
            L.xo_eval_marginal_likelihood.argtypes = [
                C.c_double, C.c_size_t, P, C.c_size_t, P, C.c_size_t, P, P, P, P,
                P, P, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                P, C.c_double, P, C.c_uint, P, P, P, P]
            L.xo_expected_counts.restype = None
            L.xo_expected_counts.argtypes = [C.c_double, C.c_size_t, P, C.c_size_t, C.c_size_t,
                                             P, P, P, P, P, P, P]
            L.xo_phase_integrator.restype = None
            L.xo_phase_integrator.argtypes = [C.c_double, C.c_size_t, P, C.c_size_t, C.c_size_t,
                                              P, P, C.c_double, C.c_int, P]
            L.xo_lnfact.restype = C.c_double
            L.xo_lnfact.argtypes = [C.c_uint]
            D_ = C.c_double
            L.xo_allocate_cells.restype = None
            L.xo_allocate_cells.argtypes = [C.c_size_t, C.c_size_t, C.c_size_t, D_, D_, D_, D_,
                                            C.c_int] + [D_] * 8 + [P]
            L.xo_cell_mesh.restype = C.c_int
            L.xo_cell_mesh.argtypes = [C.c_int, C.c_size_t, C.c_size_t, D_, D_, D_, C.c_int,
                                       D_, D_, D_, D_, D_, C.c_int] + [P] * 7
            L.xo_closed_cell_mesh.restype = C.c_int
            L.xo_closed_cell_mesh.argtypes = [C.c_size_t, C.c_size_t, D_, D_, D_, C.c_int,
                                              C.c_int] + [P] * 7
            _lib = L
    return _lib


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def allocate_cells(num_cells, min_sqrt_num_cells, max_sqrt_num_cells, mass, r_s, R_eq,
                   Omega, zeta, epsilon, star_shape_ind, superRadius, cedeRadius,
                   superColatitude, cedeColatitude, superAzimuth, holeColatitude,
                   holeRadius, holeAzimuth):
    """mesh_tools.allocate_cells (mesh_tools.pyx:892-1099): (super_sqrt,
    super_num, cede_sqrt, cede_num), integer zeros for the ceding region when
    there is none, as the reference returns."""
    out = np.zeros(4)
    lib().xo_allocate_cells(int(num_cells), int(min_sqrt_num_cells), int(max_sqrt_num_cells),
                            float(R_eq), float(Omega), float(zeta), float(epsilon),
                            int(star_shape_ind), float(superRadius), float(cedeRadius),
                            float(superColatitude), float(cedeColatitude), float(superAzimuth),
                            float(holeColatitude), float(holeRadius), float(holeAzimuth),
                            _p(out))
    if abs(float(cedeRadius)) < 1.0e-12:
        return (float(out[0]), float(out[1]), 0, 0)
    return tuple(float(x) for x in out)


def _cell_mesh(polar, numThreads, numCell, sqrt_numCell, mass, r_s, R_eq, zeta, epsilon,
               star_shape_ind, cedeRadius, cedeColatitude, superRadius, superColatitude,
               superAzimuth):
    S = int(sqrt_numCell)
    th, ph, r, ma, cg, g = (np.empty(S) for _ in range(6))
    A = np.empty((S, S))
    rc = lib().xo_cell_mesh(int(polar), int(numCell), S, float(R_eq), float(zeta),
                            float(epsilon), int(star_shape_ind), float(cedeRadius),
                            float(cedeColatitude), float(superRadius), float(superColatitude),
                            float(superAzimuth), int(numThreads), _p(th), _p(ph), _p(r), _p(A),
                            _p(ma), _p(cg), _p(g))
    if rc:
        raise ValueError("mesh needs at least 2 cells per side")
    phi, theta = np.meshgrid(ph, th)
    return theta, phi, r, A, ma, cg, g


def construct_spot_cellMesh(*args):
    """mesh.construct_spot_cellMesh (mesh.pyx:23-417): (theta, phi, r,
    cellArea, maxEmissionAngle, cos_gamma, effGrav)."""
    return _cell_mesh(0, *args)


def construct_polar_cellMesh(*args):
    """polar_mesh.construct_polar_cellMesh (polar_mesh.pyx:23-430)."""
    return _cell_mesh(1, *args)


def construct_closed_cellMesh(numThreads, sqrt_numCell, numCell, mass, r_s, R_eq, zeta,
                              epsilon, star_shape_ind):
    """global_mesh.construct_closed_cellMesh (global_mesh.pyx:21-137):
    (theta, phi, r, cellArea (scalar), maxEmissionAngle, cos_gamma, effGrav)."""
    S = int(sqrt_numCell)
    th, ph, r, ma, cg, g = (np.empty(S) for _ in range(6))
    area = np.zeros(1)
    rc = lib().xo_closed_cell_mesh(S, int(numCell), float(R_eq), float(zeta), float(epsilon),
                                   int(star_shape_ind), int(numThreads), _p(th), _p(ph), _p(r),
                                   _p(area), _p(ma), _p(cg), _p(g))
    if rc:
        raise ValueError("closed mesh needs at least 4 cells per side")
    phi, theta = np.meshgrid(ph, th)
    return theta, phi, r, float(area[0]), ma, cg, g


def compute_rays(N_T, N_u, r_s, r_s_over_R, maxAlpha, N_R):
    """rays.compute_rays (rays.pyx:249-390); maxAlpha is clamped in place."""
    u = _c(r_s_over_R)
    assert maxAlpha.dtype == np.float64 and maxAlpha.flags.c_contiguous
    D = np.empty((N_u, N_R)); CA = np.empty((N_u, N_R)); L = np.empty((N_u, N_R))
    MD = np.empty(N_u)
    t = lib().xo_compute_rays(int(N_T), N_u, float(r_s), _p(u), _p(maxAlpha), N_R,
                              _p(D), _p(CA), _p(L), _p(MD))
    return t, D, CA, L, MD


def _atmos_struct(hot_atmosphere, atm_ext=2, hot_atmosphere_Q=None):
    """The C struct of a preloaded atmosphere: the 4-D table (logT, logg, mu,
    logE, I), or for atm_ext 4 (Pol_Num2D) the 2-D table (mu, logE, I) with
    the Q table of hot_atmosphere_Q on the same grids."""
    if not hot_atmosphere:
        return None, ()
    keep = tuple(_c(a) for a in hot_atmosphere)
    if int(atm_ext) == 4:
        q = None
        if hot_atmosphere_Q:
            qk = tuple(_c(a) for a in hot_atmosphere_Q)
            if not (np.array_equal(qk[0], keep[0]) and np.array_equal(qk[1], keep[1])):
                raise NotImplementedError("I and Q tables on different grids")
            keep = keep + (qk[2],)
            q = _p(qk[2]).value
        s = Atmos4D(None, None, _p(keep[0]).value, _p(keep[1]).value, _p(keep[2]).value,
                    0, 0, keep[0].size, keep[1].size, q)
        return s, keep
    s = Atmos4D(*(_p(a).value for a in keep[:5]), keep[0].size, keep[1].size,
                keep[2].size, keep[3].size, None)
    return s, keep


def integrate(numThreads, R, omega, r_s, inclination, cellArea,
              radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams,
              CELL_RADIATES, correction_srcCellParams, numRays, deflection,
              cos_alpha, lag, maxDeflection, cos_gammaArray, energies, leaves,
              phases, hot_atmosphere, elsewhere_atmosphere, hot_atm_ext,
              else_atm_ext, beam_opt, image_order_limit=None, R_in=1e6):
    """integrator_for_azimuthal_invariance.integrate (:70-665) for the
    uniform BB / Num4D / Pol_Num2D (I) hot regions, with the
    correction for a blackbody elsewhere (else_atm_ext 1) when
    correction_srcCellParams is given."""
    if beam_opt != 0 or R_in < 1e6:
        raise NotImplementedError("oracle covers the default hot-region path")
    corr = None
    if correction_srcCellParams is not None:
        if int(else_atm_ext) != 1:
            raise NotImplementedError("oracle corrects for a blackbody elsewhere only")
        corr = _c(correction_srcCellParams)
    A = _c(cellArea); S0, S1 = A.shape
    par = _c(srcCellParams)
    rad = _c(CELL_RADIATES, np.int32)
    E = _c(energies); Lv = _c(leaves); P = _c(phases)
    out = np.zeros((E.size, P.size))
    st, keep = _atmos_struct(hot_atmosphere, hot_atm_ext)
    arrs = [_c(radialCoords_of_parallels), _c(r_s_over_r), _c(theta), _c(phi),
            _c(deflection), _c(cos_alpha), _c(lag), _c(maxDeflection),
            _c(cos_gammaArray)]
    status = lib().xo_integrate(
        int(numThreads), float(R), float(omega), float(r_s), float(inclination),
        S0, S1, _p(A), _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), _p(arrs[3]),
        _p(par), par.shape[2], _p(rad), _p(corr) if corr is not None else None,
        corr.shape[2] if corr is not None else 0, int(numRays), _p(arrs[4]), _p(arrs[5]),
        _p(arrs[6]), _p(arrs[7]), _p(arrs[8]), E.size, _p(E), Lv.size, _p(Lv),
        P.size, _p(P), int(hot_atm_ext),
        C.cast(C.pointer(st), C.c_void_p) if st is not None else None,
        int(image_order_limit or 0), _p(out), None, None)
    del keep
    if status != 0:
        return (1, None)
    return (0, out)


def integrate_iqu(numThreads, R, omega, r_s, inclination, cellArea,
                  radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams,
                  CELL_RADIATES, correction_srcCellParams, numRays, deflection, cos_alpha, lag,
                  maxDeflection, cos_gammaArray, energies, leaves, phases, hot_atmosphere_I,
                  hot_atmosphere_Q, elsewhere_atmosphere, hot_atm_ext, else_atm_ext, beam_opt,
                  image_order_limit=None, R_in=1e6):
    """integratorIQU_for_azimuthal_invariance.integrate (:68-743):
    (0, flux_I, flux_Q, flux_U) or (1, None) for the blackbody (1), Num4D (2),
    burst blackbody (3) and Pol_Num2D (4) atmospheres."""
    if beam_opt != 0 or R_in < 1e6:
        raise NotImplementedError("oracle covers beam_opt 0 without a disk")
    if int(hot_atm_ext) not in (1, 2, 3, 4):
        raise NotImplementedError("oracle covers atmospheres 1 to 4")
    corr = None
    if correction_srcCellParams is not None:
        if int(else_atm_ext) != 1:
            raise NotImplementedError("oracle corrects for a blackbody elsewhere only")
        corr = _c(correction_srcCellParams)
    A = _c(cellArea); S0, S1 = A.shape
    par = _c(srcCellParams)
    rad = _c(CELL_RADIATES, np.int32)
    E = _c(energies); Lv = _c(leaves); P = _c(phases)
    out = [np.zeros((E.size, P.size)) for _ in range(3)]
    st, keep = _atmos_struct(hot_atmosphere_I if int(hot_atm_ext) in (2, 4) else (),
                             hot_atm_ext, hot_atmosphere_Q)
    arrs = [_c(radialCoords_of_parallels), _c(r_s_over_r), _c(theta), _c(phi),
            _c(deflection), _c(cos_alpha), _c(lag), _c(maxDeflection),
            _c(cos_gammaArray)]
    status = lib().xo_integrate(
        int(numThreads), float(R), float(omega), float(r_s), float(inclination),
        S0, S1, _p(A), _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), _p(arrs[3]),
        _p(par), par.shape[2], _p(rad), _p(corr) if corr is not None else None,
        corr.shape[2] if corr is not None else 0, int(numRays), _p(arrs[4]), _p(arrs[5]),
        _p(arrs[6]), _p(arrs[7]), _p(arrs[8]), E.size, _p(E), Lv.size, _p(Lv),
        P.size, _p(P), int(hot_atm_ext),
        C.cast(C.pointer(st), C.c_void_p) if st is not None else None,
        int(image_order_limit or 0), _p(out[0]), _p(out[1]), _p(out[2]))
    del keep
    if status != 0:
        return (1, None)
    return (0, out[0], out[1], out[2])


def _general(numThreads, R, omega, r_s, inclination, cellArea, radialCoords_of_parallels,
             r_s_over_r, theta, phi, srcCellParams, CELL_RADIATES, correction_srcCellParams,
             numRays, deflection, cos_alpha, lag, maxDeflection, cos_gammaArray, energies,
             leaves, phases, hot_atmosphere, hot_atmosphere_Q, hot_atm_ext, else_atm_ext,
             beam_opt, image_order_limit, R_in, stokes):
    if beam_opt != 0 or R_in < 1e6:
        raise NotImplementedError("oracle covers beam_opt 0 without a disk")
    if int(hot_atm_ext) not in (1, 2, 3, 4):
        raise NotImplementedError("oracle covers atmospheres 1 to 4")
    corr = None
    if correction_srcCellParams is not None:
        if int(else_atm_ext) != 1:
            raise NotImplementedError("oracle corrects for a blackbody elsewhere only")
        corr = _c(correction_srcCellParams)
    A = _c(cellArea); S0, S1 = A.shape
    par = _c(srcCellParams)
    rad = _c(CELL_RADIATES, np.int32)
    E = _c(energies); Lv = _c(leaves); P = _c(phases)
    out = [np.zeros((E.size, P.size)) for _ in range(3 if stokes else 1)]
    st, keep = _atmos_struct(hot_atmosphere if int(hot_atm_ext) in (2, 4) else (),
                             hot_atm_ext, hot_atmosphere_Q)
    arrs = [_c(radialCoords_of_parallels), _c(r_s_over_r), _c(theta), _c(phi),
            _c(deflection), _c(cos_alpha), _c(lag), _c(maxDeflection),
            _c(cos_gammaArray)]
    status = lib().xo_integrate_general(
        int(numThreads), float(R), float(omega), float(r_s), float(inclination),
        S0, S1, _p(A), _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), _p(arrs[3]),
        _p(par), par.shape[2], _p(rad), _p(corr) if corr is not None else None,
        corr.shape[2] if corr is not None else 0, int(numRays), _p(arrs[4]), _p(arrs[5]),
        _p(arrs[6]), _p(arrs[7]), _p(arrs[8]), E.size, _p(E), Lv.size, _p(Lv),
        P.size, _p(P), int(hot_atm_ext),
        C.cast(C.pointer(st), C.c_void_p) if st is not None else None,
        int(image_order_limit or 0), _p(out[0]), _p(out[1]) if stokes else None,
        _p(out[2]) if stokes else None)
    del keep
    if status != 0:
        return (1, None)
    return (0,) + tuple(out)


def integrate_general(numThreads, R, omega, r_s, inclination, cellArea,
                      radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams,
                      CELL_RADIATES, correction_srcCellParams, numRays, deflection,
                      cos_alpha, lag, maxDeflection, cos_gammaArray, energies, leaves,
                      phases, hot_atmosphere, elsewhere_atmosphere, hot_atm_ext,
                      else_atm_ext, beam_opt, image_order_limit=None, R_in=1e6):
    """integrator.integrate (integrator.pyx:48-667), the general integrator
    of HotRegion(symmetry=False), with the blackbody elsewhere correction
    when correction_srcCellParams is given; atmospheres 1 to 4."""
    return _general(numThreads, R, omega, r_s, inclination, cellArea,
                    radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams,
                    CELL_RADIATES, correction_srcCellParams, numRays, deflection, cos_alpha,
                    lag, maxDeflection, cos_gammaArray, energies, leaves, phases,
                    hot_atmosphere, None, hot_atm_ext, else_atm_ext, beam_opt,
                    image_order_limit, R_in, False)


def integrate_general_iqu(numThreads, R, omega, r_s, inclination, cellArea,
                          radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams,
                          CELL_RADIATES, correction_srcCellParams, numRays, deflection,
                          cos_alpha, lag, maxDeflection, cos_gammaArray, energies, leaves,
                          phases, hot_atmosphere_I, hot_atmosphere_Q, elsewhere_atmosphere,
                          hot_atm_ext, else_atm_ext, beam_opt, image_order_limit=None,
                          R_in=1e6):
    """integratorIQU.integrate (integratorIQU.pyx:76-717), the general Stokes
    integrator: (0, flux_I, flux_Q, flux_U) or (1, None)."""
    return _general(numThreads, R, omega, r_s, inclination, cellArea,
                    radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams,
                    CELL_RADIATES, correction_srcCellParams, numRays, deflection, cos_alpha,
                    lag, maxDeflection, cos_gammaArray, energies, leaves, phases,
                    hot_atmosphere_I, hot_atmosphere_Q, hot_atm_ext, else_atm_ext, beam_opt,
                    image_order_limit, R_in, True)


def integrate_time_invariant(numThreads, R, omega, r_s, inclination, sqrt_numPix,
                             cellArea, radialCoords_of_parallels, r_s_over_r, theta,
                             phi, srcCellParams, numRays, deflection, cos_alpha,
                             maxDeflection, cos_gammaArray, energies, atmosphere,
                             atm_ext, image_order_limit=None, *args):
    """integrator_for_time_invariance.integrate (:59-338): the photosphere
    elsewhere, blackbody (atm_ext 1) or numerical 4-D (2)."""
    if int(atm_ext) not in (1, 2):
        raise NotImplementedError("oracle covers atm_ext 1 and 2")
    S = int(sqrt_numPix)
    par = _c(srcCellParams)
    E = _c(energies)
    out = np.zeros(E.size)
    st, keep = _atmos_struct(atmosphere if int(atm_ext) == 2 else ())
    arrs = [_c(radialCoords_of_parallels), _c(r_s_over_r), _c(theta), _c(phi),
            _c(deflection), _c(cos_alpha), _c(maxDeflection), _c(cos_gammaArray)]
    status = lib().xo_integrate_time_invariant(
        int(numThreads), float(R), float(omega), float(r_s), float(inclination), S,
        float(cellArea), _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), _p(arrs[3]), _p(par),
        par.shape[2], int(numRays), _p(arrs[4]), _p(arrs[5]), _p(arrs[6]), _p(arrs[7]),
        E.size, _p(E), int(atm_ext),
        C.cast(C.pointer(st), C.c_void_p) if st is not None else None,
        int(image_order_limit or 0), _p(out))
    del keep
    if status != 0:
        return (1, None)
    return (0, out)


def energy_integrator(N_Ts, signal, energies, energy_edges):
    """tools.energy_integrator (energy_integrator.pyx:27-114)."""
    S = _c(signal); E = _c(energies); ed = _c(energy_edges)
    out = np.zeros((ed.size - 1, S.shape[1]))
    lib().xo_energy_integrator(int(N_Ts), E.size, S.shape[1], _p(S), _p(E), ed.size,
                               _p(ed), _p(out))
    return out


def precomputation(data):
    d = _c(data, np.int32)
    out = np.zeros(d.shape[0])
    lib().xo_precomputation(d.shape[0], d.shape[1], _p(d), _p(out))
    return out


def eval_marginal_likelihood(exposure_time, phases, counts, components,
                             component_phases, phase_shifts,
                             neg_sum_ln_data_factorial, support,
                             workspace_intervals, epsabs, epsrel, epsilon, sigmas,
                             llzero, allow_negative=False, slim=20.0,
                             background=None, seed=12345, return_status=False):
    """default_background_marginalisation.eval_marginal_likelihood (:450-734)."""
    ph = _c(phases); cnt = _c(counts)
    comps = [_c(c) for c in components]
    cph = [_c(c) for c in component_phases]
    H = len(comps)
    K, B = cnt.shape
    sup = _c(support)
    if sup.shape[0] != K:
        raise TypeError('The number of energy channels in the background support '
                        'does not match to that of the data.')
    for i in range(K):
        if sup[i, 1] == 0:
            raise TypeError('Background upper limit cannot be set to 0.')
        if sup[i, 1] > 0 and sup[i, 1] - sup[i, 0] < 0:
            raise TypeError('Background upper limit must be higher than the lower limit.')
    if isinstance(allow_negative, bool):
        an = np.full(H, int(allow_negative), dtype=np.int32)
    else:
        an = _c([int(x) for x in allow_negative], np.int32)
    ptrs = (C.c_void_p * H)(*[_p(c).value for c in comps])
    pptrs = (C.c_void_p * H)(*[_p(c).value for c in cph])
    nph = np.array([c.shape[1] for c in comps], dtype=np.uint64)
    sh = _c(phase_shifts)
    pre = _c(neg_sum_ln_data_factorial)
    bg = _c(background) if background is not None else None
    STAR = np.zeros((K, B)); mb = np.zeros(K); mbs = np.zeros(K)
    ll = C.c_double(0.0)
    st = lib().xo_eval_marginal_likelihood(
        float(exposure_time), B, _p(ph), K, _p(cnt), H, C.cast(ptrs, C.c_void_p),
        _p(nph), C.cast(pptrs, C.c_void_p), _p(sh), _p(pre), _p(sup), float(epsabs),
        float(epsrel), float(epsilon), float(sigmas), float(llzero), _p(an),
        float(slim), _p(bg) if bg is not None else None, int(seed), C.byref(ll),
        _p(STAR), _p(mb), _p(mbs))
    res = (ll.value, STAR, mb, mbs)
    return (res, st) if return_status else res


def compute_expected_counts(exposure_time, phases, components, component_phases, phase_shifts,
                            background=None, allow_negative=False):
    """compute_expected_counts (compute_expected_counts.pyx:200-276): [K, B]
    expected counts; background is a count-rate array [K, B] or None."""
    ph = _c(phases)
    comps = [_c(c) for c in components]
    cph = [_c(c) for c in component_phases]
    H = len(comps)
    K = comps[0].shape[0]
    B = ph.size - 1
    if isinstance(allow_negative, bool):
        an = np.full(H, int(allow_negative), dtype=np.int32)
    else:
        an = _c([int(x) for x in allow_negative], np.int32)
    ptrs = (C.c_void_p * H)(*[_p(c).value for c in comps])
    pptrs = (C.c_void_p * H)(*[_p(c).value for c in cph])
    nph = np.array([c.shape[1] for c in comps], dtype=np.uint64)
    sh = _c(phase_shifts)
    bg = _c(background) if background is not None else None
    out = np.zeros((K, B))
    lib().xo_expected_counts(float(exposure_time), B, _p(ph), K, H, C.cast(ptrs, C.c_void_p),
                             _p(nph), C.cast(pptrs, C.c_void_p), _p(sh),
                             _p(bg) if bg is not None else None, _p(an), _p(out))
    return out


def phase_integrator(exposure_time, phases, signal, signal_phases, phase_shift,
                     allow_negative=False):
    """tools.phase_integrator.phase_integrator (phase_integrator.pyx:23-121)."""
    ph = _c(phases); S = _c(signal); sp = _c(signal_phases)
    out = np.zeros((S.shape[0], ph.size - 1))
    lib().xo_phase_integrator(float(exposure_time), ph.size, _p(ph), S.shape[0], S.shape[1],
                              _p(S), _p(sp), float(phase_shift), int(bool(allow_negative)),
                              _p(out))
    return out


def gaussian_loglike(model, counts, errors):
    """The Gaussian log-likelihood of _gaussian_likelihood_given_background_IQU
    .pyx:70-78 and _gaussian_likelihood_QnUn.pyx:31-36, summed in the
    reference's order; `model` is [rows, cols] or one row [cols]."""
    import math
    d = _c(counts)
    e = _c(errors)
    m = _c(model)
    L = 0.0
    for i in range(d.shape[0]):
        row = m[i] if m.ndim == 2 else m
        for j in range(d.shape[1]):
            s2 = math.pow(e[i, j], 2.0)
            norm = 0.5 * math.log(2.0 * math.pi * s2)
            L -= (row[j] - d[i, j]) ** 2 / (2.0 * s2) + norm
    return L


class Atmos5D(C.Structure):
    _fields_ = [("grid", C.c_void_p * 5), ("n", C.c_size_t * 5), ("I", C.c_void_p)]


def integrate_split(numThreads, R, omega, r_s, inclination, cellArea,
                    radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams,
                    CELL_RADIATES, correction_srcCellParams, numRays, deflection, cos_alpha,
                    lag, maxDeflection, cos_gammaArray, energies, leaves, phases,
                    hot_atmosphere, elsewhere_atmosphere, hot_atm_ext, else_atm_ext, beam_opt,
                    image_order_limit=None, R_in=1e6):
    """integrator_for_azimuthal_invariance_split.integrate: the 5-D split
    atmosphere hot_atmosphere = (t_e, t_bb, tau, mu, E grids, intensity)."""
    if beam_opt != 0 or R_in < 1e6:
        raise NotImplementedError("oracle covers beam_opt 0 without a disk")
    corr = None
    if correction_srcCellParams is not None:
        if int(else_atm_ext) != 1:
            raise NotImplementedError("oracle corrects for a blackbody elsewhere only")
        corr = _c(correction_srcCellParams)
    A = _c(cellArea); S0, S1 = A.shape
    par = _c(srcCellParams)
    rad = _c(CELL_RADIATES, np.int32)
    E = _c(energies); Lv = _c(leaves); P_ = _c(phases)
    out = np.zeros((E.size, P_.size))
    keep = tuple(_c(a) for a in hot_atmosphere)
    a5 = Atmos5D((C.c_void_p * 5)(*[_p(k).value for k in keep[:5]]),
                 (C.c_size_t * 5)(*[k.size for k in keep[:5]]), _p(keep[5]).value)
    arrs = [_c(radialCoords_of_parallels), _c(r_s_over_r), _c(theta), _c(phi),
            _c(deflection), _c(cos_alpha), _c(lag), _c(maxDeflection),
            _c(cos_gammaArray)]
    status = lib().xo_integrate_split(
        int(numThreads), float(R), float(omega), float(r_s), float(inclination),
        S0, S1, _p(A), _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), _p(arrs[3]),
        _p(par), par.shape[2], _p(rad), _p(corr) if corr is not None else None,
        corr.shape[2] if corr is not None else 0, int(numRays), _p(arrs[4]), _p(arrs[5]),
        _p(arrs[6]), _p(arrs[7]), _p(arrs[8]), E.size, _p(E), Lv.size, _p(Lv),
        P_.size, _p(P_), C.cast(C.pointer(a5), C.c_void_p), int(image_order_limit or 0),
        _p(out))
    del keep
    if status != 0:
        return (1, None)
    return (0, out)


def integrate_split_iqu(numThreads, R, omega, r_s, inclination, cellArea,
                        radialCoords_of_parallels, r_s_over_r, theta, phi, srcCellParams,
                        CELL_RADIATES, correction_srcCellParams, numRays, deflection,
                        cos_alpha, lag, maxDeflection, cos_gammaArray, energies, leaves,
                        phases, hot_atmosphere_I, hot_atmosphere_Q, elsewhere_atmosphere,
                        hot_atm_ext, else_atm_ext, beam_opt, image_order_limit=None,
                        R_in=1e6):
    """integratorIQU_for_azimuthal_invariance_split.integrate (:75-758):
    (0, flux_I, flux_Q, flux_U) or (1, None) for split I and Q tables
    (t_e, t_bb, tau, mu, E grids, values)."""
    if beam_opt != 0 or R_in < 1e6:
        raise NotImplementedError("oracle covers beam_opt 0 without a disk")
    corr = None
    if correction_srcCellParams is not None:
        if int(else_atm_ext) != 1:
            raise NotImplementedError("oracle corrects for a blackbody elsewhere only")
        corr = _c(correction_srcCellParams)
    A = _c(cellArea); S0, S1 = A.shape
    par = _c(srcCellParams)
    rad = _c(CELL_RADIATES, np.int32)
    E = _c(energies); Lv = _c(leaves); P_ = _c(phases)
    out = [np.zeros((E.size, P_.size)) for _ in range(3)]
    kI = tuple(_c(a) for a in hot_atmosphere_I)
    kQ = tuple(_c(a) for a in hot_atmosphere_Q)
    aI = Atmos5D((C.c_void_p * 5)(*[_p(k).value for k in kI[:5]]),
                 (C.c_size_t * 5)(*[k.size for k in kI[:5]]), _p(kI[5]).value)
    aQ = Atmos5D((C.c_void_p * 5)(*[_p(k).value for k in kQ[:5]]),
                 (C.c_size_t * 5)(*[k.size for k in kQ[:5]]), _p(kQ[5]).value)
    arrs = [_c(radialCoords_of_parallels), _c(r_s_over_r), _c(theta), _c(phi),
            _c(deflection), _c(cos_alpha), _c(lag), _c(maxDeflection),
            _c(cos_gammaArray)]
    status = lib().xo_integrate_split_iqu(
        int(numThreads), float(R), float(omega), float(r_s), float(inclination),
        S0, S1, _p(A), _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), _p(arrs[3]),
        _p(par), par.shape[2], _p(rad), _p(corr) if corr is not None else None,
        corr.shape[2] if corr is not None else 0, int(numRays), _p(arrs[4]), _p(arrs[5]),
        _p(arrs[6]), _p(arrs[7]), _p(arrs[8]), E.size, _p(E), Lv.size, _p(Lv),
        P_.size, _p(P_), C.cast(C.pointer(aI), C.c_void_p), C.cast(C.pointer(aQ), C.c_void_p),
        int(image_order_limit or 0), _p(out[0]), _p(out[1]), _p(out[2]))
    del kI, kQ
    if status < 0:
        raise NotImplementedError("I and Q split tables on different (mu, E) grids")
    if status != 0:
        return (1, None)
    return (0, out[0], out[1], out[2])


def phase_interpolator(new_phases, phases, signal, phase_shift, allow_negative=0):
    """tools/phase_interpolator.pyx:25-95 (Akima periodic)."""
    nf = _c(new_phases); ph = _c(phases); sig = _c(signal)
    out = np.zeros((sig.shape[0], nf.size))
    lib().xo_phase_interpolator(nf.size, _p(nf), ph.size, _p(ph), sig.shape[0], _p(sig),
                                float(phase_shift), int(bool(allow_negative)), _p(out))
    return out


def energy_interpolator(N_Ts, signal, energies, new_energies):
    """tools/energy_interpolator.pyx:27-113 (Steffen); energies and
    new_energies are log10 of the energies."""
    sig = _c(signal); E = _c(energies); nE = _c(new_energies)
    out = np.zeros((sig.shape[1], nE.size))
    lib().xo_energy_interpolator(E.size, sig.shape[1], _p(sig), _p(E), nE.size, _p(nE),
                                 _p(out))
    return np.ascontiguousarray(out.T)  # :125, [new energies][columns]


def pol_angle(*args):
    """cellmesh/common_functions.pyx:7-66, compute_pol_ang (17 arguments)."""
    return lib().xo_pol_angle(*[float(a) for a in args])
