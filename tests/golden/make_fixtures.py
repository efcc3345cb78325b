"""Generate the golden fixtures under tests/golden/ from the REFERENCE itself.

Runs where the reference checkout and its extension build exist
(`python oracle/build_ref.py` first).  Every array saved here is an input or
an output of the reference's own code (X-PSI's Cython compiled by
oracle/build_ref.py, Python model classes imported from the checkout), so
the GPU tests compare against the reference, not against a restatement.

Cases
  meshes         the reference's cell budgets and spot / polar-cap meshes at the
                 full-size resolution for the prior vectors of the full-size
                 parity test (polar caps on either member, omitted crescents)
                 and three hand-set members.
  examples_fast  the model of xpsi/tests/test_likelihood.py (blackbody spot,
                 golden log L -47881.27817666349); all stage inputs/outputs.
  num4d_omit     a spot with an omitted (crescent) region and a small seeded
                 numerical 4-D atmosphere; fast spin so that mu*eta > 1 and the
                 reference's history-dependent clamp is exercised.
  elsewhere      the photosphere elsewhere: closed mesh, rays and the
                 time-invariant integrator, blackbody and numerical 4-D, with
                 1 and 4 threads.
  elsewhere_correction  the hot-region integrator with a blackbody
                 elsewhere's correction, on config1's and num4d_omit's inputs.
  general_integrator  the general integrator (HotRegion symmetry=False) with a
                 temperature varying across the mesh, on config1's and
                 num4d_omit's inputs.
  synthesis      expected counts of the reference's synthesis routines and
                 its phase integrator on config1's folded signal.
  stokes         the Stokes I/Q/U integrator for the burst blackbody and the
                 plain blackbody with a correction.
  gaussian       the Gaussian likelihoods of polarimetry.
  split          the split integrator with a synthetic 5-D split atmosphere.
  energy_arrays  the integrators' energies over several wavebands (gaps, a
                 maximum energy) and the waveband a response and channel range
                 select.
  poisson_given_background  the Poisson likelihood with a known background
                 on config1's signal and data.
  beaming        the integrator with beaming options 1-3 on config1's and
                 num4d_omit's inputs.
  config1        the blackbody workload of the small plain configuration
                 (M 1.4, R 12 km, 300 Hz, i 1 rad, 1 kpc; spot 1.0/0.075/6.1;
                 32 cells, 64 leaves, 512 rays, 64 energies; 300 x 64 response;
                 32 phase bins, 1e6 s, seeded Poisson data) with a reduced
                 phase/energy grid only where noted.

Usage:  python tests/golden/make_fixtures.py [case ...]   (all cases by default)
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_harness as H  # noqa: E402
from xpsi_gb300 import synthetic  # noqa: E402


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in arrays.items()})
    print("wrote", path, "%.0f kB" % (os.path.getsize(path) / 1024))


def examples_fast(xpsi):
    H.examples_fast_modules()
    src = open(os.path.join(H.REF, "xpsi", "tests", "test_likelihood.py")).read()
    src = src.replace(
        "assert np.isclose(-47881.27817666349, likelihood(p,force=True,reinitialise=True), rtol=1.0e-5)",
        "G['v'] = likelihood(p,force=True,reinitialise=True); G['lik'] = likelihood")
    g = {"__file__": os.path.join(H.REF, "xpsi", "tests", "test_likelihood.py"),
         "__name__": "tl", "G": {}}
    exec(compile(src, "test_likelihood.py", "exec"), g)
    g["TestLikelihoodCheck"]().test_likelihood_is_correct()
    lik, v = g["G"]["lik"], g["G"]["v"]
    st = lik._star.spacetime
    hot = lik._star.photospheres[0].hot
    sig = lik._signals[0][0]
    from xpsi.cellmesh.rays import compute_rays
    from xpsi.cellmesh.integrator_for_azimuthal_invariance import integrate
    from xpsi.tools.energy_integrator import energy_integrator
    from xpsi.likelihoods.default_background_marginalisation import (
        eval_marginal_likelihood, precomputation)
    u = np.ascontiguousarray(st.r_s / hot._super_r)
    maxAlpha_in = np.pi / 2.0 + np.arccos(hot._super_cos_gamma)
    ma = maxAlpha_in.copy()
    S = int(hot._super_sqrt_num_cells)
    rt = compute_rays(1, S, st.r_s, u, ma, hot._num_rays)
    E = sig.energies
    fl = integrate(1, st.R, st.Omega, st.r_s, st.i, hot._super_cellArea, hot._super_r,
                   hot._super_r_s_over_r, hot._super_theta, hot._super_phi,
                   hot._super_cellParamVecs, hot._super_radiates, None, hot._num_rays,
                   hot._super_deflection, hot._super_cos_alpha, hot._super_lag,
                   hot._super_maxDeflection, hot._super_cos_gamma, E, hot.leaves,
                   hot.phases, (), None, hot.atm_ext, None, hot.beam_opt,
                   hot._image_order_limit)
    sflux = fl[1] / st.d_sq
    logE, logEd = np.log10(E), np.log10(sig._energy_edges)
    ei = energy_integrator(1, sflux, logE, logEd)
    matrix = sig._instrument.construct_matrix()
    folded = np.dot(matrix, ei)
    counts = sig._data.counts
    pre = precomputation(counts.astype(np.int32))
    ml = eval_marginal_likelihood(sig._data.exposure_time, sig._data.phases, counts,
                                  sig.signals, [hot.phases_in_cycles], sig.shifts, pre,
                                  sig._support, 1000, 0.0, 1.0e-8, 1.0e-3, 10.0, -1.0e90)
    save("examples_fast",
         golden_logL=-47881.27817666349, ref_logL=v,
         R=st.R, Omega=st.Omega, r_s=st.r_s, inclination=st.i, d_sq=st.d_sq,
         cellArea=hot._super_cellArea, radius=hot._super_r, u=hot._super_r_s_over_r,
         theta=hot._super_theta, phi=hot._super_phi, params=hot._super_cellParamVecs,
         radiates=hot._super_radiates, N_R=hot._num_rays,
         maxAlpha_in=maxAlpha_in, rays_u=u, rays_maxAlpha_out=ma,
         rays_deflection=rt[1], rays_cos_alpha=rt[2], rays_lag=rt[3], rays_maxDefl=rt[4],
         deflection=hot._super_deflection, cos_alpha=hot._super_cos_alpha,
         lag=hot._super_lag, maxDeflection=hot._super_maxDeflection,
         cos_gamma=hot._super_cos_gamma, energies=E, leaves=hot.leaves, phases=hot.phases,
         atm_ext=hot.atm_ext, image_order_limit=hot._image_order_limit, flux=fl[1],
         log10_energies=logE, log10_edges=logEd, signal_in=sflux, energy_out=ei,
         matrix=matrix, folded=folded, registered=sig.signals[0],
         exposure=sig._data.exposure_time, phase_edges=sig._data.phases, counts=counts,
         comp_phases=hot.phases_in_cycles, shifts=sig.shifts, precomp=pre,
         support=sig._support, logL=ml[0], star=ml[1], mcl_bg=ml[2], mcl_bg_s=ml[3])


def mesh_member(xpsi, *, M_sun, R_km, f_hz, cos_i, colat, radius, logT, omit=None,
                sqrt_num_cells, min_cells, max_cells, N_R, antiphased=False):
    """Mesh, rays and source parameters of one hot region via the reference's
    own cellmesh functions, with the glue HotRegion applies
    (HotRegion.py:774-1017)."""
    from xpsi.global_imports import _GM, _csq, _G, _km, _2pi, _c
    from xpsi.cellmesh.mesh_tools import allocate_cells
    from xpsi.cellmesh.mesh import construct_spot_cellMesh
    from xpsi.cellmesh.rays import compute_rays
    r_g = M_sun * _GM
    r_s = 2.0 * r_g
    R = R_km * _km
    Mkg = M_sun * _GM * _csq / _G
    Omega = _2pi * f_hz
    zeta = r_g / R
    eps = Omega ** 2.0 * R ** 3.0 / (_G * Mkg)
    o_r, o_c, o_a = omit if omit is not None else (0.0, 0.0, 0.0)
    S, N, _, _ = allocate_cells(sqrt_num_cells ** 2, min_cells, max_cells, Mkg, r_s, R, Omega,
                                zeta, eps, 0, radius, 0.0, colat, colat, -0.0, o_c, o_r, o_a)
    S = int(S)
    th, ph, r, A, maxA, cg, g = construct_spot_cellMesh(1, int(N), S, Mkg, r_s, R, zeta, eps,
                                                        0, radius, colat, o_r, o_c, o_a)
    ph = ph - o_a
    if antiphased:
        ph = ph + math.pi
    u = np.ascontiguousarray(r_s / r)
    ma_in = np.array(maxA, copy=True)
    ma = ma_in.copy()
    t, D, CA, L, MD = compute_rays(1, S, r_s, u, ma, N_R)
    assert t == 0
    raw_lag = L.copy()
    R_i = R / r_s
    C = (1.0 / u - R_i)
    C += np.log((1.0 / u - 1.0) / (R_i - 1.0))
    C *= r_s / _c
    for j in range(L.shape[1]):
        L[:, j] -= C
    L *= f_hz * _2pi
    radiates = np.greater(A, 0.0).astype(np.int32)
    params = np.ones((S, S, 2))
    params[..., :-1] *= logT
    for j in range(S):
        params[:, j, -1] *= g
    return dict(R=R, Omega=Omega, r_s=r_s, inclination=math.acos(cos_i), S=S,
                cellArea=A, radius=r, u=u, theta=th, phi=ph, params=params,
                radiates=radiates, maxAlpha_in=ma_in, rays_maxAlpha_out=ma,
                deflection=D, cos_alpha=CA, raw_lag=raw_lag, lag=L, maxDeflection=MD,
                cos_gamma=cg, effGrav=g, N_R=N_R)


# prior vectors of the batched configuration (config3_vectors(64, seed=3))
# used by the full-size parity test: 4, 5, 18 carry a polar-cap mesh on the
# member with an omitted crescent, 17 and 26 on the circular member, 20 on
# both; 0, 1, 2 are ordinary spots
FULL_SIZE_VECTORS = (0, 1, 2, 4, 5, 17, 18, 20, 26)


def meshes(xpsi):
    """Reference meshes at the full-size resolution (sqrt_num_cells 64,
    min 10, max 128): the cell budget (mesh_tools.allocate_cells) and the
    spot or polar-cap mesh (mesh.construct_spot_cellMesh,
    polar_mesh.construct_polar_cellMesh), chosen and called as
    HotRegion.__construct_cellMesh does (HotRegion.py:774-836), for every
    hot-region member of the parameter vectors FULL_SIZE_VECTORS, plus three
    hand-set members: a south polar cap with an omitted region over the
    pole, a north polar cap at a fast spin, and a spot of the smallest
    prior radius."""
    from xpsi.global_imports import _GM, _csq, _G, _km, _2pi
    from xpsi.cellmesh.mesh_tools import allocate_cells
    from xpsi.cellmesh.mesh import construct_spot_cellMesh
    from xpsi.cellmesh.polar_mesh import construct_polar_cellMesh
    from xpsi_gb300 import batch as BT
    model = synthetic.config2_model()
    names = BT.param_names(model)
    col = {n: i for i, n in enumerate(names)}
    params = synthetic.config3_vectors(64, seed=3)[list(FULL_SIZE_VECTORS)]
    members = []
    for v in range(params.shape[0]):
        p = params[v]
        for h, r in enumerate(model.regions):
            om = (p[col[f"h{h}_omit_radius"]], p[col[f"h{h}_omit_colatitude"]],
                  p[col[f"h{h}_omit_azimuth"]]) if r.omit else (0.0, 0.0, 0.0)
            members.append((p[0], p[1], p[2], p[col[f"h{h}_colatitude"]],
                            p[col[f"h{h}_radius"]]) + om)
    members += [(1.8, 13.0, 450.0, 2.9, 0.45, 0.2, 3.05, 0.4),
                (1.2, 15.5, 600.0, 0.3, 0.48, 0.0, 0.0, 0.0),
                (2.6, 12.5, 250.0, 1.4, 0.01, 0.0, 0.0, 0.0)]
    out = dict(params=params, vector_index=np.array(FULL_SIZE_VECTORS),
               members=np.array(members), sqrt_num_cells=64, min_sqrt_num_cells=10,
               max_sqrt_num_cells=128)
    for k, (M_sun, R_km, f_hz, colat, rad, o_r, o_c, o_a) in enumerate(members):
        r_g = M_sun * _GM
        r_s = 2.0 * r_g
        R = R_km * _km
        Mkg = M_sun * _GM * _csq / _G
        Omega = _2pi * f_hz
        zeta = r_g / R
        eps = Omega ** 2.0 * R ** 3.0 / (_G * Mkg)
        S, N, _, _ = allocate_cells(64 ** 2, 10, 128, Mkg, r_s, R, Omega, zeta, eps, 0, rad,
                                    0.0, colat, colat, -0.0, o_c, o_r, o_a)
        polar = colat - rad < 0.0 or colat + rad > math.pi
        fn = construct_polar_cellMesh if polar else construct_spot_cellMesh
        th, ph, r, A, maxA, cg, g = fn(1, int(N), int(S), Mkg, r_s, R, zeta, eps, 0, rad, colat,
                                       o_r, o_c, o_a)
        assert np.all(th == th[:, :1]) and np.all(ph == ph[:1, :])
        out[f"m{k}_S"] = int(S)
        out[f"m{k}_num_cells"] = int(N)
        out[f"m{k}_polar"] = int(polar)
        out[f"m{k}_theta"] = th[:, 0]
        out[f"m{k}_phi"] = ph[0, :]
        out[f"m{k}_cellArea"] = A
        out[f"m{k}_radius"] = r
        out[f"m{k}_maxAlpha"] = maxA
        out[f"m{k}_cos_gamma"] = cg
        out[f"m{k}_effGrav"] = g
    out["n_members"] = len(members)
    save("meshes", **out)


# beaming-modification parameters (abb, bbb, cbb, dbb, nimu) appended to the
# cell vectors for the beaming fixture
BEAM_PARAMS = (0.3, -0.2, 0.5, 0.3, 20.0)


# waveband sets for the energy-array fixture: (num_energies, max_energy,
# [(lower, upper, n_edges), ...])
ENERGY_CASES = (
    (64, None, [(0.1, 10.0, 65)]),
    (100, None, [(0.3, 12.0, 40), (0.1, 3.0, 30)]),
    (128, None, [(0.6, 10.0, 50), (0.1, 0.5, 20)]),
    (200, None, [(2.2, 12.0, 30), (0.8, 2.0, 25), (0.2, 0.7, 10)]),
    (200, 2.1, [(2.2, 12.0, 30), (0.8, 2.0, 25), (0.2, 0.7, 10)]),
    (200, 1.5, [(2.2, 12.0, 30), (0.8, 2.0, 25), (0.2, 0.7, 10)]),
    (128, 20.0, [(0.6, 10.0, 50), (0.1, 0.5, 20)]),
    (90, None, [(0.5, 8.0, 17), (0.2, 0.9, 9), (8.5, 15.0, 12)]),
)
# (the reference subtracts the gaps' widths in keV from a log10 span, so
# gaps are kept narrow here: wide ones drive its interval negative)


def energy_arrays(xpsi):
    """The reference's construct_energy_array (Signal.py:1092-1197) over the
    waveband sets of ENERGY_CASES (overlapping bands, coverage gaps, a
    maximum energy inside a gap, inside a band and above all bands), and its
    Signal._identify_waveband (Signal.py:324-354) on responses whose edge
    channels have leading and trailing zero columns."""
    from types import SimpleNamespace
    from xpsi.Signal import Signal, construct_energy_array

    class _Sig:  # compared by identity, as list.remove in the reference needs
        def __init__(self, e):
            self.energy_edges = e
    rng = np.random.default_rng(8)
    out = {"n_cases": len(ENERGY_CASES)}
    for c, (num, emax, bands) in enumerate(ENERGY_CASES):
        sigs = []
        for b, (lo, hi, n) in enumerate(bands):
            e = np.sort(np.exp(rng.uniform(np.log(lo), np.log(hi), n)))
            e[0], e[-1] = lo, hi
            out[f"c{c}_band{b}"] = e
            sigs.append(_Sig(e))
        out[f"c{c}_energies"] = construct_energy_array(num, list(sigs), emax)
    for c, (K, q, rng_ch) in enumerate(((40, 30, (0, 40)), (40, 30, (5, 33)), (25, 50, (3, 4)))):
        M = rng.uniform(0.1, 1.0, (K, q))
        M[:, :3] = 0.0
        M[:, -4:] = 0.0
        M[rng_ch[0], 3:6] = 0.0
        M[rng_ch[1] - 1, -8:] = 0.0
        edges = np.logspace(-1, 1, q + 1)
        obj = SimpleNamespace(_data=SimpleNamespace(index_range=rng_ch),
                              _instrument=SimpleNamespace(matrix=M, energy_edges=edges))
        Signal._identify_waveband(obj)
        out[f"w{c}_matrix"] = M
        out[f"w{c}_edges"] = edges
        out[f"w{c}_index_range"] = np.array(rng_ch)
        out[f"w{c}_range"] = np.array(obj._input_interval_range)
        out[f"w{c}_energy_edges"] = obj._energy_edges
    out["n_wave"] = 3
    save("energy_arrays", **out)


def poisson_given_background(xpsi):
    """The reference's poisson_likelihood_given_background
    (_poisson_likelihood_given_background.pyx:14-113) on config1's registered
    signal, data and phases: a background of 10 % of each channel's mean
    source rate, with and without the data-factorial constants, and a case
    whose first channels have no signal, no background and no counts (no
    penalty).  (The penalty branch, :107-108, converts a 1-element array to
    a C double, which numpy >= 2 refuses; the reference pins numpy < 2, so
    that branch is not run here.)"""
    from xpsi.likelihoods._poisson_likelihood_given_background import (
        poisson_likelihood_given_background as plgb)
    with np.load(os.path.join(HERE, "config1.npz")) as z:
        f = {k: z[k] for k in z.files}
    reg = np.ascontiguousarray(f["folded"])  # the registered count rates [K, N_P]
    counts = np.ascontiguousarray(f["counts"].astype(np.float64))
    B = f["phase_edges"].size - 1
    bg = np.ascontiguousarray(np.repeat(0.1 * reg.mean(axis=1, keepdims=True), B, axis=1))
    args = lambda r, c, b: (float(f["exposure"]), f["phase_edges"], c, [r], [f["comp_phases"]],
                            np.ascontiguousarray(f["shifts"]), b)
    out = dict(registered=reg, counts=counts, background=bg, exposure=f["exposure"],
               phase_edges=f["phase_edges"], comp_phases=f["comp_phases"], shifts=f["shifts"],
               precomp=f["precomp"])
    out["ll_nopre"], out["expec"] = plgb(*args(reg, counts, bg))
    out["ll_pre"], _ = plgb(*args(reg, counts, bg), f["precomp"])
    r0, c0, b0 = reg.copy(), counts.copy(), bg.copy()
    r0[:3] = 0.0
    c0[:3] = 0.0
    b0[:3] = 0.0
    out["ll_zero"], out["expec_zero"] = plgb(*args(r0, c0, b0), f["precomp"])
    save("poisson_given_background", **out)


def beaming(xpsi):
    """The hot-region integrator with the reference's beaming options 1-3
    (hot_wrapper.pyx:153-199) on config1's blackbody inputs and num4d_omit's
    Num4D inputs (read from their fixtures), the cell vectors extended with
    BEAM_PARAMS as columns 2-6."""
    from xpsi.cellmesh.integrator_for_azimuthal_invariance import integrate
    out = {"beam_params": np.array(BEAM_PARAMS)}
    for case in ("config1", "num4d_omit"):
        with np.load(os.path.join(HERE, case + ".npz")) as z:
            f = {k: z[k] for k in z.files}
        prm = np.ascontiguousarray(np.concatenate(
            [f["params"], np.broadcast_to(np.array(BEAM_PARAMS), f["params"].shape[:2] + (5,))],
            axis=2))
        atm = ((f["atm_logT"], f["atm_logg"], f["atm_mu"], f["atm_logE"], f["atm_I"])
               if case == "num4d_omit" else ())
        for opt in (1, 2, 3):
            st, flux = integrate(1, float(f["R"]), float(f["Omega"]), float(f["r_s"]),
                                 float(f["inclination"]), f["cellArea"], f["radius"], f["u"],
                                 f["theta"], f["phi"], prm, f["radiates"], None, int(f["N_R"]),
                                 f["deflection"], f["cos_alpha"], f["lag"], f["maxDeflection"],
                                 f["cos_gamma"], f["energies"], f["leaves"], f["phases"], atm,
                                 None, int(f["atm_ext"]), None, opt,
                                 int(f["image_order_limit"]) or None)
            assert st == 0
            out[f"{case}_opt{opt}"] = flux
    save("beaming", **out)


def num4d_omit(xpsi):
    from xpsi.cellmesh.integrator_for_azimuthal_invariance import integrate
    atm = synthetic.num4d_table(shape=(12, 8, 20, 40), seed=2)
    m = mesh_member(xpsi, M_sun=1.6, R_km=14.0, f_hz=600.0, cos_i=0.55, colat=1.2,
                    radius=0.3, logT=6.3, omit=(0.12, 1.25, 0.1), sqrt_num_cells=20,
                    min_cells=10, max_cells=40, N_R=256)
    E = np.logspace(-1.0, 1.0, 48)
    leaves = np.linspace(0.0, 2 * math.pi, 40)
    phases = 2 * math.pi * np.linspace(0.0, 1.0, 40)
    args = lambda nt: (nt, m["R"], m["Omega"], m["r_s"], m["inclination"], m["cellArea"],
                       m["radius"], m["u"], m["theta"], m["phi"], m["params"],
                       m["radiates"], None, m["N_R"], m["deflection"], m["cos_alpha"],
                       m["lag"], m["maxDeflection"], m["cos_gamma"], E, leaves, phases,
                       atm, None, 2, None, 0, None)
    st1, flux1 = integrate(*args(1))
    st4, flux4 = integrate(*args(4))
    assert st1 == 0
    save("num4d_omit", **{k: v for k, v in m.items()}, energies=E, leaves=leaves,
         phases=phases, atm_logT=atm[0], atm_logg=atm[1], atm_mu=atm[2], atm_logE=atm[3],
         atm_I=atm[4], atm_ext=2, image_order_limit=0, flux=flux1,
         flux_threads4=flux4 if st4 == 0 else np.zeros(0))


def config1(xpsi):
    from xpsi.cellmesh.integrator_for_azimuthal_invariance import integrate
    from xpsi.tools.energy_integrator import energy_integrator
    from xpsi.likelihoods.default_background_marginalisation import (
        eval_marginal_likelihood, precomputation)
    w = synthetic.config1_workload()
    m = mesh_member(xpsi, M_sun=w["mass"], R_km=w["radius_km"], f_hz=w["frequency"],
                    cos_i=math.cos(w["inclination"]), colat=w["colatitude"],
                    radius=w["spot_radius"], logT=w["logT"], sqrt_num_cells=32,
                    min_cells=10, max_cells=80, N_R=512)
    E = w["energies"]
    leaves = np.linspace(0.0, 2 * math.pi, 64)
    phases = 2 * math.pi * np.linspace(0.0, 1.0, 64)
    st, flux = integrate(1, m["R"], m["Omega"], m["r_s"], m["inclination"], m["cellArea"],
                         m["radius"], m["u"], m["theta"], m["phi"], m["params"],
                         m["radiates"], None, m["N_R"], m["deflection"], m["cos_alpha"],
                         m["lag"], m["maxDeflection"], m["cos_gamma"], E, leaves, phases,
                         (), None, 1, None, 0, None)
    assert st == 0
    d_sq = w["d_sq"]
    sflux = flux / d_sq
    logE, logEd = np.log10(E), np.log10(w["input_edges"])
    ei = energy_integrator(1, sflux, logE, logEd)
    folded = np.dot(w["matrix"], ei)
    comp_phases = np.linspace(0.0, 1.0, 64)
    counts = synthetic.poisson_data(folded, comp_phases, w["phase_edges"], w["exposure"],
                                    seed=20261203)
    pre = precomputation(counts.astype(np.int32))
    support = -1.0 * np.ones((counts.shape[0], 2))
    support[:, 0] = 0.0
    ml = eval_marginal_likelihood(w["exposure"], w["phase_edges"], counts.astype(np.float64),
                                  [folded], [comp_phases], np.array([0.0]), pre, support,
                                  1000, 0.0, 1.0e-8, 1.0e-3, 10.0, -1.0e90)
    save("config1", **{k: v for k, v in m.items()}, energies=E, leaves=leaves, phases=phases,
         atm_ext=1, image_order_limit=0, flux=flux, d_sq=d_sq, signal_in=sflux,
         log10_energies=logE, log10_edges=logEd, energy_out=ei, matrix=w["matrix"],
         folded=folded, exposure=w["exposure"], phase_edges=w["phase_edges"],
         counts=counts, comp_phases=comp_phases, shifts=np.array([0.0]), precomp=pre,
         support=support, logL=ml[0], star=ml[1], mcl_bg=ml[2], mcl_bg_s=ml[3])


def closed_mesh(xpsi, *, M_sun, R_km, f_hz, sqrt_num_cells, N_R, star_shape_ind=0):
    """Closed mesh and rays of the photosphere elsewhere via the reference's
    own functions, with the glue Elsewhere applies (Elsewhere.py:254-303)."""
    from xpsi.global_imports import _GM, _csq, _G, _km, _2pi
    from xpsi.cellmesh.global_mesh import construct_closed_cellMesh
    from xpsi.cellmesh.rays import compute_rays
    r_g = M_sun * _GM
    r_s = 2.0 * r_g
    R = R_km * _km
    Mkg = M_sun * _GM * _csq / _G
    Omega = _2pi * f_hz
    zeta = r_g / R
    eps = Omega ** 2.0 * R ** 3.0 / (_G * Mkg)
    S = int(sqrt_num_cells)
    th, ph, r, cA, maxA, cg, g = construct_closed_cellMesh(1, S, S * S, Mkg, r_s, R, zeta, eps,
                                                           star_shape_ind)
    u = np.ascontiguousarray(r_s / r)
    ma_in = np.array(maxA, copy=True)
    ma = ma_in.copy()
    t, D, CA, L, MD = compute_rays(1, S, r_s, u, ma, N_R)
    assert t == 0
    return dict(mass=Mkg, R=R, Omega=Omega, r_s=r_s, zeta=zeta, epsilon=eps,
                star_shape_ind=star_shape_ind, S=S, theta=th, phi=ph, radius=r,
                cellArea=cA, maxAlpha_in=ma_in, rays_maxAlpha_out=ma, cos_gamma=cg,
                effGrav=g, u=u, deflection=D, cos_alpha=CA, maxDeflection=MD, N_R=N_R)


def elsewhere(xpsi):
    """The photosphere elsewhere: closed mesh, rays and the time-invariant
    integrator (integrator_for_time_invariance.pyx:59-338) for a blackbody
    and for the small numerical 4-D table, at 600 Hz so that mu * eta > 1
    on the approaching limb (the Num4D clamp history)."""
    from xpsi.cellmesh.integrator_for_time_invariance import integrate
    m = closed_mesh(xpsi, M_sun=1.6, R_km=14.0, f_hz=600.0, sqrt_num_cells=24, N_R=256)
    S = m["S"]
    E = np.logspace(-1.0, 1.0, 48)
    inclination = math.acos(0.55)
    out = {}
    # the numerical 4-D table num4d_omit.npz stores (not duplicated here)
    ref = np.load(os.path.join(HERE, "num4d_omit.npz"))
    atm = tuple(np.ascontiguousarray(ref[k]) for k in
                ("atm_logT", "atm_logg", "atm_mu", "atm_logE", "atm_I"))
    # the same table on a mu grid that tops out at 0.9, so that many queries
    # lie above it and the evaluator's clamp history decides their value
    atm09 = (atm[0], atm[1], np.ascontiguousarray(0.9 * atm[2]), atm[3], atm[4])
    for tag, logT, ext, atmos in (("bb", 6.0, 1, ()), ("num4d", 6.1, 2, atm),
                                  ("num4d_mu09", 6.1, 2, atm09)):
        params = np.ones((S, S, 2))
        params[..., :-1] *= logT
        for j in range(S):
            params[:, j, -1] *= m["effGrav"]
        for nt in (1, 4):
            st, flux = integrate(nt, m["R"], m["Omega"], m["r_s"], inclination, S,
                                 m["cellArea"], m["radius"], m["u"], m["theta"], m["phi"],
                                 params, m["N_R"], m["deflection"], m["cos_alpha"],
                                 m["maxDeflection"], m["cos_gamma"], E, atmos, ext, None)
            assert st == 0
            out["%s_flux_threads%d" % (tag, nt)] = flux
        out[tag + "_params"] = params
    save("elsewhere", **m, inclination=inclination, energies=E, **out)


def elsewhere_correction(xpsi):
    """The hot-region integrator with the elsewhere correction
    (integrator_for_azimuthal_invariance.pyx:257-261,469-478,593-594): a
    blackbody elsewhere at log T 6.0 (config1's blackbody spot) and 6.2
    (num4d_omit's numerical spot), correction vectors as Elsewhere and
    HotRegion.embed build them (Elsewhere.py:305-330, HotRegion.py:1052-1067).
    Inputs are the stored fixtures' own."""
    from xpsi.cellmesh.integrator_for_azimuthal_invariance import integrate
    out = {}
    for case, logT_else in (("config1", 6.0), ("num4d_omit", 6.2)):
        f = np.load(os.path.join(HERE, case + ".npz"))
        S = int(f["S"])
        corr = np.ones((S, S, 2))
        corr[..., :-1] *= logT_else
        for j in range(S):
            corr[:, j, -1] *= f["effGrav"]
        atm = ()
        if int(f["atm_ext"]) == 2:
            atm = tuple(np.ascontiguousarray(f[k]) for k in
                        ("atm_logT", "atm_logg", "atm_mu", "atm_logE", "atm_I"))
        st, flux = integrate(1, float(f["R"]), float(f["Omega"]), float(f["r_s"]),
                             float(f["inclination"]), f["cellArea"], f["radius"], f["u"],
                             f["theta"], f["phi"], f["params"], f["radiates"], corr,
                             int(f["N_R"]), f["deflection"], f["cos_alpha"], f["lag"],
                             f["maxDeflection"], f["cos_gamma"], f["energies"], f["leaves"],
                             f["phases"], atm, (), int(f["atm_ext"]), 1, 0,
                             int(f["image_order_limit"]) or None)
        assert st == 0
        out[case + "_correction"] = corr
        out[case + "_flux"] = flux
    save("elsewhere_correction", **out)


def general_integrator(xpsi):
    """The general integrator of HotRegion(symmetry=False)
    (cellmesh/integrator.pyx:48-667) on stored fixtures' meshes and rays,
    with a temperature that varies from cell to cell (the non-uniform hot
    region it exists for): config1's blackbody spot (with and without a
    blackbody elsewhere's correction) and num4d_omit's numerical spot at
    600 Hz (1 and 4 threads)."""
    from xpsi.cellmesh.integrator import integrate
    out = {}
    for case in ("config1", "num4d_omit"):
        f = np.load(os.path.join(HERE, case + ".npz"))
        S = int(f["S"])
        params = np.array(f["params"], copy=True)
        # log T rising by 0.1 dex across the mesh's azimuth and colatitude
        jj, ii = np.meshgrid(np.arange(S), np.arange(S))
        params[..., 0] += 0.1 * (jj / max(S - 1, 1)) - 0.05 * (ii / max(S - 1, 1))
        atm = ()
        if int(f["atm_ext"]) == 2:
            atm = tuple(np.ascontiguousarray(f[k]) for k in
                        ("atm_logT", "atm_logg", "atm_mu", "atm_logE", "atm_I"))
        corr_cases = [("", None)]
        if case == "config1":
            corr = np.ones((S, S, 2))
            corr[..., 0] = 6.0
            corr[..., 1] = f["effGrav"][:, None]
            corr_cases.append(("_corrected", corr))
        for tag, corr in corr_cases:
            for nt in ((1, 4) if case == "num4d_omit" else (1,)):
                st, flux = integrate(nt, float(f["R"]), float(f["Omega"]), float(f["r_s"]),
                                     float(f["inclination"]), f["cellArea"], f["radius"],
                                     f["u"], f["theta"], f["phi"], params, f["radiates"], corr,
                                     int(f["N_R"]), f["deflection"], f["cos_alpha"], f["lag"],
                                     f["maxDeflection"], f["cos_gamma"], f["energies"],
                                     f["leaves"], f["phases"], atm, (), int(f["atm_ext"]),
                                     1 if corr is not None else None, 0,
                                     int(f["image_order_limit"]) or None)
                assert st == 0
                out["%s%s_flux_threads%d" % (case, tag, nt)] = flux
            if corr is not None:
                out[case + tag + "_correction"] = corr
        out[case + "_params"] = params
        if case == "num4d_omit":
            # the same table on a mu grid topped at 0.9: many evaluations lie
            # above it and the evaluator's clamp history decides their value
            atm09 = (atm[0], atm[1], np.ascontiguousarray(0.9 * atm[2]), atm[3], atm[4])
            st, flux = integrate(1, float(f["R"]), float(f["Omega"]), float(f["r_s"]),
                                 float(f["inclination"]), f["cellArea"], f["radius"], f["u"],
                                 f["theta"], f["phi"], params, f["radiates"], None,
                                 int(f["N_R"]), f["deflection"], f["cos_alpha"], f["lag"],
                                 f["maxDeflection"], f["cos_gamma"], f["energies"],
                                 f["leaves"], f["phases"], atm09, (), 2, None, 0,
                                 int(f["image_order_limit"]) or None)
            assert st == 0
            out["num4d_omit_mu09_flux_threads1"] = flux
    save("general_integrator", **out)


def synthesis(xpsi):
    """Expected counts of the reference's synthesis routines
    (tools/synthesise.pyx: synthesise_exposure and
    synthesise_given_total_count_number, both through
    compute_expected_counts.pyx:200-276) and tools/phase_integrator.pyx on
    config1's folded signal: two components on different phase grids (the
    second a shifted copy sampled on a coarser grid), negative parts allowed for the
    second, a phase-dependent background.  The realisations (SYNTHETIC) come
    from the random stream of the build and are not stored."""
    from xpsi.tools.synthesise import synthesise_exposure, synthesise_given_total_count_number
    from xpsi.tools.phase_integrator import phase_integrator
    f = np.load(os.path.join(HERE, "config1.npz"))
    c1 = np.ascontiguousarray(f["folded"])
    p1 = np.ascontiguousarray(f["comp_phases"])
    p2 = np.linspace(0.0, 1.0, 33)
    c2 = np.ascontiguousarray(
        [0.3 * np.interp((p2 + 0.11) % 1.0, p1, row) for row in c1])
    edges = np.ascontiguousarray(f["phase_edges"])
    K, B = c1.shape[0], edges.size - 1
    rng = np.random.default_rng(5)
    bkg = np.ascontiguousarray(rng.uniform(0.5, 1.5, (K, B)) * c1.mean(axis=1)[:, None])
    shifts = np.array([0.1, -0.3])
    ex = synthesise_exposure(2.0e5, edges, (c1, c2), (p1, p2), shifts, 3.0e4, bkg,
                             allow_negative=[False, True], gsl_seed=7)
    tc = synthesise_given_total_count_number(edges, 1.0e6, (c1, c2), (p1, p2), shifts, 2.0e5,
                                             bkg, allow_negative=[False, True], gsl_seed=7)
    pi = phase_integrator(1.0e5, edges, c1, p1, 0.25)
    pi_neg = phase_integrator(1.0e5, edges, c2, p2, -0.7, True)
    # c1, p1 and the bin edges are config1.npz's folded, comp_phases, phase_edges
    save("synthesis", c2=c2, p2=p2, bkg=bkg, shifts=shifts,
         exposure_expec=ex[0], exposure_scale_background=ex[2], total_expec=tc[0],
         total_scale_star=tc[2], total_scale_ratio=tc[3], phase_integrated=pi,
         phase_integrated_neg=pi_neg)


def stokes(xpsi):
    """The Stokes integrator (integratorIQU_for_azimuthal_invariance.pyx:
    68-743) on config1's mesh and rays: the burst blackbody (atm_ext 3,
    hot_BB_burst.pyx: limb-darkened, polarised), also at 600 Hz on
    num4d_omit's mesh (a fast, oblate star), and the plain blackbody
    (Q = U = 0) with a blackbody elsewhere's correction."""
    from xpsi.cellmesh.integratorIQU_for_azimuthal_invariance import integrate
    out = {}
    for case, ext, corr_T in (("config1", 3, None), ("num4d_omit", 3, None),
                              ("config1", 1, 6.0)):
        f = np.load(os.path.join(HERE, case + ".npz"))
        S = int(f["S"])
        params = np.array(f["params"], copy=True)
        corr = None
        if corr_T is not None:
            corr = np.ones((S, S, 2))
            corr[..., 0] = corr_T
            corr[..., 1] = f["effGrav"][:, None]
        res = integrate(1, float(f["R"]), float(f["Omega"]), float(f["r_s"]),
                        float(f["inclination"]), f["cellArea"], f["radius"], f["u"], f["theta"],
                        f["phi"], params, f["radiates"], corr, int(f["N_R"]), f["deflection"],
                        f["cos_alpha"], f["lag"], f["maxDeflection"], f["cos_gamma"],
                        f["energies"], f["leaves"], f["phases"], (), (), (), ext,
                        1 if corr is not None else None, 0, int(f["image_order_limit"]) or None)
        assert res[0] == 0
        tag = "%s_ext%d%s" % (case, ext, "_corrected" if corr is not None else "")
        out[tag + "_I"], out[tag + "_Q"], out[tag + "_U"] = res[1], res[2], res[3]
        if corr is not None:
            out[tag + "_correction"] = corr
    save("stokes", **out)


def gaussian(xpsi):
    """The Gaussian likelihoods of polarimetry
    (likelihoods/_gaussian_likelihood_given_background_IQU.pyx,
    likelihoods/_gaussian_likelihood_QnUn.pyx) on config1's folded signal
    with seeded counts and errors."""
    from xpsi.likelihoods._gaussian_likelihood_given_background_IQU import (
        gaussian_likelihood_given_background)
    from xpsi.likelihoods._gaussian_likelihood_QnUn import gaussian_likelihood_QnUn
    f = np.load(os.path.join(HERE, "config1.npz"))
    c1 = np.ascontiguousarray(f["folded"][:40])
    p1 = np.ascontiguousarray(f["comp_phases"])
    edges = np.ascontiguousarray(f["phase_edges"])
    K, B = c1.shape[0], edges.size - 1
    rng = np.random.default_rng(8)
    bkg = np.ascontiguousarray(rng.uniform(0.5, 1.5, (K, B)) * c1.mean(axis=1)[:, None])
    T = 1.0e4
    counts = np.ascontiguousarray(rng.uniform(0.5, 2.0, (K, B)) * c1.mean(axis=1)[:, None] * T)
    errors = np.ascontiguousarray(np.sqrt(counts) * rng.uniform(0.8, 1.2, (K, B)))
    ll, expec = gaussian_likelihood_given_background(T, edges, counts, errors, (c1,), (p1,),
                                                     np.array([0.2]), bkg)
    qn = np.ascontiguousarray(rng.normal(0.0, 0.05, (3, B)))
    qn_err = np.ascontiguousarray(rng.uniform(0.02, 0.08, (3, B)))
    star = np.ascontiguousarray(rng.normal(0.0, 0.05, B))
    ll_qn, _ = gaussian_likelihood_QnUn(edges, qn, qn_err, star)
    save("gaussian", bkg=bkg, counts=counts, errors=errors, exposure=T, loglike=ll,
         expec=expec, qn=qn, qn_err=qn_err, star=star, loglike_qn=ll_qn)


def split(xpsi):
    """The split integrator (integrator_for_azimuthal_invariance_split.pyx):
    the 5-D split atmosphere of synthetic.split_table reduced to (mu, E) at
    the first cell's (t_e, t_bb, tau) (hot_Num5D_split.pyx:566-640) and
    interpolated per leaf and energy (hot_Num2D_split.pyx:200-384), on
    config1's mesh (300 Hz) and num4d_omit's (600 Hz), with a blackbody
    elsewhere's correction, and with (t_e, t_bb, tau) outside the table
    (above, above, below: the cached walk clamps the first query only)."""
    from xpsi.cellmesh.integrator_for_azimuthal_invariance_split import integrate
    atm = synthetic.split_table()
    out = {}
    for tag, case, vec, corr_T in (("config1", "config1", (0.7, 0.004, 1.5), None),
                                   ("num4d_omit", "num4d_omit", (0.45, 0.0035, 2.2), None),
                                   ("config1_corrected", "config1", (0.7, 0.004, 1.5), 5.9),
                                   ("config1_outside", "config1", (1.35, 0.0063, 0.4), None)):
        f = np.load(os.path.join(HERE, case + ".npz"))
        S = int(f["S"])
        params = np.ones((S, S, 3)) * np.array(vec)
        corr = None
        if corr_T is not None:
            corr = np.ones((S, S, 2))
            corr[..., 0] = corr_T
            corr[..., 1] = f["effGrav"][:, None]
        st, flux = integrate(1, float(f["R"]), float(f["Omega"]), float(f["r_s"]),
                             float(f["inclination"]), f["cellArea"], f["radius"], f["u"],
                             f["theta"], f["phi"], params, f["radiates"], corr, int(f["N_R"]),
                             f["deflection"], f["cos_alpha"], f["lag"], f["maxDeflection"],
                             f["cos_gamma"], f["energies"], f["leaves"], f["phases"], atm, (),
                             None, 1 if corr is not None else None, 0,
                             int(f["image_order_limit"]) or None)
        assert st == 0
        out[tag + "_flux"] = flux
        out[tag + "_vec"] = np.array(vec)
        if corr is not None:
            out[tag + "_correction"] = corr
    save("split", **out)


def pol_num2d(xpsi):
    """The numerical polarised 2-D atmosphere (atm_ext 4, "Pol_Num2D",
    hot_Num2D.pyx) of synthetic.pol2d_tables: the plain integrator
    (integrator_for_azimuthal_invariance.pyx, I only) and the Stokes
    integrator (integratorIQU_for_azimuthal_invariance.pyx, I and Q tables)
    on config1's mesh (300 Hz) and num4d_omit's (600 Hz), with a blackbody
    elsewhere's correction, and on a mu grid topped at 0.9 (queries above
    the table: the cached walk's clamp history)."""
    from xpsi.cellmesh.integrator_for_azimuthal_invariance import integrate as plain
    from xpsi.cellmesh.integratorIQU_for_azimuthal_invariance import integrate as iqu
    out = {}
    for tag, case, corr_T, mu_top in (("config1", "config1", None, 1.0),
                                      ("num4d_omit", "num4d_omit", None, 1.0),
                                      ("config1_corrected", "config1", 6.0, 1.0),
                                      ("config1_mu09", "config1", None, 0.9)):
        f = np.load(os.path.join(HERE, case + ".npz"))
        S = int(f["S"])
        atm_I, atm_Q = synthetic.pol2d_tables(mu_top=mu_top)
        corr = None
        if corr_T is not None:
            corr = np.ones((S, S, 2))
            corr[..., 0] = corr_T
            corr[..., 1] = f["effGrav"][:, None]
        common = (float(f["R"]), float(f["Omega"]), float(f["r_s"]), float(f["inclination"]),
                  f["cellArea"], f["radius"], f["u"], f["theta"], f["phi"],
                  np.array(f["params"], copy=True), f["radiates"], corr, int(f["N_R"]),
                  f["deflection"], f["cos_alpha"], f["lag"], f["maxDeflection"], f["cos_gamma"],
                  f["energies"], f["leaves"], f["phases"])
        iol = int(f["image_order_limit"]) or None
        st, flux = plain(1, *common, atm_I, (), 4, 1 if corr is not None else None, 0, iol)
        assert st == 0
        res = iqu(1, *common, atm_I, atm_Q, (), 4, 1 if corr is not None else None, 0, iol)
        assert res[0] == 0
        out[tag + "_plain"] = flux
        out[tag + "_I"], out[tag + "_Q"], out[tag + "_U"] = res[1], res[2], res[3]
        out[tag + "_mu_top"] = np.array(mu_top)
        if corr is not None:
            out[tag + "_correction"] = corr
    save("pol_num2d", **out)


def split_iqu(xpsi):
    """The split Stokes integrator
    (integratorIQU_for_azimuthal_invariance_split.pyx): I and Q split tables
    (synthetic.split_table, split_table_q), each reduced to (mu, E) at the
    first cell's (t_e, t_bb, tau), on config1's and num4d_omit's meshes,
    with a blackbody elsewhere's correction, and outside the table."""
    from xpsi.cellmesh.integratorIQU_for_azimuthal_invariance_split import integrate
    atm_I = synthetic.split_table()
    atm_Q = synthetic.split_table_q()
    out = {}
    for tag, case, vec, corr_T in (("config1", "config1", (0.7, 0.004, 1.5), None),
                                   ("num4d_omit", "num4d_omit", (0.45, 0.0035, 2.2), None),
                                   ("config1_corrected", "config1", (0.7, 0.004, 1.5), 5.9),
                                   ("config1_outside", "config1", (1.35, 0.0063, 0.4), None)):
        f = np.load(os.path.join(HERE, case + ".npz"))
        S = int(f["S"])
        params = np.ones((S, S, 3)) * np.array(vec)
        corr = None
        if corr_T is not None:
            corr = np.ones((S, S, 2))
            corr[..., 0] = corr_T
            corr[..., 1] = f["effGrav"][:, None]
        res = integrate(1, float(f["R"]), float(f["Omega"]), float(f["r_s"]),
                        float(f["inclination"]), f["cellArea"], f["radius"], f["u"],
                        f["theta"], f["phi"], params, f["radiates"], corr, int(f["N_R"]),
                        f["deflection"], f["cos_alpha"], f["lag"], f["maxDeflection"],
                        f["cos_gamma"], f["energies"], f["leaves"], f["phases"], atm_I, atm_Q,
                        (), None, 1 if corr is not None else None, 0,
                        int(f["image_order_limit"]) or None)
        assert res[0] == 0
        out[tag + "_I"], out[tag + "_Q"], out[tag + "_U"] = res[1], res[2], res[3]
        out[tag + "_vec"] = np.array(vec)
        if corr is not None:
            out[tag + "_correction"] = corr
    save("split_iqu", **out)


def general_iqu(xpsi):
    """The general Stokes integrator of HotRegion(symmetry=False)
    (cellmesh/integratorIQU.pyx) and, for the same atmospheres, the general
    intensity integrator (cellmesh/integrator.pyx), on the general
    integrator's cell-varying temperatures: the burst blackbody (atm_ext 3)
    at 300 and 600 Hz, the blackbody with a blackbody elsewhere's
    correction, and Pol_Num2D (atm_ext 4) on full and 0.9-topped mu grids."""
    from xpsi.cellmesh.integrator import integrate as plain
    from xpsi.cellmesh.integratorIQU import integrate as iqu
    g = np.load(os.path.join(HERE, "general_integrator.npz"))
    out = {}
    for tag, case, ext, corr_T, mu_top in (("config1_ext3", "config1", 3, None, 1.0),
                                           ("num4d_omit_ext3", "num4d_omit", 3, None, 1.0),
                                           ("config1_ext1_corrected", "config1", 1, 6.0, 1.0),
                                           ("config1_ext4", "config1", 4, None, 1.0),
                                           ("num4d_omit_ext4_mu09", "num4d_omit", 4, None, 0.9)):
        f = np.load(os.path.join(HERE, case + ".npz"))
        S = int(f["S"])
        params = np.ascontiguousarray(g[case + "_params"])
        corr = None
        if corr_T is not None:
            corr = np.ones((S, S, 2))
            corr[..., 0] = corr_T
            corr[..., 1] = f["effGrav"][:, None]
        atm_I, atm_Q = synthetic.pol2d_tables(mu_top=mu_top) if ext == 4 else ((), ())
        common = (float(f["R"]), float(f["Omega"]), float(f["r_s"]), float(f["inclination"]),
                  f["cellArea"], f["radius"], f["u"], f["theta"], f["phi"], params,
                  f["radiates"], corr, int(f["N_R"]), f["deflection"], f["cos_alpha"],
                  f["lag"], f["maxDeflection"], f["cos_gamma"], f["energies"], f["leaves"],
                  f["phases"])
        iol = int(f["image_order_limit"]) or None
        res = iqu(1, *common, atm_I, atm_Q, (), ext, 1 if corr is not None else None, 0, iol)
        assert res[0] == 0
        st, flux = plain(1, *common, atm_I, (), ext, 1 if corr is not None else None, 0, iol)
        assert st == 0
        out[tag + "_I"], out[tag + "_Q"], out[tag + "_U"] = res[1], res[2], res[3]
        out[tag + "_plain"] = flux
        out[tag + "_mu_top"] = np.array(mu_top)
        if corr is not None:
            out[tag + "_correction"] = corr
    save("general_iqu", **out)


def interpolators(xpsi):
    """The phase and energy interpolators (tools/phase_interpolator.pyx,
    tools/energy_interpolator.pyx, with the default Akima-periodic and
    Steffen interpolants) on config1's folded signal (phases in cycles,
    shifted; negative parts dropped or kept) and its photon flux (log10
    energies, new energies inside and above the grid; one column made
    non-positive so that it is splined without the logarithm)."""
    from xpsi.tools.phase_interpolator import phase_interpolator
    from xpsi.tools.energy_interpolator import energy_interpolator
    f = np.load(os.path.join(HERE, "config1.npz"))
    folded = np.ascontiguousarray(f["folded"][:60])
    ph = np.ascontiguousarray(f["comp_phases"])
    rng = np.random.default_rng(11)
    new_ph = np.ascontiguousarray(np.sort(rng.uniform(-0.3, 1.3, 97)))
    # a row with an oscillation, so that the interpolant dips below zero
    osc = np.ascontiguousarray(np.vstack([folded, np.sin(2 * np.pi * 3 * ph[None, :]) * 0.1]))
    out = {"phase_signal": osc, "phase_phases": ph, "phase_new": new_ph}
    for tag, shift, neg in (("shift", 0.23, 0), ("neg", -0.41, 1)):
        out["phase_" + tag] = phase_interpolator(new_ph, ph, osc, shift, neg)
        out["phase_%s_shift" % tag] = np.array(shift)
    flux = np.array(f["flux"], copy=True)
    flux[:, 5] = flux[:, 5] - flux[:, 5].max() * 0.5  # a column with non-positive entries
    flux = np.ascontiguousarray(flux)
    lgE = np.ascontiguousarray(f["log10_energies"])
    new_lgE = np.ascontiguousarray(np.linspace(lgE[0], lgE[-1] + 0.1, 150))
    out["energy_signal"] = flux
    out["energy_log10"] = lgE
    out["energy_new"] = new_lgE
    out["energy_out"] = energy_interpolator(1, flux, lgE, new_lgE)
    save("interpolators", **out)


def main():
    xpsi = H.load()
    if len(sys.argv) > 1:
        for name in sys.argv[1:]:
            globals()[name](xpsi)
        return
    meshes(xpsi)
    examples_fast(xpsi)
    num4d_omit(xpsi)
    config1(xpsi)
    elsewhere(xpsi)
    elsewhere_correction(xpsi)
    general_integrator(xpsi)
    synthesis(xpsi)
    stokes(xpsi)
    gaussian(xpsi)
    split(xpsi)
    pol_num2d(xpsi)
    split_iqu(xpsi)
    general_iqu(xpsi)
    interpolators(xpsi)
    beaming(xpsi)
    energy_arrays(xpsi)
    poisson_given_background(xpsi)


if __name__ == "__main__":
    main()
