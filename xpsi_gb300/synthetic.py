"""Seeded synthetic workloads with the shapes of the pulse-likelihood
benchmarks: numerical atmosphere table, synthetic instrument response,
star/spot parameters and Poisson data.  No external data files are needed.
"""
import math

import numpy as np

# xpsi/global_imports.py constants
KPC = 3.08567758e19


def num4d_table(shape=(35, 14, 67, 166), seed=2,
                ranges=((5.0, 7.0), (13.4, 15.6), (0.0, 1.0), (-1.5, 2.7))):
    """A numerical 4-D hot atmosphere (logT, logg, mu, log10(E/kT)) filled with
    a limb-darkened modified blackbody plus 1e-3 seeded noise:
    I = P x^3/(e^x - 1) (0.42 + 0.58 mu) (1 + 0.05 (logg - 14.5)) (1 + 1e-3 N(0,1)),
    x = 10^logE, with P = 2 k^3 / (h^2 c^2) in cgs so that I T^3 is a specific
    intensity per Hz (the units the Num4D evaluator expects,
    hot_Num4D.pyx:437-461).  Returns the tuple X-PSI preloads:
    (logT, logg, mu, logE, I)."""
    nT, ng, nmu, nE = shape
    logT = np.linspace(*ranges[0], nT)
    logg = np.linspace(*ranges[1], ng)
    mu = np.linspace(*ranges[2], nmu)
    logE = np.linspace(*ranges[3], nE)
    rng = np.random.default_rng(seed)
    x = 10.0 ** logE
    k_B, h, c = 1.380649e-16, 6.62607015e-27, 2.99792458e10
    planck = (2.0 * k_B ** 3 / (h * h * c * c)) * x ** 3 / np.expm1(x)
    I = (planck[None, None, None, :] * (0.42 + 0.58 * mu)[None, None, :, None]
         * (1.0 + 0.05 * (logg - 14.5))[None, :, None, None]
         * np.ones((nT, 1, 1, 1)))
    I = I * (1.0 + 1.0e-3 * rng.standard_normal(I.shape))
    return (logT, logg, mu, logE, np.ascontiguousarray(I.reshape(-1)))


def split_table(shape=(6, 5, 5, 12, 64), seed=4,
                ranges=((0.2, 1.2), (0.002, 0.006), (0.5, 3.0), (0.0, 1.0), (5e-5, 0.03))):
    """A 5-D split atmosphere (t_e, t_bb, tau, mu, E in electron rest energies)
    for the split integrator: a Comptonised-blackbody-like shape
    x^2 exp(-E / t_bb') (1 + tau (0.3 + 0.7 mu)) (1 + 0.1 t_e) with
    t_bb' = t_bb (1 + 0.2 tau), times 1 + 1e-3 seeded noise; positive
    everywhere.  Returns the tuple X-PSI preloads (5 grids, intensity)."""
    g = [np.linspace(lo, hi, n) for (lo, hi), n in zip(ranges, shape)]
    te, tbb, tau, mu, E = np.meshgrid(*g, indexing="ij")
    tb = tbb * (1.0 + 0.2 * tau)
    I = (E / tb) ** 2 * np.exp(-E / tb) * (1.0 + tau * (0.3 + 0.7 * mu)) * (1.0 + 0.1 * te)
    I = I * (1.0 + 1.0e-3 * np.random.default_rng(seed).standard_normal(I.shape))
    return tuple(np.ascontiguousarray(x) for x in g) + (np.ascontiguousarray(I.reshape(-1)),)


def split_table_q(shape=(6, 5, 5, 12, 64), seed=9, **kw):
    """Stokes Q of a split atmosphere on split_table's grids: the intensity
    times -(0.05 + 0.1 (1 - mu)) (polarisation across the surface normal,
    strongest at the limb), times 1 + 1e-3 seeded noise.  Returns the tuple
    (5 grids, Q)."""
    g = split_table(shape=shape, **kw)
    I = g[5].reshape(shape)
    mu = g[3][None, None, None, :, None]
    Q = -(0.05 + 0.1 * (1.0 - mu)) * I
    Q = Q * (1.0 + 1.0e-3 * np.random.default_rng(seed).standard_normal(Q.shape))
    return g[:5] + (np.ascontiguousarray(Q.reshape(-1)),)


def pol2d_tables(shape=(12, 80), seed=6, kT=0.6, mu_top=1.0, logE_range=(-1.3, 1.3)):
    """A numerical polarised 2-D atmosphere (HotRegion atm_ext "Pol_Num2D",
    hot_Num2D.pyx): I and Q on a (mu, log10 E/keV) grid.  I = E^3 /
    (exp(E/kT) - 1) (0.421 + 0.868 mu), Q = 0.1171 (mu - 1) / (1 + 3.582 mu)
    (1 + 0.2 log10 E) I (the burst approximation with an energy trend), each
    times 1 + 1e-3 seeded noise; the mu grid runs over [0, mu_top].  Returns
    ((mu, logE, I), (mu, logE, Q)) as X-PSI preloads them."""
    mu = np.linspace(0.0, mu_top, shape[0])
    lgE = np.linspace(logE_range[0], logE_range[1], shape[1])
    M, L = np.meshgrid(mu, lgE, indexing="ij")
    E = 10.0 ** L
    I = E ** 3 / np.expm1(E / kT) * (0.421 + 0.868 * M)
    Q = 0.1171 * (M - 1.0) / (1.0 + 3.582 * M) * (1.0 + 0.2 * L) * I
    rng = np.random.default_rng(seed)
    I = I * (1.0 + 1.0e-3 * rng.standard_normal(I.shape))
    Q = Q * (1.0 + 1.0e-3 * rng.standard_normal(Q.shape))
    mu, lgE = np.ascontiguousarray(mu), np.ascontiguousarray(lgE)
    return ((mu, lgE, np.ascontiguousarray(I.reshape(-1))),
            (mu.copy(), lgE.copy(), np.ascontiguousarray(Q.reshape(-1))))


def gaussian_response(n_channels, n_inputs, e_lo=0.1, e_hi=10.0, width=0.1):
    """Synthetic response matrix [channels, inputs]: Gaussian redistribution
    (sigma = width * E) times a smooth effective area of 100-1000 cm^2,
    A(E) = 100 + 900 exp(-(log10(E / 1.5 keV) / 0.6)^2).  Returns
    (matrix, input_edges, channel_edges)."""
    in_edges = np.logspace(math.log10(e_lo), math.log10(e_hi), n_inputs + 1)
    ch_edges = np.logspace(math.log10(e_lo), math.log10(e_hi), n_channels + 1)
    Em = np.sqrt(in_edges[:-1] * in_edges[1:])
    area = 100.0 + 900.0 * np.exp(-(np.log10(Em / 1.5) / 0.6) ** 2)
    sig = width * Em
    from math import erf
    verf = np.vectorize(erf)
    lo = (ch_edges[:-1, None] - Em[None, :]) / (math.sqrt(2.0) * sig[None, :])
    hi = (ch_edges[1:, None] - Em[None, :]) / (math.sqrt(2.0) * sig[None, :])
    M = 0.5 * (verf(hi) - verf(lo)) * area[None, :]
    assert (M.max(axis=0) > 0).all() and (M.max(axis=1) > 0).all()
    return np.ascontiguousarray(M), in_edges, ch_edges


def config1_workload(n_channels=300, n_inputs=64, n_energies=64):
    """The small plain configuration: star, spot, grids and instrument."""
    M, in_edges, ch_edges = gaussian_response(n_channels, n_inputs)
    energies = np.logspace(math.log10(in_edges[0]), math.log10(in_edges[-1]), n_energies)
    return dict(mass=1.4, radius_km=12.0, frequency=300.0, inclination=1.0,
                distance_kpc=1.0, d_sq=(1.0 * KPC) ** 2, colatitude=1.0,
                spot_radius=0.075, logT=6.1, matrix=M, input_edges=in_edges,
                channel_edges=ch_edges, energies=energies,
                phase_edges=np.linspace(0.0, 1.0, 33), exposure=1.0e6)


def config1_model():
    """Model of the small plain configuration: one blackbody hot region
    (sqrt_num_cells 32, min 10, max 80; 64 leaves, 512 rays), 64 energies,
    the 300 x 64 response, 32 phase bins, exposure 1e6 s; data are attached
    later (attach_data).  Its parameter vector is config1_vector()."""
    from .batch import Data, HotRegionSpec, Instrument, Model
    w = config1_workload()
    return Model(regions=[HotRegionSpec(atm_ext=1, sqrt_num_cells=32, min_sqrt_num_cells=10,
                                        max_sqrt_num_cells=80, num_leaves=64, num_rays=512)],
                 instrument=Instrument(w["matrix"], w["input_edges"]),
                 data=Data(np.zeros((300, 32), np.int32), w["phase_edges"], w["exposure"]),
                 num_energies=64)


def config1_vector():
    """M 1.4, R 12 km, 300 Hz, i 1 rad, 1 kpc; spot colatitude 1.0, radius
    0.075, log T 6.1, no phase shift."""
    w = config1_workload()
    return np.array([w["mass"], w["radius_km"], w["frequency"], math.cos(w["inclination"]),
                     w["distance_kpc"], w["colatitude"], w["spot_radius"], w["logT"], 0.0])


def poisson_data(registered, comp_phases, phase_edges, exposure, seed=20261203,
                 bg_fraction=0.1):
    """Counts [channels, bins]: Poisson draws of the source counts per phase
    bin plus a flat background at `bg_fraction` of each channel's
    phase-summed source counts."""
    fine = np.linspace(0.0, 1.0, 4097)
    B = len(phase_edges) - 1
    src = np.zeros((registered.shape[0], B))
    for c in range(registered.shape[0]):
        r = np.interp(fine, comp_phases, registered[c])
        cum = np.concatenate([[0.0], np.cumsum(0.5 * (r[1:] + r[:-1]) * np.diff(fine))])
        src[c] = np.diff(np.interp(phase_edges, fine, cum)) * exposure
    src = np.clip(src, 0.0, None)
    bg = bg_fraction * src.sum(axis=1, keepdims=True) / B
    rng = np.random.default_rng(seed)
    return rng.poisson(src + bg).astype(np.int32)


def _offset_point(colat, dist, chi):
    """Point at angular distance `dist` from the spot centre (colat, azimuth 0)
    in direction chi on the sphere; returns (colatitude, azimuth)."""
    c = np.array([math.sin(colat), 0.0, math.cos(colat)])
    e_t = np.array([math.cos(colat), 0.0, -math.sin(colat)])
    e_p = np.array([0.0, 1.0, 0.0])
    x = math.cos(dist) * c + math.sin(dist) * (math.cos(chi) * e_t + math.sin(chi) * e_p)
    return math.acos(max(-1.0, min(1.0, x[2]))), math.atan2(x[1], x[0])


def draw_spots(rng):
    """Spot parameters of the full-size plain configuration: a circular spot
    and a spot with an omitted crescent; colatitudes U(0, pi), radii
    U(0.01, 0.5), log T U(5.8, 6.6), omit radius U(0.3, 0.9) x radius, omit
    centre offset U(0.2, 0.8) x radius inside the spot, phase shifts U(0, 1)."""
    out = []
    for h in range(2):
        colat = rng.uniform(0.0, math.pi)
        rad = rng.uniform(0.01, 0.5)
        logT = rng.uniform(5.8, 6.6)
        shift = rng.uniform(0.0, 1.0)
        out += [colat, rad, logT, shift]
        if h == 1:
            o_r = rng.uniform(0.3, 0.9) * rad
            off = rng.uniform(0.2, 0.8) * rad
            chi = rng.uniform(0.0, 2 * math.pi)
            o_c, o_a = _offset_point(colat, off, chi)
            out += [o_r, o_c, o_a]
    return out


def prior_vector(rng, fixed_star=None):
    """One parameter vector of the batched configuration: M U(1, 3) Msun,
    R U(3 r_g(M), 16 km), spin U(200, 600) Hz, cos i U(0, 1), D = 1 kpc,
    spots as draw_spots."""
    if fixed_star is not None:
        star = list(fixed_star)
    else:
        M = rng.uniform(1.0, 3.0)
        r_g_km = M * 0.5 * 2.95325024e3 / 1.0e3
        R = rng.uniform(3.0 * r_g_km, 16.0)
        star = [M, R, rng.uniform(200.0, 600.0), rng.uniform(0.0, 1.0), 1.0]
    return star + draw_spots(rng)


def config2_model(K=1500, q=128, num_energies=128, sqrt_num_cells=64, num_leaves=128,
                  num_rays=1024, max_sqrt_num_cells=128, table_shape=(35, 14, 67, 166),
                  data_seed=20261203):
    """Model of the full-size plain configuration (two Num4D hot regions, one
    with an omitted crescent) with synthetic instrument K x q; data are drawn
    later by draw_data()."""
    from .batch import Data, HotRegionSpec, Instrument, Model
    M, in_edges, _ = gaussian_response(K, q)
    regions = [HotRegionSpec(atm_ext=2, sqrt_num_cells=sqrt_num_cells, min_sqrt_num_cells=10,
                             max_sqrt_num_cells=max_sqrt_num_cells, num_leaves=num_leaves,
                             num_rays=num_rays),
               HotRegionSpec(atm_ext=2, sqrt_num_cells=sqrt_num_cells, min_sqrt_num_cells=10,
                             max_sqrt_num_cells=max_sqrt_num_cells, num_leaves=num_leaves,
                             num_rays=num_rays, omit=True)]
    data = Data(counts=np.zeros((K, 32), dtype=np.int32), phase_edges=np.linspace(0, 1, 33),
                exposure=1.0e6)
    return Model(regions=regions, instrument=Instrument(M, in_edges), data=data,
                 num_energies=num_energies, atmosphere=num4d_table(table_shape, seed=2))


def config2_vector(seed=1):
    """The full-size configuration's parameter vector: the small configuration's
    star (M 1.4, R 12 km, 300 Hz, i 1 rad, 1 kpc) and spots drawn with `seed`."""
    rng = np.random.default_rng(seed)
    return np.array(prior_vector(rng, fixed_star=[1.4, 12.0, 300.0, math.cos(1.0), 1.0]))


def config3_vectors(V=4096, seed=3):
    rng = np.random.default_rng(seed)
    return np.array([prior_vector(rng) for _ in range(V)])


def attach_data(model, registered_by_region, shifts, seed=20261203):
    """Replace the model's counts by Poisson draws from the summed registered
    signals of its hot regions (each [K, N_P]).  The likelihood integrates a
    region's signal over [edge + shift, edge' + shift]
    (compute_expected_counts.pyx:146-152), so the count rate at data phase x
    is signal(x + shift)."""
    N_P = registered_by_region[0].shape[1]
    ph = np.linspace(0.0, 1.0, N_P)
    total = np.zeros_like(registered_by_region[0])
    fine = np.linspace(0.0, 1.0, N_P)
    for reg, s in zip(registered_by_region, shifts):
        for c in range(reg.shape[0]):
            total[c] += np.interp((fine + s) % 1.0, ph, reg[c])
    model.data.counts = poisson_data(total, ph, model.data.phase_edges, model.data.exposure,
                                     seed=seed)
    return model
