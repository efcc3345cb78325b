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
    I = x^3/(e^x - 1) (0.42 + 0.58 mu) (1 + 0.05 (logg - 14.5)) (1 + 1e-3 N(0,1)),
    x = 10^logE.  Returns the tuple X-PSI preloads: (logT, logg, mu, logE, I)."""
    nT, ng, nmu, nE = shape
    logT = np.linspace(*ranges[0], nT)
    logg = np.linspace(*ranges[1], ng)
    mu = np.linspace(*ranges[2], nmu)
    logE = np.linspace(*ranges[3], nE)
    rng = np.random.default_rng(seed)
    x = 10.0 ** logE
    planck = x ** 3 / np.expm1(x)
    I = (planck[None, None, None, :] * (0.42 + 0.58 * mu)[None, None, :, None]
         * (1.0 + 0.05 * (logg - 14.5))[None, :, None, None]
         * np.ones((nT, 1, 1, 1)))
    I = I * (1.0 + 1.0e-3 * rng.standard_normal(I.shape))
    return (logT, logg, mu, logE, np.ascontiguousarray(I.reshape(-1)))


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
