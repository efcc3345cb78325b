"""CPU oracle of the batched likelihood (test infrastructure and the timed
CPU baseline): per vector and hot region, the oracle's restatement of the
reference stages on the inputs the batched path packs:
rays (rays.pyx) -> lag calibration (HotRegion.py:880-901) -> integrator
(integrator_for_azimuthal_invariance.pyx) -> /d^2 and energy integration
(Likelihood.py:361-364, energy_integrator.pyx) -> numpy dot fold
(Instrument.py:192-197) -> background-marginalised likelihood
(default_background_marginalisation.pyx).  With an elsewhere: its rays, the
time-invariant integrator (integrator_for_time_invariance.pyx), the hot
regions' correction and the spectrum added to the first hot region's signal
(Photosphere.py:588-592).

P is a prepared batch: oracle/prepare.py builds one with the oracle's own
meshes (so nothing of the GPU library runs), and the batched path's
preparation gives the same fields (to check the GPU stages on identical
inputs)."""
import math

import numpy as np

from oracle import oracle as O

_C = 2.99792458e8


def loglike(model, P, n_threads=1, return_stages=False):
    V, H = P.V, P.H
    N_L = model.regions[0].num_leaves
    N_R = model.regions[0].num_rays
    leaves = np.linspace(0.0, 2 * math.pi, N_L)
    phases = 2 * math.pi * np.linspace(0.0, 1.0, N_L)
    comp_phases = np.linspace(0.0, 1.0, N_L)
    logE = np.log10(model.energies)
    logEd = np.log10(model.instrument.energy_edges)
    atm = model.atmosphere
    counts = np.asarray(model.data.counts, dtype=np.float64)
    pre = O.precomputation(np.asarray(model.data.counts, np.int32))
    K = counts.shape[0]
    sup = model.data.support
    if sup is None:
        sup = -1.0 * np.ones((K, 2))
        sup[:, 0] = 0.0
    out = np.zeros(V)
    status = np.zeros(V, dtype=np.int32)
    stages = []
    else_V = getattr(P, "else_V", 0)
    for v in range(V):
        regs = []
        spectrum = None
        if else_V:
            spectrum, est = _elsewhere(model, P, v, n_threads)
            if est:
                status[v] = est
                continue
        for h in range(H):
            mi = v * H + h
            mesh = P.meshes[mi]
            S = mesh.S0
            r0, c0 = mesh.row_off, mesh.cell_off
            rs = slice(r0, r0 + S)
            cs = slice(c0, c0 + S * S)
            u = P.row["u"][rs].copy()
            ma = P.row["maxAlpha"][rs].copy()
            r_s = P.row["r_s"][r0]
            t, D, CA, L, MD = O.compute_rays(n_threads, S, r_s, u, ma, N_R)
            if t:
                status[v] = 1
                break
            for j in range(L.shape[1]):
                L[:, j] -= P.row["lag_C"][rs]
            L *= P.row["lag_scale"][r0]
            theta = np.repeat(P.row["theta0"][rs][:, None], S, axis=1)
            spec = model.regions[h]
            corr = P.correction[cs].reshape(S, S, 2) if else_V else None
            st, flux = O.integrate(n_threads, 0.0, mesh.omega, r_s, mesh.inclination,
                                   P.cellArea[cs].reshape(S, S), P.row["radius"][rs], u,
                                   theta, P.phi[cs].reshape(S, S),
                                   P.params[cs].reshape(S, S, 2),
                                   P.radiates[cs].reshape(S, S), corr, N_R, D, CA, L, MD,
                                   P.row["cos_gamma"][rs], model.energies, leaves, phases,
                                   atm if spec.atm_ext == 2 else (), None, spec.atm_ext,
                                   1 if else_V else None, 0, spec.image_order_limit)
            if st:
                status[v] = 2
                break
            if spectrum is not None and h == 0:
                flux = flux + spectrum[:, None]
            ei = O.energy_integrator(n_threads, flux / P.d_sq[mi], logE, logEd)
            regs.append(np.dot(model.instrument.matrix, ei))
            if return_stages:
                stages.append(dict(v=v, h=h, flux=flux, energy=ei, folded=regs[-1],
                                   deflection=D, lag=L))
        if status[v]:
            continue
        (ll, star, mb, mbs), st = O.eval_marginal_likelihood(
            model.data.exposure, model.data.phase_edges, counts, regs, [comp_phases] * H,
            P.shifts[v], pre, sup, 1000, 0.0, model.epsrel, model.epsilon, model.sigmas,
            model.llzero, slim=model.slim, return_status=True)
        out[v] = ll
        if st:
            status[v] = 5 if st == 1 else 4
    if P.status is not None:
        status[P.status != 0] = P.status[P.status != 0]
    return (out, status, stages) if return_stages else (out, status)


def _elsewhere(model, P, v, n_threads):
    """The spectrum of vector v's elsewhere and a status (0, 1 ray failure,
    7 integration failure)."""
    spec = model.elsewhere
    S = P.else_S
    rs = slice(v * S, (v + 1) * S)
    cs = slice(v * S * S, (v + 1) * S * S)
    er = P.else_row
    u = er["u"][rs].copy()
    ma = er["maxAlpha"][rs].copy()
    r_s = er["r_s"][v * S]
    t, D, CA, L, MD = O.compute_rays(n_threads, S, r_s, u, ma, spec.num_rays)
    if t:
        return None, 1
    m = P.else_meshes[v]
    theta = np.repeat(er["theta0"][rs][:, None], S, axis=1)
    st, spectrum = O.integrate_time_invariant(
        n_threads, 0.0, m.omega, r_s, m.inclination, S, m.cellArea, er["radius"][rs], u,
        theta, P.else_phi[cs].reshape(S, S), P.else_params[cs].reshape(S, S, 2),
        spec.num_rays, D, CA, MD, er["cos_gamma"][rs], model.energies, (), spec.atm_ext,
        spec.image_order_limit)
    if st:
        return None, 7
    return spectrum, 0
