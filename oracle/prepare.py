"""The oracle's own preparation of a batch of parameter vectors: what the
reference's model classes do before the numerical stages, restated here so
that the CPU oracle (and the timed CPU baseline) runs nothing of the GPU
library -- not even its host mesh builder.

TEST INFRASTRUCTURE.  Per vector and hot-region member:

  Spacetime derived quantities          Spacetime.py:110-187
  atmosphere-bounds check (status 3)    Photosphere.py:486-507
  cell budget and mesh                  HotRegion.py:774-836 with the oracle's
                                        mesh restatement (xpsi_oracle_mesh.c)
  lag calibration constants             HotRegion.py:880-901
  source parameters, radiating cells    HotRegion.py:953-1017

and, with an elsewhere, its closed mesh (Elsewhere.py:254-330,
global_mesh.pyx).  The result carries the fields oracle/pipeline.py reads,
in the same packed layout as the batched path's host preparation.
"""
import math
from types import SimpleNamespace

import numpy as np

from oracle import oracle as O

# xpsi/global_imports.py:68-79
_GM = 0.5 * 2.95325024e3
_C = 2.99792458e8
_CSQ = _C * _C
_G = 6.6740831e-11
_KM = 1.0e3
_KPC = 3.08567758e19
_2PI = 2.0 * math.pi


def _log_g(mu, R, zeta, eps):
    """effective_gravity_universal.pyx:10-71 (oblate star)."""
    x = zeta
    g_0 = x * _C * _C / (R * math.sqrt(1.0 - 2.0 * x))
    c_e, c_p = -0.791 + 0.776 * x, 1.138 - 1.431 * x
    d_e, d_p = (-1.315 + 2.431 * x) * eps * x, (0.653 - 2.864 * x) * eps * x
    d_60 = (13.47 - 27.13 * x) * eps * x
    f_e, f_p = -1.172 * x * eps * eps, 0.975 * x * eps * eps
    g = 1.0
    g += (c_e + d_e + f_e) * eps * (1.0 - mu * mu)
    g += (c_p + d_p + f_p - d_60) * eps * mu * mu
    g += d_60 * eps * abs(mu)
    return math.log10(g * g_0) + 2.0


def _names(model):
    names = ["mass", "radius", "frequency", "cos_inclination", "distance"]
    for h, r in enumerate(model.regions):
        names += [f"h{h}_colatitude", f"h{h}_radius", f"h{h}_temperature", f"h{h}_phase_shift"]
        if r.omit:
            names += [f"h{h}_omit_radius", f"h{h}_omit_colatitude", f"h{h}_omit_azimuth"]
    if getattr(model, "elsewhere", None) is not None:
        names.append("elsewhere_temperature")
    return names


def prepare(model, params, n_threads=1):
    params = np.atleast_2d(np.asarray(params, dtype=np.float64))
    V, H = params.shape[0], len(model.regions)
    names = _names(model)
    if params.shape[1] != len(names):
        raise ValueError("expected %d parameters per vector" % len(names))
    col = {n: i for i, n in enumerate(names)}
    atm = model.atmosphere
    status = np.zeros(V, dtype=np.int32)
    members, stars = [], []
    for v in range(V):
        p = params[v]
        M_sun, R_km, f = p[col["mass"]], p[col["radius"]], p[col["frequency"]]
        r_g = M_sun * _GM
        st = dict(M=M_sun * _GM * _CSQ / _G, r_s=2.0 * r_g, R=R_km * _KM, Omega=_2PI * f, f=f,
                  i=math.acos(p[col["cos_inclination"]]),
                  d_sq=(p[col["distance"]] * _KPC) * (p[col["distance"]] * _KPC))
        st["zeta"] = r_g / st["R"]
        st["epsilon"] = st["Omega"] ** 2.0 * st["R"] ** 3.0 / (_G * st["M"])
        stars.append(st)
        if atm is not None and any(r.atm_ext == 2 for r in model.regions):
            T_lo, T_hi = atm[0][0], atm[0][-1]
            g_lo, g_hi = atm[1][0], atm[1][-1]
            for h, r in enumerate(model.regions):
                if r.atm_ext == 2 and not T_lo <= p[col[f"h{h}_temperature"]] <= T_hi:
                    status[v] = 3
            for mu in (1.0, 0.0):
                if not g_lo <= _log_g(mu, st["R"], st["zeta"], st["epsilon"]) <= g_hi:
                    status[v] = 3
        for h, r in enumerate(model.regions):
            colat, rad = p[col[f"h{h}_colatitude"]], p[col[f"h{h}_radius"]]
            o_r = p[col[f"h{h}_omit_radius"]] if r.omit else 0.0
            o_c = p[col[f"h{h}_omit_colatitude"]] if r.omit else 0.0
            o_a = p[col[f"h{h}_omit_azimuth"]] if r.omit else 0.0
            S, N, _, _ = O.allocate_cells(r.sqrt_num_cells ** 2, r.min_sqrt_num_cells,
                                          r.max_sqrt_num_cells, st["M"], st["r_s"], st["R"],
                                          st["Omega"], st["zeta"], st["epsilon"], 0, rad, 0.0,
                                          colat, colat, -0.0, o_c, o_r, o_a)
            polar = colat - rad < 0.0 or colat + rad > math.pi
            fn = O.construct_polar_cellMesh if polar else O.construct_spot_cellMesh
            th, ph, rr, A, ma, cg, g = fn(n_threads, int(N), int(S), st["M"], st["r_s"],
                                          st["R"], st["zeta"], st["epsilon"], 0, rad, colat,
                                          o_r, o_c, o_a)
            ph = ph - o_a
            if r.is_antiphased:
                ph = ph + math.pi
            members.append(dict(v=v, h=h, S=int(S), theta=th, phi=ph, r=rr, area=A, maxAlpha=ma,
                                cos_gamma=cg, effGrav=g, logT=p[col[f"h{h}_temperature"]],
                                shift=p[col[f"h{h}_phase_shift"]], star=st))
    P = SimpleNamespace(V=V, H=H, status=status, else_V=0)
    n_rows = sum(m["S"] for m in members)
    n_cells = sum(m["S"] * m["S"] for m in members)
    P.row = {k: np.empty(n_rows) for k in ("u", "r_s", "maxAlpha", "radius", "cos_gamma",
                                           "theta0", "lag_C", "lag_scale")}
    P.cellArea, P.phi = np.empty(n_cells), np.empty(n_cells)
    P.params = np.empty((n_cells, 2))
    P.radiates = np.empty(n_cells, dtype=np.int32)
    P.d_sq = np.empty(len(members))
    P.shifts = np.empty((V, H))
    P.meshes = []
    ro = co = 0
    for mi, m in enumerate(members):
        S, st = m["S"], m["star"]
        rs = slice(ro, ro + S)
        u = st["r_s"] / m["r"]
        P.row["u"][rs] = u
        P.row["r_s"][rs] = st["r_s"]
        P.row["maxAlpha"][rs] = m["maxAlpha"]
        P.row["radius"][rs] = m["r"]
        P.row["cos_gamma"][rs] = m["cos_gamma"]
        P.row["theta0"][rs] = m["theta"][:, 0]
        # HotRegion.py:880-901
        R_i = st["R"] / st["r_s"]
        C_ = (1.0 / u - R_i)
        C_ += np.log((1.0 / u - 1.0) / (R_i - 1.0))
        C_ *= st["r_s"] / _C
        P.row["lag_C"][rs] = C_
        P.row["lag_scale"][rs] = st["f"] * _2PI
        cs = slice(co, co + S * S)
        P.cellArea[cs] = m["area"].reshape(-1)
        P.phi[cs] = m["phi"].reshape(-1)
        # HotRegion.py:953-1017: (log T, log g of the parallel) per cell
        prm = np.ones((S, S, 2))
        prm[..., :-1] *= m["logT"]
        for j in range(S):
            prm[:, j, -1] *= m["effGrav"]
        P.params[cs] = prm.reshape(-1, 2)
        P.radiates[cs] = np.greater(m["area"], 0.0).astype(np.int32).reshape(-1)
        P.d_sq[mi] = st["d_sq"]
        P.shifts[m["v"], m["h"]] = m["shift"]
        P.meshes.append(SimpleNamespace(S0=S, S1=S, row_off=ro, cell_off=co, omega=st["Omega"],
                                        inclination=st["i"]))
        ro += S
        co += S * S
    if getattr(model, "elsewhere", None) is not None:
        _elsewhere(model, P, params, col, stars, n_threads)
        # the hot regions' correction vectors: the elsewhere's log T with the
        # hot mesh's effective gravity (Elsewhere.py:305-330)
        P.correction = P.params.copy()
        P.correction[:, 0] = np.repeat(P.else_logT[[m["v"] for m in members]],
                                       [m["S"] * m["S"] for m in members])
    return P


def _elsewhere(model, P, params, col, stars, n_threads):
    spec = model.elsewhere
    V, S = P.V, int(spec.sqrt_num_cells)
    P.else_V, P.else_S = V, S
    P.else_logT = np.ascontiguousarray(params[:, col["elsewhere_temperature"]])
    P.else_row = {k: np.empty(V * S) for k in ("u", "r_s", "maxAlpha", "radius", "cos_gamma",
                                               "theta0")}
    P.else_phi = np.empty(V * S * S)
    P.else_params = np.empty((V * S * S, 2))
    P.else_meshes = []
    for v, st in enumerate(stars):
        th, ph, r, A, ma, cg, g = O.construct_closed_cellMesh(
            n_threads, S, S * S, st["M"], st["r_s"], st["R"], st["zeta"], st["epsilon"], 0)
        rs = slice(v * S, (v + 1) * S)
        P.else_row["u"][rs] = st["r_s"] / r
        P.else_row["r_s"][rs] = st["r_s"]
        P.else_row["maxAlpha"][rs] = ma
        P.else_row["radius"][rs] = r
        P.else_row["cos_gamma"][rs] = cg
        P.else_row["theta0"][rs] = th[:, 0]
        cs = slice(v * S * S, (v + 1) * S * S)
        P.else_phi[cs] = ph.reshape(-1)
        prm = P.else_params[cs].reshape(S, S, 2)
        prm[..., 0] = P.else_logT[v]
        prm[..., 1] = g[:, None]
        P.else_meshes.append(SimpleNamespace(omega=st["Omega"], inclination=st["i"],
                                             cellArea=A))
