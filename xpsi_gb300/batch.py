"""Batched likelihood evaluation: many parameter vectors per launch.

The model mirrors X-PSI's Likelihood/Star/Photosphere/HotRegion/Signal stack
for uniform-temperature hot regions (HotRegion.py, Signal.py, Likelihood.py),
with the per-vector geometry prepared on the host and every numerical stage
on the GPU:

    host   Spacetime derived quantities (Spacetime.py:110-187), cell budget and
           meshes (mesh_tools.pyx:892-1099, mesh.pyx, polar_mesh.pyx), lag
           calibration constants (HotRegion.py:880-901), source parameters
           (HotRegion.py:953-1017)
    GPU    rays (K1) -> integrator (K2/K3) -> energy integration over the
           instrument's input intervals with the 1/d^2 factor (K4,
           Likelihood.py:361-364) -> response fold (K5) -> background-
           marginalised log-likelihood of every vector (K6)

With an Elsewhere (a blackbody photosphere outside the hot regions,
Elsewhere.py) each vector also gets a closed mesh (host C++), its rays, the
time-invariant integrator, the correction of the hot regions' intensities
(integrator_for_azimuthal_invariance.pyx:469-478) and the spectrum added to
the first hot region's signal (Photosphere.py:588-592).

PyTorch supplies device buffers and the stream; the kernels are reached
through the C ABI only.
"""
import ctypes as C
import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from ._native import (AllocRequest, Atmos4D, Component, ElsewhereBatchData, ElsewhereMesh,
                      IntegrateBatchData, LikelihoodBatchData, Mesh, MeshBatchOut, MeshMember,
                      check, lib)
from .cellmesh import global_mesh as _global_mesh
from .cellmesh import mesh as _mesh

# xpsi/global_imports.py
_GM = 0.5 * 2.95325024e3
_C = 2.99792458e8
_CSQ = _C * _C
_G = 6.6740831e-11
_KM = 1.0e3
_KPC = 3.08567758e19
_2PI = 2.0 * math.pi

STATUS_NAMES = {0: "ok", 1: "RayError", 2: "PulseError", 3: "AtmosError", 4: "QuadFail",
                5: "SlimCut", 6: "BadInput", 7: "IntegrationError", 8: "DeviceTimeout"}


@dataclass
class HotRegionSpec:
    """Resolution and kind of one hot region (HotRegion.__init__ arguments)."""
    atm_ext: int = 1                 # 1 blackbody, 2 numerical 4-D
    sqrt_num_cells: int = 32
    min_sqrt_num_cells: int = 10
    max_sqrt_num_cells: int = 80
    num_leaves: int = 64
    num_rays: int = 512
    image_order_limit: Optional[int] = None
    omit: bool = False
    is_antiphased: bool = False


@dataclass
class ElsewhereSpec:
    """Resolution and kind of the photosphere elsewhere (Elsewhere.__init__
    arguments).  Only the blackbody (atm_ext 1) is batched: the hot regions'
    correction for a numerical elsewhere is not on the GPU path."""
    atm_ext: int = 1
    sqrt_num_cells: int = 64
    num_rays: int = 1000
    image_order_limit: Optional[int] = None


def identify_waveband(matrix, energy_edges, index_range=None):
    """The input intervals a signal integrates over (Signal._identify_waveband,
    Signal.py:324-354): from the data's channel range [a, b), the first input
    column with a nonzero response in channel a and the last with one in
    channel b - 1.  Returns ((first, end) input-interval range, the energy
    edges [end - first + 1])."""
    M = np.asarray(matrix)
    a, b = (0, M.shape[0]) if index_range is None else index_range

    def search(i, j, k):
        while M[i, j] == 0.0:
            j += k
        return j

    lo = search(a, 0, 1)
    hi = M.shape[1] + search(b - 1, -1, -1) + 1
    return (lo, hi), np.asarray(energy_edges)[lo:hi + 1]


def construct_energy_array(num_energies, wavebands, max_energy=None):
    """Photon energies for the integrators, distributed over the union of the
    signals' wavebands (Signal.construct_energy_array, Signal.py:1092-1197).

    wavebands: the energy-edge arrays of the signals (any order).  As the
    reference does: the bands are ordered by upper limit; a gap between a
    band's upper limit and the lowest lower limit of the bands above it is a
    coverage gap; max_energy (if below the highest limit) caps the range,
    falling to the bottom of a gap it lands in; the log10 span less the gaps'
    widths (the reference subtracts the gaps' widths in keV, not in log10)
    shares num_energies between the covered intervals, each getting
    ceil(fraction x num_energies) log-spaced energies.  Returns them
    ascending."""
    bands = [np.asarray(e, dtype=np.float64) for e in wavebands]
    if not bands:
        raise ValueError("at least one waveband is needed")
    ordered, gaps = [], []
    remaining = list(bands)
    MIN = None
    while remaining:
        k = 0
        for i in range(1, len(remaining)):
            if remaining[i][-1] > remaining[k][-1]:
                k = i
        top = remaining.pop(k)
        ordered.append(top)
        if len(ordered) > 1:
            for e in ordered[:-1]:
                if MIN is None or e[0] < MIN:
                    MIN = e[0]
            if top[-1] < MIN:
                gaps.append((top[-1], MIN))
    hi = ordered[0][-1]
    if max_energy is not None and max_energy < hi:
        MAX = max_energy
        kept = []
        for g in gaps:
            if g[0] < MAX <= g[1]:
                MAX = g[0]
            if MAX > g[1]:
                kept.append(g)
        gaps = kept
    else:
        MAX = hi
    for e in ordered:
        if MIN is None or e[0] < MIN:
            MIN = e[0]
    interval = np.log10(MAX) - np.log10(MIN)
    for g in gaps:
        interval -= (g[1] - g[0])
    energies = np.array([])
    for i in range(len(gaps) + 1):
        U = MAX if i == 0 else gaps[i - 1][0]
        L = MIN if i == len(gaps) else gaps[i][1]
        frac = (np.log10(U) - np.log10(L)) / interval
        num = int(math.ceil(frac * num_energies))
        energies = np.append(energies, np.logspace(np.log10(L), np.log10(U), int(num),
                                                   base=10.0)[::-1])
    return np.ascontiguousarray(energies[::-1])


@dataclass
class Instrument:
    matrix: np.ndarray               # [K, q] response (channels x input intervals)
    energy_edges: np.ndarray         # [q + 1] keV


@dataclass
class Data:
    counts: np.ndarray               # [K, B]
    phase_edges: np.ndarray          # [B + 1] cycles
    exposure: float
    support: Optional[np.ndarray] = None  # [K, 2]; default unbounded


@dataclass
class Model:
    regions: List[HotRegionSpec]
    instrument: Instrument
    data: Data
    num_energies: int = 64
    atmosphere: Optional[tuple] = None   # (logT, logg, mu, logE, I) for Num4D
    llzero: float = -1.0e90
    epsrel: float = 1.0e-8
    epsilon: float = 1.0e-3
    sigmas: float = 10.0
    slim: float = 20.0
    energies: np.ndarray = field(default=None)
    elsewhere: Optional[ElsewhereSpec] = None

    def __post_init__(self):
        if self.elsewhere is not None:
            e = self.elsewhere
            if e.atm_ext != 1:
                raise NotImplementedError("a batched elsewhere is a blackbody (atm_ext 1)")
            if e.sqrt_num_cells < 10 or e.sqrt_num_cells % 2 != 0:
                raise ValueError("elsewhere sqrt_num_cells must be an even integer >= 10")
            if e.num_rays < 3:
                raise ValueError("elsewhere num_rays must be at least 3")
        if self.energies is None:
            # the signal's waveband and the integrators' energies
            # (Signal.py:324-354, 1092-1197; Likelihood.py:102-104)
            _, edges = identify_waveband(self.instrument.matrix, self.instrument.energy_edges)
            self.energies = construct_energy_array(self.num_energies, [edges])
        leaves = {r.num_leaves for r in self.regions}
        rays = {r.num_rays for r in self.regions}
        if len(leaves) != 1 or len(rays) != 1:
            raise ValueError("all hot regions of one model share num_leaves and num_rays")


# parameter vector layout per vector:
#   mass, radius_km, frequency, cos_inclination, distance_kpc,
#   then per region: colatitude, angular radius, log10 T, phase shift,
#   and for an omit region additionally omit radius, omit colatitude, omit azimuth;
#   last, with an elsewhere, its log10 T
def param_names(model):
    names = ["mass", "radius", "frequency", "cos_inclination", "distance"]
    for h, r in enumerate(model.regions):
        names += [f"h{h}_colatitude", f"h{h}_radius", f"h{h}_temperature", f"h{h}_phase_shift"]
        if r.omit:
            names += [f"h{h}_omit_radius", f"h{h}_omit_colatitude", f"h{h}_omit_azimuth"]
    if getattr(model, "elsewhere", None) is not None:
        names.append("elsewhere_temperature")
    return names


def spacetime(mass, radius, frequency, cos_inclination, distance):
    """The derived quantities of xpsi.Spacetime (Spacetime.py:110-187) from
    its five parameters (solar masses, km, Hz, cos i, kpc): M (kg), r_g,
    r_s, R, R_r_s, f, Omega, i, d, d_sq (SI), zeta and epsilon of the
    universal relations (Morsink et al. 2007; AlGendy & Morsink 2014)."""
    r_g = mass * _GM
    M = mass * _GM * _CSQ / _G
    R = radius * _KM
    Omega = _2PI * frequency
    d = distance * _KPC
    return dict(M=M, r_g=r_g, r_s=2.0 * r_g, R=R, R_r_s=R / (2.0 * r_g), f=frequency,
                Omega=Omega, i=math.acos(cos_inclination), d=d, d_sq=d * d, zeta=r_g / R,
                epsilon=Omega ** 2.0 * R ** 3.0 / (_G * M))


def _effective_gravity_bounds(R, zeta, eps):
    c = _C
    out = []
    for mu in (1.0, 0.0):
        x = zeta
        g0 = x * c * c / (R * math.sqrt(1.0 - 2.0 * x))
        c_e, c_p = -0.791 + 0.776 * x, 1.138 - 1.431 * x
        d_e, d_p = (-1.315 + 2.431 * x) * eps * x, (0.653 - 2.864 * x) * eps * x
        d_60 = (13.47 - 27.13 * x) * eps * x
        f_e, f_p = -1.172 * x * eps * eps, 0.975 * x * eps * eps
        g = 1.0 + (c_e + d_e + f_e) * eps * (1.0 - mu * mu)
        g += (c_p + d_p + f_p - d_60) * eps * mu * mu + d_60 * eps * abs(mu)
        out.append(math.log10(g * g0) + 2.0)
    return out


class Prepared:
    """Host-packed inputs of one batch (numpy), ready to upload."""


def prepare(model: Model, params: np.ndarray, n_threads: int = 0,
            meshes: str = "host") -> Prepared:
    """Derived quantities and meshes of every (vector, hot region) member,
    packed into the flat arrays the kernels read.

    meshes="host": the meshes are built here on the host's cores (C++) and
    packed in numpy.  meshes="gpu": only the cell budget of each member is
    computed here; BatchEvaluator.upload builds the meshes on the GPU
    (xgpu_mesh_batch) straight into the packed device arrays."""
    if meshes not in ("host", "gpu"):
        raise ValueError("meshes must be 'host' or 'gpu'")
    params = np.atleast_2d(np.asarray(params, dtype=np.float64))
    V = params.shape[0]
    H = len(model.regions)
    names = param_names(model)
    if params.shape[1] != len(names):
        raise ValueError("expected %d parameters per vector: %s" % (len(names), names))
    col = {n: i for i, n in enumerate(names)}
    reqs, members, pend, status = [], [], [], np.zeros(V, dtype=np.int32)
    stars = []
    atm = model.atmosphere
    for v in range(V):
        p = params[v]
        Msun, Rkm, f, cosi, Dkpc = (p[col[k]] for k in ("mass", "radius", "frequency",
                                                         "cos_inclination", "distance"))
        sp = spacetime(Msun, Rkm, f, cosi, Dkpc)
        R, zeta, eps = sp["R"], sp["zeta"], sp["epsilon"]
        star = dict(r_s=sp["r_s"], R=R, Omega=sp["Omega"], zeta=zeta, eps=eps,
                    inclination=sp["i"], d_sq=sp["d_sq"], f=f)
        stars.append(star)
        if atm is not None and any(r.atm_ext == 2 for r in model.regions):
            # Photosphere.py:486-507
            gl = _effective_gravity_bounds(R, zeta, eps)
            for h, r in enumerate(model.regions):
                T = p[col[f"h{h}_temperature"]]
                if r.atm_ext == 2 and not (atm[0][0] <= T <= atm[0][-1]):
                    status[v] = 3
            if any(not (atm[1][0] <= g <= atm[1][-1]) for g in gl):
                status[v] = 3
        for h, r in enumerate(model.regions):
            colat, rad = p[col[f"h{h}_colatitude"]], p[col[f"h{h}_radius"]]
            logT, shift = p[col[f"h{h}_temperature"]], p[col[f"h{h}_phase_shift"]]
            if r.omit:
                o_r = p[col[f"h{h}_omit_radius"]]
                o_c = p[col[f"h{h}_omit_colatitude"]]
                o_a = p[col[f"h{h}_omit_azimuth"]]
            else:
                o_r = o_c = o_a = 0.0
            pend.append((AllocRequest(r.sqrt_num_cells ** 2, r.min_sqrt_num_cells,
                                      r.max_sqrt_num_cells, R, sp["Omega"], zeta, eps, 0, rad,
                                      0.0,
                                      colat, colat, -0.0, o_c, o_r, o_a),
                         dict(colat=colat, rad=rad, o_r=o_r, o_c=o_c, o_a=o_a),
                         dict(v=v, h=h, logT=logT, shift=shift, omit_azimuth=o_a,
                              antiphased=r.is_antiphased, spec=r, **star)))
    # cell budgets of all members at once (mesh_tools.pyx:892-1099), on the
    # host's cores
    alloc = (AllocRequest * len(pend))(*[q for q, _, _ in pend])
    if pend:
        check(lib().xgpu_allocate_cells_many(len(pend), alloc, int(n_threads)))
    for k, (_, g, mem) in enumerate(pend):
        S = int(alloc[k].out[0])
        colat, rad = g["colat"], g["rad"]
        polar = (colat - rad < 0.0) or (colat + rad > math.pi)
        reqs.append(dict(polar=polar, num_cells=int(alloc[k].out[1]), S=S, R_eq=mem["R"],
                         zeta=mem["zeta"], epsilon=mem["eps"], star_shape_ind=0,
                         cede_radius=rad, cede_colatitude=colat, super_radius=g["o_r"],
                         super_colatitude=g["o_c"], super_azimuth=g["o_a"]))
        members.append(dict(S=S, **mem))
    n_rows = sum(m["S"] for m in members)
    n_cells = sum(m["S"] * m["S"] for m in members)
    P = Prepared()
    P.V, P.H, P.n_rows, P.n_cells = V, H, n_rows, n_cells
    P.status = status
    N_E, N_P = len(model.energies), model.regions[0].num_leaves
    P.meshes = (Mesh * len(members))()
    P.d_sq = np.empty(len(members))
    P.shifts = np.empty((V, H))
    P.members = members
    P.else_V = 0
    if model.elsewhere is not None:
        _prepare_elsewhere(model, P, params, col, stars, n_threads)
    if meshes == "gpu":
        P.mesh_members = (MeshMember * len(members))()
        ro = co = 0
        for m_i, (m, q) in enumerate(zip(members, reqs)):
            S = m["S"]
            P.mesh_members[m_i] = MeshMember(
                int(q["polar"]), int(q["num_cells"]), S, float(q["R_eq"]), float(q["zeta"]),
                float(q["epsilon"]), int(q["star_shape_ind"]), float(q["cede_radius"]),
                float(q["cede_colatitude"]), float(q["super_radius"]),
                float(q["super_colatitude"]), float(q["super_azimuth"]), ro, co,
                float(m["r_s"]), float(m["f"] * _2PI), float(m["omit_azimuth"]),
                float(m["logT"]), int(bool(m["antiphased"])))
            _member_meta(P, m_i, m, ro, co, N_E, N_P)
            ro += S
            co += S * S
        P.row = None
        P.correction = None  # formed on the device from the GPU-built params
        return P
    P.mesh_members = None
    _mesh.build_many(reqs, n_threads)
    P.row = {k: np.empty(n_rows) for k in ("u", "r_s", "maxAlpha", "radius", "cos_gamma",
                                           "theta0", "lag_C", "lag_scale")}
    P.row_mesh = np.empty(n_rows, dtype=np.int32)
    P.cellArea = np.empty(n_cells)
    P.phi = np.empty(n_cells)
    P.params = np.empty((n_cells, 2))
    P.radiates = np.empty(n_cells, dtype=np.int32)
    ro = co = 0
    for m_i, (m, q) in enumerate(zip(members, reqs)):
        S = m["S"]
        sl = slice(ro, ro + S)
        u = m["r_s"] / q["r"]
        P.row["u"][sl] = u
        P.row["r_s"][sl] = m["r_s"]
        P.row["maxAlpha"][sl] = q["maxAlpha"]
        P.row["radius"][sl] = q["r"]
        P.row["cos_gamma"][sl] = q["cos_gamma"]
        P.row["theta0"][sl] = q["theta"][:, 0]
        R_i = m["R"] / m["r_s"]
        C_ = (1.0 / u - R_i)
        C_ += np.log((1.0 / u - 1.0) / (R_i - 1.0))
        C_ *= m["r_s"] / _C
        P.row["lag_C"][sl] = C_
        P.row["lag_scale"][sl] = m["f"] * _2PI
        P.row_mesh[sl] = m_i
        cs = slice(co, co + S * S)
        A = q["area"]
        P.cellArea[cs] = A.reshape(-1)
        ph = q["phi"] - m["omit_azimuth"]
        if m["antiphased"]:
            ph = ph + math.pi
        P.phi[cs] = ph.reshape(-1)
        prm = np.ones((S, S, 2))
        prm[..., :-1] *= m["logT"]
        for j in range(S):
            prm[:, j, -1] *= q["effGrav"]
        P.params[cs] = prm.reshape(-1, 2)
        P.radiates[cs] = np.greater(A, 0.0).astype(np.int32).reshape(-1)
        _member_meta(P, m_i, m, ro, co, N_E, N_P)
        ro += S
        co += S * S
    if P.else_V:
        # the hot regions' correction vectors: the elsewhere's log T with the
        # hot mesh's effective gravity (Elsewhere.py:305-330, HotRegion.py:1052-1067)
        P.correction = P.params.copy()
        P.correction[:, 0] = np.repeat(P.else_logT[[m["v"] for m in members]],
                                       [m["S"] * m["S"] for m in members])
    return P


def _prepare_elsewhere(model, P, params, col, stars, n_threads):
    """Closed meshes of every vector's elsewhere (host C++,
    global_mesh.pyx:21-137) packed like the hot meshes: per parallel u, r_s,
    maxAlpha, radius, cos_gamma, theta0; per cell phi and (log T, log10
    effective gravity of the parallel) (Elsewhere.py:254-330)."""
    spec = model.elsewhere
    V = P.V
    S = int(spec.sqrt_num_cells)
    reqs = [dict(S=S, num_cells=S * S, R_eq=st["R"], zeta=st["zeta"], epsilon=st["eps"],
                 star_shape_ind=0) for st in stars]
    _global_mesh.build_many(reqs, n_threads)
    P.else_V, P.else_S = V, S
    P.else_logT = np.ascontiguousarray(params[:, col["elsewhere_temperature"]])
    rows = V * S
    P.else_row = {k: np.empty(rows) for k in ("u", "r_s", "maxAlpha", "radius", "cos_gamma",
                                              "theta0")}
    P.else_row_mesh = np.repeat(np.arange(V, dtype=np.int32), S)
    P.else_phi = np.empty(V * S * S)
    P.else_params = np.empty((V * S * S, 2))
    P.else_meshes = (ElsewhereMesh * V)()
    for v, (q, st) in enumerate(zip(reqs, stars)):
        sl = slice(v * S, (v + 1) * S)
        P.else_row["u"][sl] = st["r_s"] / q["r"]
        P.else_row["r_s"][sl] = st["r_s"]
        P.else_row["maxAlpha"][sl] = q["maxAlpha"]
        P.else_row["radius"][sl] = q["r"]
        P.else_row["cos_gamma"][sl] = q["cos_gamma"]
        P.else_row["theta0"][sl] = q["theta"][:, 0]
        cs = slice(v * S * S, (v + 1) * S * S)
        P.else_phi[cs] = q["phi"].reshape(-1)
        prm = P.else_params[cs].reshape(S, S, 2)
        prm[..., 0] = P.else_logT[v]
        prm[..., 1] = q["effGrav"][:, None]
        P.else_meshes[v] = ElsewhereMesh(S, v * S, v * S * S, st["Omega"], st["inclination"],
                                         q["cellArea"], int(spec.image_order_limit or 0),
                                         int(spec.atm_ext))


def _member_meta(P, m_i, m, ro, co, N_E, N_P):
    S, spec = m["S"], m["spec"]
    P.meshes[m_i] = Mesh(S, S, ro, co, m["Omega"], m["inclination"],
                         int(spec.image_order_limit or 0), int(spec.atm_ext), m_i * N_E * N_P)
    P.d_sq[m_i] = m["d_sq"]
    P.shifts[m["v"], m["h"]] = m["shift"]


class BatchEvaluator:
    """Device-resident model (tables, response, data) plus per-batch buffers.

    precision "plain": every stage in FP64 (the drop-in's numerics).
    precision "mixed": the integrator's atmosphere interpolation (from an
    FP32 copy of the table), splines and cell x phase sums in FP32
    (xgpu_integrate_batch_mixed) and the response fold on the tensor cores
    in 3xTF32 split products with FP32 accumulation (xgpu_fold_batch_tc);
    rays, energy integration and the likelihood as in the plain form."""

    def __init__(self, model: Model, device=0, precision="plain"):
        import torch
        if precision not in ("plain", "mixed"):
            raise ValueError("precision is 'plain' or 'mixed'")
        if precision == "mixed" and model.elsewhere is not None:
            raise NotImplementedError("the elsewhere correction is computed by the FP64 "
                                      "integrator only (precision 'plain')")
        self.precision = precision
        # the integrator's work plan aims at about 4 x target_ctas chunks of
        # parallels (xgpu_integrate_batch; 0: 8 per SM)
        self.target_ctas = 0
        self.torch = torch
        self.model = model
        self.dev = torch.device("cuda", device)
        t = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt,
                                                          device=self.dev)
        self.energies = t(model.energies)
        r0 = model.regions[0]
        self.N_L = r0.num_leaves
        self.N_R = r0.num_rays
        self.leaves = t(np.linspace(0.0, _2PI, self.N_L))
        self.phases = t(_2PI * np.linspace(0.0, 1.0, self.N_L))
        self.comp_phases = t(np.linspace(0.0, 1.0, self.N_L))
        self.log10E = t(np.log10(model.energies))
        self.log10edges = t(np.log10(model.instrument.energy_edges))
        self.matrix = t(model.instrument.matrix)
        self.K, self.q = model.instrument.matrix.shape
        d = model.data
        self.counts = t(np.asarray(d.counts, dtype=np.float64))
        self.phase_edges = t(d.phase_edges)
        self.B = len(d.phase_edges) - 1
        sup = d.support
        if sup is None:
            sup = -1.0 * np.ones((self.K, 2))
            sup[:, 0] = 0.0
        self.support = t(sup)
        self.allow_negative = t(np.zeros(len(model.regions)), torch.int32)
        self.precomp = torch.empty(self.K, dtype=torch.float64, device=self.dev)
        from .likelihoods.default_background_marginalisation import precomputation
        self.precomp.copy_(torch.as_tensor(precomputation(np.asarray(d.counts, np.int32))))
        self.atmos = None
        if model.atmosphere is not None:
            self.atm_t = [t(a) for a in model.atmosphere]
            a = self.atm_t
            self.atm_f32 = a[4].to(torch.float32) if precision == "mixed" else None
            self.atmos = Atmos4D(a[0].data_ptr(), a[1].data_ptr(), a[2].data_ptr(),
                                 a[3].data_ptr(), a[4].data_ptr(), a[0].numel(),
                                 a[1].numel(), a[2].numel(), a[3].numel(),
                                 self.atm_f32.data_ptr() if self.atm_f32 is not None else None)

    # ---------------------------------------------------------------- upload
    def upload(self, P: Prepared, pinned=None):
        """Copy a prepared batch to the device (non-blocking from pinned
        memory when given) and allocate its work buffers."""
        torch = self.torch
        dev = self.dev
        f64 = torch.float64

        def put(a, dt=f64):
            h = torch.from_numpy(np.ascontiguousarray(a))
            if pinned is not None:
                h = h.pin_memory()
            return h.to(dev, non_blocking=True)
        B = dict()
        if P.mesh_members is not None:
            self._gpu_meshes(P, B)
        else:
            B["row"] = {k: put(v) for k, v in P.row.items()}
            B["row_mesh"] = put(P.row_mesh)
            B["cellArea"], B["phi"] = put(P.cellArea), put(P.phi)
            B["params"], B["radiates"] = put(P.params), put(P.radiates)
        B["d_sq"], B["shifts"] = put(P.d_sq), put(P.shifts)
        if P.else_V:
            B["else_row"] = {k: put(v) for k, v in P.else_row.items()}
            B["else_row_mesh"] = put(P.else_row_mesh)
            B["else_phi"], B["else_params"] = put(P.else_phi), put(P.else_params)
            if P.correction is not None:
                B["correction"] = put(P.correction)
            else:
                # the elsewhere's log T over each hot member's cells, with the
                # hot mesh's effective gravity
                torch = self.torch
                corr = B["params"].clone()
                per = torch.from_numpy(P.else_logT[[m["v"] for m in P.members]])
                counts = torch.tensor([m["S"] * m["S"] for m in P.members])
                corr[:, 0] = torch.repeat_interleave(per, counts).to(self.dev)
                B["correction"] = corr
        self.alloc(P, B)
        return B

    def _gpu_meshes(self, P, B):
        """Build the batch's meshes on the device (xgpu_mesh_batch) into the
        packed row and cell arrays, on torch's current stream."""
        torch = self.torch
        dev, f64, i32 = self.dev, torch.float64, torch.int32
        R, C_ = P.n_rows, P.n_cells
        B["row"] = {k: torch.empty(R, dtype=f64, device=dev)
                    for k in ("u", "r_s", "maxAlpha", "radius", "cos_gamma", "theta0",
                              "lag_C", "lag_scale")}
        B["row_mesh"] = torch.empty(R, dtype=i32, device=dev)
        B["cellArea"] = torch.empty(C_, dtype=f64, device=dev)
        B["phi"] = torch.empty(C_, dtype=f64, device=dev)
        B["params"] = torch.empty((C_, 2), dtype=f64, device=dev)
        B["radiates"] = torch.empty(C_, dtype=i32, device=dev)
        p = lambda x: x.data_ptr()
        row = B["row"]
        o = MeshBatchOut(p(row["u"]), p(row["r_s"]), p(row["maxAlpha"]), p(row["radius"]),
                         p(row["cos_gamma"]), p(row["theta0"]), p(row["lag_C"]),
                         p(row["lag_scale"]), p(B["row_mesh"]), p(B["cellArea"]), p(B["phi"]),
                         p(B["params"]), p(B["radiates"]))
        st = torch.cuda.current_stream(dev).cuda_stream
        check(lib().xgpu_mesh_batch(len(P.mesh_members), P.mesh_members, R, C_, C.byref(o), st))

    def h2d_bytes(self, P: Prepared):
        n = 0
        if P.else_V:
            n += (sum(v.nbytes for v in P.else_row.values()) + P.else_row_mesh.nbytes
                  + P.else_phi.nbytes + P.else_params.nbytes)
            if P.correction is not None:
                n += P.correction.nbytes
            else:
                n += 8 * len(P.members)
        if P.mesh_members is not None:
            return int(n + C.sizeof(P.mesh_members) + P.d_sq.nbytes + P.shifts.nbytes)
        return int(n + sum(v.nbytes for v in P.row.values()) + P.row_mesh.nbytes
                   + P.cellArea.nbytes + P.phi.nbytes + P.params.nbytes + P.radiates.nbytes
                   + P.d_sq.nbytes + P.shifts.nbytes)

    def alloc(self, P, B):
        torch = self.torch
        dev, f64 = self.dev, torch.float64
        n_m = P.V * P.H
        N_E, N_P = len(self.model.energies), self.N_L
        tab = (P.n_rows, self.N_R)
        B["defl"] = torch.empty(tab, dtype=f64, device=dev)
        B["ca"] = torch.empty(tab, dtype=f64, device=dev)
        B["lag"] = torch.empty(tab, dtype=f64, device=dev)
        B["maxDefl"] = torch.empty(P.n_rows, dtype=f64, device=dev)
        B["row_status"] = torch.empty(P.n_rows, dtype=torch.int32, device=dev)
        B["maxAlpha"] = B["row"]["maxAlpha"]
        B["flux"] = torch.empty((n_m, N_E, N_P), dtype=f64, device=dev)
        B["mesh_status"] = torch.empty(n_m, dtype=torch.int32, device=dev)
        B["off_in"] = torch.arange(n_m, dtype=torch.int64, device=dev) * (N_E * N_P)
        B["off_out"] = torch.arange(n_m, dtype=torch.int64, device=dev) * (self.q * N_P)
        B["integrated"] = torch.empty((n_m, self.q, N_P), dtype=f64, device=dev)
        B["folded"] = torch.empty((n_m, self.K, N_P), dtype=f64, device=dev)
        B["chan_ll"] = torch.empty((P.V, self.K), dtype=f64, device=dev)
        B["chan_flag"] = torch.empty((P.V, self.K), dtype=torch.int32, device=dev)
        B["loglike"] = torch.empty(P.V, dtype=f64, device=dev)
        B["status"] = torch.empty(P.V, dtype=torch.int32, device=dev)
        if P.else_V:
            n_er = P.else_V * P.else_S
            etab = (n_er, self.model.elsewhere.num_rays)
            for k in ("else_defl", "else_ca", "else_lag"):
                B[k] = torch.empty(etab, dtype=f64, device=dev)
            B["else_maxDefl"] = torch.empty(n_er, dtype=f64, device=dev)
            B["else_row_status"] = torch.empty(n_er, dtype=torch.int32, device=dev)
            B["else_flux"] = torch.empty((P.else_V, N_E), dtype=f64, device=dev)
            B["else_status"] = torch.empty(P.else_V, dtype=torch.int32, device=dev)
        B["P"] = P

    # ---------------------------------------------------------------- run
    def run(self, B, stream=None, probe=None, likelihood=True):
        """Enqueue the five stages on `stream` (default: torch's current).
        `probe` (optional dict) receives CUDA events around the integrator
        launch and its algorithmic FLOP count (key "flops", a device tensor).
        likelihood=False stops after the response fold (B["folded"])."""
        torch = self.torch
        P = B["P"]
        strm = stream or torch.cuda.current_stream(self.dev)
        st = strm.cuda_stream
        p = lambda x: x.data_ptr()
        L = lib()
        row = B["row"]
        check(L.xgpu_rays_batch(P.n_rows, self.N_R, p(row["u"]), p(row["r_s"]),
                                p(B["maxAlpha"]), p(B["defl"]), p(B["ca"]), p(B["lag"]),
                                p(B["maxDefl"]), p(B["row_status"]), p(row["lag_C"]),
                                p(row["lag_scale"]), st))
        d = IntegrateBatchData()
        d.row_mesh = p(B["row_mesh"])
        d.radius, d.u, d.cos_gamma = p(row["radius"]), p(row["u"]), p(row["cos_gamma"])
        d.theta0, d.maxDeflection = p(row["theta0"]), p(B["maxDefl"])
        d.deflection, d.cos_alpha, d.lag = p(B["defl"]), p(B["ca"]), p(B["lag"])
        d.cellArea, d.phi, d.params = p(B["cellArea"]), p(B["phi"]), p(B["params"])
        d.n_params = 2
        d.radiates = p(B["radiates"])
        d.energies, d.leaves, d.phases = p(self.energies), p(self.leaves), p(self.phases)
        if self.atmos is not None:
            d.atmos = self.atmos
        d.flux = p(B["flux"])
        d.mesh_status = p(B["mesh_status"])
        n_m = P.V * P.H
        N_E, N_P = len(self.model.energies), self.N_L
        if P.else_V:
            er = B["else_row"]
            N_Re = self.model.elsewhere.num_rays
            check(L.xgpu_rays_batch(P.else_V * P.else_S, N_Re, p(er["u"]), p(er["r_s"]),
                                    p(er["maxAlpha"]), p(B["else_defl"]), p(B["else_ca"]),
                                    p(B["else_lag"]), p(B["else_maxDefl"]),
                                    p(B["else_row_status"]), None, None, st))
            d.correction = p(B["correction"])
            d.n_correction = 2
        if probe is not None:
            d.flop_counter = p(probe["flops"])
            probe["start"] = torch.cuda.Event(enable_timing=True)
            probe["end"] = torch.cuda.Event(enable_timing=True)
            probe["start"].record(strm)
        integ = L.xgpu_integrate_batch_mixed if self.precision == "mixed" \
            else L.xgpu_integrate_batch
        check(integ(n_m, P.meshes, P.n_rows, self.N_R, N_E, self.N_L, N_P, C.byref(d),
                    int(self.target_ctas), st))
        if probe is not None:
            probe["end"].record(strm)
        if P.else_V:
            # the time-invariant spectrum of every vector, added to its first
            # hot region's signal (integrator_for_time_invariance.pyx:59-338,
            # Photosphere.py:588-592)
            ed = ElsewhereBatchData()
            ed.row_mesh = p(B["else_row_mesh"])
            ed.radius, ed.u = p(er["radius"]), p(er["u"])
            ed.cos_gamma, ed.theta0 = p(er["cos_gamma"]), p(er["theta0"])
            ed.maxDeflection = p(B["else_maxDefl"])
            ed.deflection, ed.cos_alpha = p(B["else_defl"]), p(B["else_ca"])
            ed.phi, ed.params, ed.n_params = p(B["else_phi"]), p(B["else_params"]), 2
            ed.energies = p(self.energies)
            ed.flux, ed.mesh_status = p(B["else_flux"]), p(B["else_status"])
            ed.signal, ed.signal_stride, ed.signal_N_P = p(B["flux"]), P.H * N_E * N_P, N_P
            check(L.xgpu_elsewhere_batch(P.else_V, P.else_meshes, P.else_V * P.else_S, N_Re,
                                         N_E, 0, C.byref(ed), st))
        check(L.xgpu_energy_batch(n_m, N_E, N_P, self.log10edges.numel(), p(B["flux"]),
                                  p(B["off_in"]), p(self.log10E), p(self.log10edges),
                                  p(B["d_sq"]), p(B["integrated"]), p(B["off_out"]), 0, st))
        if self.precision == "mixed":
            if "fold_status" not in B:
                B["fold_status"] = self.torch.zeros(1, dtype=self.torch.int32, device=self.dev)
            else:
                B["fold_status"].zero_()
            check(L.xgpu_fold_batch_tc(n_m, self.K, self.q, N_P, p(self.matrix), self.q,
                                       p(B["integrated"]), p(B["folded"]), p(B["fold_status"]),
                                       st))
        else:
            check(L.xgpu_fold_batch(n_m, self.K, self.q, N_P, p(self.matrix), self.q,
                                    p(B["integrated"]), p(B["folded"]), st))
        if not likelihood:
            return
        m = self.model
        ld = LikelihoodBatchData()
        ld.n_vec, ld.K, ld.B, ld.H, ld.N_P = P.V, self.K, self.B, P.H, N_P
        ld.exposure, ld.epsabs, ld.epsrel = m.data.exposure, 0.0, m.epsrel
        ld.epsilon, ld.sigmas, ld.llzero, ld.slim = m.epsilon, m.sigmas, m.llzero, m.slim
        ld.phase_edges, ld.comp_phases = p(self.phase_edges), p(self.comp_phases)
        ld.counts, ld.precomp, ld.support = p(self.counts), p(self.precomp), p(self.support)
        ld.background = None
        ld.signals, ld.shifts = p(B["folded"]), p(B["shifts"])
        ld.allow_negative = p(self.allow_negative)
        ld.chan_ll, ld.chan_flag = p(B["chan_ll"]), p(B["chan_flag"])
        ld.star = ld.mcl_bg = ld.mcl_bg_support = None
        ld.loglike, ld.status = p(B["loglike"]), p(B["status"])
        check(L.xgpu_likelihood_batch(C.byref(ld), st))

    def synthesise(self, params, exposure_time, background=None, seed=0, n_threads=0,
                   meshes="gpu"):
        """Synthetic data sets for many parameter vectors in one pass, as
        Signal.synthesise does for one (Signal.py:725-855 with an exposure
        time, tools/synthesise.pyx:35-140): the signal of every vector, its
        expected counts per (channel, phase bin) =
        exposure x (the hot regions' bin-integrated count rates, clamped at
        zero, + `background` count rates [K, B]), and a Poisson realisation
        of each, drawn on the GPU from Philox4x32-10 keyed by `seed` at the
        element's index in the batch.  Returns host arrays (expected
        [V, K, B], counts [V, K, B], status [V]); vectors with a non-zero
        status (ray or integration failure, atmosphere bounds) carry no data
        set."""
        torch = self.torch
        P = prepare(self.model, params, n_threads, meshes=meshes)
        B = self.upload(P)
        self.run(B, likelihood=False)
        p = lambda x: x.data_ptr()
        N_P = self.N_L
        n_m = P.V * P.H
        comps = (Component * n_m)()
        base = p(B["folded"])
        for i in range(n_m):
            comps[i] = Component(base + 8 * i * self.K * N_P, p(self.comp_phases), N_P, N_P,
                                 float(P.shifts[i // P.H, i % P.H]))
        bg = None
        if background is not None:
            bg = torch.as_tensor(np.ascontiguousarray(background, dtype=np.float64),
                                 device=self.dev)
            if tuple(bg.shape) != (self.K, self.B):
                raise ValueError("background must be [channels, phase bins]")
        expec = torch.empty((P.V, self.K, self.B), dtype=torch.float64, device=self.dev)
        counts = torch.empty_like(expec)
        fail = torch.zeros(1, dtype=torch.int32, device=self.dev)
        st = torch.cuda.current_stream(self.dev).cuda_stream
        L = lib()
        check(L.xgpu_expected_counts_batch(P.V, self.K, self.B, P.H, float(exposure_time),
                                           p(self.phase_edges), comps, p(self.allow_negative),
                                           p(bg) if bg is not None else None, p(expec), st))
        check(L.xgpu_poisson_batch(expec.numel(), p(expec), p(counts),
                                   int(seed) & (2 ** 64 - 1), 0, p(fail), st))
        status = self.statuses_no_likelihood(B)
        if int(fail.item()):
            raise RuntimeError("a Poisson draw hit the rejection loop's bound")
        return expec.cpu().numpy(), counts.cpu().numpy(), status

    def statuses_no_likelihood(self, B):
        """Per-vector status of a run stopped after the fold (ray, pulse,
        atmosphere and elsewhere failures)."""
        B["status"].zero_()
        return self.statuses(B)

    def statuses(self, B):
        """Per-vector status word (ray, pulse, atmosphere, quadrature, slim)."""
        torch = self.torch
        P = B["P"]
        st = B["status"].cpu().numpy().copy()
        rs = B["row_status"].cpu().numpy()
        ms = B["mesh_status"].cpu().numpy()
        rm = B["row_mesh"].cpu().numpy()
        vec_of_mesh = np.repeat(np.arange(P.V), P.H)
        bad_rows = np.unique(rm[rs != 0])
        for mi in bad_rows:
            st[vec_of_mesh[mi]] = 1
        for mi in np.nonzero(ms)[0]:
            if st[vec_of_mesh[mi]] == 0:
                st[vec_of_mesh[mi]] = 2
        if P.else_V:
            ers = B["else_row_status"].cpu().numpy()
            erm = B["else_row_mesh"].cpu().numpy()
            est = B["else_status"].cpu().numpy()
            for v in np.unique(erm[ers != 0]):
                st[v] = 1
            for v in np.nonzero(est)[0]:
                if st[v] == 0:
                    st[v] = 7
        if "fold_status" in B and int(B["fold_status"].item()) != 0:
            # a bounded wait in the tensor-core fold ran out: every vector's
            # folded signal is void
            st[st == 0] = 8
        st[P.status != 0] = P.status[P.status != 0]
        return st

    def loglikelihood_pipelined(self, batches, n_threads=0, meshes="gpu", depth=3):
        """log L and statuses of a sequence of parameter batches, yielded in
        order, with up to `depth` batches in flight on separate CUDA streams:
        batch i+1's host preparation, copies and GPU mesh build overlap batch
        i's stages.  Each yielded pair is as loglikelihood() returns."""
        from collections import deque
        torch = self.torch
        streams = [torch.cuda.Stream(device=self.dev) for _ in range(max(1, int(depth)))]
        inflight = deque()
        for i, params in enumerate(batches):
            s = streams[i % len(streams)]
            P = prepare(self.model, params, n_threads, meshes=meshes)
            with torch.cuda.stream(s):
                B = self.upload(P, pinned=True)
                self.run(B, stream=s)
                ll = torch.empty(P.V, dtype=torch.float64, pin_memory=True)
                ll.copy_(B["loglike"], non_blocking=True)
                done = torch.cuda.Event()
                done.record(s)
            inflight.append((done, B, ll))
            if len(inflight) >= len(streams):
                yield self._finish(*inflight.popleft())
        while inflight:
            yield self._finish(*inflight.popleft())

    def _finish(self, done, B, ll):
        done.synchronize()
        ll = ll.numpy().copy()
        st = self.statuses(B)
        bad = st != 0
        if bad.any():
            rng = np.random.default_rng(12345)
            ll[bad] = self.model.llzero * (0.1 + 0.9 * rng.random(int(bad.sum())))
        return ll, st

    def loglikelihood(self, params, n_threads=0, meshes="gpu"):
        """log L of every parameter vector (host in, host out) and statuses.
        Vectors whose status is not 0 get a value near llzero, as
        Likelihood.random_near_llzero does (Likelihood.py:268-271).  The
        meshes are built on the GPU unless meshes="host"."""
        P = prepare(self.model, params, n_threads, meshes=meshes)
        B = self.upload(P)
        self.run(B)
        ll = B["loglike"].cpu().numpy().copy()
        st = self.statuses(B)
        bad = st != 0
        if bad.any():
            rng = np.random.default_rng(12345)
            ll[bad] = self.model.llzero * (0.1 + 0.9 * rng.random(int(bad.sum())))
        return ll, st


def concat_prepared(parts, model: Model) -> Prepared:
    """One packed batch from several prepared batches of the same model
    (offsets re-based; no mesh is rebuilt)."""
    if len(parts) == 1:
        return parts[0]
    N_E, N_P = len(model.energies), model.regions[0].num_leaves
    gpu = parts[0].mesh_members is not None
    if any((p.mesh_members is not None) != gpu for p in parts):
        raise ValueError("cannot merge host-meshed and GPU-meshed batches")
    P = Prepared()
    P.H = parts[0].H
    P.V = sum(p.V for p in parts)
    P.n_rows = sum(p.n_rows for p in parts)
    P.n_cells = sum(p.n_cells for p in parts)
    P.status = np.concatenate([p.status for p in parts])
    if gpu:
        P.row = None
    else:
        P.row = {k: np.concatenate([p.row[k] for p in parts]) for k in parts[0].row}
        P.cellArea = np.concatenate([p.cellArea for p in parts])
        P.phi = np.concatenate([p.phi for p in parts])
        P.params = np.concatenate([p.params for p in parts])
        P.radiates = np.concatenate([p.radiates for p in parts])
    P.d_sq = np.concatenate([p.d_sq for p in parts])
    P.shifts = np.concatenate([p.shifts for p in parts])
    n_m = sum(len(p.meshes) for p in parts)
    P.meshes = (Mesh * n_m)()
    P.mesh_members = (MeshMember * n_m)() if gpu else None
    rm, members = [], []
    ro = co = mo = vb = 0
    for p in parts:
        for i in range(len(p.meshes)):
            q = p.meshes[i]
            P.meshes[mo + i] = Mesh(q.S0, q.S1, q.row_off + ro, q.cell_off + co, q.omega,
                                    q.inclination, q.image_order_limit, q.atm_ext,
                                    (mo + i) * N_E * N_P)
            if gpu:
                mm = MeshMember()
                C.memmove(C.byref(mm), C.byref(p.mesh_members[i]), C.sizeof(MeshMember))
                mm.row_off += ro
                mm.cell_off += co
                P.mesh_members[mo + i] = mm
        if not gpu:
            rm.append(p.row_mesh + mo)
        members += [dict(m, v=m["v"] + vb) for m in p.members]
        vb += p.V
        ro += p.n_rows
        co += p.n_cells
        mo += len(p.meshes)
    if not gpu:
        P.row_mesh = np.concatenate(rm).astype(np.int32)
    P.members = members
    P.else_V = sum(p.else_V for p in parts)
    if P.else_V:
        _concat_elsewhere(P, parts)
    return P


def _concat_elsewhere(P, parts):
    S = parts[0].else_S
    P.else_S = S
    P.else_logT = np.concatenate([p.else_logT for p in parts])
    P.else_row = {k: np.concatenate([p.else_row[k] for p in parts]) for k in parts[0].else_row}
    P.else_row_mesh = np.repeat(np.arange(P.else_V, dtype=np.int32), S)
    P.else_phi = np.concatenate([p.else_phi for p in parts])
    P.else_params = np.concatenate([p.else_params for p in parts])
    P.else_meshes = (ElsewhereMesh * P.else_V)()
    v0 = 0
    for p in parts:
        for i in range(p.else_V):
            q = p.else_meshes[i]
            P.else_meshes[v0 + i] = ElsewhereMesh(q.S, (v0 + i) * S, (v0 + i) * S * S, q.omega,
                                                  q.inclination, q.cellArea,
                                                  q.image_order_limit, q.atm_ext)
        v0 += p.else_V
    if all(p.correction is not None for p in parts):
        P.correction = np.concatenate([p.correction for p in parts])
    else:
        P.correction = None
