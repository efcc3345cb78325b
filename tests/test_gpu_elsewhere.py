"""The photosphere elsewhere on the GPU (through the C ABI): the
time-invariant integrator against the reference's own spectra and against
the oracle on variations of the fixture's geometry.  FP64 throughout; the
only difference from the reference is the order of the final sum over
parallels, so the bar is 1e-12 relative per energy."""
import ctypes as C
import math

import numpy as np
import pytest

from conftest import ELSEWHERE_CASES, elsewhere_args, elsewhere_atmos, spectrum_rel
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.fixture(scope="module")
def tinv():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import xpsi_gb300
    xpsi_gb300.lib()
    from xpsi_gb300.cellmesh import integrator_for_time_invariance
    return integrator_for_time_invariance


@pytest.mark.parametrize("case", ELSEWHERE_CASES)
def test_time_invariant_vs_reference(tinv, golden, case):
    f = golden("elsewhere")
    st, flux = tinv.integrate(*elsewhere_args(f, case, elsewhere_atmos(golden, case)))
    assert st == 0
    assert spectrum_rel(flux, f[case + "_flux_threads1"]) <= RTOL


@pytest.mark.parametrize("case", ELSEWHERE_CASES)
@pytest.mark.parametrize("image_order_limit,inclination,omega", [
    (1, None, None), (2, None, None), (None, 0.15, None), (None, 2.9, None),
    (None, math.pi / 2, 2 * math.pi * 716.0), (None, 1.0, 0.0)])
def test_time_invariant_vs_oracle(tinv, golden, case, image_order_limit, inclination, omega):
    """Image-order limits, observers near either pole (whole hemispheres of
    parallels without a visible cell: the Num4D call history then crosses
    them), an equatorial observer at 716 Hz and a static star."""
    f = golden("elsewhere")
    args = elsewhere_args(f, case, elsewhere_atmos(golden, case),
                          image_order_limit=image_order_limit, inclination=inclination,
                          omega=omega)
    st_o, ref = O.integrate_time_invariant(*args)
    st, flux = tinv.integrate(*args)
    assert st == st_o == 0
    assert spectrum_rel(flux, ref) <= RTOL


def test_time_invariant_bitwise_reproducible(tinv, golden):
    f = golden("elsewhere")
    args = elsewhere_args(f, "num4d_mu09", elsewhere_atmos(golden, "num4d_mu09"))
    a = tinv.integrate(*args)[1]
    b = tinv.integrate(*args)[1]
    np.testing.assert_array_equal(a, b)


def test_user_extension_not_silently_replaced(tinv, golden):
    f = golden("elsewhere")
    args = list(elsewhere_args(f, "bb", ()))
    args[19] = 3
    with pytest.raises(NotImplementedError):
        tinv.integrate(*args)


def test_elsewhere_batch_matches_single_calls(tinv, golden):
    """Three closed meshes (two sizes, both atmospheres) in one batched
    launch give the drop-in's spectra bit for bit."""
    import torch
    from xpsi_gb300 import _native as N
    from xpsi_gb300.cellmesh.global_mesh import construct_closed_cellMesh
    from xpsi_gb300.cellmesh.rays import compute_rays
    f = golden("elsewhere")
    atm = elsewhere_atmos(golden, "num4d")
    E = f["energies"]
    N_R = 128
    specs = []
    for S, ext, incl in ((12, 1, 0.7), (16, 2, 1.1), (12, 2, 2.4)):
        th, ph, r, cA, ma, cg, g = construct_closed_cellMesh(
            1, S, S * S, float(f["mass"]), float(f["r_s"]), float(f["R"]), float(f["zeta"]),
            float(f["epsilon"]), 0)
        u = np.ascontiguousarray(float(f["r_s"]) / r)
        t, D, CA, L, MD = compute_rays(1, S, float(f["r_s"]), u, ma, N_R)
        assert t == 0
        params = np.ones((S, S, 2))
        params[..., 0] = 6.1
        params[..., 1] = g[:, None]
        single = tinv.integrate(1, float(f["R"]), float(f["Omega"]), float(f["r_s"]), incl, S,
                                cA, r, u, th, ph, params, N_R, D, CA, MD, cg, E,
                                atm if ext == 2 else (), ext, None)
        assert single[0] == 0
        specs.append(dict(S=S, ext=ext, incl=incl, th=th, ph=ph, r=r, cA=cA, cg=cg, u=u, D=D,
                          CA=CA, MD=MD, params=params, flux=single[1]))
    dev = torch.device("cuda")
    cat = lambda key: torch.tensor(np.concatenate([np.ravel(s[key]) for s in specs]),
                                   device=dev, dtype=torch.float64)
    rows = sum(s["S"] for s in specs)
    meshes = (N.ElsewhereMesh * len(specs))()
    row_off = cell_off = 0
    row_mesh = []
    for m, s in enumerate(specs):
        meshes[m] = N.ElsewhereMesh(s["S"], row_off, cell_off, float(f["Omega"]), s["incl"],
                                    s["cA"], 0, s["ext"])
        row_mesh += [m] * s["S"]
        row_off += s["S"]
        cell_off += s["S"] ** 2
    t_rm = torch.tensor(row_mesh, dtype=torch.int32, device=dev)
    theta0 = torch.tensor(np.concatenate([s["th"][:, 0] for s in specs]), device=dev,
                          dtype=torch.float64)
    bufs = dict(radius=cat("r"), u=cat("u"), cg=cat("cg"), MD=cat("MD"), D=cat("D"),
                CA=cat("CA"), ph=cat("ph"), params=cat("params"))
    tE = torch.tensor(E, device=dev, dtype=torch.float64)
    tatm = [torch.tensor(np.ascontiguousarray(a), device=dev, dtype=torch.float64) for a in atm]
    flux = torch.zeros(len(specs), E.size, device=dev, dtype=torch.float64)
    status = torch.full((len(specs),), -1, device=dev, dtype=torch.int32)
    d = N.ElsewhereBatchData(
        t_rm.data_ptr(), bufs["radius"].data_ptr(), bufs["u"].data_ptr(), bufs["cg"].data_ptr(),
        theta0.data_ptr(), bufs["MD"].data_ptr(), bufs["D"].data_ptr(), bufs["CA"].data_ptr(),
        bufs["ph"].data_ptr(), bufs["params"].data_ptr(), 2, tE.data_ptr(),
        N.Atmos4D(*(t.data_ptr() for t in tatm), tatm[0].numel(), tatm[1].numel(),
                  tatm[2].numel(), tatm[3].numel(), None),
        flux.data_ptr(), status.data_ptr())
    stream = torch.cuda.current_stream().cuda_stream
    N.check(N.lib().xgpu_elsewhere_batch(len(specs), meshes, rows, N_R, E.size, 0,
                                         C.byref(d), C.c_void_p(stream)))
    torch.cuda.synchronize()
    assert status.cpu().tolist() == [0, 0, 0]
    out = flux.cpu().numpy()
    for m, s in enumerate(specs):
        np.testing.assert_array_equal(out[m], s["flux"])


@pytest.mark.parametrize("case", ["config1", "num4d_omit"])
def test_corrected_integrator_vs_reference(tinv, golden, case):
    """The hot-region integrator with a blackbody elsewhere's correction
    against the reference; 1e-9 relative to each energy row's largest value,
    the bar of the uncorrected integrator."""
    from conftest import atmos_of, row_rel
    from test_elsewhere_host import _corrected_args
    from xpsi_gb300.cellmesh import integrator_for_azimuthal_invariance as integ
    f = golden(case)
    c = golden("elsewhere_correction")
    atmos = atmos_of(f) if int(f["atm_ext"]) == 2 else ()
    st, flux = integ.integrate(*_corrected_args(f, c[case + "_correction"], atmos))
    assert st == 0
    assert row_rel(flux, c[case + "_flux"]) <= 1e-9
    # the negative values the correction leaves are summed, not dropped
    if case == "num4d_omit":
        assert flux.min() < 0.0


def test_corrected_integrator_rejects_num4d_elsewhere(tinv, golden):
    from test_elsewhere_host import _corrected_args
    from xpsi_gb300.cellmesh import integrator_for_azimuthal_invariance as integ
    f = golden("config1")
    c = golden("elsewhere_correction")
    args = list(_corrected_args(f, c["config1_correction"], ()))
    args[25] = 2
    with pytest.raises(NotImplementedError):
        integ.integrate(*args)


@pytest.mark.parametrize("num4d", [False, True])
@pytest.mark.parametrize("meshes", ["host", "gpu"])
def test_batch_with_elsewhere_vs_oracle(tinv, num4d, meshes):
    """The batched likelihood of a hot region plus a blackbody elsewhere
    against the oracle pipeline on the same packed inputs: the corrected hot
    signal with the spectrum added (1e-9 per energy row) and log L (1e-7)."""
    import torch
    from batch_cases import small_elsewhere
    from conftest import row_rel
    from oracle import pipeline as OP
    from xpsi_gb300 import batch as BT
    m, params = small_elsewhere(V=3, num4d=num4d)
    P_host = BT.prepare(m, params)
    ref, ref_st, stages = OP.loglike(m, P_host, return_stages=True)
    ev = BT.BatchEvaluator(m)
    P = BT.prepare(m, params, meshes=meshes)
    B = ev.upload(P)
    ev.run(B)
    torch.cuda.synchronize()
    st = ev.statuses(B)
    np.testing.assert_array_equal(st, ref_st)
    ok = st == 0
    assert ok.all()
    ll = B["loglike"].cpu().numpy()
    assert np.max(np.abs(ll - ref)) <= 1e-7
    flux = B["flux"].cpu().numpy()
    for v in range(P.V):
        assert row_rel(flux[v], stages[v]["flux"]) <= 1e-9


def test_batch_with_elsewhere_rejects_mixed(tinv):
    from batch_cases import small_elsewhere
    from xpsi_gb300 import batch as BT
    m, _ = small_elsewhere(V=1)
    with pytest.raises(NotImplementedError):
        BT.BatchEvaluator(m, precision="mixed")
