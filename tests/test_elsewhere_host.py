"""The photosphere elsewhere on the host: the oracle's time-invariant
integrator and the native library's closed mesh against the reference's own
outputs (tests/golden/elsewhere.npz, made by tests/golden/make_fixtures.py).
CPU only: the closed mesh is host C++, no CUDA call is made."""
import numpy as np
import pytest

from conftest import ELSEWHERE_CASES, elsewhere_args, elsewhere_atmos, spectrum_rel
from oracle import oracle as O


@pytest.mark.parametrize("case", ELSEWHERE_CASES)
@pytest.mark.parametrize("threads", [1, 4])
def test_oracle_time_invariant_vs_reference(golden, case, threads):
    """integrator_for_time_invariance.pyx:59-338; with 4 threads the
    oracle keeps the reference's per-thread Num4D stencil state too."""
    f = golden("elsewhere")
    st, flux = O.integrate_time_invariant(
        *elsewhere_args(f, case, elsewhere_atmos(golden, case), threads=threads))
    assert st == 0
    assert spectrum_rel(flux, f["%s_flux_threads%d" % (case, threads)]) <= 1e-13


def test_closed_mesh_vs_reference(golden):
    """global_mesh.pyx:21-137 through the C ABI's host builder."""
    from xpsi_gb300.cellmesh.global_mesh import construct_closed_cellMesh
    f = golden("elsewhere")
    S = int(f["S"])
    th, ph, r, cA, ma, cg, g = construct_closed_cellMesh(
        1, S, S * S, float(f["mass"]), float(f["r_s"]), float(f["R"]), float(f["zeta"]),
        float(f["epsilon"]), int(f["star_shape_ind"]))
    np.testing.assert_allclose(th, f["theta"], rtol=1e-13, atol=0)
    np.testing.assert_array_equal(ph, f["phi"])
    np.testing.assert_allclose(r, f["radius"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(ma, f["maxAlpha_in"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(cg, f["cos_gamma"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(g, f["effGrav"], rtol=1e-13, atol=0)
    assert abs(cA / float(f["cellArea"]) - 1.0) <= 1e-13


def test_closed_mesh_many_matches_single(golden):
    from xpsi_gb300.cellmesh import global_mesh as G
    f = golden("elsewhere")
    reqs = []
    for S, shape in ((10, 0), (24, 0), (16, 1)):
        reqs.append(dict(S=S, num_cells=S * S, R_eq=float(f["R"]), zeta=float(f["zeta"]),
                         epsilon=float(f["epsilon"]), star_shape_ind=shape))
    G.build_many(reqs, n_threads=3)
    for q in reqs:
        one = G.construct_closed_cellMesh(1, q["S"], q["num_cells"], 0.0, 0.0, q["R_eq"],
                                          q["zeta"], q["epsilon"], q["star_shape_ind"])
        for k, v in zip(("theta", "phi", "r", "cellArea", "maxAlpha", "cos_gamma", "effGrav"),
                        one):
            np.testing.assert_array_equal(q[k], v)
        # the southern hemisphere mirrors the northern one
        S = q["S"]
        np.testing.assert_allclose(q["theta"][::-1, 0], np.pi - q["theta"][:, 0], rtol=0,
                                   atol=1e-15)
        np.testing.assert_array_equal(q["r"][::-1], q["r"])


@pytest.mark.parametrize("S", [0, 3, 7])
def test_closed_mesh_rejects_odd_sizes(S):
    from xpsi_gb300.cellmesh.global_mesh import construct_closed_cellMesh
    with pytest.raises(ValueError):
        construct_closed_cellMesh(1, S, S * S, 1.0, 1.0, 1.2e4, 0.1, 0.1, 0)


def _corrected_args(f, corr, atmos):
    return (1, float(f["R"]), float(f["Omega"]), float(f["r_s"]), float(f["inclination"]),
            f["cellArea"], f["radius"], f["u"], f["theta"], f["phi"], f["params"],
            f["radiates"], corr, int(f["N_R"]), f["deflection"], f["cos_alpha"], f["lag"],
            f["maxDeflection"], f["cos_gamma"], f["energies"], f["leaves"], f["phases"],
            atmos, None, int(f["atm_ext"]), 1, 0, int(f["image_order_limit"]) or None)


@pytest.mark.parametrize("case", ["config1", "num4d_omit"])
def test_oracle_corrected_integrator_vs_reference(golden, case):
    """The hot-region integrator with a blackbody elsewhere's correction
    (integrator_for_azimuthal_invariance.pyx:257-261,469-478,593-594)."""
    from conftest import atmos_of, row_rel
    f = golden(case)
    c = golden("elsewhere_correction")
    atmos = atmos_of(f) if int(f["atm_ext"]) == 2 else ()
    st, flux = O.integrate(*_corrected_args(f, c[case + "_correction"], atmos))
    assert st == 0
    assert row_rel(flux, c[case + "_flux"]) <= 1e-13
