"""The host mesh builder (the drop-in cell budget and spot / polar-cap mesh
functions) against the reference's own meshes at the full-size resolution:
the members of the full-size parity test's prior vectors (polar caps on
either member, omitted crescents) and three hand-set members
(tests/golden/meshes.npz, written by make_fixtures.py from
mesh_tools.allocate_cells, mesh.construct_spot_cellMesh and
polar_mesh.construct_polar_cellMesh).  CPU only."""
import math

import numpy as np
import pytest

from conftest import load_golden
from xpsi_gb300.cellmesh import mesh as MESH

# xpsi/global_imports.py:68-79
_GM, _C, _G = 0.5 * 2.95325024e3, 2.99792458e8, 6.6740831e-11
_CSQ = _C * _C


def star(M_sun, R_km, f_hz):
    """Spacetime derived quantities (Spacetime.py:110-187): M in kg, r_s,
    R, Omega, zeta, epsilon."""
    r_g = M_sun * _GM
    R = R_km * 1.0e3
    Mkg = M_sun * _GM * _CSQ / _G
    Om = 2.0 * math.pi * f_hz
    return Mkg, 2.0 * r_g, R, Om, r_g / R, Om ** 2 * R ** 3 / (_G * Mkg)


def fixture_members():
    f = load_golden("meshes")
    return f, int(f["n_members"])


def check_mesh(f, k, th, ph, r, A, ma, cg, g):
    """Mesh k of the fixture against arrays (th, ph per row / column)."""
    np.testing.assert_allclose(A, f[f"m{k}_cellArea"], rtol=1e-12,
                               atol=1e-12 * np.max(f[f"m{k}_cellArea"]))
    assert np.array_equal(A > 0.0, f[f"m{k}_cellArea"] > 0.0)
    # the cell colatitudes are quadratures (relative 1e-8 requested of CQUAD,
    # whose stand-in here converges far tighter): 3e-13 is the largest
    # deviation seen
    np.testing.assert_allclose(th, f[f"m{k}_theta"], rtol=1e-12)
    np.testing.assert_allclose(ph, f[f"m{k}_phi"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(r, f[f"m{k}_radius"], rtol=1e-13)
    np.testing.assert_allclose(cg, f[f"m{k}_cos_gamma"], rtol=1e-13)
    np.testing.assert_allclose(ma, f[f"m{k}_maxAlpha"], rtol=1e-13)
    np.testing.assert_allclose(g, f[f"m{k}_effGrav"], rtol=1e-13)


def test_fixture_covers_polar_caps_and_omits():
    f, n = fixture_members()
    polar = [int(f[f"m{k}_polar"]) for k in range(n)]
    assert sum(polar) >= 6
    mem = f["members"]
    assert any(polar[k] and mem[k, 5] > 0.0 for k in range(n))  # polar cap with a hole
    assert any(mem[k, 3] > math.pi / 2 and polar[k] for k in range(n))  # south cap


@pytest.mark.parametrize("k", range(21))
def test_host_mesh_vs_reference(k):
    f, n = fixture_members()
    if k >= n:
        pytest.skip("fixture has fewer members")
    M_sun, R_km, f_hz, colat, rad, o_r, o_c, o_a = f["members"][k]
    Mkg, r_s, R, Om, zeta, eps = star(M_sun, R_km, f_hz)
    S, N, _, _ = MESH.allocate_cells(64 ** 2, 10, 128, Mkg, r_s, R, Om, zeta, eps, 0, rad, 0.0,
                                     colat, colat, -0.0, o_c, o_r, o_a)
    assert int(S) == int(f[f"m{k}_S"]) and int(N) == int(f[f"m{k}_num_cells"])
    polar = colat - rad < 0.0 or colat + rad > math.pi
    assert int(polar) == int(f[f"m{k}_polar"])
    fn = MESH.construct_polar_cellMesh if polar else MESH.construct_spot_cellMesh
    th, ph, r, A, ma, cg, g = fn(1, int(N), int(S), Mkg, r_s, R, zeta, eps, 0, rad, colat, o_r,
                                 o_c, o_a)
    check_mesh(f, k, th[:, 0], ph[0, :], r, A, ma, cg, g)


@pytest.mark.parametrize("k", range(21))
def test_oracle_mesh_bit_exact_vs_reference(k):
    """The oracle's own mesh restatement (oracle/xpsi_oracle_mesh.c) runs the
    same floating-point steps through the same GSL-API subset as the
    reference's build: its cell budgets and meshes are bit-identical, on 1
    and on 4 threads."""
    from oracle import oracle as O
    f, n = fixture_members()
    if k >= n:
        pytest.skip("fixture has fewer members")
    M_sun, R_km, f_hz, colat, rad, o_r, o_c, o_a = f["members"][k]
    Mkg, r_s, R, Om, zeta, eps = star(M_sun, R_km, f_hz)
    S, N, cs, cn = O.allocate_cells(64 ** 2, 10, 128, Mkg, r_s, R, Om, zeta, eps, 0, rad, 0.0,
                                    colat, colat, -0.0, o_c, o_r, o_a)
    assert (S, N) == (float(f[f"m{k}_S"]), float(f[f"m{k}_num_cells"])) and (cs, cn) == (0, 0)
    polar = colat - rad < 0.0 or colat + rad > math.pi
    fn = O.construct_polar_cellMesh if polar else O.construct_spot_cellMesh
    for nt in (1, 4):
        th, ph, r, A, ma, cg, g = fn(nt, int(N), int(S), Mkg, r_s, R, zeta, eps, 0, rad, colat,
                                     o_r, o_c, o_a)
        for got, key in ((A, "cellArea"), (th[:, 0], "theta"), (ph[0], "phi"), (r, "radius"),
                         (ma, "maxAlpha"), (cg, "cos_gamma"), (g, "effGrav")):
            np.testing.assert_array_equal(got, f[f"m{k}_{key}"], err_msg=key)


def test_oracle_closed_mesh_bit_exact_vs_reference():
    """global_mesh.construct_closed_cellMesh of the elsewhere fixture."""
    from oracle import oracle as O
    f = load_golden("elsewhere")
    S = int(f["S"])
    th, ph, r, A, ma, cg, g = O.construct_closed_cellMesh(
        4, S, S * S, float(f["mass"]), float(f["r_s"]), float(f["R"]), float(f["zeta"]),
        float(f["epsilon"]), int(f["star_shape_ind"]))
    np.testing.assert_array_equal(th, f["theta"])
    np.testing.assert_array_equal(ph, f["phi"])
    np.testing.assert_array_equal(r, f["radius"])
    assert A == float(f["cellArea"])
    np.testing.assert_array_equal(ma, f["maxAlpha_in"])
    np.testing.assert_array_equal(cg, f["cos_gamma"])
    np.testing.assert_array_equal(g, f["effGrav"])
