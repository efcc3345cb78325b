"""Host side of the batched path with an elsewhere: parameter layout, the
packed closed meshes and correction vectors, and batch concatenation.  CPU
only (the closed meshes are host C++; no CUDA call)."""
import numpy as np
import pytest

from xpsi_gb300 import batch as BT
from xpsi_gb300.cellmesh import global_mesh as G


@pytest.fixture(scope="module")
def case():
    from batch_cases import small_elsewhere
    return small_elsewhere(V=3)


def test_param_names_end_with_elsewhere_temperature(case):
    m, params = case
    names = BT.param_names(m)
    assert names[-1] == "elsewhere_temperature"
    assert params.shape[1] == len(names)


def test_packed_closed_meshes(case):
    m, params = case
    P = BT.prepare(m, params)
    S = m.elsewhere.sqrt_num_cells
    assert P.else_V == 3 and P.else_S == S
    for v in range(P.V):
        M = P.else_meshes[v]
        assert (M.S, M.row_off, M.cell_off, M.atm_ext) == (S, v * S, v * S * S, 1)
        R = params[v, 1] * 1e3
        r_g = params[v, 0] * BT._GM
        Mkg = params[v, 0] * BT._GM * BT._CSQ / BT._G
        Om = 2 * np.pi * params[v, 2]
        th, ph, r, cA, ma, cg, g = G.construct_closed_cellMesh(
            1, S, S * S, Mkg, 2 * r_g, R, r_g / R, Om ** 2 * R ** 3 / (BT._G * Mkg), 0)
        sl = slice(v * S, (v + 1) * S)
        np.testing.assert_array_equal(P.else_row["radius"][sl], r)
        np.testing.assert_array_equal(P.else_row["theta0"][sl], th[:, 0])
        np.testing.assert_array_equal(P.else_row["maxAlpha"][sl], ma)
        assert M.cellArea == cA
        cs = slice(v * S * S, (v + 1) * S * S)
        np.testing.assert_array_equal(P.else_phi[cs], ph.reshape(-1))
        prm = P.else_params[cs].reshape(S, S, 2)
        assert np.all(prm[..., 0] == params[v, -1])
        np.testing.assert_array_equal(prm[:, 0, 1], g)


def test_correction_vectors(case):
    m, params = case
    P = BT.prepare(m, params)
    c0 = 0
    for mem in P.members:
        n = mem["S"] ** 2
        cs = slice(c0, c0 + n)
        assert np.all(P.correction[cs, 0] == params[mem["v"], -1])
        np.testing.assert_array_equal(P.correction[cs, 1], P.params[cs, 1])
        c0 += n


def test_concat_matches_one_prepare(case):
    m, params = case
    whole = BT.prepare(m, params)
    parts = BT.concat_prepared([BT.prepare(m, params[:1]), BT.prepare(m, params[1:])], m)
    for k in whole.else_row:
        np.testing.assert_array_equal(parts.else_row[k], whole.else_row[k])
    np.testing.assert_array_equal(parts.else_row_mesh, whole.else_row_mesh)
    np.testing.assert_array_equal(parts.else_params, whole.else_params)
    np.testing.assert_array_equal(parts.correction, whole.correction)
    for v in range(whole.V):
        a, b = parts.else_meshes[v], whole.else_meshes[v]
        assert (a.S, a.row_off, a.cell_off, a.cellArea) == (b.S, b.row_off, b.cell_off,
                                                           b.cellArea)
    assert [mm["v"] for mm in parts.members] == [mm["v"] for mm in whole.members]


def test_numerical_elsewhere_not_batched():
    with pytest.raises(NotImplementedError):
        BT.ElsewhereSpec(atm_ext=2) and BT.Model(
            regions=[BT.HotRegionSpec()], instrument=BT.Instrument(np.eye(2), np.arange(3.0)),
            data=BT.Data(np.zeros((2, 2), np.int32), np.linspace(0, 1, 3), 1.0),
            elsewhere=BT.ElsewhereSpec(atm_ext=2))
