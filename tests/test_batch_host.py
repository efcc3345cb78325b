"""Host-side logic of the batched path: packing of meshes into the flat
layout the kernels read, atmosphere-bounds statuses, and the mesh builder
against the reference's meshes.  CPU only."""
import math

import numpy as np

from batch_cases import small_num4d
from conftest import load_golden
from xpsi_gb300 import batch as BT
from xpsi_gb300 import synthetic as SY
from xpsi_gb300.cellmesh import mesh as MESH


def test_packing_offsets():
    m, params = small_num4d(V=3)
    P = BT.prepare(m, params)
    assert P.V == 3 and P.H == 2
    ro = co = 0
    for i in range(P.V * P.H):
        mesh = P.meshes[i]
        assert mesh.row_off == ro and mesh.cell_off == co
        assert mesh.flux_off == i * len(m.energies) * m.regions[0].num_leaves
        assert (P.row_mesh[ro:ro + mesh.S0] == i).all()
        ro += mesh.S0
        co += mesh.S0 * mesh.S1
    assert ro == P.n_rows and co == P.n_cells
    assert np.array_equal(P.radiates, (P.cellArea > 0).astype(np.int32))


def test_atmosphere_bounds_status():
    m = SY.config2_model(K=20, q=8, num_energies=8, sqrt_num_cells=8, num_leaves=8,
                         num_rays=16, max_sqrt_num_cells=16, table_shape=(6, 5, 6, 8))
    rng = np.random.default_rng(3)
    v = np.array(SY.prior_vector(rng))
    v[7] = 7.5  # log T of the first region above the table
    P = BT.prepare(m, v[None, :])
    assert P.status[0] == 3


def test_mesh_builder_vs_reference_fixtures():
    for case in ("examples_fast", "num4d_omit", "config1"):
        f = load_golden(case)
        if "S" not in f:
            continue
        S = int(f["S"])
        assert f["cellArea"].shape == (S, S)
    f = load_golden("num4d_omit")
    # the reference mesh of this fixture: M 1.6, R 14 km, 600 Hz, spot 1.2/0.3,
    # omit (0.12, 1.25, 0.1)
    _GM, _C, _G = 0.5 * 2.95325024e3, 2.99792458e8, 6.6740831e-11
    r_g = 1.6 * _GM
    R = 14e3
    Mkg = 1.6 * _GM * _C * _C / _G
    Om = 2 * math.pi * 600.0
    zeta, eps = r_g / R, Om ** 2 * R ** 3 / (_G * Mkg)
    S = int(f["S"])
    a = MESH.allocate_cells(400, 10, 40, Mkg, 2 * r_g, R, Om, zeta, eps, 0, 0.3, 0.0, 1.2, 1.2,
                            -0.0, 1.25, 0.12, 0.1)
    assert int(a[0]) == S
    th, ph, r, A, ma, cg, g = MESH.construct_spot_cellMesh(1, int(a[1]), S, Mkg, 2 * r_g, R,
                                                           zeta, eps, 0, 0.3, 1.2, 0.12, 1.25,
                                                           0.1)
    np.testing.assert_allclose(A, f["cellArea"], rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(th, f["theta"], rtol=1e-13)
    np.testing.assert_allclose(ph - 0.1, f["phi"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(r, f["radius"], rtol=1e-14)
    np.testing.assert_allclose(cg, f["cos_gamma"], rtol=1e-14)
    np.testing.assert_allclose(ma, f["maxAlpha_in"], rtol=1e-14)


def test_allocate_cells_drop_in_matches_reference_types():
    """The drop-in cell budget returns the reference's values and types."""
    from oracle import ref_harness as H
    if not H.available():
        import pytest
        pytest.skip("reference checkout not present")
    H.load()
    import xpsi.cellmesh.mesh_tools as MT
    from xpsi_gb300.cellmesh import mesh as M
    for cede in (0.0, 0.35):
        args = (400, 10, 40, 2.8e30, 4136.0, 12000.0, 2 * 3.14159 * 300, 0.2, 0.05, 0, 0.3,
                cede, 1.2, 1.25, 0.0, 0.0, 0.0, 0.0)
        ref = MT.allocate_cells(*args)
        ours = M.allocate_cells(*args)
        assert ours == ref
        assert [type(x) for x in ours] == [type(x) for x in ref]
