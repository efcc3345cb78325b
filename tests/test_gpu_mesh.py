"""Meshes built on the GPU (xgpu_mesh_batch) against the host builder on the
same batch: the packed row and cell arrays agree to round-off (the two
builders run the same steps; the device's trigonometric functions may
differ from the host's in the last bit), and the log-likelihoods agree."""
import numpy as np
import pytest

from xpsi_gb300 import batch as BT
from xpsi_gb300 import synthetic as SY

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _both(cuda, model, params):
    ev = BT.BatchEvaluator(model)
    Ph = BT.prepare(model, params, meshes="host")
    Pg = BT.prepare(model, params, meshes="gpu")
    Bh, Bg = ev.upload(Ph), ev.upload(Pg)
    cuda.cuda.synchronize()
    return ev, Ph, Pg, Bh, Bg


def test_gpu_meshes_match_host_meshes(cuda):
    model = SY.config2_model()
    params = SY.config3_vectors(12, seed=11)
    ev, Ph, Pg, Bh, Bg = _both(cuda, model, params)
    polar = sum(int(m.polar) for m in Pg.mesh_members)
    assert polar >= 1 and Pg.n_rows == Ph.n_rows and Pg.n_cells == Ph.n_cells
    for k in ("u", "r_s", "maxAlpha", "radius", "cos_gamma", "theta0", "lag_scale"):
        np.testing.assert_allclose(Bg["row"][k].cpu().numpy(), Ph.row[k], rtol=1e-12, err_msg=k)
    # lag_C = (1/u - R/r_s + ln(...)) r_s / c nearly cancels where r ~ R
    lc = Ph.row["lag_C"]
    np.testing.assert_allclose(Bg["row"]["lag_C"].cpu().numpy(), lc, rtol=1e-11,
                               atol=1e-12 * np.max(np.abs(lc)))
    np.testing.assert_array_equal(Bg["row_mesh"].cpu().numpy(), Ph.row_mesh)
    A = Bg["cellArea"].cpu().numpy()
    scale = np.max(Ph.cellArea)
    np.testing.assert_allclose(A, Ph.cellArea, rtol=1e-12, atol=1e-12 * scale)
    np.testing.assert_allclose(Bg["phi"].cpu().numpy(), Ph.phi, rtol=0, atol=1e-14)
    np.testing.assert_allclose(Bg["params"].cpu().numpy(), Ph.params, rtol=1e-14)
    assert (Bg["radiates"].cpu().numpy() != Ph.radiates).sum() == 0


def test_loglike_with_gpu_meshes(cuda):
    model = SY.config2_model()
    # counts drawn from the model of the full-size configuration's vector
    ev = BT.BatchEvaluator(model)
    P0 = BT.prepare(model, SY.config2_vector(seed=1)[None, :])
    B0 = ev.upload(P0)
    ev.run(B0)
    cuda.cuda.synchronize()
    f = B0["folded"].cpu().numpy()
    SY.attach_data(model, [f[0], f[1]], P0.shifts[0])
    params = SY.config3_vectors(6, seed=3)
    ev, Ph, Pg, Bh, Bg = _both(cuda, model, params)
    ev.run(Bh)
    ev.run(Bg)
    cuda.cuda.synchronize()
    st_h, st_g = ev.statuses(Bh), ev.statuses(Bg)
    np.testing.assert_array_equal(st_h, st_g)
    ok = st_h == 0
    assert ok.any()
    lh, lg = Bh["loglike"].cpu().numpy(), Bg["loglike"].cpu().numpy()
    assert np.max(np.abs(lh[ok] - lg[ok])) <= 1e-7
