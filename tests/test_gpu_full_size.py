"""The benchmarked workload itself, vector by vector: the full-size plain
model (two Num4D hot regions, one with an omitted crescent; the
35 x 14 x 67 x 166 table, sqrt_num_cells 64 (max 128), 128 leaves, 1024
rays, 128 energies, a 1500 x 128 response, 32 phase bins) at prior vectors
of the batched configuration that include polar caps on either member and
on both (tests/golden/meshes.npz carries the vectors and the reference's
meshes of all their members).

  * the GPU mesh builder against the reference's meshes (per-parallel values
    1e-12, cell areas 1e-10, each mesh's total area 1e-12);
  * the batched plain path, with host-built and with GPU-built meshes,
    against the oracle's restatement of every stage, meshes included
    (oracle/prepare.py, oracle/pipeline.py), on the same vectors:
    statuses equal, log L within 1e-7 absolute where the status is 0, and
    every member's flux within 1e-9 of the largest value of its energy row."""
import os

import numpy as np
import pytest

from conftest import load_golden, row_rel
from oracle import pipeline as OP
from oracle import prepare as OPR
from xpsi_gb300 import batch as BT
from xpsi_gb300 import synthetic as SY

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def workload(cuda):
    model = SY.config2_model()
    # counts drawn from the oracle's model of the full-size configuration's
    # vector (not from the GPU, so the data do not depend on the code tested)
    P0 = OPR.prepare(model, SY.config2_vector(seed=1)[None, :], n_threads=NT)
    _, _, st0 = OP.loglike(model, P0, n_threads=NT, return_stages=True)
    SY.attach_data(model, [st0[0]["folded"], st0[1]["folded"]], P0.shifts[0])
    f = load_golden("meshes")
    params = f["params"]
    Ph = BT.prepare(model, params)
    # the oracle end to end, its own meshes included
    Po = OPR.prepare(model, params, n_threads=NT)
    ref, ref_st, stages = OP.loglike(model, Po, n_threads=NT, return_stages=True)
    return dict(model=model, params=params, f=f, Ph=Ph, ref=ref, ref_st=ref_st,
                stages={(s["v"], s["h"]): s for s in stages})


def test_gpu_and_oracle_draw_the_same_counts(cuda, workload):
    """The benchmark's arms draw their data from the GPU's and from the
    oracle's model of the same vector: the seeded Poisson counts agree."""
    model = SY.config2_model()
    ev = BT.BatchEvaluator(model)
    P0 = BT.prepare(model, SY.config2_vector(seed=1)[None, :])
    B0 = ev.upload(P0)
    ev.run(B0)
    cuda.cuda.synchronize()
    f = B0["folded"].cpu().numpy()
    SY.attach_data(model, [f[0], f[1]], P0.shifts[0])
    np.testing.assert_array_equal(model.data.counts, workload["model"].data.counts)


def test_full_size_workload_has_polar_caps(workload):
    Ph = workload["Ph"]
    f = workload["f"]
    n = Ph.V * Ph.H
    polar = [int(f[f"m{k}_polar"]) for k in range(n)]
    assert sum(polar[0::2]) >= 1 and sum(polar[1::2]) >= 2
    assert any(polar[2 * v] and polar[2 * v + 1] for v in range(Ph.V))
    assert (workload["ref_st"] == 0).sum() >= 6


def test_gpu_meshes_vs_reference_meshes(cuda, workload):
    model, params, f = workload["model"], workload["params"], workload["f"]
    ev = BT.BatchEvaluator(model)
    Pg = BT.prepare(model, params, meshes="gpu")
    B = ev.upload(Pg)
    cuda.cuda.synchronize()
    row = {k: v.cpu().numpy() for k, v in B["row"].items()}
    A_all = B["cellArea"].cpu().numpy()
    phi_all = B["phi"].cpu().numpy()
    prm = B["params"].cpu().numpy()
    mem = f["members"]
    for mi in range(Pg.V * Pg.H):
        m = Pg.meshes[mi]
        S = m.S0
        assert S == int(f[f"m{mi}_S"])
        rs = slice(m.row_off, m.row_off + S)
        cs = slice(m.cell_off, m.cell_off + S * S)
        A = A_all[cs].reshape(S, S)
        Ar = f[f"m{mi}_cellArea"]
        # cells cut by a region boundary are adaptive quadratures of an
        # integrand with kinks and square-root endpoints; the GPU's
        # lane-parallel Kronrod sums round differently from the serial ones,
        # so its bisection stops at different (equally converged) points:
        # 2.6e-11 of such a cell at most has been seen.  Whole cells are exact.
        np.testing.assert_allclose(A, Ar, rtol=1e-10, atol=1e-12 * Ar.max(), err_msg=str(mi))
        assert np.array_equal(A > 0.0, Ar > 0.0)
        assert abs(A.sum() - Ar.sum()) <= 1e-12 * Ar.sum()
        np.testing.assert_allclose(row["theta0"][rs], f[f"m{mi}_theta"], rtol=1e-12)
        np.testing.assert_allclose(row["radius"][rs], f[f"m{mi}_radius"], rtol=1e-13)
        np.testing.assert_allclose(row["cos_gamma"][rs], f[f"m{mi}_cos_gamma"], rtol=1e-13)
        np.testing.assert_allclose(row["maxAlpha"][rs], f[f"m{mi}_maxAlpha"], rtol=1e-13)
        # the mesh azimuths less the omitted region's azimuth (HotRegion.py:836)
        ph = phi_all[cs].reshape(S, S)
        np.testing.assert_allclose(ph, np.broadcast_to(f[f"m{mi}_phi"] - mem[mi, 7], (S, S)),
                                   rtol=0, atol=1e-14)
        g = prm[cs, 1].reshape(S, S)
        np.testing.assert_allclose(g, np.broadcast_to(f[f"m{mi}_effGrav"][:, None], (S, S)),
                                   rtol=1e-13)


@pytest.mark.parametrize("meshes", ["host", "gpu"])
def test_full_size_batch_vs_oracle(cuda, workload, meshes):
    model, params = workload["model"], workload["params"]
    ref, ref_st, stages = workload["ref"], workload["ref_st"], workload["stages"]
    ev = BT.BatchEvaluator(model)
    P = BT.prepare(model, params, meshes=meshes)
    B = ev.upload(P)
    ev.run(B)
    cuda.cuda.synchronize()
    st = ev.statuses(B)
    ll = B["loglike"].cpu().numpy()
    np.testing.assert_array_equal(st, ref_st)
    ok = st == 0
    assert np.max(np.abs(ll[ok] - ref[ok])) <= 1e-7
    # every member the oracle integrated, including those of vectors the
    # likelihood's slim cut rejects afterwards
    flux = B["flux"].cpu().numpy()
    assert len(stages) == 2 * P.V
    worst = 0.0
    for (v, h), s in stages.items():
        worst = max(worst, row_rel(flux[v * P.H + h], s["flux"]))
    assert worst <= 1e-9, worst
