"""Synthesis on the GPU: expected counts and phase integration against the
reference's own outputs, the Poisson draws against a restatement of the
generator (small means, bit for bit) and against the Poisson law (all
means), and batched synthesis against the oracle pipeline."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from philox_ref import first_uniform, poisson_small

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def syn():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import xpsi_gb300
    xpsi_gb300.lib()
    from xpsi_gb300.tools import phase_integrator, synthesise
    return synthesise, phase_integrator


def _inputs(golden):
    f, z = golden("config1"), golden("synthesis")
    return f["folded"], f["comp_phases"], f["phase_edges"], z


def test_synthesise_exposure_expected(syn, golden):
    S, _ = syn
    c1, p1, edges, z = _inputs(golden)
    E, D, scale = S.synthesise_exposure(2.0e5, edges, (c1, z["c2"]), (p1, z["p2"]),
                                        z["shifts"], 3.0e4, z["bkg"], [False, True], gsl_seed=7)
    assert abs(scale / float(z["exposure_scale_background"]) - 1.0) <= 1e-14
    np.testing.assert_allclose(E, z["exposure_expec"], rtol=1e-12, atol=0)
    assert D.shape == E.shape and np.all(D >= 0) and np.all(D == np.floor(D))
    # the realisation is a Poisson draw of the expectation (sums within 5 sigma)
    assert abs(D.sum() - E.sum()) <= 5.0 * math.sqrt(E.sum())


def test_synthesise_given_total_expected(syn, golden):
    S, _ = syn
    c1, p1, edges, z = _inputs(golden)
    E, D, s_star, ratio = S.synthesise_given_total_count_number(
        edges, 1.0e6, (c1, z["c2"]), (p1, z["p2"]), z["shifts"], 2.0e5, z["bkg"],
        [False, True], gsl_seed=7)
    assert abs(s_star / float(z["total_scale_star"]) - 1.0) <= 1e-12
    assert abs(ratio / float(z["total_scale_ratio"]) - 1.0) <= 1e-12
    np.testing.assert_allclose(E, z["total_expec"], rtol=1e-12, atol=0)
    assert abs(D.sum() - E.sum()) <= 5.0 * math.sqrt(E.sum())


@pytest.mark.parametrize("which", ["phase_integrated", "phase_integrated_neg"])
def test_phase_integrator_vs_reference(syn, golden, which):
    _, PI = syn
    c1, p1, edges, z = _inputs(golden)
    if which == "phase_integrated":
        out = PI.phase_integrator(1e5, edges, c1, p1, 0.25)
    else:
        out = PI.phase_integrator(1e5, edges, z["c2"], z["p2"], -0.7, True)
    np.testing.assert_allclose(out, z[which], rtol=1e-12, atol=1e-12 * np.abs(z[which]).max())


def test_poisson_small_means_bitwise(syn):
    """Means below 10: every draw equals the restatement's inversion of the
    element's first uniform."""
    S, _ = syn
    rng = np.random.default_rng(1)
    mu = rng.uniform(0.0, 9.999, 4000)
    mu[:5] = [0.0, 1e-12, 0.5, 9.999, 3.0]
    seed = 0x1234_5678_9abc_def0
    d = S.poisson(mu, seed, offset=17)
    ref = [0 if m == 0.0 else poisson_small(m, first_uniform(seed, 17 + i))
           for i, m in enumerate(mu)]
    np.testing.assert_array_equal(d, np.array(ref, dtype=float))


@pytest.mark.parametrize("mu", [0.3, 4.0, 9.99, 10.0, 37.5, 2500.0, 1.0e6])
def test_poisson_moments(syn, mu):
    S, _ = syn
    n = 200_000
    d = S.poisson(np.full(n, mu), seed=99)
    m, v = d.mean(), d.var()
    assert abs(m - mu) <= 5.0 * math.sqrt(mu / n)
    # the variance of the sample variance of a Poisson law is ~ (mu + 2 mu^2) / n
    assert abs(v - mu) <= 5.0 * math.sqrt((mu + 2.0 * mu * mu) / n)


def test_poisson_law_chi_square(syn):
    """The histogram at a mean of 37.5 (the rejection sampler) against the
    Poisson probabilities: chi-square below its 99.9 % point."""
    from scipy import stats
    S, _ = syn
    n, mu = 400_000, 37.5
    d = S.poisson(np.full(n, mu), seed=2024).astype(int)
    lo, hi = 15, 65
    obs = np.array([(d < lo).sum()] + [(d == k).sum() for k in range(lo, hi)] +
                   [(d >= hi).sum()], dtype=float)
    p = np.array([stats.poisson.cdf(lo - 1, mu)] + [stats.poisson.pmf(k, mu)
                                                    for k in range(lo, hi)] +
                 [stats.poisson.sf(hi - 1, mu)])
    chi2 = float(((obs - n * p) ** 2 / (n * p)).sum())
    assert chi2 < stats.chi2.ppf(0.999, len(obs) - 1)


def test_poisson_stream_keys(syn):
    S, _ = syn
    mu = np.full(1000, 25.0)
    a = S.poisson(mu, seed=5)
    np.testing.assert_array_equal(a, S.poisson(mu, seed=5))
    assert np.any(a != S.poisson(mu, seed=6))
    # element i at offset 10 is element i + 10 at offset 0
    np.testing.assert_array_equal(S.poisson(mu[:990], seed=5, offset=10), a[10:])


def test_batch_synthesise_vs_oracle(syn):
    """Synthetic data sets of a batch: expected counts against the oracle
    pipeline's folded signals through the oracle's compute_expected_counts."""
    from batch_cases import small_blackbody
    from oracle import pipeline as OP
    from xpsi_gb300 import batch as BT
    m, params = small_blackbody(V=3)
    P = BT.prepare(m, params)
    _, ref_st, stages = OP.loglike(m, P, return_stages=True)
    ev = BT.BatchEvaluator(m)
    K, Bn = m.instrument.matrix.shape[0], len(m.data.phase_edges) - 1
    bkg = np.full((K, Bn), 0.01)
    E, D, st = ev.synthesise(params, 1.0e5, background=bkg, seed=3)
    np.testing.assert_array_equal(st, ref_st)
    comp_phases = np.linspace(0.0, 1.0, m.regions[0].num_leaves)
    for v in range(P.V):
        ref = O.compute_expected_counts(1.0e5, m.data.phase_edges, [stages[v]["folded"]],
                                        [comp_phases], P.shifts[v], bkg)
        np.testing.assert_allclose(E[v], ref, rtol=1e-8, atol=1e-9 * np.abs(ref).max())
    assert abs(D.sum() - E.sum()) <= 5.0 * math.sqrt(E.sum())
