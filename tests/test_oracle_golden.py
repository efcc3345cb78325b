"""The oracle (CPU restatement, oracle/xpsi_oracle.c) against the golden
fixtures produced by the reference itself (tests/golden/make_fixtures.py).
CPU only."""
import numpy as np
import pytest

from conftest import atmos_of, row_rel
from oracle import oracle as O


def _integrate_args(f, atmos=()):
    return (1, float(f["R"]), float(f["Omega"]), float(f["r_s"]), float(f["inclination"]),
            f["cellArea"], f["radius"], f["u"], f["theta"], f["phi"], f["params"],
            f["radiates"], None, int(f["N_R"]), f["deflection"], f["cos_alpha"], f["lag"],
            f["maxDeflection"], f["cos_gamma"], f["energies"], f["leaves"], f["phases"],
            atmos, None, int(f["atm_ext"]), None, 0,
            int(f["image_order_limit"]) or None)


def test_rays_examples_fast(golden):
    f = golden("examples_fast")
    ma = f["maxAlpha_in"].copy()
    S = f["rays_u"].size
    t, D, CA, L, MD = O.compute_rays(1, S, float(f["r_s"]), f["rays_u"], ma, int(f["N_R"]))
    assert t == 0
    np.testing.assert_array_equal(ma, f["rays_maxAlpha_out"])
    np.testing.assert_array_equal(D, f["rays_deflection"])
    np.testing.assert_array_equal(CA, f["rays_cos_alpha"])
    np.testing.assert_array_equal(L, f["rays_lag"])
    np.testing.assert_array_equal(MD, f["rays_maxDefl"])


@pytest.mark.parametrize("case", ["examples_fast", "config1"])
def test_integrator_blackbody(golden, case):
    f = golden(case)
    st, flux = O.integrate(*_integrate_args(f))
    assert st == 0
    assert row_rel(flux, f["flux"]) <= 1e-13


def test_integrator_num4d_history(golden):
    """The oracle keeps the reference's per-thread Num4D stencil state, so it
    matches the reference for one thread and for four threads."""
    f = golden("num4d_omit")
    st, flux = O.integrate(*_integrate_args(f, atmos_of(f)))
    assert st == 0
    assert row_rel(flux, f["flux"]) <= 1e-13
    args = list(_integrate_args(f, atmos_of(f)))
    args[0] = 4
    st, flux4 = O.integrate(*args)
    assert row_rel(flux4, f["flux_threads4"]) <= 1e-13


@pytest.mark.parametrize("case", ["examples_fast", "config1"])
def test_energy_integrator(golden, case):
    f = golden(case)
    out = O.energy_integrator(1, f["signal_in"], f["log10_energies"], f["log10_edges"])
    np.testing.assert_allclose(out, f["energy_out"], rtol=0, atol=1e-13 * np.abs(f["energy_out"]).max())


@pytest.mark.parametrize("case", ["examples_fast", "config1"])
def test_likelihood(golden, case):
    f = golden(case)
    reg = f["registered"] if "registered" in f else f["folded"]
    pre = O.precomputation(f["counts"].astype(np.int32))
    np.testing.assert_allclose(pre, f["precomp"], rtol=1e-14)
    ll, star, mb, mbs = O.eval_marginal_likelihood(
        float(f["exposure"]), f["phase_edges"], f["counts"], [reg], [f["comp_phases"]],
        f["shifts"], f["precomp"], f["support"], 1000, 0.0, 1e-8, 1e-3, 10.0, -1e90)
    assert abs(ll - float(f["logL"])) <= 1e-9 * abs(float(f["logL"]))
    np.testing.assert_allclose(star, f["star"], rtol=1e-12, atol=1e-300)


def test_examples_fast_golden_value(golden):
    """The reference's published check (xpsi/tests/test_likelihood.py:131-134)."""
    f = golden("examples_fast")
    assert np.isclose(float(f["golden_logL"]), float(f["ref_logL"]), rtol=1e-5)
    assert abs(float(f["ref_logL"]) - float(f["logL"])) < 1e-6


def test_gk_nodes_exactness():
    """Gauss-Kronrod tables integrate monomials exactly to their degree."""
    import importlib.util, os, re
    from conftest import ROOT
    txt = open(os.path.join(ROOT, "oracle", "gslsub", "include", "gk_nodes.h")).read()
    for K, deg in ((21, 31), (61, 91)):
        def arr(name):
            body = re.search(r"GSLSUB_K%d_%s\[\d+\] = \{([^}]*)\}" % (K, name), txt).group(1)
            return np.array([float(v) for v in body.replace("\n", "").split(",") if v.strip()])
        x, wk, wg = arr("X"), arr("WK"), arr("WG")
        xs = np.concatenate([-x[:-1], x[::-1]])
        ws = np.concatenate([wk[:-1], wk[::-1]])
        wgs = np.concatenate([wg[:-1], wg[::-1]])
        for p in range(0, deg + 1, 2):
            assert abs(np.sum(ws * xs ** p) - 2.0 / (p + 1)) < 1e-14
        n_g = (K - 1) // 2
        for p in range(0, 2 * n_g, 2):
            assert abs(np.sum(wgs * xs ** p) - 2.0 / (p + 1)) < 1e-14
