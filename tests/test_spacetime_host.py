"""The batched path's spacetime quantities (batch.spacetime, restating
Spacetime.py:110-187) against the closed forms of the reference's own tests
(xpsi/tests/test_spacetime.py:83-205: f 100 Hz, M 1 Msun, R 10 km, D 3 kpc,
cos i -1, with the same tolerances), against the reference's Spacetime class
where its checkout is present, and the packing that prepare() does with
them.  CPU only."""
import math

import numpy as np
import pytest

from xpsi_gb300 import batch as BT

F, M, R, D, COSI = 100.0, 1.0, 10.0, 3.0, -1.0
RG_SUN, MSUN = 2.95 * 10 ** 3, 1.989 * 10 ** 30


@pytest.fixture(scope="module")
def st():
    return BT.spacetime(M, R, F, COSI, D)


def test_mass(st):
    assert np.isclose(MSUN, st["M"], rtol=0.001)


def test_gravitational_and_schwarzschild_radii(st):
    # the reference's r_g is half the solar Schwarzschild radius
    assert np.isclose(RG_SUN / 2, st["r_g"], rtol=0.002)
    assert np.isclose(RG_SUN, st["r_s"], rtol=0.002)


def test_radius_and_ratio(st):
    assert st["R"] == R * 1000
    assert np.isclose(st["R_r_s"], R * 1000.0 / RG_SUN, rtol=0.002)


def test_frequency_and_angular_frequency(st):
    assert st["f"] == F
    assert st["Omega"] == 2 * np.pi * F


def test_inclination(st):
    assert st["i"] == np.pi


def test_distance(st):
    dist = D * 3.086 * 10 ** 16 * 1000.0
    assert np.isclose(st["d"], dist, rtol=0.001)
    assert np.isclose(st["d_sq"], dist ** 2.0, rtol=0.001)


def test_zeta_and_epsilon(st):
    assert np.isclose((RG_SUN / 2.) / (R * 1000.0), st["zeta"], rtol=0.002)
    eps = (2. * np.pi * F) ** 2.0 * (R * 1000) ** 3.0 / (6.6743e-11 * MSUN)
    assert np.isclose(eps, st["epsilon"], rtol=0.001)


def test_prepare_uses_spacetime():
    """prepare() packs r_s, the inclination, the distance and the lag
    constants of every member from these quantities."""
    from batch_cases import small_num4d
    m, params = small_num4d(V=2)
    P = BT.prepare(m, params)
    for v in range(P.V):
        sp = BT.spacetime(*params[v, :5])
        for h in range(P.H):
            mesh = P.meshes[v * P.H + h]
            assert P.row["r_s"][mesh.row_off] == sp["r_s"]
            assert mesh.omega == sp["Omega"] and mesh.inclination == sp["i"]
            assert P.d_sq[v * P.H + h] == sp["d_sq"]
            assert P.row["lag_scale"][mesh.row_off] == sp["f"] * 2.0 * math.pi


def test_matches_reference_spacetime_class():
    """Every quantity equals the reference's Spacetime property bit for bit
    (needs the reference checkout and its build)."""
    from oracle import ref_harness as H
    if not H.available():
        pytest.skip("reference checkout not present")
    H.load()
    from xpsi.Spacetime import Spacetime
    rng = np.random.default_rng(4)
    for _ in range(20):
        vals = {"mass": rng.uniform(1.0, 2.4), "radius": rng.uniform(8.0, 15.0),
                "frequency": rng.uniform(1.0, 700.0), "distance": rng.uniform(0.1, 20.0),
                "cos_inclination": rng.uniform(-1.0, 0.9)}
        bounds = {"mass": (0.01, 2.5), "radius": (5.0, 15.0), "frequency": (0.1, 750.0),
                  "distance": (0.05, 25.0), "cos_inclination": (-1.0, 0.9)}
        ref = Spacetime(bounds, vals)
        ours = BT.spacetime(vals["mass"], vals["radius"], vals["frequency"],
                            vals["cos_inclination"], vals["distance"])
        for k in ("M", "r_g", "r_s", "R", "R_r_s", "f", "Omega", "i", "d", "d_sq", "zeta",
                  "epsilon"):
            assert ours[k] == getattr(ref, k), k
