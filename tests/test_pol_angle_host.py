"""The polarisation angle (cellmesh/common_functions.pyx:7-66) of the
oracle, which the Stokes kernels restate: the reference's own unit tests
(xpsi/tests/test_cellmesh.py: a finite result; the non-relativistic limit,
where the angle is the analytic one) and, where the reference builds here,
equality with its compute_pol_ang_py.  CPU only."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import ref_harness as H


def test_pol_angle_finite():
    assert np.isfinite(O.pol_angle(0.1, 0.2, 0.98, 0.3, 0.95, 0.4, 0.92, 0.5, 0.86, 0.6, 0.8,
                                   1.0, 0.7, 1.0, 0.2, 1.1, 0.9))


def test_pol_angle_non_relativistic_limit():
    rng = np.random.default_rng(1234)
    for _ in range(10):
        theta = rng.uniform(0.001, np.pi - 0.001)
        phi = rng.uniform(0, 2 * np.pi)
        i = rng.uniform(0.001, np.pi - 0.001)
        chi = O.pol_angle(phi, 0.3, np.sqrt(1 - 0.09), 0.4, np.sqrt(1 - 0.16), np.sin(theta),
                          np.cos(theta), np.sin(i), np.cos(i), 0.0, 1.0, 1.0, 0.5, 1.0, 0.0,
                          1.0, 0.5)
        expected = np.arctan2(-np.sin(theta) * np.sin(phi),
                              np.sin(i) * np.cos(theta) - np.cos(i) * np.sin(theta) * np.cos(phi))
        assert np.isclose(chi, expected, atol=1e-12)


@pytest.mark.skipif(not H.available(), reason="reference checkout not present")
def test_pol_angle_equals_reference():
    H.load()
    from xpsi.cellmesh.common_functions import compute_pol_ang_py
    rng = np.random.default_rng(7)
    for _ in range(200):
        a = rng.uniform(-1.0, 1.0, 17)
        a[[1, 3, 5, 7, 9]] = np.abs(a[[1, 3, 5, 7, 9]])
        a[[11, 13, 15]] = 1.0 + np.abs(a[[11, 13, 15]])
        assert O.pol_angle(*a) == compute_pol_ang_py(*a)
