"""The oracle's Gaussian likelihoods of polarimetry against the reference's
own values (tests/golden/gaussian.npz).  CPU only."""
import numpy as np

from oracle import oracle as O


def test_oracle_gaussian_given_background(golden):
    f, z = golden("config1"), golden("gaussian")
    expec = O.compute_expected_counts(float(z["exposure"]), f["phase_edges"],
                                      [f["folded"][:40]], [f["comp_phases"]], [0.2], z["bkg"])
    np.testing.assert_allclose(expec, z["expec"], rtol=1e-13, atol=0)
    assert abs(O.gaussian_loglike(expec, z["counts"], z["errors"]) - float(z["loglike"])) <= \
        1e-12 * abs(float(z["loglike"]))


def test_oracle_gaussian_QnUn(golden):
    z = golden("gaussian")
    assert abs(O.gaussian_loglike(z["star"], z["qn"], z["qn_err"]) - float(z["loglike_qn"])) <= \
        1e-12 * abs(float(z["loglike_qn"]))
