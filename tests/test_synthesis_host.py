"""Synthesis on the host: the oracle's compute_expected_counts and
phase_integrator against the reference's own outputs
(tests/golden/synthesis.npz), and the test-side Philox restatement against
the generator's published known answers.  CPU only."""
import numpy as np
import pytest

from oracle import oracle as O
from philox_ref import philox4x32_10


def synthesis_inputs(golden):
    f, z = golden("config1"), golden("synthesis")
    return (f["folded"], f["comp_phases"], f["phase_edges"], z)


def test_oracle_expected_counts_exposure(golden):
    c1, p1, edges, z = synthesis_inputs(golden)
    T = 2.0e5
    rate = z["bkg"] * float(z["exposure_scale_background"]) / T
    e = O.compute_expected_counts(T, edges, (c1, z["c2"]), (p1, z["p2"]), z["shifts"], rate,
                                  [False, True])
    np.testing.assert_allclose(e, z["exposure_expec"], rtol=1e-13, atol=0)


def test_oracle_expected_counts_total(golden):
    c1, p1, edges, z = synthesis_inputs(golden)
    star = O.compute_expected_counts(1e5, edges, (c1, z["c2"]), (p1, z["p2"]), z["shifts"],
                                     np.zeros_like(z["bkg"]), [False, True])
    scale_star = float(z["total_scale_star"])
    scale_bkg = float(z["total_scale_ratio"]) * scale_star
    np.testing.assert_allclose(star * scale_star + z["bkg"] * scale_bkg, z["total_expec"],
                               rtol=1e-12, atol=0)


@pytest.mark.parametrize("which", ["phase_integrated", "phase_integrated_neg"])
def test_oracle_phase_integrator(golden, which):
    c1, p1, edges, z = synthesis_inputs(golden)
    if which == "phase_integrated":
        out = O.phase_integrator(1e5, edges, c1, p1, 0.25)
    else:
        out = O.phase_integrator(1e5, edges, z["c2"], z["p2"], -0.7, True)
    np.testing.assert_array_equal(out, z[which])


@pytest.mark.parametrize("c,k,expected", [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1])])
def test_philox_known_answers(c, k, expected):
    assert philox4x32_10(c, k) == expected
