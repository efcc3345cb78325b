"""The phase and energy interpolators: the oracle against the reference's
own output (tests/golden/interpolators.npz); the drop-ins' argument checks.
CPU only."""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.mark.parametrize("tag", ["shift", "neg"])
def test_oracle_phase_interpolator_vs_reference(golden, tag):
    z = golden("interpolators")
    out = O.phase_interpolator(z["phase_new"], z["phase_phases"], z["phase_signal"],
                               float(z["phase_%s_shift" % tag]), tag == "neg")
    assert np.array_equal(out, z["phase_" + tag])


def test_oracle_energy_interpolator_vs_reference(golden):
    z = golden("interpolators")
    out = O.energy_interpolator(1, z["energy_signal"], z["energy_log10"], z["energy_new"])
    assert out.shape == z["energy_out"].shape
    assert np.array_equal(out, z["energy_out"])


def test_fixture_exercises_both_modes(golden):
    """A column with non-positive entries (splined without the logarithm),
    new energies above the grid (zero), and negative interpolant values."""
    z = golden("interpolators")
    assert (z["energy_signal"] <= 0).any(axis=0).sum() == 1
    assert (z["energy_new"] > z["energy_log10"][-1]).any()
    assert (z["phase_neg"] < 0).any() and not (z["phase_shift"] < 0).any()


def test_drop_in_shapes_are_checked():
    from xpsi_gb300.tools.energy_interpolator import energy_interpolator
    from xpsi_gb300.tools.phase_interpolator import phase_interpolator
    with pytest.raises(ValueError):
        phase_interpolator(np.zeros(3), np.linspace(0, 1, 8), np.zeros((2, 7)), 0.0)
    with pytest.raises(ValueError):
        energy_interpolator(1, np.zeros((5, 3)), np.zeros(4), np.zeros(2))
