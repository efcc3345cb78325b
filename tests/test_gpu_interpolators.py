"""The phase and energy interpolators on the GPU (through the C ABI) against
the reference's own output (tests/golden/interpolators.npz): 1e-12 of each
row's (column's) largest value."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tools():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import xpsi_gb300
    xpsi_gb300.lib()
    from xpsi_gb300.tools import energy_interpolator, phase_interpolator
    return phase_interpolator.phase_interpolator, energy_interpolator.energy_interpolator


@pytest.mark.parametrize("tag", ["shift", "neg"])
def test_phase_interpolator_vs_reference(tools, golden, tag):
    z = golden("interpolators")
    out = tools[0](z["phase_new"], z["phase_phases"], z["phase_signal"],
                   float(z["phase_%s_shift" % tag]), tag == "neg")
    ref = z["phase_" + tag]
    scale = np.abs(ref).max(axis=1, keepdims=True)
    assert np.all(np.abs(out - ref) <= 1e-12 * scale)
    assert np.array_equal(out == 0.0, ref == 0.0)


def test_energy_interpolator_vs_reference(tools, golden):
    z = golden("interpolators")
    out = tools[1](1, z["energy_signal"], z["energy_log10"], z["energy_new"])
    ref = z["energy_out"]
    scale = np.abs(ref).max(axis=0, keepdims=True)
    assert out.shape == ref.shape
    assert np.all(np.abs(out - ref) <= 1e-12 * scale)
    assert np.array_equal(out == 0.0, ref == 0.0)
