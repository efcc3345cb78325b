"""The integrators' energy grid over the union of the signals' wavebands
(batch.construct_energy_array) and the waveband a response and channel range
select (batch.identify_waveband), against the reference's own
construct_energy_array (Signal.py:1092-1197) and Signal._identify_waveband
(Signal.py:324-354) on the cases of tests/golden/energy_arrays.npz:
overlapping bands, coverage gaps, a maximum energy inside a gap, inside a
band and above every band.  CPU only."""
import numpy as np
import pytest

from conftest import load_golden
from xpsi_gb300 import batch as BT


@pytest.mark.parametrize("c", range(8))
def test_energy_array_vs_reference(c):
    f = load_golden("energy_arrays")
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_fixtures import ENERGY_CASES
    num, emax, bands = ENERGY_CASES[c]
    edges = [f[f"c{c}_band{b}"] for b in range(len(bands))]
    got = BT.construct_energy_array(num, edges, emax)
    np.testing.assert_array_equal(got, f[f"c{c}_energies"])
    # any order of the wavebands gives the same grid
    np.testing.assert_array_equal(BT.construct_energy_array(num, edges[::-1], emax), got)


@pytest.mark.parametrize("c", range(3))
def test_identify_waveband_vs_reference(c):
    f = load_golden("energy_arrays")
    rng, edges = BT.identify_waveband(f[f"w{c}_matrix"], f[f"w{c}_edges"],
                                      tuple(int(x) for x in f[f"w{c}_index_range"]))
    assert rng == tuple(int(x) for x in f[f"w{c}_range"])
    np.testing.assert_array_equal(edges, f[f"w{c}_energy_edges"])


def test_model_energies_follow_its_waveband():
    """A model whose response has zero input columns at both ends integrates
    over the trimmed waveband only."""
    from xpsi_gb300 import synthetic as SY
    M, edges, _ = SY.gaussian_response(40, 30)
    M[:, :2] = 0.0
    M[:, -3:] = 0.0
    m = BT.Model(regions=[BT.HotRegionSpec()], instrument=BT.Instrument(M, edges),
                 data=BT.Data(np.zeros((40, 32), np.int32), np.linspace(0, 1, 33), 1e6),
                 num_energies=50)
    assert np.isclose(m.energies[0], edges[2]) and np.isclose(m.energies[-1], edges[-4])
    assert m.energies.size == 50
