"""The oracle's Stokes integrator (integratorIQU_for_azimuthal_invariance.pyx:
68-743, burst blackbody and blackbody with a correction) against the
reference's own outputs (tests/golden/stokes.npz).  CPU only."""
import pytest

from conftest import STOKES_CASES, row_rel, stokes_args
from oracle import oracle as O


@pytest.mark.parametrize("case,ext,corrected", STOKES_CASES)
def test_oracle_stokes_vs_reference(golden, case, ext, corrected):
    tag, args = stokes_args(golden, case, ext, corrected)
    out = O.integrate_iqu(*args)
    assert out[0] == 0
    z = golden("stokes")
    for k, s in enumerate("IQU"):
        assert row_rel(out[k + 1], z[tag + "_" + s]) <= 1e-13


@pytest.mark.parametrize("case", ["config1", "num4d_omit"])
def test_oracle_plain_burst_intensity_is_the_reference_stokes_i(golden, case):
    """The azimuthal intensity integrator with the burst blackbody (atm_ext
    3) gives the reference Stokes integrator's I."""
    tag, args = stokes_args(golden, case, 3, False)
    st, flux = O.integrate(*(args[:22] + (args[22],) + args[24:]))
    assert st == 0
    assert row_rel(flux, golden("stokes")[tag + "_I"]) <= 1e-13
