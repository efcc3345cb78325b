"""The oracle's general integrator (HotRegion symmetry=False,
cellmesh/integrator.pyx:48-667) against the reference's own outputs
(tests/golden/general_integrator.npz).  CPU only."""
import pytest

from conftest import GENERAL_CASES, general_args, row_rel
from oracle import oracle as O


@pytest.mark.parametrize("case,corrected,mu09,key", GENERAL_CASES)
def test_oracle_general_vs_reference(golden, case, corrected, mu09, key):
    st, flux = O.integrate_general(*general_args(golden, case, corrected=corrected, mu09=mu09))
    assert st == 0
    assert row_rel(flux, golden("general_integrator")[key]) <= 1e-13


def test_oracle_general_num4d_four_threads(golden):
    """The per-thread Num4D stencil state of the reference at 4 threads."""
    st, flux = O.integrate_general(*general_args(golden, "num4d_omit", threads=4))
    assert st == 0
    assert row_rel(flux, golden("general_integrator")["num4d_omit_flux_threads4"]) <= 1e-13
