"""The oracle's numerical polarised atmospheres against the reference's own
output on the same inputs: Pol_Num2D (atm_ext 4, hot_Num2D.pyx) in the plain
and Stokes integrators (tests/golden/pol_num2d.npz) and the split Stokes
integrator (integratorIQU_for_azimuthal_invariance_split.pyx,
tests/golden/split_iqu.npz).  CPU only."""
import pytest

from conftest import (GENERAL_IQU_CASES, POL2D_CASES, SPLIT_CASES, general_iqu_args, pol2d_args,
                      row_rel, split_iqu_args)
from oracle import oracle as O


@pytest.mark.parametrize("tag,case", POL2D_CASES)
def test_oracle_pol_num2d_vs_reference(golden, tag, case):
    z = golden("pol_num2d")
    st, flux = O.integrate(*pol2d_args(golden, tag, case, stokes=False))
    assert st == 0
    assert row_rel(flux, z[tag + "_plain"]) <= 1e-13
    res = O.integrate_iqu(*pol2d_args(golden, tag, case, stokes=True))
    assert res[0] == 0
    for k, s in enumerate("IQU"):
        assert row_rel(res[k + 1], z[tag + "_" + s]) <= 1e-13, s


@pytest.mark.parametrize("tag,case", SPLIT_CASES)
def test_oracle_split_iqu_vs_reference(golden, tag, case):
    z = golden("split_iqu")
    res = O.integrate_split_iqu(*split_iqu_args(golden, tag, case))
    assert res[0] == 0
    for k, s in enumerate("IQU"):
        assert row_rel(res[k + 1], z[tag + "_" + s]) <= 1e-13, s


def test_split_iqu_rejects_tables_on_different_grids(golden):
    from xpsi_gb300 import synthetic
    a = list(split_iqu_args(golden, "config1", "config1"))
    q = list(synthetic.split_table_q())
    q[3] = q[3] * 0.95
    a[23] = tuple(q)
    with pytest.raises(NotImplementedError):
        O.integrate_split_iqu(*a)


@pytest.mark.parametrize("tag,case,ext", GENERAL_IQU_CASES)
def test_oracle_general_iqu_vs_reference(golden, tag, case, ext):
    """The general Stokes integrator (integratorIQU.pyx), whose polarisation
    angle reads the leaf loop's last values, and the general intensity
    integrator with the same atmospheres."""
    z = golden("general_iqu")
    res = O.integrate_general_iqu(*general_iqu_args(golden, tag, case, ext))
    assert res[0] == 0
    for k, s in enumerate("IQU"):
        assert row_rel(res[k + 1], z[tag + "_" + s]) <= 1e-13, s
    st, flux = O.integrate_general(*general_iqu_args(golden, tag, case, ext, stokes=False))
    assert st == 0
    assert row_rel(flux, z[tag + "_plain"]) <= 1e-13
