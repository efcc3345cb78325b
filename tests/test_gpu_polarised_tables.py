"""Numerical polarised atmospheres on the GPU (through the C ABI) against the
reference's own output and the oracle: Pol_Num2D (atm_ext 4) in the plain
and Stokes integrators (tests/golden/pol_num2d.npz) and the split Stokes
integrator (tests/golden/split_iqu.npz).  Every energy row of I, Q and U to
1e-9 of its largest value, the integrator's bar."""
import pytest

from conftest import (GENERAL_IQU_CASES, POL2D_CASES, SPLIT_CASES, general_iqu_args, pol2d_args,
                      row_rel, row_rel_floor, split_iqu_args)
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-9


@pytest.fixture(scope="module")
def mods():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import xpsi_gb300
    xpsi_gb300.lib()
    from xpsi_gb300.cellmesh import (integrator_for_azimuthal_invariance as plain,
                                     integratorIQU_for_azimuthal_invariance as iqu,
                                     integratorIQU_for_azimuthal_invariance_split as iqu_split)
    return plain, iqu, iqu_split


@pytest.mark.parametrize("tag,case", POL2D_CASES)
def test_pol_num2d_vs_reference(mods, golden, tag, case):
    plain, iqu, _ = mods
    z = golden("pol_num2d")
    st, flux = plain.integrate(*pol2d_args(golden, tag, case, stokes=False))
    assert st == 0
    assert row_rel(flux, z[tag + "_plain"]) <= RTOL
    res = iqu.integrate(*pol2d_args(golden, tag, case, stokes=True))
    assert res[0] == 0
    for k, s in enumerate("IQU"):
        assert row_rel(res[k + 1], z[tag + "_" + s]) <= RTOL, s
    # the Stokes I is the plain integrator's (two kernels, two summation orders)
    assert row_rel(res[1], flux) <= 1e-12


@pytest.mark.parametrize("image_order_limit", [1, 2])
def test_pol_num2d_vs_oracle_image_orders(mods, golden, image_order_limit):
    _, iqu, _ = mods
    args = pol2d_args(golden, "config1_mu09", "config1", True, image_order_limit)
    ref = O.integrate_iqu(*args)
    out = iqu.integrate(*args)
    assert out[0] == ref[0] == 0
    for k in range(3):
        assert row_rel(out[k + 1], ref[k + 1]) <= RTOL


@pytest.mark.parametrize("tag,case", SPLIT_CASES)
def test_split_stokes_vs_reference(mods, golden, tag, case):
    _, _, iqu_split = mods
    z = golden("split_iqu")
    res = iqu_split.integrate(*split_iqu_args(golden, tag, case))
    assert res[0] == 0
    for k, s in enumerate("IQU"):
        assert row_rel(res[k + 1], z[tag + "_" + s]) <= RTOL, s


def test_split_stokes_intensity_is_the_split_integrators(mods, golden):
    from xpsi_gb300.cellmesh import integrator_for_azimuthal_invariance_split as split
    from conftest import split_args
    _, _, iqu_split = mods
    res = iqu_split.integrate(*split_iqu_args(golden, "num4d_omit", "num4d_omit"))
    st, flux = split.integrate(*split_args(golden, "num4d_omit", "num4d_omit"))
    assert res[0] == st == 0
    assert row_rel(res[1], flux) <= 1e-12


@pytest.mark.parametrize("tag,case,ext", GENERAL_IQU_CASES)
def test_general_stokes_vs_reference(golden, tag, case, ext):
    """The general Stokes integrator (integratorIQU.pyx) and the general
    intensity integrator with the same atmospheres, on the GPU."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xpsi_gb300.cellmesh import integrator, integratorIQU
    z = golden("general_iqu")
    res = integratorIQU.integrate(*general_iqu_args(golden, tag, case, ext))
    assert res[0] == 0
    for k, s in enumerate("IQU"):
        assert row_rel_floor(res[k + 1], z[tag + "_" + s]) <= RTOL, s
    st, flux = integrator.integrate(*general_iqu_args(golden, tag, case, ext, stokes=False))
    assert st == 0
    assert row_rel_floor(flux, z[tag + "_plain"]) <= RTOL
