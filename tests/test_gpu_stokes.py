"""The Stokes integrator on the GPU (through the C ABI) against the
reference's own I, Q, U and against the oracle; each Stokes parameter is
held to 1e-9 of its energy row's largest value, the integrator's bar."""
import numpy as np
import pytest

from conftest import STOKES_CASES, atmos_of, row_rel, stokes_args
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-9


@pytest.fixture(scope="module")
def iqu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import xpsi_gb300
    xpsi_gb300.lib()
    from xpsi_gb300.cellmesh import integratorIQU_for_azimuthal_invariance
    return integratorIQU_for_azimuthal_invariance


@pytest.mark.parametrize("case,ext,corrected", STOKES_CASES)
def test_stokes_vs_reference(iqu, golden, case, ext, corrected):
    tag, args = stokes_args(golden, case, ext, corrected)
    out = iqu.integrate(*args)
    assert out[0] == 0
    z = golden("stokes")
    for k, s in enumerate("IQU"):
        assert row_rel(out[k + 1], z[tag + "_" + s]) <= RTOL, s
    if ext == 1:
        assert not np.any(out[2]) and not np.any(out[3])


@pytest.mark.parametrize("image_order_limit", [1, 2])
def test_stokes_vs_oracle_image_orders(iqu, golden, image_order_limit):
    _, args = stokes_args(golden, "num4d_omit", 3, False, image_order_limit)
    ref = O.integrate_iqu(*args)
    out = iqu.integrate(*args)
    assert out[0] == ref[0] == 0
    for k in range(3):
        assert row_rel(out[k + 1], ref[k + 1]) <= RTOL


def test_stokes_num4d_is_the_intensity_integrator(iqu, golden):
    """For the numerical 4-D atmosphere the reference's Q is zero and its I is
    the azimuthal integrator's."""
    f = golden("num4d_omit")
    _, args = stokes_args(golden, "num4d_omit", 3, False)
    args = list(args)
    args[22] = atmos_of(f)
    args[25] = 2
    out = iqu.integrate(*args)
    assert out[0] == 0
    assert row_rel(out[1], f["flux"]) <= RTOL
    assert not np.any(out[2]) and not np.any(out[3])


def test_stokes_bitwise_reproducible(iqu, golden):
    _, args = stokes_args(golden, "num4d_omit", 3, False)
    a = iqu.integrate(*args)
    b = iqu.integrate(*args)
    for k in range(1, 4):
        np.testing.assert_array_equal(a[k], b[k])


@pytest.mark.parametrize("case", ["config1", "num4d_omit"])
def test_plain_integrator_burst_intensity(iqu, golden, case):
    """The azimuthal intensity integrator with the burst blackbody (atm_ext 3)
    against the reference Stokes integrator's I and the oracle."""
    from xpsi_gb300.cellmesh import integrator_for_azimuthal_invariance as az
    tag, args = stokes_args(golden, case, 3, False)
    plain = args[:22] + (args[22],) + args[24:]
    st, flux = az.integrate(*plain)
    assert st == 0
    assert row_rel(flux, golden("stokes")[tag + "_I"]) <= RTOL
    ref = O.integrate(*plain)
    assert ref[0] == 0 and row_rel(flux, ref[1]) <= RTOL
