"""The general integrator (HotRegion symmetry=False) on the GPU through the
C ABI, against the reference's own outputs and the oracle.  FP64 throughout;
the bar is the integrator's: 1e-9 relative to each energy row's largest
value, with that scale floored at 1e-15 of the spectrum's peak.  (In the
Num4D case the top energy rows lie 1e-18 to 1e-26 below the peak, where the
table's 4-point stencil cancels terms ~1e6 times larger than its result;
there the reference's own value is rounding residue, and the GPU agrees with
it to 2e-12 of the row at 1e-18 and 2e-8 of the row at 1e-26.)"""
import numpy as np
import pytest

from conftest import GENERAL_CASES, general_args, row_rel, row_rel_floor
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-9


@pytest.fixture(scope="module")
def gen():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import xpsi_gb300
    xpsi_gb300.lib()
    from xpsi_gb300.cellmesh import integrator
    return integrator


@pytest.mark.parametrize("case,corrected,mu09,key", GENERAL_CASES)
def test_general_vs_reference(gen, golden, case, corrected, mu09, key):
    st, flux = gen.integrate(*general_args(golden, case, corrected=corrected, mu09=mu09))
    assert st == 0
    assert row_rel_floor(flux, golden("general_integrator")[key]) <= RTOL


@pytest.mark.parametrize("case,mu09", [("config1", False), ("num4d_omit", True)])
@pytest.mark.parametrize("image_order_limit", [1, 2])
def test_general_vs_oracle_image_orders(gen, golden, case, mu09, image_order_limit):
    args = general_args(golden, case, mu09=mu09, image_order_limit=image_order_limit)
    st_o, ref = O.integrate_general(*args)
    st, flux = gen.integrate(*args)
    assert st == st_o == 0
    assert row_rel_floor(flux, ref) <= RTOL


def test_general_uniform_equals_azimuthal(gen, golden):
    """With one temperature on every cell the general integrator computes the
    azimuthally invariant one's signal by another route (per-cell splines of
    Z, mu eta and the geometric factor instead of per-energy profile splines
    with the negative part dropped): they agree to the spline difference."""
    from xpsi_gb300.cellmesh import integrator_for_azimuthal_invariance as az
    f = golden("config1")
    args = list(general_args(golden, "config1"))
    args[10] = f["params"]
    st, flux = gen.integrate(*args)
    st2, ref = az.integrate(*args)
    assert st == st2 == 0
    assert row_rel(flux, ref) <= 2e-3


def test_general_bitwise_reproducible(gen, golden):
    args = general_args(golden, "num4d_omit", mu09=True)
    a = gen.integrate(*args)[1]
    b = gen.integrate(*args)[1]
    np.testing.assert_array_equal(a, b)
