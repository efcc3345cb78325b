"""The split integrator on the GPU (through the C ABI) against the
reference's own output (tests/golden/split.npz) and the oracle: every energy
row to 1e-9 of its largest value, the integrator's bar."""
import numpy as np
import pytest

from conftest import SPLIT_CASES, row_rel, split_args
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-9


@pytest.fixture(scope="module")
def split():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import xpsi_gb300
    xpsi_gb300.lib()
    from xpsi_gb300.cellmesh import integrator_for_azimuthal_invariance_split
    return integrator_for_azimuthal_invariance_split


@pytest.mark.parametrize("tag,case", SPLIT_CASES)
def test_split_vs_reference(split, golden, tag, case):
    st, flux = split.integrate(*split_args(golden, tag, case))
    assert st == 0
    assert row_rel(flux, golden("split")[tag + "_flux"]) <= RTOL


@pytest.mark.parametrize("image_order_limit", [1, 2])
def test_split_vs_oracle_image_orders(split, golden, image_order_limit):
    args = split_args(golden, "num4d_omit", "num4d_omit", image_order_limit)
    ref = O.integrate_split(*args)
    out = split.integrate(*args)
    assert out[0] == ref[0] == 0
    assert row_rel(out[1], ref[1]) <= RTOL


def test_split_reduction_vs_oracle_on_a_uniform_slab(split, golden):
    """A table constant along (t_e, t_bb, tau) reduces to its (mu, E) slice
    exactly wherever the vector lies, so the split integrator equals itself
    on the slice-replicated table whatever (t_e, t_bb, tau)."""
    from xpsi_gb300 import synthetic
    g = synthetic.split_table()
    n = [x.size for x in g[:5]]
    I = g[5].reshape(n)
    flat = np.ascontiguousarray(np.broadcast_to(I[:1, :1, :1], n)).reshape(-1)
    args = list(split_args(golden, "config1", "config1"))
    args[22] = g[:5] + (flat,)
    a = split.integrate(*args)[1]
    args[10] = np.ones_like(args[10]) * np.array([1.0, 0.005, 2.9])
    b = split.integrate(*args)[1]
    assert row_rel(a, b) <= 1e-12
