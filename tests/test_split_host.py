"""The oracle's split integrator (integrator_for_azimuthal_invariance_split.pyx
with hot_Num5D_split.pyx and hot_Num2D_split.pyx) against the reference's
own output on the same inputs (tests/golden/split.npz).  CPU only."""
import numpy as np
import pytest

from conftest import SPLIT_CASES, row_rel, split_args
from oracle import oracle as O


@pytest.mark.parametrize("tag,case", SPLIT_CASES)
def test_oracle_split_vs_reference(golden, tag, case):
    st, flux = O.integrate_split(*split_args(golden, tag, case))
    assert st == 0
    ref = golden("split")[tag + "_flux"]
    assert flux.shape == ref.shape
    assert row_rel(flux, ref) <= 1e-13


def test_split_table_is_positive_and_seeded():
    from xpsi_gb300 import synthetic
    a = synthetic.split_table()
    b = synthetic.split_table()
    assert len(a) == 6
    assert a[5].size == np.prod([g.size for g in a[:5]])
    assert (a[5] > 0).all()
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


def test_split_shim_rejects_unsupported_options(golden):
    """The drop-in refuses what the GPU path does not compute, before any
    library call."""
    from xpsi_gb300.cellmesh import integrator_for_azimuthal_invariance_split as S
    args = list(split_args(golden, "config1", "config1"))
    bad = list(args)
    bad[26] = 1  # beam_opt
    with pytest.raises(NotImplementedError):
        S.integrate(*bad)
    bad = list(args)
    bad[22] = bad[22][:5]  # no intensity table
    with pytest.raises(ValueError):
        S.integrate(*bad)
