"""Host logic of the serving loop: request streams and batch packing."""
import numpy as np

from batch_cases import small_num4d
from xpsi_gb300 import batch as BT
from xpsi_gb300.serving import poisson_stream


def test_poisson_stream_sizes():
    s = poisson_stream(200.0, 2.0, 4096, seed=5)
    assert 250 < len(s) < 550
    sizes = np.array([v for _, v in s])
    assert sizes.min() >= 1 and sizes.max() <= 4096
    times = np.array([t for t, _ in s])
    assert (np.diff(times) > 0).all()


def test_concat_prepared_equals_joint_prepare():
    m, params = small_num4d(V=4)
    a = BT.prepare(m, params[:1])
    b = BT.prepare(m, params[1:])
    c = BT.concat_prepared([a, b], m)
    j = BT.prepare(m, params)
    assert c.V == j.V and c.n_rows == j.n_rows and c.n_cells == j.n_cells
    for k in j.row:
        np.testing.assert_array_equal(c.row[k], j.row[k])
    np.testing.assert_array_equal(c.cellArea, j.cellArea)
    np.testing.assert_array_equal(c.row_mesh, j.row_mesh)
    np.testing.assert_array_equal(c.shifts, j.shifts)
    for i in range(len(j.meshes)):
        x, y = c.meshes[i], j.meshes[i]
        assert (x.S0, x.row_off, x.cell_off, x.flux_off) == (y.S0, y.row_off, y.cell_off,
                                                              y.flux_off)
