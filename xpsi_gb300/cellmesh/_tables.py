"""Host-side packing of numerical atmosphere tables for the C ABI: the 2-D
tables of Pol_Num2D (hot_Num2D.pyx) and the 5-D split tables
(hot_Num5D_split.pyx), with the arrays kept alive beside the structs."""
import ctypes as C

import numpy as np

from .._arr import f64
from .._native import Atmos4D, Atmos5D


def table2d(preloaded, name="hot_atmosphere"):
    """(struct, keep) for a preloaded 2-D table (mu, log10 E/keV, values)."""
    if not preloaded or len(preloaded) < 3:
        raise ValueError("%s: the 2-D table (mu, logE, values) was not preloaded" % name)
    mu, lgE, v = (f64(x) for x in preloaded[:3])
    if v.size != mu.size * lgE.size:
        raise ValueError("%s: table has %d values, grids give %d"
                         % (name, v.size, mu.size * lgE.size))
    s = Atmos4D(None, None, mu.ctypes.data, lgE.ctypes.data, v.ctypes.data, 0, 0,
                mu.size, lgE.size, None)
    return s, (mu, lgE, v)


def table5d(preloaded, name="hot_atmosphere"):
    """(struct, keep) for a preloaded split table (5 grids, values)."""
    if not preloaded or len(preloaded) < 6:
        raise ValueError("%s: split atmosphere data (5 grids and the values) were not "
                         "preloaded" % name)
    grids = tuple(f64(g) for g in preloaded[:5])
    v = f64(preloaded[5])
    n = [g.size for g in grids]
    if v.size != int(np.prod(n)):
        raise ValueError("%s: split table has %d values, grids give %d"
                         % (name, v.size, int(np.prod(n))))
    s = Atmos5D((C.c_void_p * 5)(*(g.ctypes.data for g in grids)), (C.c_size_t * 5)(*n),
                v.ctypes.data)
    return s, grids + (v,)


def same_grids(a, b, dims):
    """Whether two preloaded tables share their grids on `dims`."""
    return all(np.array_equal(f64(a[d]), f64(b[d])) for d in dims)
