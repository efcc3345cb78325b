"""numpy helpers for the C ABI: contiguous float64/int32 views and pointers."""
import ctypes as C

import numpy as np


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)
