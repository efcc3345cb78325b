import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "reference: needs the reference checkout and its build")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as f:
        return {k: f[k] for k in f.files}


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = load_golden(name)
        return cache[name]
    return get


def row_rel(a, b):
    """max |a-b| relative to the max |b| of each energy row (rows of zeros
    must match to 1e-300 absolute)."""
    a = np.asarray(a)
    b = np.asarray(b)
    scale = np.max(np.abs(b), axis=1, keepdims=True)
    scale = np.where(scale > 0, scale, 1e300)
    return float(np.max(np.abs(a - b) / scale))


def atmos_of(f):
    return (f["atm_logT"], f["atm_logg"], f["atm_mu"], f["atm_logE"], f["atm_I"])
