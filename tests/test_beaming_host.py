"""Argument checks of the drop-in integrator's beaming options, made before
any GPU call (CPU only): options 1-3 need the five beaming parameters in
the cell vectors, option 3 takes the blackbody or Num4D atmosphere, and an
unknown option is rejected."""
import numpy as np
import pytest

from conftest import load_golden
from test_gpu_beaming import _run


def test_beaming_needs_the_parameters():
    f = load_golden("config1")
    with pytest.raises(ValueError):
        _run(f, f["params"], 1)


def test_unknown_option():
    f = load_golden("config1")
    with pytest.raises(ValueError):
        _run(f, f["params"], 4)


def test_option_3_atmospheres():
    f = dict(load_golden("config1"))
    f["atm_ext"] = np.array(3)
    prm = np.concatenate([f["params"], np.ones(f["params"].shape[:2] + (5,))], axis=2)
    with pytest.raises(NotImplementedError):
        _run(f, prm, 3)
