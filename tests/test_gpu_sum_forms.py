"""The FP64 integrator's two forms of the cell x phase sums -- the per-cell
form (the default) and the power sums over runs of cells
(XGPU_CELL_SUMS=runs) -- give the same fluxes to round-off (1e-12 of each
energy row's largest value) on the small Num4D and blackbody batches, the
latter with an omitted crescent and polar caps among the members."""
import os
import subprocess
import sys

import numpy as np
import pytest

from batch_cases import small_blackbody, small_num4d
from conftest import ROOT, row_rel

pytestmark = pytest.mark.gpu

_CHILD = r"""
import json, sys
sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
import numpy as np, torch
from batch_cases import small_blackbody, small_num4d
from xpsi_gb300 import batch as BT
m, params = {builder}()
ev = BT.BatchEvaluator(m)
B = ev.upload(BT.prepare(m, params))
ev.run(B)
torch.cuda.synchronize()
np.save({out!r}, B["flux"].cpu().numpy())
"""


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("builder", ["small_num4d", "small_blackbody"])
def test_power_sums_equal_cell_sums(cuda, tmp_path, builder):
    assert os.environ.get("XGPU_CELL_SUMS", "cells") == "cells"
    from xpsi_gb300 import batch as BT
    out = str(tmp_path / "runs.npy")
    code = _CHILD.format(root=ROOT, tests=os.path.join(ROOT, "tests"), builder=builder, out=out)
    env = dict(os.environ, XGPU_CELL_SUMS="runs")
    subprocess.run([sys.executable, "-c", code], check=True, env=env, timeout=600)
    m, params = {"small_num4d": small_num4d, "small_blackbody": small_blackbody}[builder]()
    ev = BT.BatchEvaluator(m)
    B = ev.upload(BT.prepare(m, params))
    ev.run(B)
    cuda.cuda.synchronize()
    fc = B["flux"].cpu().numpy()
    fw = np.load(out)
    assert np.abs(fc).max() > 0
    for i in range(fw.shape[0]):
        assert row_rel(fw[i], fc[i]) <= 1e-12
