"""Beaming options 1-3 of the hot intensity (hot_wrapper.pyx:153-199)
through the drop-in integrator against the reference's own integrator on
the same inputs (tests/golden/beaming.npz): the small plain configuration's
blackbody spot and the Num4D spot with an omitted crescent at 600 Hz, the
cell vectors carrying (abb, bbb, cbb, dbb, nimu) in columns 2-6.  Each
energy row within 1e-9 of its largest value."""
import numpy as np
import pytest

from conftest import load_golden, row_rel
from xpsi_gb300.cellmesh import integrator_for_azimuthal_invariance as I

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _run(f, prm, opt):
    atm = ((f["atm_logT"], f["atm_logg"], f["atm_mu"], f["atm_logE"], f["atm_I"])
           if "atm_I" in f else ())
    return I.integrate(1, float(f["R"]), float(f["Omega"]), float(f["r_s"]),
                       float(f["inclination"]), f["cellArea"], f["radius"], f["u"], f["theta"],
                       f["phi"], prm, f["radiates"], None, int(f["N_R"]), f["deflection"],
                       f["cos_alpha"], f["lag"], f["maxDeflection"], f["cos_gamma"],
                       f["energies"], f["leaves"], f["phases"], atm, None, int(f["atm_ext"]),
                       None, opt, int(f["image_order_limit"]) or None)


@pytest.mark.parametrize("case", ["config1", "num4d_omit"])
@pytest.mark.parametrize("opt", [0, 1, 2, 3])
def test_beaming_vs_reference(cuda, case, opt):
    f = load_golden(case)
    b = load_golden("beaming")
    prm = np.ascontiguousarray(np.concatenate(
        [f["params"], np.broadcast_to(b["beam_params"], f["params"].shape[:2] + (5,))], axis=2))
    st, flux = _run(f, prm, opt)
    assert st == 0
    ref = f["flux"] if opt == 0 else b[f"{case}_opt{opt}"]
    assert row_rel(flux, ref) <= 1e-9
