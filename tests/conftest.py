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


def spectrum_rel(a, b):
    """max |a-b| / |b| over the energies where b != 0 (where b == 0 the
    value must be 0 too, else inf)."""
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    nz = b != 0
    if np.any(a[~nz] != 0):
        return float("inf")
    return float(np.max(np.abs(a[nz] / b[nz] - 1.0))) if nz.any() else 0.0


# the photosphere-elsewhere fixture's cases: (parameter key, atm_ext, table)
ELSEWHERE_CASES = ("bb", "num4d", "num4d_mu09")


def elsewhere_atmos(golden, case):
    """The atmosphere argument of an elsewhere fixture case: () for the
    blackbody, else the numerical table num4d_omit.npz stores (for
    num4d_mu09 on a mu grid scaled to [0, 0.9])."""
    if case == "bb":
        return ()
    t = atmos_of(golden("num4d_omit"))
    if case == "num4d_mu09":
        t = (t[0], t[1], np.ascontiguousarray(0.9 * t[2]), t[3], t[4])
    return t


def elsewhere_args(f, case, atmos, threads=1, image_order_limit=None, inclination=None,
                   omega=None):
    """Arguments of integrator_for_time_invariance.integrate for a fixture case."""
    return (threads, float(f["R"]), float(f["Omega"] if omega is None else omega),
            float(f["r_s"]), float(f["inclination"] if inclination is None else inclination),
            int(f["S"]), float(f["cellArea"]), f["radius"], f["u"], f["theta"], f["phi"],
            f[("num4d" if case != "bb" else "bb") + "_params"], int(f["N_R"]),
            f["deflection"], f["cos_alpha"], f["maxDeflection"], f["cos_gamma"],
            f["energies"], atmos, 1 if case == "bb" else 2, image_order_limit)


def general_args(golden, case, threads=1, corrected=False, mu09=False, image_order_limit=None):
    """Arguments of integrator.integrate (the general integrator) for a
    general_integrator.npz case on its base fixture's mesh and rays."""
    f = golden(case)
    g = golden("general_integrator")
    atmos = ()
    if int(f["atm_ext"]) == 2:
        atmos = atmos_of(f)
        if mu09:
            atmos = (atmos[0], atmos[1], np.ascontiguousarray(0.9 * atmos[2]), atmos[3],
                     atmos[4])
    corr = g[case + "_corrected_correction"] if corrected else None
    iol = image_order_limit if image_order_limit is not None else (
        int(f["image_order_limit"]) or None)
    return (threads, float(f["R"]), float(f["Omega"]), float(f["r_s"]),
            float(f["inclination"]), f["cellArea"], f["radius"], f["u"], f["theta"],
            f["phi"], g[case + "_params"], f["radiates"], corr, int(f["N_R"]),
            f["deflection"], f["cos_alpha"], f["lag"], f["maxDeflection"], f["cos_gamma"],
            f["energies"], f["leaves"], f["phases"], atmos, None, int(f["atm_ext"]),
            1 if corrected else None, 0, iol)


# the general-integrator fixture's cases: (base fixture, corrected, mu09, key)
GENERAL_CASES = (("config1", False, False, "config1_flux_threads1"),
                 ("config1", True, False, "config1_corrected_flux_threads1"),
                 ("num4d_omit", False, False, "num4d_omit_flux_threads1"),
                 ("num4d_omit", False, True, "num4d_omit_mu09_flux_threads1"))


def row_rel_floor(a, b, floor=1e-15):
    """row_rel with each energy row's scale floored at `floor` times the
    spectrum's largest value: rows many orders of magnitude below the peak
    (the 4-point Lagrange stencil cancelling in the Num4D table's exponential
    tail, where the reference's own value is rounding residue) are held
    against that floor instead of their own maximum."""
    a = np.asarray(a)
    b = np.asarray(b)
    peak = np.max(np.abs(b))
    scale = np.maximum(np.max(np.abs(b), axis=1, keepdims=True), floor * peak)
    scale = np.where(scale > 0, scale, 1e300)
    return float(np.max(np.abs(a - b) / scale))


# the Stokes fixture's cases: (base fixture, atm_ext, corrected)
STOKES_CASES = (("config1", 3, False), ("num4d_omit", 3, False), ("config1", 1, True))


def stokes_args(golden, case, ext, corrected, image_order_limit=None):
    """Arguments of integratorIQU_for_azimuthal_invariance.integrate for a
    stokes.npz case on its base fixture's mesh and rays."""
    f = golden(case)
    z = golden("stokes")
    tag = "%s_ext%d%s" % (case, ext, "_corrected" if corrected else "")
    corr = z[tag + "_correction"] if corrected else None
    iol = image_order_limit if image_order_limit is not None else (
        int(f["image_order_limit"]) or None)
    return tag, (1, float(f["R"]), float(f["Omega"]), float(f["r_s"]), float(f["inclination"]),
                 f["cellArea"], f["radius"], f["u"], f["theta"], f["phi"], f["params"],
                 f["radiates"], corr, int(f["N_R"]), f["deflection"], f["cos_alpha"], f["lag"],
                 f["maxDeflection"], f["cos_gamma"], f["energies"], f["leaves"], f["phases"],
                 (), (), (), ext, 1 if corrected else None, 0, iol)


# the split fixture's cases: (tag, base fixture)
SPLIT_CASES = (("config1", "config1"), ("num4d_omit", "num4d_omit"),
               ("config1_corrected", "config1"), ("config1_outside", "config1"))


def split_args(golden, tag, case, image_order_limit=None):
    """Arguments of integrator_for_azimuthal_invariance_split.integrate for a
    split.npz case on its base fixture's mesh and rays (uniform (t_e, t_bb,
    tau) over the cells, the table of synthetic.split_table)."""
    from xpsi_gb300 import synthetic
    f = golden(case)
    z = golden("split")
    S = int(f["S"])
    params = np.ones((S, S, 3)) * z[tag + "_vec"]
    corr = z.get(tag + "_correction")
    iol = image_order_limit if image_order_limit is not None else (
        int(f["image_order_limit"]) or None)
    return (1, float(f["R"]), float(f["Omega"]), float(f["r_s"]), float(f["inclination"]),
            f["cellArea"], f["radius"], f["u"], f["theta"], f["phi"], params, f["radiates"],
            corr, int(f["N_R"]), f["deflection"], f["cos_alpha"], f["lag"], f["maxDeflection"],
            f["cos_gamma"], f["energies"], f["leaves"], f["phases"], synthetic.split_table(),
            (), None, 1 if corr is not None else None, 0, iol)


# the Pol_Num2D fixture's cases: (tag, base fixture)
POL2D_CASES = (("config1", "config1"), ("num4d_omit", "num4d_omit"),
               ("config1_corrected", "config1"), ("config1_mu09", "config1"))


def pol2d_args(golden, tag, case, stokes, image_order_limit=None):
    """Arguments of the plain (stokes False) or Stokes integrator for a
    pol_num2d.npz case: atm_ext 4 with synthetic.pol2d_tables on the base
    fixture's mesh and rays."""
    from xpsi_gb300 import synthetic
    f = golden(case)
    z = golden("pol_num2d")
    atm_I, atm_Q = synthetic.pol2d_tables(mu_top=float(z[tag + "_mu_top"]))
    corr = z.get(tag + "_correction")
    iol = image_order_limit if image_order_limit is not None else (
        int(f["image_order_limit"]) or None)
    common = (1, float(f["R"]), float(f["Omega"]), float(f["r_s"]), float(f["inclination"]),
              f["cellArea"], f["radius"], f["u"], f["theta"], f["phi"], f["params"],
              f["radiates"], corr, int(f["N_R"]), f["deflection"], f["cos_alpha"], f["lag"],
              f["maxDeflection"], f["cos_gamma"], f["energies"], f["leaves"], f["phases"])
    atm = (atm_I, atm_Q) if stokes else (atm_I,)
    return common + atm + ((), 4, 1 if corr is not None else None, 0, iol)


def split_iqu_args(golden, tag, case, image_order_limit=None):
    """Arguments of integratorIQU_for_azimuthal_invariance_split.integrate for
    a split_iqu.npz case (synthetic.split_table and split_table_q)."""
    from xpsi_gb300 import synthetic
    a = list(split_args(golden, tag, case, image_order_limit))
    z = golden("split_iqu")
    a[10] = np.ones_like(a[10]) * z[tag + "_vec"]
    a[12] = z.get(tag + "_correction")
    a[25] = 1 if a[12] is not None else None
    return tuple(a[:23]) + (synthetic.split_table_q(),) + tuple(a[23:])


# the general Stokes fixture's cases: (tag, base fixture, atm_ext)
GENERAL_IQU_CASES = (("config1_ext3", "config1", 3), ("num4d_omit_ext3", "num4d_omit", 3),
                     ("config1_ext1_corrected", "config1", 1), ("config1_ext4", "config1", 4),
                     ("num4d_omit_ext4_mu09", "num4d_omit", 4))


def general_iqu_args(golden, tag, case, ext, stokes=True, image_order_limit=None):
    """Arguments of the general Stokes (stokes True) or intensity integrator
    for a general_iqu.npz case on the general integrator's cell-varying
    temperatures."""
    from xpsi_gb300 import synthetic
    f = golden(case)
    z = golden("general_iqu")
    g = golden("general_integrator")
    corr = z.get(tag + "_correction")
    atm_I, atm_Q = (synthetic.pol2d_tables(mu_top=float(z[tag + "_mu_top"])) if ext == 4
                    else ((), ()))
    iol = image_order_limit if image_order_limit is not None else (
        int(f["image_order_limit"]) or None)
    common = (1, float(f["R"]), float(f["Omega"]), float(f["r_s"]), float(f["inclination"]),
              f["cellArea"], f["radius"], f["u"], f["theta"], f["phi"], g[case + "_params"],
              f["radiates"], corr, int(f["N_R"]), f["deflection"], f["cos_alpha"], f["lag"],
              f["maxDeflection"], f["cos_gamma"], f["energies"], f["leaves"], f["phases"])
    atm = (atm_I, atm_Q) if stokes else (atm_I,)
    return common + atm + ((), ext, 1 if corr is not None else None, 0, iol)
