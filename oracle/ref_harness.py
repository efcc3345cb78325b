"""Import harness for the reference X-PSI package built by build_ref.py.

TEST INFRASTRUCTURE.  Makes `import xpsi` resolve to the reference's own
Python sources (read in place from the reference checkout) plus the
extension modules compiled into oracle/_ref/ against the oracle's GSL-API
subset.  Only the pieces the likelihood path needs are loaded:

* the top-level xpsi/__init__.py is replaced by a module carrying the
  attributes the model classes read (_comm, _rank, _size, _verbose, ...),
  because it imports plotting, post-processing and sampler stacks;
* astropy (FITS I/O only) and pandas/matplotlib users (shell_interpolator)
  are stubbed: they are not on the path;
* numpy 2 removed `numpy.infty`, which the reference evaluates in two
  constructors; it is aliased to `numpy.inf`;
* modules for Stokes integrators (and the closed mesh / time-invariant
  integrator, when they were not built) are stubbed, since the model classes
  import them at construction but the path never calls them.

Available only where the reference checkout exists (not on the GPU host).
"""
import importlib
import importlib.util
import os
import sys
import sysconfig
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILT = os.path.join(HERE, "_ref")


def _reference_path():
    """The checkout: $XPSI_REFERENCE, else the one oracle/build_ref.py built
    from (recorded in oracle/_ref/REFERENCE_PATH), else none."""
    env = os.environ.get("XPSI_REFERENCE")
    if env:
        return env
    try:
        with open(os.path.join(BUILT, "REFERENCE_PATH")) as f:
            return f.read().strip()
    except OSError:
        return ""


REF = _reference_path()


def available():
    return (bool(REF) and os.path.isdir(os.path.join(REF, "xpsi"))
            and os.path.isdir(os.path.join(BUILT, "xpsi", "cellmesh")))


def _stub(name, **attrs):
    m = types.ModuleType(name)
    m.__dict__.update(attrs)
    sys.modules[name] = m
    return m


def _package(name, rel, run_init=True):
    paths = [os.path.join(BUILT, *rel), os.path.join(REF, *rel)]
    init = os.path.join(REF, *rel, "__init__.py")
    if run_init and os.path.exists(init):
        spec = importlib.util.spec_from_file_location(
            name, init, submodule_search_locations=paths)
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    else:
        mod = types.ModuleType(name)
        mod.__path__ = paths
        sys.modules[name] = mod
    parent, _, leaf = name.rpartition(".")
    if parent:
        setattr(sys.modules[parent], leaf, mod)
    return mod


def _effective_gravity(cos_colatitude, R_eq, zeta, epsilon, star_shape="AGM_14"):
    """log10 g_eff [cgs] (surface_radiation_field/core.pyx:517,
    effective_gravity_universal.pyx:10-71), used by the Num4D bounds check."""
    c = 2.99792458e8
    mu = np.asarray(cos_colatitude, dtype=float)
    x = np.asarray(zeta, dtype=float)
    R = np.asarray(R_eq, dtype=float)
    e = np.asarray(epsilon, dtype=float)
    g0 = x * c * c / (R * np.sqrt(1.0 - 2.0 * x))
    c_e = -0.791 + 0.776 * x
    c_p = 1.138 - 1.431 * x
    d_e = (-1.315 + 2.431 * x) * e * x
    d_p = (0.653 - 2.864 * x) * e * x
    d_60 = (13.47 - 27.13 * x) * e * x
    f_e = -1.172 * x * e * e
    f_p = 0.975 * x * e * e
    g = 1.0 + (c_e + d_e + f_e) * e * (1.0 - mu * mu)
    g = g + (c_p + d_p + f_p - d_60) * e * mu * mu + d_60 * e * np.abs(mu)
    if star_shape == "AGM_14":
        return np.log10(g * g0) + 2.0
    return np.log10(g0) + 2.0


_loaded = None


def load():
    """Return the reference `xpsi` package (importing it once)."""
    global _loaded
    if _loaded is not None:
        return _loaded
    if not available():
        raise RuntimeError("reference checkout or oracle/_ref build missing; "
                           "run oracle/build_ref.py")
    if not hasattr(np, "infty"):
        np.infty = np.inf
    # FITS I/O is not on the path
    astropy = _stub("astropy")
    astropy.io = _stub("astropy.io")
    astropy.io.fits = _stub("astropy.io.fits")
    astropy.table = _stub("astropy.table", Table=object)

    xpsi = _package("xpsi", ("xpsi",), run_init=False)
    xpsi.__version__ = "3.3.0"
    xpsi.__XPSI_SETUP__ = True
    xpsi._comm, xpsi._rank, xpsi._size, xpsi._verbose = None, 0, 1, False
    xpsi._warning = lambda msg: None
    gi = importlib.import_module("xpsi.global_imports")
    xpsi.global_imports = gi

    _package("xpsi.tools", ("xpsi", "tools"))
    tools = sys.modules["xpsi.tools"]
    tools.set_phase_interpolant("Akima")
    tools.set_energy_interpolant("Steffen")
    srf = _package("xpsi.surface_radiation_field", ("xpsi", "surface_radiation_field"),
                   run_init=False)
    srf.effective_gravity = _effective_gravity
    _package("xpsi.cellmesh", ("xpsi", "cellmesh"))
    _package("xpsi.likelihoods", ("xpsi", "likelihoods"))

    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    for name in ("integratorIQU_for_azimuthal_invariance", "integratorIQU",
                 "integrator_for_azimuthal_invariance_split",
                 "integratorIQU_for_azimuthal_invariance_split",
                 "global_mesh", "integrator_for_time_invariance"):
        if os.path.exists(os.path.join(BUILT, "xpsi", "cellmesh", name + suffix)):
            continue
        _stub("xpsi.cellmesh." + name, integrate=None,
              construct_closed_cellMesh=None)
    _stub("xpsi.shell_interpolator", Temp_Interpolator_shells=None)

    for name in ("Parameter", "ParameterSubspace", "Spacetime", "HotRegion",
                 "HotRegions", "Elsewhere", "Everywhere", "Photosphere", "Star",
                 "Instrument", "Data", "Signal", "Background", "Interstellar",
                 "EmissionModels", "Prior", "Likelihood"):
        mod = importlib.import_module("xpsi." + name)
        setattr(xpsi, name, mod)
    from xpsi.Parameter import Parameter, Derive
    from xpsi.ParameterSubspace import ParameterSubspace
    xpsi.Parameter, xpsi.Derive, xpsi.ParameterSubspace = Parameter, Derive, ParameterSubspace
    for cls_mod, cls in (("Likelihood", "Likelihood"), ("Data", "Data"),
                         ("Instrument", "Instrument"), ("Signal", "Signal"),
                         ("Star", "Star"), ("Spacetime", "Spacetime"),
                         ("Photosphere", "Photosphere"), ("HotRegion", "HotRegion"),
                         ("HotRegions", "HotRegions"), ("Elsewhere", "Elsewhere"),
                         ("Everywhere", "Everywhere"), ("Background", "Background"),
                         ("Interstellar", "Interstellar"), ("Prior", "Prior")):
        setattr(xpsi, cls, getattr(sys.modules["xpsi." + cls_mod], cls))
    _loaded = xpsi
    return xpsi


def examples_fast_modules():
    """Put the reference's examples_fast model modules on sys.path."""
    p = os.path.join(REF, "examples", "examples_fast", "Modules")
    if p not in sys.path:
        sys.path.insert(0, p)
    return p
