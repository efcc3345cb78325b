"""GB300-native pulse-likelihood hot path for X-PSI.

Drop-in replacements for the native callables on X-PSI's likelihood path
(same names, arguments, return values and error statuses), backed by
hand-written sm_103a CUDA kernels behind the C ABI in include/xpsi_gb300.h:

    xpsi_gb300.cellmesh.rays.compute_rays
    xpsi_gb300.cellmesh.mesh.{construct_spot_cellMesh, construct_polar_cellMesh,
                              allocate_cells}         (host C++, threaded)
    xpsi_gb300.cellmesh.integrator_for_azimuthal_invariance.integrate
    xpsi_gb300.cellmesh.integrator.integrate          (HotRegion symmetry=False)
    xpsi_gb300.cellmesh.integratorIQU.integrate       (the same, Stokes)
    xpsi_gb300.cellmesh.integrator_for_azimuthal_invariance_split.integrate
    xpsi_gb300.cellmesh.integratorIQU_for_azimuthal_invariance_split.integrate
                                                      (HotRegion split=True)
    xpsi_gb300.cellmesh.integratorIQU_for_azimuthal_invariance.integrate (Stokes)
    xpsi_gb300.cellmesh.global_mesh.construct_closed_cellMesh   (elsewhere)
    xpsi_gb300.cellmesh.integrator_for_time_invariance.integrate (elsewhere)
    xpsi_gb300.tools.energy_integrator.energy_integrator
    xpsi_gb300.tools.phase_integrator.phase_integrator
    xpsi_gb300.tools.{phase_interpolator,energy_interpolator}
    xpsi_gb300.tools.synthesise.{synthesise_exposure,
                                 synthesise_given_total_count_number}
    xpsi_gb300.likelihoods.default_background_marginalisation.{precomputation,
                                                              eval_marginal_likelihood}
    xpsi_gb300.instrument.fold        (Instrument.__call__'s matrix product)

`install(xpsi)` rebinds them inside an imported X-PSI package, and
`xpsi_gb300.batch` evaluates many parameter vectors per launch.
"""
from ._native import GPUError, build, lib  # noqa: F401

__version__ = "0.1.0"


def install(xpsi_module):
    """Route an imported X-PSI package's likelihood path through the GPU.

    Rebinds the module-level callables that X-PSI's model classes import
    (HotRegion.py:3-6 and :557-572, Signal.py:10, CustomSignal modules) so
    that Likelihood.__call__ runs the CUDA kernels.  Returns the list of
    rebound names.
    """
    import importlib
    from .cellmesh import rays, integrator_for_azimuthal_invariance as integ
    from .cellmesh import global_mesh, integrator_for_time_invariance as tinv
    from .cellmesh import mesh as hot_mesh
    from .cellmesh import integrator as general
    from .cellmesh import integratorIQU as general_iqu
    from .cellmesh import integrator_for_azimuthal_invariance_split as split
    from .cellmesh import integratorIQU_for_azimuthal_invariance_split as iqu_split
    from .cellmesh import integratorIQU_for_azimuthal_invariance as iqu
    from .tools import energy_integrator as ei
    from .tools import phase_integrator as pint, synthesise as syn
    from .tools import phase_interpolator as pinterp, energy_interpolator as einterp
    from .likelihoods import default_background_marginalisation as dbm
    from .likelihoods import _gaussian_likelihood_given_background_IQU as gbg
    from .likelihoods import _gaussian_likelihood_QnUn as gqu
    done = []
    targets = [
        ("xpsi.cellmesh.rays", "compute_rays", rays.compute_rays),
        ("xpsi.cellmesh.mesh_tools", "allocate_cells", hot_mesh.allocate_cells),
        ("xpsi.cellmesh.mesh", "construct_spot_cellMesh", hot_mesh.construct_spot_cellMesh),
        ("xpsi.cellmesh.polar_mesh", "construct_polar_cellMesh",
         hot_mesh.construct_polar_cellMesh),
        ("xpsi.cellmesh.integrator_for_azimuthal_invariance", "integrate", integ.integrate),
        ("xpsi.tools.energy_integrator", "energy_integrator", ei.energy_integrator),
        ("xpsi.likelihoods.default_background_marginalisation", "eval_marginal_likelihood",
         dbm.eval_marginal_likelihood),
        ("xpsi.likelihoods.default_background_marginalisation", "precomputation",
         dbm.precomputation),
        ("xpsi.cellmesh.global_mesh", "construct_closed_cellMesh",
         global_mesh.construct_closed_cellMesh),
        ("xpsi.cellmesh.integrator_for_time_invariance", "integrate", tinv.integrate),
        ("xpsi.cellmesh.integrator", "integrate", general.integrate),
        ("xpsi.cellmesh.integratorIQU", "integrate", general_iqu.integrate),
        ("xpsi.cellmesh.integrator_for_azimuthal_invariance_split", "integrate",
         split.integrate),
        ("xpsi.cellmesh.integratorIQU_for_azimuthal_invariance_split", "integrate",
         iqu_split.integrate),
        ("xpsi.cellmesh.integratorIQU_for_azimuthal_invariance", "integrate", iqu.integrate),
        ("xpsi.tools.phase_integrator", "phase_integrator", pint.phase_integrator),
        ("xpsi.tools.phase_interpolator", "phase_interpolator", pinterp.phase_interpolator),
        ("xpsi.tools.energy_interpolator", "energy_interpolator",
         einterp.energy_interpolator),
        ("xpsi.likelihoods._gaussian_likelihood_given_background_IQU",
         "gaussian_likelihood_given_background", gbg.gaussian_likelihood_given_background),
        ("xpsi.likelihoods._gaussian_likelihood_QnUn", "gaussian_likelihood_QnUn",
         gqu.gaussian_likelihood_QnUn),
        ("xpsi.tools.synthesise", "synthesise_exposure", syn.synthesise_exposure),
        ("xpsi.tools.synthesise", "synthesise_given_total_count_number",
         syn.synthesise_given_total_count_number),
    ]
    for modname, attr, fn in targets:
        try:
            mod = importlib.import_module(modname)
        except ImportError:
            continue
        setattr(mod, attr, fn)
        done.append(modname + "." + attr)
    # names bound at import time by the model classes
    for modname, attr, fn in (("xpsi.HotRegion", "_compute_rays", rays.compute_rays),
                              ("xpsi.HotRegion", "_allocate_cells", hot_mesh.allocate_cells),
                              ("xpsi.HotRegion", "_construct_spot_cellMesh",
                               hot_mesh.construct_spot_cellMesh),
                              ("xpsi.HotRegion", "_construct_polar_cellMesh",
                               hot_mesh.construct_polar_cellMesh),
                              ("xpsi.Signal", "energy_integrator", ei.energy_integrator),
                              ("xpsi.Signal", "phase_integrator", pint.phase_integrator),
                              ("xpsi.Signal", "_synthesise_expo", syn.synthesise_exposure),
                              ("xpsi.Signal", "_synthesise_given_total_count_number",
                               syn.synthesise_given_total_count_number),
                              ("xpsi.Elsewhere", "_compute_rays", rays.compute_rays),
                              ("xpsi.Elsewhere", "_construct_closed_cellMesh",
                               global_mesh.construct_closed_cellMesh),
                              ("xpsi.Elsewhere", "_integrator", tinv.integrate),
                              ("xpsi.PostProcessing._pulse", "interp",
                               pinterp.phase_interpolator),
                              ("xpsi.PostProcessing._spectrum", "interp",
                               pinterp.phase_interpolator),
                              ("xpsi.PostProcessing._spectrum", "energy_interpolator",
                               einterp.energy_interpolator)):
        try:
            mod = importlib.import_module(modname)
        except ImportError:
            continue
        setattr(mod, attr, fn)
        done.append(modname + "." + attr)
    HotRegion = importlib.import_module("xpsi.HotRegion").HotRegion
    orig = HotRegion.symmetry.fset

    def _symmetry(self, declaration, _orig=orig):
        _orig(self, declaration)
        if not getattr(self, "_split", False):
            self._integrator = integ.integrate if declaration else general.integrate
            self._integratorIQU = iqu.integrate if declaration else general_iqu.integrate
        elif declaration:
            # split=True and symmetry=False raise in the original setter
            self._integrator = split.integrate
            self._integratorIQU = iqu_split.integrate
    HotRegion.symmetry = property(HotRegion.symmetry.fget, _symmetry)
    done.append("xpsi.HotRegion.HotRegion.symmetry")
    return done
