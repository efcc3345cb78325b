"""xpsi_gb300.install rebinds the native callables inside the reference
package (imported from its checkout through oracle/ref_harness.py; skipped
where the checkout is absent).  CPU only: no compute call is made."""
import pytest

from oracle import ref_harness as H

pytestmark = pytest.mark.skipif(not H.available(), reason="reference checkout not present")


def test_install_rebinds_path_callables():
    import importlib
    xpsi = H.load()
    import xpsi_gb300
    from xpsi_gb300.cellmesh import (global_mesh, integrator, integrator_for_azimuthal_invariance,
                                     integrator_for_time_invariance,
                                     integratorIQU_for_azimuthal_invariance, rays)
    from xpsi_gb300.tools import energy_integrator, phase_integrator, synthesise
    done = xpsi_gb300.install(xpsi)
    assert "xpsi.Elsewhere._integrator" in done
    E = importlib.import_module("xpsi.Elsewhere")
    assert E._integrator is integrator_for_time_invariance.integrate
    assert E._construct_closed_cellMesh is global_mesh.construct_closed_cellMesh
    assert E._compute_rays is rays.compute_rays
    S = importlib.import_module("xpsi.Signal")
    assert S.energy_integrator is energy_integrator.energy_integrator
    assert S.phase_integrator is phase_integrator.phase_integrator
    assert S._synthesise_expo is synthesise.synthesise_exposure
    assert S._synthesise_given_total_count_number is synthesise.synthesise_given_total_count_number
    assert importlib.import_module("xpsi.HotRegion")._compute_rays is rays.compute_rays
    from xpsi_gb300.cellmesh import mesh as hot_mesh
    HRm = importlib.import_module("xpsi.HotRegion")
    assert HRm._allocate_cells is hot_mesh.allocate_cells
    assert HRm._construct_spot_cellMesh is hot_mesh.construct_spot_cellMesh
    assert HRm._construct_polar_cellMesh is hot_mesh.construct_polar_cellMesh
    # the symmetry setter picks the GPU integrators
    HR = importlib.import_module("xpsi.HotRegion").HotRegion
    hr = object.__new__(HR)
    hr._split = False
    hr.symmetry = True
    assert hr._integrator is integrator_for_azimuthal_invariance.integrate
    assert hr._integratorIQU is integratorIQU_for_azimuthal_invariance.integrate
    hr.symmetry = False
    assert hr._integrator is integrator.integrate
    from xpsi_gb300.cellmesh import integratorIQU
    assert hr._integratorIQU is integratorIQU.integrate


def test_install_binds_split_integrator():
    import importlib
    xpsi = H.load()
    import xpsi_gb300
    from xpsi_gb300.cellmesh import integrator_for_azimuthal_invariance_split as split
    from xpsi_gb300.cellmesh import integratorIQU_for_azimuthal_invariance_split as iqu_split
    done = xpsi_gb300.install(xpsi)
    HR = importlib.import_module("xpsi.HotRegion").HotRegion
    hr = object.__new__(HR)
    hr._split = True
    hr.symmetry = True
    assert hr._integrator is split.integrate
    assert hr._integratorIQU is iqu_split.integrate
    if "xpsi.cellmesh.integrator_for_azimuthal_invariance_split.integrate" in done:
        mod = importlib.import_module("xpsi.cellmesh.integrator_for_azimuthal_invariance_split")
        assert mod.integrate is split.integrate


def test_drop_ins_refuse_other_interpolants():
    """X-PSI's global interpolant settings (tools/core.pyx) other than the
    defaults are refused, not silently replaced by the defaults."""
    import numpy as np
    H.load()
    import xpsi.tools.core as core
    from xpsi_gb300.tools import energy_interpolator, phase_interpolator
    try:
        core.set_phase_interpolant("Steffen")
        with pytest.raises(NotImplementedError):
            phase_interpolator.phase_interpolator(np.zeros(3), np.linspace(0, 1, 8),
                                                  np.zeros((2, 8)), 0.0)
        core.set_phase_interpolant("Akima")
        core.set_energy_interpolant("Cubic")
        with pytest.raises(NotImplementedError):
            energy_interpolator.energy_interpolator(1, np.ones((5, 3)), np.arange(5.0),
                                                    np.arange(2.0))
    finally:
        core.set_phase_interpolant("Akima")
        core.set_energy_interpolant("Steffen")
