"""Drop-in for xpsi.tools.energy_interpolator.energy_interpolator
(xpsi/tools/energy_interpolator.pyx:27-125) on the GPU."""
import numpy as np

from .._arr import f64, ptr
from .._interp import require_default_interpolants
from .._native import check, lib


def energy_interpolator(N_Ts, signal, energies, new_energies):
    """[len(new_energies), columns]: each column of `signal` [energies,
    columns] splined (Steffen) in log10 E -- in log10 of the signal when the
    column is positive throughout -- at `new_energies` (log10); zero above
    the last energy.  N_Ts (the reference's thread count) is not used."""
    require_default_interpolants(phase=False, energy=True)
    S = f64(signal)
    E = f64(energies)
    nE = f64(new_energies)
    if S.ndim != 2 or S.shape[0] != E.size:
        raise ValueError("signal must be [len(energies), columns]")
    out = np.empty((nE.size, S.shape[1]))
    check(lib().xgpu_energy_interpolator(E.size, S.shape[1], ptr(S), ptr(E), nE.size, ptr(nE),
                                         ptr(out)))
    return out
