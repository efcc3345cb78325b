"""Drop-in for xpsi.tools.energy_integrator (xpsi/tools/energy_integrator.pyx:27-114)."""
import numpy as np

from .._arr import f64, ptr
from .._interp import require_default_interpolants
from .._native import check, lib


def energy_integrator(N_Ts, signal, energies, energy_edges):
    """Integrate a signal over energy intervals on the GPU.

    signal[N_E, N_P] (energy increases with row), log10 energies and log10
    interval edges; returns [len(edges)-1, N_P] like the reference.
    """
    require_default_interpolants(phase=True, energy=False)
    S = f64(signal)
    E = f64(energies)
    ed = f64(energy_edges)
    out = np.zeros((ed.size - 1, S.shape[1]))
    check(lib().xgpu_energy_integrator(E.size, S.shape[1], ptr(S), ptr(E), ed.size, ptr(ed),
                                       ptr(out)))
    return out
