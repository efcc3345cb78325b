"""Drop-in for xpsi.tools.phase_integrator.phase_integrator
(xpsi/tools/phase_integrator.pyx:23-121) on the GPU."""
import numpy as np

from .._arr import f64, ptr
from .._interp import require_default_interpolants
from .._native import check, lib


def phase_integrator(exposure_time, phases, signal, signal_phases, phase_shift,
                     allow_negative=0):
    """[rows, len(phases) - 1]: each row of `signal` integrated over the
    phase-shifted intervals (Akima periodic), times the exposure time."""
    require_default_interpolants(phase=True, energy=False)
    ph = f64(phases)
    S = f64(signal)
    sp = f64(signal_phases)
    if S.ndim != 2 or S.shape[1] != sp.size:
        raise ValueError("signal must be [rows, len(signal_phases)]")
    out = np.empty((S.shape[0], ph.size - 1))
    check(lib().xgpu_phase_integrator(float(exposure_time), ph.size, ptr(ph), S.shape[0],
                                      S.shape[1], ptr(S), ptr(sp), float(phase_shift),
                                      int(bool(allow_negative)), ptr(out)))
    return out
