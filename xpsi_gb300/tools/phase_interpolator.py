"""Drop-in for xpsi.tools.phase_interpolator.phase_interpolator
(xpsi/tools/phase_interpolator.pyx:25-95) on the GPU."""
import numpy as np

from .._arr import f64, ptr
from .._interp import require_default_interpolants
from .._native import check, lib


def phase_interpolator(new_phases, phases, signal, phase_shift, allow_negative=0):
    """[rows, len(new_phases)]: each row of `signal` (Akima periodic on
    `phases`, cycles in [0, 1]) at new_phases + phase_shift wrapped into
    [0, 1); values <= 0 are 0 unless allow_negative."""
    require_default_interpolants(phase=True, energy=False)
    nf = f64(new_phases)
    ph = f64(phases)
    S = f64(signal)
    if S.ndim != 2 or S.shape[1] != ph.size:
        raise ValueError("signal must be [rows, len(phases)]")
    out = np.empty((S.shape[0], nf.size))
    check(lib().xgpu_phase_interpolator(nf.size, ptr(nf), ph.size, ptr(ph), S.shape[0], ptr(S),
                                        float(phase_shift), int(bool(allow_negative)),
                                        ptr(out)))
    return out
