"""The interpolants the GPU path implements, checked against X-PSI's global
settings (xpsi/tools/core.pyx: set_phase_interpolant, default Akima periodic;
set_energy_interpolant, default Steffen).  A drop-in whose reference reads a
setting refuses any other choice instead of computing with the default."""
import sys

_NAMES = {0: "Akima", 1: "Steffen", 2: "Cubic"}


def require_default_interpolants(phase=True, energy=False):
    core = sys.modules.get("xpsi.tools.core")
    if core is None:
        return
    if phase:
        v = getattr(core, "__phase_interpolant__", 0)
        if v != 0:
            raise NotImplementedError(
                "the GPU path splines in phase with the Akima periodic interpolant only "
                "(X-PSI's phase interpolant is set to %r)" % _NAMES.get(v, v))
    if energy:
        v = getattr(core, "__energy_interpolant__", 1)
        if v != 1:
            raise NotImplementedError(
                "the GPU path splines in energy with the Steffen interpolant only "
                "(X-PSI's energy interpolant is set to %r)" % _NAMES.get(v, v))
