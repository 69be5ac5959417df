"""GB300 (sm_103a) state-vector simulator core for ProjectQ.

A drop-in for the native engine behind ``projectq.backends.Simulator``
(``projectq.backends._sim._cppsim.Simulator``): the CUDA library
``libgb300sim.so`` behind the C ABI of ``include/gb300sim.h``, and the Python
class `Simulator` with the reference engine's method surface.
"""

from ._lib import load as load_library  # noqa: F401
from .simulator import Simulator  # noqa: F401

__all__ = ["Simulator", "load_library"]
