"""pytest plugin: serve ``projectq.backends._sim._cppsim`` from this project.

Loaded with ``-p ref_suite_plugin`` when running ProjectQ's own test modules
(projectq/backends/_sim/_simulator_test.py, projectq/tests/_factoring_test.py):
their "cpp_simulator" parametrisation then constructs our engine exactly where
it would construct the reference's pybind11 class.

Environment:
  GSIM_BACKEND    "gpu" (default; libgb300sim.so) or "oracle" (CPU restatement)
  GSIM_PRECISION  "c128" (default) or "c64"
  GSIM_FUSION     "reference" (default), "none" or "staged"
  GSIM_UNITARY    "1": also serve projectq.backends.UnitarySimulator
                  (backends/_unitary.py) from projectq_gb300.unitary
"""

import os
import sys
import types


def pytest_configure(config):
    backend = os.environ.get("GSIM_BACKEND", "gpu")
    prec = os.environ.get("GSIM_PRECISION", "c128")
    fusion = os.environ.get("GSIM_FUSION", "reference")
    from projectq_gb300 import Simulator

    from _backends import oracle_api

    if backend == "oracle":
        api = oracle_api()

        def factory(seed=1, *args):
            return Simulator(seed, _api=api)
    else:

        def factory(seed=1, *args):
            return Simulator(seed, precision=prec, fusion=fusion)

    mod = types.ModuleType("projectq.backends._sim._cppsim")
    mod.Simulator = factory
    mod.__file__ = __file__
    sys.modules["projectq.backends._sim._cppsim"] = mod
    import projectq.backends._sim as pkg

    pkg._cppsim = mod
    if os.environ.get("GSIM_UNITARY") == "1":
        import projectq.backends as backends
        import projectq.backends._unitary as umod
        from projectq_gb300.unitary import UnitarySimulator

        uapi = oracle_api() if backend == "oracle" else None

        class ServedUnitarySimulator(UnitarySimulator):
            def __init__(self):
                super().__init__(precision=prec, _api=uapi)

        umod.UnitarySimulator = ServedUnitarySimulator
        backends.UnitarySimulator = ServedUnitarySimulator
