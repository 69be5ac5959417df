"""Run ProjectQ's own simulator test modules against one of our backends."""

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
REF_PY = ROOT / "baseline" / "_ref"
MODULES = ["projectq/backends/_sim/_simulator_test.py", "projectq/tests/_factoring_test.py"]
# NumPy 2 rejects numpy.array(list, copy=False) in the reference test itself
# (_simulator_test.py:562-563); our restated copy of that check runs elsewhere.
DESELECT = ["projectq/backends/_sim/_simulator_test.py::test_simulator_time_evolution[cpp_simulator]",
            "projectq/backends/_sim/_simulator_test.py::test_simulator_time_evolution[py_simulator]"]


def available():
    return all((REF_PY / m).exists() for m in MODULES)


UNITARY_MODULE = "projectq/backends/_unitary_test.py"


def run(backend, precision="c128", fusion="reference", extra=(), unitary=False):
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([str(HERE / "_stubs"), str(REF_PY), str(HERE), str(ROOT),
                                         env.get("PYTHONPATH", "")])
    env.update(GSIM_BACKEND=backend, GSIM_PRECISION=precision, GSIM_FUSION=fusion,
               GSIM_UNITARY="1" if unitary else "0")
    modules = [UNITARY_MODULE] if unitary else MODULES
    cmd = [sys.executable, "-m", "pytest", "-q", "-p", "ref_suite_plugin", "-p", "no:cacheprovider",
           "--rootdir", str(REF_PY), *[str(REF_PY / m) for m in modules]]
    for d in ([] if unitary else DESELECT):
        cmd += ["--deselect", str(REF_PY / d)]
    cmd += list(extra)
    res = subprocess.run(cmd, cwd=str(REF_PY), env=env, capture_output=True, text=True, timeout=1800)
    out = res.stdout + res.stderr
    m = re.search(r"(\d+) passed", out)
    return res.returncode, (int(m.group(1)) if m else 0), out
