"""Construct simulators over the product library, the oracle, or the
reference build, all through projectq_gb300.Simulator's Python surface."""

import ctypes as C
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

from projectq_gb300 import _lib  # noqa: E402
from projectq_gb300.simulator import Simulator  # noqa: E402

ORACLE_LIB = ROOT / "oracle" / "_build" / "liboracle_sim.so"
REF_LIB = ROOT / "oracle" / "_ref" / "libref_sim.so"
# the reference engine built with the flags of ProjectQ's setup.py (the CPU baseline)
REF_SETUP_LIB = ROOT / "oracle" / "_ref" / "libref_sim_setup.so"
STUBS = Path(__file__).resolve().parent / "_stubs"
REF_PY = ROOT / "baseline" / "_ref"

_cache = {}


def build_oracle():
    subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh")], check=True)


def oracle_api():
    if "oracle" not in _cache:
        if not ORACLE_LIB.exists():
            build_oracle()
        _cache["oracle"] = _lib.bind(ORACLE_LIB, "osim_")
    return _cache["oracle"]


def ref_api():
    if "ref" not in _cache:
        _cache["ref"] = _lib.bind(REF_LIB, "rsim_") if REF_LIB.exists() else None
    return _cache["ref"]


def ref_setup_api():
    if "ref_setup" not in _cache:
        _cache["ref_setup"] = _lib.bind(REF_SETUP_LIB, "rsim_") if REF_SETUP_LIB.exists() else None
    return _cache["ref_setup"]


def make(kind, seed=1, precision="c128", fusion="reference"):
    if kind == "gpu":
        return Simulator(seed, precision=precision, fusion=fusion)
    if kind == "oracle":
        return Simulator(seed, fusion=fusion if fusion != "staged" else "reference", _api=oracle_api())
    if kind == "ref":
        return Simulator(seed, _api=ref_api())
    if kind == "ref_setup":
        return Simulator(seed, _api=ref_setup_api())
    raise ValueError(kind)


def projectq_available():
    """Import ProjectQ's Python layers (the installed reference copy) for
    drop-in tests; returns False when they are not present."""
    if REF_PY.exists() and str(REF_PY) not in sys.path:
        sys.path.insert(0, str(STUBS))
        sys.path.insert(0, str(REF_PY))
    try:
        import projectq  # noqa: F401
        from projectq.backends import Simulator as _S  # noqa: F401
    except Exception:
        return False
    return True
