"""CPU checks of the C ABI: the product library builds, loads and exports
every entry point declared in include/gb300sim.h; without a GPU it reports
the missing device as an error status instead of crashing."""

import ctypes as C
import re
from pathlib import Path

import pytest

from projectq_gb300 import _lib
from projectq_gb300 import build as build_mod

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "gb300sim.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(gsim_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    path = build_mod.build()
    return C.CDLL(str(path))


def test_header_declares_the_reference_surface():
    names = declared_symbols()
    # _cppsim.Simulator's 19 methods (projectq/backends/_sim/_cppsim.cpp:45-66)
    for n in ["create", "allocate_qubit", "deallocate_qubit", "get_classical_value", "is_classical",
              "measure_qubits", "apply_controlled_gate", "emulate_math_table", "emulate_math_add_constant",
              "emulate_math_add_constant_modn", "emulate_math_multiply_by_constant_modn",
              "get_expectation_value", "apply_qubit_operator", "emulate_time_evolution", "get_probability",
              "get_amplitude", "set_wavefunction", "collapse_wavefunction", "run", "get_state", "get_mapping"]:
        assert "gsim_" + n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_the_abi():
    names = {s[len("gsim_"):] for s in declared_symbols()}
    bound = set(_lib.SIGNATURES) | set(_lib.PRODUCT_ONLY)
    assert names == bound, names ^ bound


def test_no_gpu_is_an_error_status_not_a_crash(lib):
    api = _lib.bind(build_mod.LIB, "gsim_", _lib.PRODUCT_ONLY)
    if api.device_count() > 0:
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = api.create(1, _lib.GSIM_C128, C.byref(h))
    assert rc == _lib.GSIM_ERR_CUDA
    assert b"device" in api.last_error()
    with pytest.raises(RuntimeError):
        _lib.check(api, rc)
