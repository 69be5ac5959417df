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


def test_launch_features_of_recorded_launches():
    """gsim_launch_features needs no GPU: the cost model's inputs for a dense
    launch and a stage launch, field by field."""
    import math

    import numpy as np

    from projectq_gb300 import costmodel as cm

    dense = {"kind": 0, "k": 2, "nctrl": 1, "nqubits": 20, "targets": 0b1010, "bytes": 2 * (1 << 19) * 8,
             "precision": _lib.GSIM_C64, "ngates": 3, "ms": 0.1, "aux": 0}
    stage = {"kind": 1, "k": 24, "nctrl": 0, "nqubits": 30, "targets": 0, "bytes": 2 * (1 << 30) * 16,
             "precision": _lib.GSIM_C128, "ngates": 30, "ms": 9.0, "aux": 5}
    f = cm.launch_features([dense, stage])
    assert f.shape == (2, cm.F)
    d, s = f
    assert d[0] == pytest.approx(20 / 32) and d[1] == 1 and d[2] == 1 and d[3:6].sum() == 0
    assert d[6] == pytest.approx(2 / 8) and d[7] == pytest.approx(1 / 8)
    assert d[8] == pytest.approx(1 / 32) and d[9] == pytest.approx(2 / 4)
    assert d[10] == pytest.approx(math.log2(1 + dense["bytes"]) / 48, rel=1e-6)
    assert d[11] == pytest.approx(math.log2(1 + 2.0 ** 19 * 4) / 48, rel=1e-6)
    assert d[14] == 1 and d[15] == 1
    assert s[1] == 0 and s[3] == 1 and s[6] == 0 and s[12] == pytest.approx(24 / 64)
    assert s[13] == pytest.approx(5 / 32) and s[14] == 0
    assert s[11] == pytest.approx(math.log2(1 + 2.0 ** 30 * 24) / 48, rel=1e-6)
    assert np.all(np.isfinite(f))
