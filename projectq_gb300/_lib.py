"""ctypes binding of the C ABI declared in include/gb300sim.h.

`bind(path, prefix)` loads a shared library that implements the ABI under a
symbol prefix and returns a table of typed functions without the prefix
(``api.create``, ``api.run`` ...).  The product library is
``projectq_gb300/_build/libgb300sim.so`` with prefix ``gsim_``; `load()`
returns it and raises if it is missing — there is no fallback path.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path
from types import SimpleNamespace

GSIM_OK = 0
GSIM_ERR_RUNTIME = 1
GSIM_ERR_VALUE = 2
GSIM_ERR_LENGTH = 3
GSIM_ERR_CUDA = 4
GSIM_ERR_MEMORY = 5

GSIM_C128 = 0
GSIM_C64 = 1

GSIM_FUSION_REFERENCE = 0
GSIM_FUSION_NONE = 1
GSIM_FUSION_STAGED = 2
GSIM_FUSION_LEARNED = 3

_u32p = C.POINTER(C.c_uint32)
_u8p = C.POINTER(C.c_uint8)
_f64p = C.POINTER(C.c_double)
_u64p = C.POINTER(C.c_uint64)
_eng = C.c_void_p
_sz = C.c_size_t

# name -> (restype, argtypes); the ABI of include/gb300sim.h.
SIGNATURES = {
    "last_error": (C.c_char_p, []),
    "create": (C.c_int, [C.c_uint32, C.c_int, C.POINTER(C.c_void_p)]),
    "destroy": (C.c_int, [_eng]),
    "allocate_qubit": (C.c_int, [_eng, C.c_uint32]),
    "deallocate_qubit": (C.c_int, [_eng, C.c_uint32]),
    "get_classical_value": (C.c_int, [_eng, C.c_uint32, C.c_double, C.POINTER(C.c_int)]),
    "is_classical": (C.c_int, [_eng, C.c_uint32, C.c_double, C.POINTER(C.c_int)]),
    "measure_qubits": (C.c_int, [_eng, _u32p, _sz, _u8p]),
    "measure_qubits_at": (C.c_int, [_eng, _u32p, _sz, C.c_double, _u8p]),
    "apply_gates": (C.c_int, [_eng, _sz, _u32p, _u32p, _u32p, _f64p, C.POINTER(_sz)]),
    # the matrix by address (c_void_p): callers pass ndarray.ctypes.data
    "apply_controlled_gate": (C.c_int, [_eng, C.c_void_p, C.c_uint32, _u32p, _u32p, _sz]),
    "run": (C.c_int, [_eng]),
    "emulate_math_add_constant": (C.c_int, [_eng, C.c_int32, _u32p, _u32p, _sz, _u32p, _sz]),
    "emulate_math_add_constant_modn": (
        C.c_int,
        [_eng, C.c_int32, C.c_int32, _u32p, _u32p, _sz, _u32p, _sz],
    ),
    "emulate_math_multiply_by_constant_modn": (
        C.c_int,
        [_eng, C.c_int32, C.c_int32, _u32p, _u32p, _sz, _u32p, _sz],
    ),
    "emulate_math_table": (C.c_int, [_eng, _u64p, _u32p, _u32p, _sz, _u32p, _sz]),
    "get_expectation_value": (
        C.c_int,
        [_eng, _u32p, _u32p, _u8p, _f64p, _sz, _u32p, _sz, _f64p],
    ),
    "apply_qubit_operator": (C.c_int, [_eng, _u32p, _u32p, _u8p, _f64p, _sz, _u32p, _sz]),
    "emulate_time_evolution": (
        C.c_int,
        [_eng, _u32p, _u32p, _u8p, _f64p, _sz, C.c_double, _u32p, _sz, _u32p, _sz],
    ),
    "get_probability": (C.c_int, [_eng, _u8p, _u32p, _sz, _f64p]),
    "get_amplitude": (C.c_int, [_eng, _u8p, _u32p, _sz, _f64p]),
    "set_wavefunction": (C.c_int, [_eng, C.c_void_p, C.c_int, _sz, _u32p, _sz]),
    "collapse_wavefunction": (C.c_int, [_eng, _u32p, _sz, _u8p, _sz]),
    "num_qubits": (C.c_int, [_eng, _u32p]),
    "get_mapping": (C.c_int, [_eng, _u32p, _u32p, _sz]),
    "get_state": (C.c_int, [_eng, C.c_void_p, C.c_int, _sz, _sz]),
    "synchronize": (C.c_int, [_eng]),
    "set_fusion": (C.c_int, [_eng, C.c_int, C.c_uint32]),
}
# Entry points only the product library has.
class LaunchRecord(C.Structure):
    """gsim_launch_record of include/gb300sim.h."""

    _fields_ = [
        ("kind", C.c_uint32),
        ("k", C.c_uint32),
        ("nctrl", C.c_uint32),
        ("nqubits", C.c_uint32),
        ("targets", C.c_uint64),
        ("bytes", C.c_uint64),
        ("precision", C.c_uint32),
        ("ngates", C.c_uint32),
        ("ms", C.c_float),
        ("aux", C.c_uint32),
    ]


PRODUCT_ONLY = {
    "device_count": (C.c_int, []),
    "state_device_ptr": (C.c_int, [_eng, C.POINTER(C.c_void_p), C.POINTER(_sz), C.POINTER(C.c_int)]),
    "reserve": (C.c_int, [_eng, C.c_uint32]),
    "get_counters": (C.c_int, [_eng, _u64p, _sz]),
    "reset_counters": (C.c_int, [_eng]),
    "set_device": (C.c_int, [C.c_int]),
    "set_tensor_cores": (C.c_int, [_eng, C.c_int]),
    "set_stage_kernel": (C.c_int, [_eng, C.c_int]),
    "set_upload_mode": (C.c_int, [_eng, C.c_int]),
    "set_time_evolution": (C.c_int, [_eng, C.c_int]),
    "compare_states": (C.c_int, [_eng, _eng, _f64p]),
    "timer_mark": (C.c_int, [_eng, C.c_int]),
    "timer_elapsed": (C.c_int, [_eng, C.c_int, C.c_int, C.POINTER(C.c_float)]),
    "profile_enable": (C.c_int, [_eng, C.c_int]),
    "profile_fetch": (C.c_int, [_eng, C.POINTER(LaunchRecord), _sz, C.POINTER(_sz)]),
    "profile_clear": (C.c_int, [_eng]),
    "host_register": (C.c_int, [C.c_void_p, _sz]),
    "host_unregister": (C.c_int, [C.c_void_p]),
    "adjoint_gradient": (
        C.c_int,
        [_eng, _sz, _u8p, _u32p, _u32p, _u32p, C.POINTER(C.c_int32), _f64p, _f64p, _sz, _u32p, _u32p, _u8p,
         _f64p, _sz, _u32p, _sz, C.c_uint32, _f64p, _f64p],
    ),
    "launch_features": (C.c_int, [C.POINTER(LaunchRecord), _sz, C.POINTER(C.c_float), _sz]),
    "set_cost_model": (C.c_int, [_eng, C.c_int, C.c_int, C.POINTER(C.c_float)]),
    "set_learned_regimes": (C.c_int, [_eng, _u8p, _sz]),
    "last_plan_choice": (C.c_int, [_eng, C.POINTER(C.c_int), _f64p]),
    "cost_model_predict": (C.c_int, [_eng, C.POINTER(C.c_float), _sz, C.POINTER(C.c_float)]),
    "mlp_create": (C.c_int, [C.c_int, C.c_int, C.c_uint32, C.POINTER(C.c_void_p)]),
    "mlp_destroy": (C.c_int, [C.c_void_p]),
    "mlp_num_params": (C.c_int, [C.c_void_p, C.POINTER(_sz)]),
    "mlp_get_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "mlp_set_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "mlp_predict": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float)]),
    "mlp_gradient": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int,
                               C.POINTER(C.c_float), C.POINTER(C.c_double)]),
    "mlp_train": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_int, C.c_float,
                            C.POINTER(C.c_double)]),
    "probability_noalloc": (
        C.c_int,
        [C.c_void_p, C.c_int, C.c_uint32, C.c_uint64, C.c_uint64, _f64p, C.c_void_p],
    ),
}

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libgb300sim.so"

_lock = threading.Lock()
_product = None


def bind(path, prefix: str, optional=()) -> SimpleNamespace:
    """Load `path` and return the ABI functions found under `prefix`."""
    lib = C.CDLL(str(path))
    ns = SimpleNamespace(_lib=lib, _path=str(path), _prefix=prefix)
    table = dict(SIGNATURES)
    for name, sig in dict(optional).items():
        table[name] = sig
    for name, (res, args) in table.items():
        try:
            fn = getattr(lib, prefix + name)
        except AttributeError:
            continue  # not every implementation of the ABI has every entry
        fn.restype = res
        fn.argtypes = args
        setattr(ns, name, fn)
    return ns


def load() -> SimpleNamespace:
    """The product library (libgb300sim.so).  Raises if it was not built."""
    global _product
    with _lock:
        if _product is None:
            if not LIB_PATH.exists():
                raise ImportError(
                    f"{LIB_PATH} is missing: build it with `python -m projectq_gb300.build` "
                    "(the simulator has no CPU fallback)"
                )
            _product = bind(LIB_PATH, "gsim_", PRODUCT_ONLY)
        return _product


def check(api, rc: int) -> None:
    """Raise the Python exception the reference's pybind11 layer would raise."""
    if rc == GSIM_OK:
        return
    msg = api.last_error()
    msg = msg.decode("utf-8", "replace") if msg else ""
    if rc in (GSIM_ERR_VALUE, GSIM_ERR_LENGTH):
        raise ValueError(msg)
    if rc == GSIM_ERR_MEMORY:
        raise MemoryError(msg)
    raise RuntimeError(msg)
