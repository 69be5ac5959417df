"""The stage planner (projectq_gb300/csrc/stage.hpp), checked on the CPU.

tests/cpp/stage_plan_check.cpp runs the planner and executes each planned
stage with the stage kernel's semantics on the host (tile gather by the
plan's local bit positions, dense operations on tile bits with local and
non-local controls, diagonal operations over global bits); the result must
equal the oracle's gate-by-gate application.  This covers the planner's
look-ahead reordering, operation merging and diagonal conversion."""

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

from _backends import make
from _circuits import allocate, random_mixed_circuit, run_circuit
from projectq_gb300.workloads import H, X, Z, config2_circuit, random_state

HERE = Path(__file__).resolve().parent
SRC = HERE / "cpp" / "stage_plan_check.cpp"
LIB = HERE.parent / "oracle" / "_build" / "libstage_plan_check.so"


@pytest.fixture(scope="module")
def lib():
    LIB.parent.mkdir(parents=True, exist_ok=True)
    if not LIB.exists() or LIB.stat().st_mtime < max(SRC.stat().st_mtime,
                                                     (HERE.parent / "projectq_gb300/csrc/stage.hpp").stat().st_mtime):
        subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", str(SRC), "-o", str(LIB)], check=True)
    lib = C.CDLL(str(LIB))
    lib.stage_plan_apply.restype = C.c_int
    return lib


def plan_apply(lib, n, L, m, gates, psi, r=0, rho=4):
    ks = np.array([len(t) for _, t, _ in gates], dtype=np.uint32)
    tg = np.array([q for _, t, _ in gates for q in t], dtype=np.uint32)
    cm = np.array([sum(1 << c for c in cs) for _, _, cs in gates], dtype=np.uint64)
    mats = np.concatenate([np.ascontiguousarray(m, dtype=np.complex128).reshape(-1) for m, _, _ in gates]).view(np.float64)
    st = np.ascontiguousarray(psi, dtype=np.complex128).copy()
    ns = C.c_uint32()
    P = lambda a, t: a.ctypes.data_as(C.POINTER(t))  # noqa: E731
    rc = lib.stage_plan_apply(C.c_uint(n), C.c_uint(L), C.c_uint(m), C.c_uint(r), C.c_uint(rho),
                              C.c_size_t(len(gates)), P(ks, C.c_uint32), P(tg, C.c_uint32), P(cm, C.c_uint64),
                              P(mats, C.c_double), P(st.view(np.float64), C.c_double), C.byref(ns))
    assert rc == 0, "planned operation metadata is inconsistent"
    return st, ns.value


def oracle_apply(n, gates, psi):
    o = make("oracle", seed=1)
    allocate(o, n)
    o.set_wavefunction(psi, list(range(n)))
    o.set_fusion("none")
    run_circuit(o, gates)
    return o.cheat()[1]


@pytest.mark.parametrize("r,rho", [(0, 4), (5, 4), (4, 4), (3, 3), (2, 3)])
@pytest.mark.parametrize("n,L,m,seed", [(9, 6, 3, 0), (10, 7, 4, 1), (11, 8, 5, 2), (6, 6, 3, 3), (12, 12, 5, 4)])
def test_planned_stages_equal_gate_by_gate(lib, n, L, m, seed, r, rho):
    """r = 0 executes the per-operation stage kernel's semantics, r > 0 the
    register-substage kernel's (swizzled tile, 2^r amplitudes per row)."""
    gates = random_mixed_circuit(n, 120, seed, kmax=3, max_ctrl=3)
    psi = random_state(n, seed=seed)
    got, nst = plan_apply(lib, n, L, m, gates, psi, r, rho)
    exp = oracle_apply(n, gates, psi)
    assert np.max(np.abs(got - exp)) < 1e-12
    assert nst >= 1


def test_random_circuit_packs_many_gates_per_stage(lib):
    n = 14
    gates = config2_circuit(n, depth=10, per_layer=14, seed=3)
    psi = random_state(n, seed=3)
    got, nst = plan_apply(lib, n, 12, 5, gates, psi, r=4, rho=4)
    exp = oracle_apply(n, gates, psi)
    assert np.max(np.abs(got - exp)) < 1e-12
    assert len(gates) / nst >= 8  # gates per pass over the state


def count_ops(lib, n, L, m, gates):
    ks = np.array([len(t) for _, t, _ in gates], dtype=np.uint32)
    tg = np.array([q for _, t, _ in gates for q in t], dtype=np.uint32)
    cm = np.array([sum(1 << c for c in cs) for _, _, cs in gates], dtype=np.uint64)
    mats = np.concatenate([np.ascontiguousarray(m_, dtype=np.complex128).reshape(-1) for m_, _, _ in gates]).view(np.float64)
    nops, ns = C.c_uint32(), C.c_uint32()
    P = lambda a, t: a.ctypes.data_as(C.POINTER(t))  # noqa: E731
    lib.stage_plan_count_ops(C.c_uint(n), C.c_uint(L), C.c_uint(m), C.c_size_t(len(gates)), P(ks, C.c_uint32),
                             P(tg, C.c_uint32), P(cm, C.c_uint64), P(mats, C.c_double), C.byref(nops), C.byref(ns))
    return nops.value, ns.value


_T = np.diag([1, np.exp(0.25j * np.pi)])
_S = np.diag([1, 1j])

# (gates, operations after merging): a gate joins an earlier operation of the
# same shape, or an earlier diagonal one, only across operations it commutes with
LOOKBACK_CASES = [
    ([(H, (0,), ()), (X, (1,), ()), (H, (0,), ())], 2),          # across a disjoint gate
    ([(H, (0,), ()), (X, (1,), (0,)), (H, (0,), ())], 3),        # a CNOT on qubit 0 blocks
    ([(_T, (0,), ()), (H, (1,), ()), (_S, (0,), ())], 2),        # diagonal across a disjoint dense gate
    ([(_T, (0,), ()), (H, (0,), ()), (_S, (0,), ())], 3),        # ... not across one on its qubit
    ([(X, (1,), (0,)), (H, (2,), ()), (X, (1,), (0,))], 2),      # same targets and controls
    ([(X, (1,), (0,)), (X, (1,), (2,)), (X, (1,), (0,))], 3),    # different controls, shared target
    ([(Z, (1,), (0,)), (Z, (3,), (2,)), (Z, (5,), (4,)), (_T, (0,), ())], 1),  # diagonals up to 6 qubits
    ([(Z, (1,), (0,)), (Z, (3,), (2,)), (Z, (5,), (4,)), (Z, (6,), (5,)), (_T, (6,), ())], 2),
]


@pytest.mark.parametrize("case", range(len(LOOKBACK_CASES)))
@pytest.mark.parametrize("r,rho", [(0, 4), (3, 3)])
def test_lookback_merging(lib, case, r, rho):
    """Operation counts of the look-back merge on crafted stages (the whole
    7-qubit state is one tile) and the merged stage's state against the
    oracle's gate-by-gate application."""
    gates, want = LOOKBACK_CASES[case]
    n = 7
    nops, ns = count_ops(lib, n, 7, 3, gates)
    assert ns == 1 and nops == want, (nops, ns)
    psi = random_state(n, seed=40 + case)
    got, _ = plan_apply(lib, n, 7, 3, gates, psi, r, rho)
    assert np.max(np.abs(got - oracle_apply(n, gates, psi))) < 1e-12
