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
from projectq_gb300.workloads import H, X, Z, random_gate_circuit, random_state

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
    gates = random_gate_circuit(n, depth=10, per_layer=14, seed=3)
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


def plan_apply_pk(lib, n, gates, psi):
    ks = np.array([len(t) for _, t, _ in gates], dtype=np.uint32)
    tg = np.array([q for _, t, _ in gates for q in t], dtype=np.uint32)
    cm = np.array([sum(1 << c for c in cs) for _, _, cs in gates], dtype=np.uint64)
    mats = np.concatenate([np.ascontiguousarray(m, dtype=np.complex128).reshape(-1) for m, _, _ in gates]).view(np.float64)
    st = np.ascontiguousarray(psi, dtype=np.complex128).copy()
    ns, npk = C.c_uint32(), C.c_uint32()
    kinds = np.zeros(3, dtype=np.uint32)
    P = lambda a, t: a.ctypes.data_as(C.POINTER(t))  # noqa: E731
    rc = lib.stage_plan_apply_pk(C.c_uint(n), C.c_size_t(len(gates)), P(ks, C.c_uint32), P(tg, C.c_uint32),
                                 P(cm, C.c_uint64), P(mats, C.c_double), P(st.view(np.float64), C.c_double),
                                 C.byref(ns), C.byref(npk), P(kinds, C.c_uint32))
    assert rc == 0, "packed-pair descriptors are inconsistent"
    return st, ns.value, npk.value, kinds


def _sprinkle(gates, extra, seed):
    rng = np.random.default_rng(seed)
    for g in extra:
        gates.insert(int(rng.integers(len(gates) + 1)), g)
    return gates


@pytest.mark.parametrize("n,seed,avoid,kind,dense2", [
    (16, 0, (0,), 0, True),          # qubit 0 left free: pairs along global bit 0
    (18, 1, (0, 17), None, True),    # free qubits 0 and 17
    (18, 2, (15,), None, True),      # qubits 0-4 all used
    (13, 3, (3,), 1, False),         # the whole state is one tile; the free qubit is inside the runs
    (20, 4, (), None, True),         # nothing left free by construction
])
def test_packed_pair_stages_equal_gate_by_gate(lib, n, seed, avoid, kind, dense2):
    """The complex64 planning path: stages with a pack bit executed with the
    packed-pair kernel's semantics (pairs along the pack bit, folded X gates as
    address XORs and offset-table permutations, FP32 matrices and diagonal
    tables), the rest with the register-substage kernel's; against the
    oracle's gate-by-gate application.  The circuits mix the headline gate
    set with controlled 1-qubit gates (register, row and non-local controls)
    and a few 2-qubit dense gates (whose stages keep the register-substage
    kernel); `avoid` lists qubits no gate touches, which
    steers the pack bit to global bit 0, inside or above the contiguous runs.
    Tolerance 2e-6 (FP32 gate data)."""
    keep = [q for q in range(n) if q not in avoid]
    relabel = lambda gs: [(m, tuple(keep[q] for q in t), tuple(keep[q] for q in c)) for m, t, c in gs]  # noqa: E731
    k = len(keep)
    # (a one-tile state holds the whole circuit in one stage: kept small enough
    # for the kernel's shared-memory budget)
    gates = relabel(random_gate_circuit(k, depth=12 if n > 13 else 4, per_layer=k, seed=seed))
    gates = _sprinkle(gates, relabel(random_mixed_circuit(k, 60 if n > 13 else 20, seed + 10, kmax=1, max_ctrl=3)),
                      seed)
    if dense2:
        gates = _sprinkle(gates, relabel(random_mixed_circuit(k, 4, seed + 20, kmax=2, max_ctrl=1)), seed + 1)
    psi = random_state(n, seed=seed)
    got, nst, npk, kinds = plan_apply_pk(lib, n, gates, psi)
    exp = oracle_apply(n, gates, psi)
    assert np.max(np.abs(got - exp)) < 2e-6
    if avoid:
        assert npk >= max(1, nst // 2), (npk, nst)
    if kind is not None:
        assert kinds[kind] >= 1, kinds


@pytest.mark.parametrize("n", [13, 16])
def test_packed_pair_register_controlled_x(lib, n):
    """X gates with 0-3 controls among four neighbouring qubits, between
    rotations on them: in a packed-pair substage each becomes the exchange of
    the pairs its register controls select (the control mask travels in the
    operation code; the emulator checks it against the pair mask).  Against
    the oracle, tolerance 2e-6."""
    rng = np.random.default_rng(200 + n)
    from projectq_gb300.workloads import Rx, Ry, X
    gates = []
    for _ in range(60 if n > 13 else 30):
        block = [int(q) for q in rng.permutation(4)] if rng.uniform() < 0.5 else [int(q) + 6 for q in rng.permutation(4)]
        nctl = int(rng.integers(0, 4))
        if rng.uniform() < 0.3:
            gates.append(((Rx, Ry)[int(rng.integers(2))](float(rng.uniform(0, 2 * np.pi))), (block[0],), ()))
        else:
            gates.append((X, (block[0],), tuple(block[1:1 + nctl])))
    psi = random_state(n, seed=n)
    got, nst, npk, kinds = plan_apply_pk(lib, n, gates, psi)
    assert npk >= 1
    assert np.max(np.abs(got - oracle_apply(n, gates, psi))) < 2e-6


def test_packed_pair_stage_with_pack_bit_above_the_runs(lib):
    """Dense gates only on qubits 0-9, diagonal gates and controls on every
    qubit but 18: each stage's dense targets leave room in the tile, and the
    planner adds the free qubit 18 as the pack bit (pairs split across two
    16-byte loads from different runs)."""
    n = 20
    rng = np.random.default_rng(7)
    from projectq_gb300.workloads import Rx, Rz, S, T as Tg
    others = [q for q in range(n) if q != 18]
    gates = []
    for _ in range(90):  # one stage (all dense targets are local), within the shared-memory budget
        kind = int(rng.integers(5))
        if kind == 0:
            gates.append((H, (int(rng.integers(10)),), ()))
        elif kind == 1:
            gates.append((Rx(float(rng.uniform(0, 6.3))), (int(rng.integers(10)),), ()))
        elif kind == 2:
            t, c = (int(v) for v in rng.choice(others, 2, replace=False))
            gates.append((X, (int(t % 10),), (c,) if c != t % 10 else ()))
        elif kind == 3:
            gates.append(([Tg, S, Rz(float(rng.uniform(0, 6.3)))][int(rng.integers(3))], (int(rng.choice(others)),), ()))
        else:
            a, b = (int(v) for v in rng.choice(others, 2, replace=False))
            gates.append((Z, (a,), (b,)))
    psi = random_state(n, seed=7)
    got, nst, npk, kinds = plan_apply_pk(lib, n, gates, psi)
    assert np.max(np.abs(got - oracle_apply(n, gates, psi))) < 2e-6
    assert kinds[2] >= 1, kinds
