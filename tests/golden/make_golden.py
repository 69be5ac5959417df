#!/usr/bin/env python3
"""Generate the golden fixtures in this directory from the reference engine.

The reference engine is ProjectQ's own C++ simulator core
(projectq/backends/_sim/_cppkernels/simulator.hpp), compiled from the
reference tree by oracle/build_ref.sh into oracle/_ref/libref_sim.so and
driven here through the same Python surface as the GB300 engine.  This script
only runs where the reference tree is present; the fixtures it writes are
committed and are what the tests compare against everywhere else.

    python tests/golden/make_golden.py

Fixtures (numpy .npz):
  layered_n10.npz  the layered Rx/Ry/Rz + CNOT circuit (10 qubits, depth 10,
                   seed 0): full final state with a run() per gate and with the
                   reference's fusion, <Z0 Z1 + X5 X6>, 8 measurement draws of
                   the engine RNG (seed 0), each on a fresh copy of the state.
  layered_n20.npz  the same circuit at 20 qubits, depth 20 (the workload the
                   reference numbers are quoted on): 4096 sampled amplitudes,
                   per-qubit probabilities, <Z0 Z1 + X5 X6>, 8 draws.
  ops_small.npz    every other entry point on small seeded inputs: a mixed
                   random circuit, emulate_math (three fast paths and a
                   tabulated function), expectation values, apply_qubit_operator,
                   time evolution, collapse / probability / amplitude and
                   deallocation.
"""

import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE.parent))

from _backends import REF_LIB, make  # noqa: E402
from _circuits import allocate, random_mixed_circuit, random_pauli_sum, run_circuit  # noqa: E402
from projectq_gb300.workloads import layered_rotation_circuit, random_state  # noqa: E402

ZZ_XX = [([(0, "Z"), (1, "Z")], 1.0), ([(5, "X"), (6, "X")], 1.0)]


def layered(n, depth, fused):
    sim = make("ref", seed=0)
    allocate(sim, n)
    run_circuit(sim, layered_rotation_circuit(n, depth, seed=0), run_each=not fused)
    return sim


def draws(sim, n, count=8):
    """`count` measurements of all qubits, each on a fresh copy of the state,
    with the engine RNG (seed 0) advancing from draw to draw."""
    ids = list(range(n))
    _, psi = sim.cheat()
    psi = psi.copy()
    out = []
    for _ in range(count):
        sim.set_wavefunction(psi, ids)
        bits = sim.measure_qubits(ids)
        out.append(sum(int(b) << i for i, b in enumerate(bits)))
    sim.set_wavefunction(psi, ids)
    return np.array(out, dtype=np.int64)


def make_layered_n10():
    n, depth = 10, 10
    res = {}
    for fused in (False, True):
        sim = layered(n, depth, fused)
        tag = "fused" if fused else "unfused"
        res["state_" + tag] = sim.cheat()[1]
        res["zz_xx_" + tag] = sim.get_expectation_value(ZZ_XX, list(range(n)))
        res["draws_" + tag] = draws(sim, n)
    np.savez_compressed(HERE / "layered_n10.npz", **res)


def make_layered_n20():
    n, depth = 20, 20
    idx = np.sort(np.random.default_rng(0).choice(1 << n, size=4096, replace=False))
    res = {"sample_index": idx}
    for fused in (False, True):
        sim = layered(n, depth, fused)
        tag = "fused" if fused else "unfused"
        psi = sim.cheat()[1]
        res["sample_" + tag] = psi[idx]
        res["zz_xx_" + tag] = sim.get_expectation_value(ZZ_XX, list(range(n)))
        res["p1_" + tag] = np.array([sim.get_probability([1], [q]) for q in range(n)])
        res["draws_" + tag] = draws(sim, n)
    np.savez_compressed(HERE / "layered_n20.npz", **res)


MATH_OPS = [
    ("addConstant", (3,), [[0, 1, 2, 3, 4]], [6]),
    ("addConstantModN", (4, 5), [[0, 1, 2, 3, 4]], [7, 8]),
    ("multiplyByConstantModN", (15, 16), [[4, 2, 0, 1, 3]], []),
    ("addConstant", (-5,), [[1, 3], [5, 6]], [0]),
]


def math_table_f(vals):
    return [(vals[0] * vals[0] + 1) % 8, vals[1] ^ vals[0]]


TE_TERMS = [([(0, "X"), (1, "Y"), (2, "Z"), (3, "Y"), (4, "X")], 0.3), ([], 1.1),
            ([(0, "Y"), (1, "Z"), (3, "X"), (5, "Y")], -1.4), ([(1, "Y"), (2, "X"), (3, "X"), (4, "Y")], -1.1)]


def make_ops():
    res = {}
    # mixed random circuit, reference fusion
    n = 8
    sim = make("ref", seed=1)
    allocate(sim, n)
    run_circuit(sim, random_mixed_circuit(n, 60, 2))
    res["mixed_state"] = sim.cheat()[1]
    ids = [4, 2, 0, 1, 3, 7, 6, 5]
    res["expect"] = np.array([sim.get_expectation_value(random_pauli_sum(n, 12, s), ids) for s in range(4)])
    cterms = [(t, complex(c, 0.3 * c)) for t, c in random_pauli_sum(n, 6, 9)]
    sim.apply_qubit_operator(cterms, ids)
    res["qubit_operator_state"] = sim.cheat()[1]
    # emulate_math on a random state
    n = 9
    psi = random_state(n, seed=31)
    for i, (name, args, regs, ctrl) in enumerate(MATH_OPS):
        s = make("ref", seed=1)
        allocate(s, n)
        s.set_wavefunction(psi, list(range(n)))
        getattr(s, "emulate_math_" + name)(*args, regs, ctrl)
        res[f"math_{i}"] = s.cheat()[1]
    s = make("ref", seed=1)
    allocate(s, n)
    s.set_wavefunction(psi, list(range(n)))
    table = np.zeros(64, dtype=np.uint64)
    for x in range(64):
        y = math_table_f([x & 7, x >> 3])
        table[x] = (y[0] & 7) | ((y[1] & 7) << 3)
    import ctypes as C
    ida = np.array([0, 1, 2, 3, 4, 5], dtype=np.uint32)
    sz = np.array([3, 3], dtype=np.uint32)
    ctrl = np.array([8], dtype=np.uint32)
    rc = s._api.emulate_math_table(s._h, table.ctypes.data_as(C.POINTER(C.c_uint64)),
                                   ida.ctypes.data_as(C.POINTER(C.c_uint32)), sz.ctypes.data_as(C.POINTER(C.c_uint32)),
                                   2, ctrl.ctypes.data_as(C.POINTER(C.c_uint32)), 1)
    assert rc == 0
    res["math_table"] = s.cheat()[1]
    # time evolution with a control qubit
    n = 8
    s = make("ref", seed=1)
    allocate(s, n)
    run_circuit(s, random_mixed_circuit(n, 30, 10))
    s.emulate_time_evolution(TE_TERMS, 1.1, list(range(7)), [7])
    res["time_evolution_state"] = s.cheat()[1]
    # collapse / probability / amplitude / deallocation
    s = make("ref", seed=1)
    allocate(s, n)
    run_circuit(s, random_mixed_circuit(n, 40, 6))
    res["prob"] = np.array([s.get_probability([0, 1, 1], [0, 5, 2]), s.get_probability([1], [3])])
    res["amp"] = np.array([s.get_amplitude([(b >> i) & 1 for i in range(8)], [3, 1, 4, 0, 7, 6, 2, 5])
                           for b in range(0, 256, 37)])
    s.collapse_wavefunction([2, 5], [1, 0])
    res["collapse_state"] = s.cheat()[1]
    s = make("ref", seed=1)
    for q in range(6):
        s.allocate_qubit(10 + q)
    from projectq_gb300.workloads import H, X
    s.apply_controlled_gate(X, [12], [])
    s.apply_controlled_gate(H, [14], [])
    s.apply_controlled_gate(X, [11], [14])
    s.run()
    for q in (12, 10, 15):
        s.deallocate_qubit(q)
    m, st = s.cheat()
    res["dealloc_state"] = st
    res["dealloc_map"] = np.array(sorted(m.items()), dtype=np.int64)
    np.savez_compressed(HERE / "ops_small.npz", **res)


def main():
    if not REF_LIB.exists():
        subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh")], check=True)
    if not REF_LIB.exists():
        sys.exit("the reference tree is needed to build oracle/_ref/libref_sim.so")
    make_layered_n10()
    make_layered_n20()
    make_ops()
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
