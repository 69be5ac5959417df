"""The CUDA engine against the fixtures made by the reference engine itself
(tests/golden/make_golden.py): the 20- and 10-qubit layered circuits, their
<Z0 Z1 + X5 X6> and seeded measurement draws, and every other entry point on
small inputs.  Tolerances: complex128 1e-12 (amplitudes), complex64 5e-6;
measurement outcomes and emulate_math results exactly."""

import sys
from pathlib import Path

import numpy as np
import pytest

from _backends import make
from _circuits import allocate, random_mixed_circuit, random_pauli_sum, run_circuit
from projectq_gb300.workloads import H, X, layered_rotation_circuit, random_state

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
from make_golden import MATH_OPS, TE_TERMS, ZZ_XX, math_table_f  # noqa: E402

pytestmark = pytest.mark.gpu
TOL = {"c128": 1e-12, "c64": 5e-6}


def draws(sim, n, count=8):
    ids = list(range(n))
    psi = sim.cheat()[1].copy()
    out = []
    for _ in range(count):
        sim.set_wavefunction(psi, ids)
        out.append(sum(int(b) << i for i, b in enumerate(sim.measure_qubits(ids))))
    return out


@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("fusion", ["reference", "none", "staged"])
def test_layered_n20(prec, fusion):
    g = np.load(GOLDEN / "layered_n20.npz")
    sim = make("gpu", seed=0, precision=prec, fusion=fusion)
    allocate(sim, 20)
    run_circuit(sim, layered_rotation_circuit(20, 20, seed=0))
    psi = sim.cheat()[1]
    assert np.max(np.abs(psi[g["sample_index"]] - g["sample_fused"])) < TOL[prec] * 10
    zz = sim.get_expectation_value(ZZ_XX, list(range(20)))
    assert zz == pytest.approx(float(g["zz_xx_fused"]), abs=1e-11 if prec == "c128" else 1e-5)
    p1 = np.array([sim.get_probability([1], [q]) for q in range(20)])
    assert np.max(np.abs(p1 - g["p1_fused"])) < (1e-12 if prec == "c128" else 1e-5)
    if prec == "c128":
        assert draws(sim, 20) == list(g["draws_fused"])


@pytest.mark.parametrize("fused", [False, True])
def test_layered_n10_full_state(fused):
    g = np.load(GOLDEN / "layered_n10.npz")
    tag = "fused" if fused else "unfused"
    sim = make("gpu", seed=0)
    allocate(sim, 10)
    run_circuit(sim, layered_rotation_circuit(10, 10, seed=0), run_each=not fused)
    assert np.max(np.abs(sim.cheat()[1] - g["state_" + tag])) < 1e-13
    assert draws(sim, 10) == list(g["draws_" + tag])


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_ops_fixture(prec):
    g = np.load(GOLDEN / "ops_small.npz")
    n = 8
    sim = make("gpu", seed=1, precision=prec)
    allocate(sim, n)
    run_circuit(sim, random_mixed_circuit(n, 60, 2))
    assert np.max(np.abs(sim.cheat()[1] - g["mixed_state"])) < TOL[prec]
    ids = [4, 2, 0, 1, 3, 7, 6, 5]
    ex = [sim.get_expectation_value(random_pauli_sum(n, 12, s), ids) for s in range(4)]
    assert np.max(np.abs(np.array(ex) - g["expect"])) < (1e-11 if prec == "c128" else 1e-5)
    sim.apply_qubit_operator([(t, complex(c, 0.3 * c)) for t, c in random_pauli_sum(n, 6, 9)], ids)
    assert np.max(np.abs(sim.cheat()[1] - g["qubit_operator_state"])) < TOL[prec] * 20


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_math_fixture(prec):
    g = np.load(GOLDEN / "ops_small.npz")
    n = 9
    psi = random_state(n, seed=31)
    for i, (name, args, regs, ctrl) in enumerate(MATH_OPS + [("table", None, None, None)]):
        s = make("gpu", seed=1, precision=prec)
        allocate(s, n)
        s.set_wavefunction(psi, list(range(n)))
        if name == "table":
            s.emulate_math(math_table_f, [[0, 1, 2], [3, 4, 5]], [8])
            ref = g["math_table"]
        else:
            getattr(s, "emulate_math_" + name)(*args, regs, ctrl)
            ref = g[f"math_{i}"]
        if prec == "c128":
            assert np.array_equal(s.cheat()[1].view(np.uint64), ref.view(np.uint64)), name
        else:
            # complex64: a bijection moves amplitudes unchanged, so the result is
            # bit-exact against the reference result rounded to complex64; maps
            # with collisions add the colliding amplitudes in FP32
            got = s.cheat(dtype=np.complex64)[1]
            exp = ref.astype(np.complex64)
            if name == "addConstant":
                assert np.array_equal(got.view(np.uint32), exp.view(np.uint32)), name
            else:
                assert np.max(np.abs(got - exp)) < 1e-7, name


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_time_evolution_collapse_dealloc_fixture(prec):
    g = np.load(GOLDEN / "ops_small.npz")
    n = 8
    s = make("gpu", seed=1, precision=prec)
    allocate(s, n)
    run_circuit(s, random_mixed_circuit(n, 30, 10))
    s.emulate_time_evolution(TE_TERMS, 1.1, list(range(7)), [7])
    assert np.max(np.abs(s.cheat()[1] - g["time_evolution_state"])) < (1e-11 if prec == "c128" else 2e-5)
    s = make("gpu", seed=1, precision=prec)
    allocate(s, n)
    run_circuit(s, random_mixed_circuit(n, 40, 6))
    assert s.get_probability([0, 1, 1], [0, 5, 2]) == pytest.approx(g["prob"][0], abs=TOL[prec])
    amps = [s.get_amplitude([(b >> i) & 1 for i in range(8)], [3, 1, 4, 0, 7, 6, 2, 5]) for b in range(0, 256, 37)]
    assert np.max(np.abs(np.array(amps) - g["amp"])) < TOL[prec]
    s.collapse_wavefunction([2, 5], [1, 0])
    assert np.max(np.abs(s.cheat()[1] - g["collapse_state"])) < TOL[prec]
    s = make("gpu", seed=1, precision=prec)
    for q in range(6):
        s.allocate_qubit(10 + q)
    s.apply_controlled_gate(X, [12], [])
    s.apply_controlled_gate(H, [14], [])
    s.apply_controlled_gate(X, [11], [14])
    s.run()
    for q in (12, 10, 15):
        s.deallocate_qubit(q)
    m, st = s.cheat()
    assert np.max(np.abs(st - g["dealloc_state"])) < TOL[prec]
    assert sorted(m.items()) == [tuple(r) for r in g["dealloc_map"]]
