"""ProjectQ's own simulator tests with the GB300 engine as the C++ engine.

ProjectQ's test module projectq/backends/_sim/_simulator_test.py runs each
test with a "cpp_simulator" parameter that constructs
projectq.backends._sim._cppsim.Simulator; ref_suite_plugin serves that name
from libgb300sim.so, so the reference's known-answer tests (GHZ amplitudes,
probabilities, amplitudes, expectation values, qubit operators, collapse,
set_wavefunction, math emulation, k-qubit gates, errors) and the Shor N=15
integration test (projectq/tests/_factoring_test.py) run against it through
MainEngine and the compiler engines, unchanged.
"""

import numpy as np
import pytest

import _refsuite
from _backends import make, projectq_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not _refsuite.available(), reason="ProjectQ's Python layers are not installed")]


@pytest.mark.parametrize("fusion", ["reference", "staged"])
def test_reference_suite_complex128(fusion):
    rc, passed, out = _refsuite.run("gpu", "c128", fusion)
    assert rc == 0, out[-6000:]
    assert passed >= 55


def test_reference_suite_complex64():
    """complex64 storage: every test of the suite passes with the reference's
    own tolerances, except two whose checks sit below complex64's rounding:
    test_simulator_functional_entangle compares amplitudes that should be
    exactly zero with pytest.approx's abs 1e-12, and test_factoring treats
    |a| > 1e-8 as nonzero after H.H, where complex64 leaves ~3e-8.  Those two
    are deselected here and run with stated bounds in
    test_complex64_entangle_and_factoring_with_stated_bounds."""
    rc, passed, out = _refsuite.run(
        "gpu", "c64", "staged",
        extra=["-k", "not (test_simulator_functional_entangle and cpp_simulator) "
                     "and not (test_factoring and cpp_simulator)"])
    assert rc == 0, out[-6000:]
    assert passed >= 50


def _main_engine(backend_sim, engine_list=None):
    from projectq import MainEngine
    from projectq.backends import Simulator

    backend = Simulator(gate_fusion=True)
    backend._simulator = backend_sim
    return MainEngine(backend, engine_list if engine_list is not None else []), backend


def test_complex64_entangle_and_factoring_with_stated_bounds():
    """The circuits of ProjectQ's test_simulator_functional_entangle (GHZ by
    CNOTs, by Toffolis, uncomputed by multi-controlled X) and test_factoring
    (Shor's order finding for N = 15, a = 2, through ProjectQ's decomposition
    engines) in complex64, next to the same circuits on the complex128 oracle.
    Stated bounds, every amplitude against the oracle's at each checkpoint:
    2e-7 for the entangling circuit (at most 14 gates), 1e-5 for each
    order-finding block (750 gates after decomposition; complex64 rounding
    accumulates to 3.5e-6 there, measured on a GB300).  The tests' own
    physical checks hold with "zero" meaning |a| <= 1e-6 and 1e-5
    respectively (complex64 leaves ~3e-8 where the reference expects 1e-12 or
    1e-8)."""
    if not projectq_available():
        pytest.skip("ProjectQ not importable")
    from projectq.libs.math import MultiplyByConstantModN
    from projectq.meta import Control
    from projectq.ops import CNOT, All, H, Measure, Toffoli, X
    from projectq.tests._factoring_test import get_main_engine

    bound, zero = 2e-7, 1e-6

    def states(backends):
        out = []
        for b in backends:
            mapping, vec = b.cheat()
            out.append((mapping, np.asarray(vec, dtype=np.complex128).copy()))
        return out

    def check_close(backends):
        (m1, v1), (m2, v2) = states(backends)
        assert m1 == m2
        assert np.max(np.abs(v1 - v2)) <= bound
        return v1

    # functional entangle
    engs = [_main_engine(make("gpu", seed=1, precision="c64", fusion="staged")),
            _main_engine(make("oracle", seed=1))]
    regs = [e.allocate_qureg(5) for e, _ in engs]
    for phase in range(3):
        for (eng, _), q in zip(engs, regs):
            if phase == 0:
                H | q[0]
                for qb in q[1:]:
                    CNOT | (q[0], qb)
            elif phase == 1:
                for qb in q[2:]:
                    CNOT | (q[0], qb)
                for qb in q[2:]:
                    Toffoli | (q[0], q[1], qb)
            else:
                for k in (1, 2, 3):
                    with Control(eng, q[0:-k]):
                        X | q[-k]
                CNOT | (q[0], q[1])
                H | q[0]
            eng.flush()
        v = check_close([b for _, b in engs])
        if phase < 2:
            assert abs(v[0]) ** 2 == pytest.approx(0.5, abs=zero)
            assert abs(v[31]) ** 2 == pytest.approx(0.5, abs=zero)
            assert np.max(np.abs(v[1:31])) <= zero
        else:
            assert abs(v[0]) ** 2 == pytest.approx(1.0, abs=zero)
            assert np.max(np.abs(v[1:])) <= zero
    for (eng, _), q in zip(engs, regs):
        All(Measure) | q
        eng.flush()

    # factoring (N = 15, a = 2)
    bound, zero = 1e-5, 1e-5
    backends = [make("gpu", seed=1, precision="c64", fusion="staged"), make("oracle", seed=1)]
    engs = [get_main_engine(_main_engine(b)[1]) for b in backends]
    ctrls, xs = [], []
    for eng in engs:
        ctrls.append(eng.allocate_qubit())
        xs.append(eng.allocate_qureg(4))
        X | xs[-1][0]
    for power, want_half in ((2**7, False), (2, True)):
        for eng, c, x in zip(engs, ctrls, xs):
            H | c
            with Control(eng, c):
                MultiplyByConstantModN(pow(2, power, 15), 15) | x
            H | c
            eng.flush()
        sims = [e.backend for e in engs]
        v = check_close(sims)
        idx = sims[0].cheat()[0][ctrls[0][0].id]
        ones = [i for i in range(len(v)) if (i >> idx) & 1]
        if not want_half:
            assert np.max(np.abs(v[ones])) <= zero  # the control is |0> with certainty
        else:
            p0 = sum(abs(v[i]) ** 2 for i in range(len(v)) if not (i >> idx) & 1 and abs(v[i]) > zero)
            assert p0 == pytest.approx(0.5, abs=zero)
        for eng, c in zip(engs, ctrls):
            Measure | c
            eng.flush()
        if not want_half:
            assert int(ctrls[0]) == 0
        else:
            break
    for eng, x in zip(engs, xs):
        All(Measure) | x
        eng.flush()


def test_reference_unitary_suite():
    """ProjectQ's UnitarySimulator tests (backends/_unitary_test.py) with
    projectq_gb300.unitary.UnitarySimulator (vec(U) on the GPU) in its place."""
    rc, passed, out = _refsuite.run("gpu", "c128", unitary=True)
    assert rc == 0, out[-6000:]
    assert passed >= 8


def test_unitary_matches_reference_class_on_random_circuits():
    """The GPU UnitarySimulator against ProjectQ's own (dense NumPy) class on
    random controlled circuits over 6 qubits (1e-12)."""
    if not projectq_available():
        pytest.skip("ProjectQ not importable")
    from projectq import MainEngine
    from projectq.backends import UnitarySimulator as RefUnitary
    from projectq.meta import Control
    from projectq.ops import CNOT, H, Rx, Ry, Rz, T, Toffoli

    from projectq_gb300.unitary import UnitarySimulator

    def build(backend, seed):
        rng = np.random.default_rng(seed)
        eng = MainEngine(backend=backend, engine_list=[])
        qureg = eng.allocate_qureg(6)
        for _ in range(60):
            kind = int(rng.integers(6))
            a, b, c = (int(v) for v in rng.choice(6, 3, replace=False))
            th = float(rng.uniform(0, 2 * np.pi))
            if kind == 0:
                H | qureg[a]
            elif kind == 1:
                Rx(th) | qureg[a]
            elif kind == 2:
                CNOT | (qureg[a], qureg[b])
            elif kind == 3:
                Toffoli | (qureg[a], qureg[b], qureg[c])
            elif kind == 4:
                with Control(eng, qureg[b]):
                    Ry(th) | qureg[a]
            else:
                T | qureg[a]
                Rz(th) | qureg[b]
        eng.flush()
        return eng, qureg

    for seed in (0, 1):
        ours, ref = UnitarySimulator(), RefUnitary()
        build(ours, seed)
        build(ref, seed)
        assert np.max(np.abs(ours.unitary - ref.unitary)) < 1e-12


@pytest.mark.parametrize("hamiltonian", ["reference", "commuting"])
def test_time_evolution_against_scipy_expm(hamiltonian):
    """The reference's time-evolution check (_simulator_test.py:514-570) with
    NumPy-2-safe array conversion: controlled exp(-i t H) on 8 qubits vs
    scipy.sparse.linalg.expm_multiply; with the reference's four-term H (the
    Taylor series) and with a Hamiltonian whose terms commute (the exact
    product of term exponentials)."""
    if not projectq_available():
        pytest.skip("ProjectQ not importable")
    import scipy.sparse
    import scipy.sparse.linalg
    from projectq import MainEngine
    from projectq.backends import Simulator
    from projectq.meta import Control
    from projectq.ops import All, H, Measure, QubitOperator, Rx, Ry, TimeEvolution

    # stated bounds on max |d psi| against expm: complex128 1e-10; complex64
    # 1e-6 (the series runs on FP64 vectors, the exact product applies each
    # term's exponential as a complex64 gate: a few complex64 roundings)
    for prec, tol in (("c128", 1e-10), ("c64", 1e-6)):
        backend = Simulator(gate_fusion=True)
        backend._simulator = make("gpu", seed=1, precision=prec)
        eng = MainEngine(backend, [])
        N, t = 8, 1.1
        qureg = eng.allocate_qureg(N)
        rng = np.random.default_rng(0)
        for qb in qureg:
            Rx(float(rng.uniform())) | qb
            Ry(float(rng.uniform())) | qb
        eng.flush()
        bitmap, init = backend.cheat()
        init = np.asarray(init).copy()
        if hamiltonian == "reference":
            op = 0.3 * QubitOperator("X0 Y1 Z2 Y3 X4") + 1.1 * QubitOperator(()) \
                - 1.4 * QubitOperator("Y0 Z1 X3 Y5") - 1.1 * QubitOperator("Y1 X2 X3 Y4")
        else:
            op = 0.5 * QubitOperator("Z0 Z1") - 0.7 * QubitOperator("X0 X1") + 0.4 * QubitOperator("Y0 Y1") \
                + 1.1 * QubitOperator(()) + 0.3 * QubitOperator("Z2 Z3 Z4") + 0.2 * QubitOperator("X5 X6 X7") \
                - 0.6 * QubitOperator("Z5 Z6")
        ctrl = eng.allocate_qubit()
        H | ctrl
        before = backend._simulator.counters()
        with Control(eng, ctrl):
            TimeEvolution(t, op) | qureg
        eng.flush()
        after = backend._simulator.counters()
        path = "evolutions_taylor" if hamiltonian == "reference" else "evolutions_exact"
        assert after[path] == before[path] + 1
        bitmap2, final = backend.cheat()
        final = np.asarray(final).copy()
        All(Measure) | qureg + ctrl
        I2 = scipy.sparse.identity(2, format="csr", dtype=complex)
        P = {"X": scipy.sparse.csr_matrix([[0, 1], [1, 0]], dtype=complex),
             "Y": scipy.sparse.csr_matrix([[0, -1j], [1j, 0]], dtype=complex),
             "Z": scipy.sparse.csr_matrix([[1, 0], [0, -1]], dtype=complex)}
        Hm = 0
        for term, c in op.terms.items():
            mats = [I2] * N
            for idx, g in term:
                mats[bitmap2[qureg[idx].id]] = P[g]
            m = mats[-1]
            for k in range(N - 2, -1, -1):
                m = scipy.sparse.kron(m, mats[k])
            Hm = Hm + c * m
        ref = scipy.sparse.linalg.expm_multiply(-1j * t * Hm, init)
        half = len(final) // 2
        assert np.max(np.abs(final[half:] - ref / np.sqrt(2.0))) <= tol
        assert np.max(np.abs(final[:half] - init / np.sqrt(2.0))) <= tol
