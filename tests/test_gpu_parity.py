"""Parity of the CUDA engine (libgb300sim.so, through the C ABI) with the
oracle, on the same seeded inputs.

Tolerances: complex128 amplitudes agree to 1e-12 absolute (normalised states)
and complex64 to 5e-6; measurement outcomes at a given uniform draw and
emulate_math permutations are compared exactly.
"""

import numpy as np
import pytest

from _backends import make
from _circuits import allocate, haar_unitary, norm2, random_mixed_circuit, random_pauli_sum, run_circuit
from projectq_gb300.workloads import H, X, Z, mt19937_uniform, random_state

pytestmark = pytest.mark.gpu

TOL = {"c128": 1e-12, "c64": 5e-6}
PRECS = ["c128", "c64"]


def pair(n, prec="c128", seed=1, fusion="reference"):
    g = make("gpu", seed=seed, precision=prec, fusion=fusion)
    o = make("oracle", seed=seed)
    allocate(g, n)
    allocate(o, n)
    return g, o


def assert_states(g, o, prec, tol=None):
    mg, sg = g.cheat()
    mo, so = o.cheat()
    assert mg == mo
    err = float(np.max(np.abs(sg - so))) if len(so) else 0.0
    assert err <= (tol or TOL[prec]), err


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("fusion", ["reference", "none", "staged"])
@pytest.mark.parametrize("n,seed", [(1, 0), (3, 1), (5, 2), (8, 3), (12, 4)])
def test_random_circuits(prec, fusion, n, seed):
    gates = random_mixed_circuit(n, 50, seed, kmax=min(5, n), max_ctrl=min(3, n - 1))
    g, o = pair(n, prec, fusion=fusion)
    run_circuit(g, gates)
    run_circuit(o, gates)
    assert_states(g, o, prec)


@pytest.mark.parametrize("prec", PRECS)
def test_every_position_one_and_two_qubit(prec):
    """Every target position (and pairs) with and without a control, n = 7."""
    n = 7
    rng = np.random.default_rng(5)
    psi = random_state(n, seed=9)
    gates = []
    for t in range(n):
        gates.append((haar_unitary(1, rng), (t,), ()))
        for c in range(n):
            if c != t:
                gates.append((haar_unitary(1, rng), (t,), (c,)))
    for a in range(n):
        for b in range(n):
            if a != b:
                gates.append((haar_unitary(2, rng), (a, b), ()))
    g, o = pair(n, prec, fusion="none")
    o.set_fusion("none")
    g.set_wavefunction(psi, list(range(n)))
    o.set_wavefunction(psi, list(range(n)))
    run_circuit(g, gates)
    run_circuit(o, gates)
    assert_states(g, o, prec, tol=TOL[prec] * 20)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("k", [3, 4, 5])
def test_wide_gates_with_controls(prec, k):
    n = 11
    rng = np.random.default_rng(k)
    psi = random_state(n, seed=k)
    gates = []
    for _ in range(12):
        qs = [int(v) for v in rng.choice(n, size=k + 2, replace=False)]
        gates.append((haar_unitary(k, rng), tuple(qs[:k]), tuple(qs[k:k + int(rng.integers(0, 3))])))
    g, o = pair(n, prec, fusion="none")
    o.set_fusion("none")
    g.set_wavefunction(psi, list(range(n)))
    o.set_wavefunction(psi, list(range(n)))
    run_circuit(g, gates)
    run_circuit(o, gates)
    assert_states(g, o, prec)


def _sequential_pick(psi, rnd):
    """The reference's sampling loop, element by element (simulator.hpp:152-160)."""
    P = 0.0
    pick = 0
    for z in psi:
        if not P < rnd:
            break
        P += norm2(z)
        pick += 1
    return pick - 1


@pytest.mark.parametrize("n", [9, 18])
def test_measure_at_draws_bit_exact(n):
    """Same state, same uniform draw -> same outcome bits as the reference's
    sequential FP64 sampling rule, including draws placed exactly on running
    sums (n = 18 exercises the blocked replay, n = 9 the host loop)."""
    psi = random_state(n, seed=21)
    norms = [norm2(z) for z in psi[: 1 << min(n, 12)]]
    running = []
    P = 0.0
    for x in norms:
        P += x
        running.append(P)
    draws = [0.0, 1e-300, 0.5, 0.999999, 0.9999999999999999, running[3], running[100],
             np.nextafter(running[200], 0), np.nextafter(running[200], 1)]
    draws += list(np.random.default_rng(1).uniform(size=20))
    ids = list(range(n))
    for rnd in draws:
        g = make("gpu", seed=1, precision="c128")
        o = make("oracle", seed=1)
        allocate(g, n)
        allocate(o, n)
        g.set_wavefunction(psi, ids)
        o.set_wavefunction(psi, ids)
        bg = g.measure_qubits_at(ids, float(rnd))
        bo = o.measure_qubits_at(ids, float(rnd))
        assert bg == bo, rnd
        if n <= 12:
            pick = _sequential_pick(psi, rnd) & ((1 << n) - 1)
            assert bg == [bool((pick >> q) & 1) for q in ids]
        assert_states(g, o, "c128")


@pytest.mark.parametrize("prec", PRECS)
def test_seeded_measurements_follow_engine_rng(prec):
    n = 6
    gates = random_mixed_circuit(n, 30, 4)
    g, o = pair(n, prec, seed=123)
    run_circuit(g, gates)
    run_circuit(o, gates)
    draws = mt19937_uniform(123, 3)
    for rnd in draws:
        bg = g.measure_qubits([0, 2, 4])
        bo = o.measure_qubits_at([0, 2, 4], rnd)
        assert bg == bo
        assert_states(g, o, prec)


@pytest.mark.parametrize("prec", PRECS)
def test_probability_amplitude_collapse(prec):
    n = 8
    gates = random_mixed_circuit(n, 40, 6)
    g, o = pair(n, prec)
    run_circuit(g, gates)
    run_circuit(o, gates)
    for bits, ids in [([1], [3]), ([0, 1, 1], [0, 5, 2]), ([1] * 8, list(range(8)))]:
        assert g.get_probability(bits, ids) == pytest.approx(o.get_probability(bits, ids), abs=TOL[prec] * 10)
    ids = [3, 1, 4, 0, 7, 6, 2, 5]
    for b in range(0, 256, 37):
        bits = [(b >> i) & 1 for i in range(8)]
        assert abs(g.get_amplitude(bits, ids) - o.get_amplitude(bits, ids)) < TOL[prec]
    with pytest.raises(RuntimeError):
        g.get_amplitude([0] * 7, ids[:7])
    g.collapse_wavefunction([2, 5], [1, 0])
    o.collapse_wavefunction([2, 5], [1, 0])
    assert_states(g, o, prec)
    with pytest.raises(ValueError):
        g.collapse_wavefunction([2, 5], [1])
    with pytest.raises(RuntimeError):
        g.collapse_wavefunction([2], [0])  # probability ~0 after the collapse above
    with pytest.raises(RuntimeError):
        g.collapse_wavefunction([99], [0])


@pytest.mark.parametrize("prec", PRECS)
def test_allocate_deallocate_classical(prec):
    g, o = pair(0, prec)
    for sim in (g, o):
        for q in range(6):
            sim.allocate_qubit(10 + q)
        sim.apply_controlled_gate(X, [12], [])
        sim.apply_controlled_gate(H, [14], [])
        sim.apply_controlled_gate(X, [11], [14])
        sim.run()
    for q in (10, 12, 13, 15):
        assert g.is_classical(q) == o.is_classical(q)
        assert g.get_classical_value(q) == o.get_classical_value(q)
    assert not g.is_classical(14)
    for q in (12, 10, 15):
        g.deallocate_qubit(q)
        o.deallocate_qubit(q)
        assert_states(g, o, prec)
    with pytest.raises(RuntimeError):
        g.deallocate_qubit(14)
    with pytest.raises(RuntimeError):
        g.allocate_qubit(11)
    g.measure_qubits_at([14], 0.75)
    o.measure_qubits_at([14], 0.75)
    g.deallocate_qubit(14)
    o.deallocate_qubit(14)
    assert_states(g, o, prec)


@pytest.mark.parametrize("prec", PRECS)
def test_expectation_and_qubit_operator(prec):
    n = 9
    gates = random_mixed_circuit(n, 40, 8)
    g, o = pair(n, prec)
    run_circuit(g, gates)
    run_circuit(o, gates)
    ids = [4, 2, 0, 1, 3, 8, 7, 6, 5]
    for seed in range(4):
        terms = random_pauli_sum(n, 12, seed)
        eg = g.get_expectation_value(terms, ids)
        eo = o.get_expectation_value(terms, ids)
        assert eg == pytest.approx(eo, abs=1e-10 if prec == "c128" else 2e-5)
    # repeated factors on one qubit compose like the gate sequence
    terms = [([(0, "X"), (0, "Y"), (3, "Z"), (3, "Z")], 0.7), ([(1, "Y"), (1, "X")], -0.4)]
    assert g.get_expectation_value(terms, ids) == pytest.approx(o.get_expectation_value(terms, ids), abs=2e-5)
    cterms = [(t, complex(c, 0.3 * c)) for t, c in random_pauli_sum(n, 6, 9)]
    g.apply_qubit_operator(cterms, ids)
    o.apply_qubit_operator(cterms, ids)
    assert_states(g, o, prec, tol=TOL[prec] * 50)
    with pytest.raises(TypeError):
        g.get_expectation_value([([(0, "X")], 1j)], ids)


@pytest.mark.parametrize("prec", PRECS)
def test_time_evolution_controlled(prec):
    n = 8
    gates = random_mixed_circuit(n, 30, 10)
    g, o = pair(n, prec)
    run_circuit(g, gates)
    run_circuit(o, gates)
    terms = [([(0, "X"), (1, "Y"), (2, "Z"), (3, "Y"), (4, "X")], 0.3), ([], 1.1),
             ([(0, "Y"), (1, "Z"), (3, "X"), (5, "Y")], -1.4), ([(1, "Y"), (2, "X"), (3, "X"), (4, "Y")], -1.1)]
    ids = list(range(7))
    g.emulate_time_evolution(terms, 1.1, ids, [7])
    o.emulate_time_evolution(terms, 1.1, ids, [7])
    assert_states(g, o, prec, tol=1e-11 if prec == "c128" else 2e-5)


@pytest.mark.parametrize("prec", PRECS)
def test_emulate_math_bit_exact(prec):
    n = 9
    psi = random_state(n, seed=31)
    ids = list(range(n))
    ops = [
        ("addConstant", (3,), [[0, 1, 2, 3, 4]], [6]),
        ("addConstantModN", (4, 5), [[0, 1, 2, 3, 4]], [7, 8]),
        ("multiplyByConstantModN", (15, 16), [[4, 2, 0, 1, 3]], []),  # not a bijection on 5 bits
        ("addConstant", (-5,), [[1, 3], [5, 6]], [0]),
    ]
    for name, args, regs, ctrl in ops:
        g = make("gpu", seed=1, precision=prec)
        o = make("oracle", seed=1)
        allocate(g, n)
        allocate(o, n)
        g.set_wavefunction(psi, ids)
        o.set_wavefunction(psi, ids)
        getattr(g, "emulate_math_" + name)(*args, regs, ctrl)
        getattr(o, "emulate_math_" + name)(*args, regs, ctrl)
        sg = g.cheat(dtype=np.complex64 if prec == "c64" else np.complex128)[1]
        so = o.cheat()[1]
        if prec == "c128":
            assert np.array_equal(sg.view(np.uint64), so.view(np.uint64)), name
        else:
            assert np.max(np.abs(sg - so)) < 1e-6, name

    def f(vals):
        return [(vals[0] * vals[0] + 1) % 8, vals[1] ^ vals[0]]

    g = make("gpu", seed=1, precision=prec)
    o = make("oracle", seed=1)
    allocate(g, n)
    allocate(o, n)
    g.set_wavefunction(psi, ids)
    o.set_wavefunction(psi, ids)
    g.emulate_math(f, [[0, 1, 2], [3, 4, 5]], [8])
    o.emulate_math(f, [[0, 1, 2], [3, 4, 5]], [8])
    assert_states(g, o, prec, tol=0.0 if prec == "c128" else 1e-6)


@pytest.mark.parametrize("prec", PRECS)
def test_set_wavefunction_cheat_roundtrip(prec):
    n = 10
    psi = random_state(n, seed=2)
    g = make("gpu", seed=1, precision=prec)
    with pytest.raises(RuntimeError):
        g.set_wavefunction(psi, list(range(n)))
    allocate(g, n)
    order = [3, 1, 4, 0, 9, 2, 6, 5, 8, 7]
    g.set_wavefunction(psi, order)
    m, s = g.cheat()
    assert m == {q: i for i, q in enumerate(order)}
    assert np.max(np.abs(s - psi)) < (0 if prec == "c128" else 1e-7) + 1e-300
    with pytest.raises(ValueError):
        g.set_wavefunction(psi[:8], order)


def test_errors_match_reference_types():
    g = make("gpu", seed=1)
    allocate(g, 3)
    with pytest.raises(RuntimeError):
        g.allocate_qubit(1)
    with pytest.raises(RuntimeError):
        g.get_probability([1], [17])
    with pytest.raises(ValueError):
        g.apply_controlled_gate(np.eye(4), [0], [])
    g.apply_controlled_gate(H, [0], [])
    g.apply_controlled_gate(Z, [1], [0])
    g.run()
    with pytest.raises(RuntimeError):
        g.deallocate_qubit(0)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("fusion", ["reference", "staged"])
def test_gate_stream_equals_per_gate_calls(prec, fusion):
    """gsim_apply_gates (one call for many gates) queues exactly what the same
    apply_controlled_gate calls queue; a malformed gate in the stream raises
    and the gates before it stay queued."""
    n = 10
    gates = random_mixed_circuit(n, 80, 7, kmax=4, max_ctrl=2)
    g, o = pair(n, prec, fusion=fusion)
    g.apply_gates(gates)
    g.run()
    run_circuit(o, gates)
    assert_states(g, o, prec)
    g2, o2 = pair(n, prec, fusion=fusion)
    bad = gates[:5] + [(np.eye(4), [0, 0], [])] + gates[5:]
    with pytest.raises(ValueError):
        g2.apply_gates(bad)
    g2.run()
    run_circuit(o2, gates[:5])
    assert_states(g2, o2, prec)


@pytest.mark.parametrize("prec", PRECS)
def test_pull_upload_of_page_locked_state(prec):
    """set_upload_mode("pull"): the SMs read a page-locked host state through
    its device view; the result equals the copy-engine upload, and pageable
    or differently typed arrays fall back to the copy paths."""
    from projectq_gb300.simulator import pin_host

    n = 14
    dt = np.complex64 if prec == "c64" else np.complex128
    psi = random_state(n, seed=11).astype(dt)
    g = make("gpu", seed=1, precision=prec)
    allocate(g, n)
    g.set_upload_mode("pull")
    pin = pin_host(psi)
    try:
        g.set_wavefunction(psi, list(range(n)))
        assert np.array_equal(g.cheat()[1].astype(dt), psi)
    finally:
        pin.close()
    g.set_wavefunction(psi[::-1].copy(), list(range(n)))  # pageable: copy engine
    assert np.array_equal(g.cheat()[1].astype(dt), psi[::-1])
    other = random_state(n, seed=12)  # complex128 into either precision
    g.set_wavefunction(other, list(range(n)))
    assert np.max(np.abs(g.cheat()[1] - other)) <= TOL[prec]


def test_headline_circuit_precision_form():
    """The 30-qubit headline circuit's family at 20 qubits: complex64 with FP64
    reductions (stage planner) against the complex128 path and the CPU oracle:
    1 - F <= 1e-6 (the stated bar; measured ~1e-12) and expectation values
    within 1e-6."""
    from projectq_gb300.workloads import random_gate_circuit

    n = 20
    gates = random_gate_circuit(n, depth=40, per_layer=40, seed=0)
    psi0 = random_state(n, seed=0)
    states, ev = {}, {}
    zz = [([(0, "Z"), (1, "Z")], 1.0), ([(5, "X"), (6, "X")], 1.0)]
    for key, kind, prec, fusion in (("c64", "gpu", "c64", "staged"), ("c128", "gpu", "c128", "staged"),
                                    ("oracle", "oracle", "c128", "reference")):
        s = make(kind, seed=1, precision=prec, fusion=fusion)
        allocate(s, n)
        if kind == "oracle":
            s.set_fusion("none")  # one pass per gate: exact FP64 reference, fast on the CPU
        s.set_wavefunction(psi0, list(range(n)))
        run_circuit(s, gates)
        ev[key] = s.get_expectation_value(zz, list(range(n)))
        states[key] = s.cheat()[1]
    ref = states["oracle"]
    assert np.max(np.abs(states["c128"] - ref)) < 1e-12
    for key in ("c64", "c128"):
        f = abs(np.vdot(ref, states[key])) ** 2 / (np.vdot(ref, ref).real * np.vdot(states[key], states[key]).real)
        assert 1 - f <= 1e-6, (key, 1 - f)
        assert abs(ev[key] - ev["oracle"]) <= 1e-6


@pytest.mark.parametrize("kmax", [1, 2, 3, 6, 7])
def test_greedy_fusion_width(kmax):
    """set_fusion("reference", kmax): the greedy fixed-size rule with clusters
    of up to kmax qubits (complex64 clusters of 5-7 run on tensor cores)
    applies the same gates as the oracle."""
    n = 16
    gates = random_mixed_circuit(n, 120, 21 + kmax, kmax=3, max_ctrl=2)
    for prec in PRECS:
        g, o = pair(n, prec)
        g.set_fusion("reference", kmax)
        run_circuit(g, gates)
        run_circuit(o, gates)
        assert_states(g, o, prec, tol=TOL[prec] * (4 if prec == "c64" else 1))


@pytest.mark.parametrize("prec", ["c64", "c128"])
def test_cuda_array_view_is_the_engine_state(prec):
    """Simulator.cuda_array() (the zero-copy __cuda_array_interface__ view of
    the flushed state) consumed by torch: same dtype, shape and values as
    cheat(), and a write through the view is seen by the engine."""
    torch = pytest.importorskip("torch")
    n = 12
    sim = make("gpu", seed=1, precision=prec, fusion="staged")
    allocate(sim, n)
    run_circuit(sim, random_mixed_circuit(n, 60, seed=4))
    t = torch.as_tensor(sim.cuda_array(), device="cuda")
    assert t.dtype == (torch.complex64 if prec == "c64" else torch.complex128)
    assert tuple(t.shape) == (1 << n,)
    dt = np.complex64 if prec == "c64" else np.complex128
    assert np.array_equal(t.cpu().numpy(), sim.cheat(dtype=dt)[1])
    t[0] = 0.25 - 0.5j
    torch.cuda.synchronize()
    assert sim.get_amplitude([0] * n, list(range(n))) == 0.25 - 0.5j


@pytest.mark.parametrize("n", [14, 18, 22])
@pytest.mark.parametrize("mode", ["packed", "register", "pass"])
def test_stage_kernels_against_oracle(n, mode):
    """The staged planner's three complex64 stage kernels on the headline
    circuit family plus controlled 1-qubit gates (register, row and
    non-local controls) against the oracle: max |d psi| 1e-5 (complex64)."""
    from projectq_gb300.workloads import random_gate_circuit

    gates = random_gate_circuit(n, depth=10, per_layer=n, seed=n)
    rng = np.random.default_rng(n)
    for g in random_mixed_circuit(n, 50, n + 1, kmax=1, max_ctrl=3):
        gates.insert(int(rng.integers(len(gates) + 1)), g)
    psi = random_state(n, seed=n)
    g = make("gpu", seed=1, precision="c64", fusion="staged")
    g.set_stage_kernel(mode)
    allocate(g, n)
    g.set_wavefunction(psi.astype(np.complex64), list(range(n)))
    run_circuit(g, gates)
    o = make("oracle", seed=1)
    allocate(o, n)
    o.set_wavefunction(psi, list(range(n)))
    run_circuit(o, gates)
    assert np.max(np.abs(g.cheat()[1] - o.cheat()[1])) < 1e-5


@pytest.mark.parametrize("n", [13, 16, 20])
def test_packed_register_controlled_x_against_oracle(n):
    """X gates with 0-3 controls all among four neighbouring qubits, between
    rotations on them: inside a packed-pair substage these are in-place
    exchanges of the pairs their register controls select (one body per
    control mask), checked against the oracle (complex64, 1e-5)."""
    rng = np.random.default_rng(100 + n)
    from projectq_gb300.workloads import Rx, Ry, X
    gates = []
    for _ in range(120):
        block = [int(q) for q in rng.permutation(4)] if rng.uniform() < 0.5 else [int(q) + 6 for q in rng.permutation(4)]
        nctl = int(rng.integers(0, 4))
        if rng.uniform() < 0.3:
            gates.append(((Rx, Ry)[int(rng.integers(2))](float(rng.uniform(0, 2 * np.pi))), (block[0],), ()))
        else:
            gates.append((X, (block[0],), tuple(block[1:1 + nctl])))
    psi = random_state(n, seed=n)
    g = make("gpu", seed=1, precision="c64", fusion="staged")
    g.set_stage_kernel("packed")
    allocate(g, n)
    g.set_wavefunction(psi.astype(np.complex64), list(range(n)))
    run_circuit(g, gates)
    o = make("oracle", seed=1)
    allocate(o, n)
    o.set_wavefunction(psi, list(range(n)))
    run_circuit(o, gates)
    assert np.max(np.abs(g.cheat()[1] - o.cheat()[1])) < 1e-5
