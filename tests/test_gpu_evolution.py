"""emulate_time_evolution for Hamiltonians whose terms commute: the exact
product of the terms' exponentials (gsim_set_time_evolution mode 1, the
default) against a dense scipy expm and against the oracle's Taylor series
(simulator.hpp:386-438), and the fall-back to the series when a pair of terms
anticommutes or a term acts on a control.

Tolerances: complex128 1e-12 against expm (the exact product rounds once per
gate) and 1e-11 against the oracle (whose series stops at an update norm of
1e-12); complex64 2e-5 (FP32 amplitudes).
"""

import numpy as np
import pytest

from _backends import make
from _circuits import allocate, random_mixed_circuit, random_pauli_sum, run_circuit

pytestmark = pytest.mark.gpu

PAULI = {
    "X": np.array([[0, 1], [1, 0]], dtype=np.complex128),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    "Z": np.array([[1, 0], [0, -1]], dtype=np.complex128),
}
TOL_EXPM = {"c128": 1e-12, "c64": 2e-5}
TOL_ORACLE = {"c128": 1e-11, "c64": 2e-5}


def symplectic(term):
    x = z = 0
    for q, p in term:
        if p in "XY":
            x |= 1 << q
        if p in "YZ":
            z |= 1 << q
    return x, z


def commute(a, b):
    (xa, za), (xb, zb) = symplectic(a), symplectic(b)
    return (bin(xa & zb).count("1") + bin(za & xb).count("1")) % 2 == 0


def random_commuting(nq, nterms, rng, wmin=1, wmax=4, paulis="XYZ", identity=True, start=()):
    """Random Pauli strings of weight wmin..wmax, each kept only if it commutes
    with every string kept before it (those of `start` included)."""
    terms = list(start) or ([([], float(rng.standard_normal()))] if identity else [])
    tries = 0
    while len(terms) < nterms and tries < 5000:
        tries += 1
        w = int(rng.integers(wmin, wmax + 1))
        qs = sorted(rng.choice(nq, size=w, replace=False).tolist())
        term = [(q, paulis[int(rng.integers(len(paulis)))]) for q in qs]
        if all(commute(term, t) for t, _ in terms if t):
            terms.append((term, float(rng.standard_normal())))
    return terms


def ising(nq, rng):
    terms = [([], 0.7)]
    for i in range(nq):
        terms.append(([(i, "Z"), ((i + 1) % nq, "Z")] if i + 1 < nq else [(0, "Z"), (i, "Z")],
                      float(rng.standard_normal())))
        terms.append(([(i, "Z")], float(rng.standard_normal())))
    return terms


def dense(terms, nq):
    h = np.zeros((1 << nq, 1 << nq), dtype=np.complex128)
    for term, c in terms:
        ops = {q: PAULI[p] for q, p in term}
        m = np.ones((1, 1), dtype=np.complex128)
        for q in reversed(range(nq)):  # bit q of the index = qubit q
            m = np.kron(m, ops.get(q, np.eye(2)))
        h += c * m
    return h


def expected(psi, terms, t, nq, ctrl_bit=None):
    """exp(-i t H) on qubits 0..nq-1 of psi, on the part where ctrl_bit is 1."""
    import scipy.linalg

    u = scipy.linalg.expm(-1j * t * dense(terms, nq))
    psi = np.asarray(psi, dtype=np.complex128).copy()
    if ctrl_bit is None:
        return u @ psi
    lo = 1 << nq
    blocks = psi.reshape(-1, lo)  # ctrl_bit = nq: block 1 holds the controlled half
    assert ctrl_bit == nq and blocks.shape[0] == 2
    blocks[1] = u @ blocks[1]
    return blocks.reshape(-1)


def prepared(n, prec, fusion="reference", seed=3):
    g = make("gpu", seed=1, precision=prec, fusion=fusion)
    allocate(g, n)
    run_circuit(g, random_mixed_circuit(n, 40, seed, kmax=2, max_ctrl=1))
    g.run()
    return g


@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("fusion", ["reference", "none", "staged"])
@pytest.mark.parametrize("kind", ["ising", "commuting"])
def test_exact_product_matches_expm(prec, fusion, kind):
    n, t = 8, 0.9
    rng = np.random.default_rng(11)
    terms = ising(n, rng) if kind == "ising" else random_commuting(n, 14, rng)
    g = prepared(n, prec, fusion)
    _, before = g.cheat()
    g.reset_counters()
    g.emulate_time_evolution(terms, t, list(range(n)), [])
    c = g.counters()
    assert c["evolutions_exact"] == 1 and c["evolutions_taylor"] == 0
    _, after = g.cheat()
    err = float(np.max(np.abs(after - expected(before, terms, t, n))))
    assert err <= TOL_EXPM[prec], err


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_exact_product_controlled_matches_oracle_series(prec):
    n = 9
    rng = np.random.default_rng(5)
    terms = random_commuting(n - 1, 12, rng, wmax=5)
    gates = random_mixed_circuit(n, 40, 7, kmax=2, max_ctrl=1)
    g = make("gpu", seed=1, precision=prec)
    o = make("oracle", seed=1)
    for s in (g, o):
        allocate(s, n)
        run_circuit(s, gates)
        s.emulate_time_evolution(terms, 1.3, list(range(n - 1)), [n - 1])
    assert g.counters()["evolutions_exact"] == 1
    assert g.cheat()[0] == o.cheat()[0]
    err = float(np.max(np.abs(g.cheat()[1] - o.cheat()[1])))
    assert err <= TOL_ORACLE[prec], err


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_wide_terms_take_the_rotation_kernel(prec):
    """Terms on 6-9 qubits (wider than a gate of the planner) are one pass of
    the rotation kernel each; diagonal ones included; controlled."""
    n = 11
    rng = np.random.default_rng(2)
    terms = random_commuting(n - 1, 6, rng, wmin=6, wmax=9)
    terms = random_commuting(n - 1, 10, rng, wmin=6, wmax=8, paulis="Z", start=terms)
    assert sum(1 for tm, _ in terms if len(tm) > 5) >= 6
    g = prepared(n, prec, seed=4)
    _, before = g.cheat()
    g.reset_counters()
    g.emulate_time_evolution(terms, 0.7, list(range(n - 1)), [n - 1])
    c = g.counters()
    assert c["evolutions_exact"] == 1
    assert c["gate_launches"] >= sum(1 for tm, _ in terms if len(tm) > 5)
    _, after = g.cheat()
    err = float(np.max(np.abs(after - expected(before, terms, 0.7, n - 1, ctrl_bit=n - 1))))
    assert err <= TOL_EXPM[prec], err


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_anticommuting_terms_use_the_series(prec):
    n = 8
    terms = random_pauli_sum(n - 1, 6, seed=9)
    assert not all(commute(a, b) for i, (a, _) in enumerate(terms) for b, _ in terms[i + 1:] if a and b)
    gates = random_mixed_circuit(n, 30, 8, kmax=2, max_ctrl=1)
    g = make("gpu", seed=1, precision=prec)
    o = make("oracle", seed=1)
    for s in (g, o):
        allocate(s, n)
        run_circuit(s, gates)
        s.emulate_time_evolution(terms, 0.8, list(range(n - 1)), [n - 1])
    c = g.counters()
    assert c["evolutions_exact"] == 0 and c["evolutions_taylor"] == 1
    err = float(np.max(np.abs(g.cheat()[1] - o.cheat()[1])))
    assert err <= TOL_ORACLE[prec], err


def test_series_mode_and_control_overlap():
    """mode "taylor" always takes the series; a term on a control qubit, or a
    Hamiltonian of identity terms only, takes it in the default mode too; all
    three agree with the oracle."""
    n = 7
    rng = np.random.default_rng(4)
    terms = random_commuting(n, 8, rng)
    cases = [
        ("taylor", terms, list(range(n)), []),
        ("exact", [([(0, "Z"), (6, "X")], 0.4), ([(1, "Y")], -0.3)], list(range(n)), [6]),
        ("exact", [([], 0.9), ([], -0.2)], list(range(n)), [2]),
    ]
    gates = random_mixed_circuit(n, 30, 2, kmax=2, max_ctrl=1)
    for mode, tm, ids, ctrl in cases:
        g = make("gpu", seed=1, precision="c128")
        o = make("oracle", seed=1)
        g.set_time_evolution(mode)
        for s in (g, o):
            allocate(s, n)
            run_circuit(s, gates)
            s.emulate_time_evolution(tm, 1.1, ids, ctrl)
        c = g.counters()
        assert c["evolutions_exact"] == 0 and c["evolutions_taylor"] == 1, (mode, c)
        err = float(np.max(np.abs(g.cheat()[1] - o.cheat()[1])))
        assert err <= 1e-11, (mode, err)
    with pytest.raises(ValueError):
        make("gpu", seed=1).set_time_evolution("trotter")


def test_qaoa_layers_share_stage_passes():
    """A p = 4 QAOA-style evolution on 20 qubits (Ising cost layer, X mixer),
    staged fusion, complex64: every term is a gate, the planner fuses them into
    a few passes per layer, and the state equals the complex128 series result."""
    n = 20
    rng = np.random.default_rng(8)
    cost = ising(n, rng)
    mixer = [([(i, "X")], 1.0) for i in range(n)]
    g = make("gpu", seed=1, precision="c64", fusion="staged")
    r = make("gpu", seed=1, precision="c128", fusion="reference")
    r.set_time_evolution("taylor")
    for s in (g, r):
        allocate(s, n)
        for q in range(n):
            s.apply_controlled_gate(np.array([[1, 1], [1, -1]]) / np.sqrt(2), [q], [])
        s.run()
        s.reset_counters()
        for layer in range(4):
            s.emulate_time_evolution(cost, 0.3 + 0.1 * layer, list(range(n)), [])
            s.emulate_time_evolution(mixer, 0.5 - 0.1 * layer, list(range(n)), [])
    c = g.counters()
    assert c["evolutions_exact"] == 8
    assert c["gate_passes"] <= 8 * 3, c
    a, b = g.cheat()[1].astype(np.complex128), r.cheat()[1]
    fid = abs(np.vdot(b, a)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)
    assert 1 - fid < 1e-6, 1 - fid


@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("t", [1.3, -0.7, 6.0])
def test_chebyshev_expansion_for_anticommuting_terms(prec, t):
    """Mode "chebyshev": non-commuting terms by the Chebyshev expansion, against
    scipy's expm (1e-12) and the oracle's series (1e-11); controlled; up to
    |t| sum|c| of about 40."""
    n = 8
    terms = random_pauli_sum(n - 1, 8, seed=21)
    gates = random_mixed_circuit(n, 30, 5, kmax=2, max_ctrl=1)
    g = make("gpu", seed=1, precision=prec)
    o = make("oracle", seed=1)
    g.set_time_evolution("chebyshev")
    for s in (g, o):
        allocate(s, n)
        run_circuit(s, gates)
    _, before = g.cheat()
    for s in (g, o):
        s.emulate_time_evolution(terms, t, list(range(n - 1)), [n - 1])
    c = g.counters()
    assert c["evolutions_chebyshev"] == 1 and c["evolutions_taylor"] == 0
    err = float(np.max(np.abs(g.cheat()[1] - o.cheat()[1])))
    assert err <= TOL_ORACLE[prec], err
    if prec == "c128":
        want = expected(before, terms, t, n - 1, ctrl_bit=n - 1)
        err = float(np.max(np.abs(g.cheat()[1] - want)))
        assert err <= 1e-12, err


def test_chebyshev_mode_identity_and_commuting():
    """Identity-only Hamiltonians (a phase) and commuting ones (the exact
    product) behave in mode "chebyshev" as in the default mode."""
    n = 6
    gates = random_mixed_circuit(n, 20, 6, kmax=2, max_ctrl=1)
    rng = np.random.default_rng(3)
    for tm, path in (([([], 0.9), ([], -0.2)], "evolutions_chebyshev"), (ising(n - 1, rng), "evolutions_exact")):
        g = make("gpu", seed=1, precision="c128")
        o = make("oracle", seed=1)
        g.set_time_evolution("chebyshev")
        for s in (g, o):
            allocate(s, n)
            run_circuit(s, gates)
            s.emulate_time_evolution(tm, 0.8, list(range(n - 1)), [n - 1])
        assert g.counters()[path] == 1
        err = float(np.max(np.abs(g.cheat()[1] - o.cheat()[1])))
        assert err <= 1e-11, err


def test_exact_product_repeated_control_id():
    """A control id given twice acts once (the reference ORs it into its
    control mask)."""
    n = 6
    rng = np.random.default_rng(12)
    terms = random_commuting(n - 1, 8, rng)
    gates = random_mixed_circuit(n, 20, 9, kmax=2, max_ctrl=1)
    g = make("gpu", seed=1, precision="c128")
    o = make("oracle", seed=1)
    for s in (g, o):
        allocate(s, n)
        run_circuit(s, gates)
        s.emulate_time_evolution(terms, 0.9, list(range(n - 1)), [n - 1, n - 1])
    assert g.counters()["evolutions_exact"] == 1
    err = float(np.max(np.abs(g.cheat()[1] - o.cheat()[1])))
    assert err <= 1e-11, err
