"""Seeded random inputs for the parity tests (shared with the fixture
generator tests/golden/make_golden.py)."""

from fractions import Fraction

import numpy as np

from projectq_gb300.workloads import H, Rx, Ry, Rz, S, T, X, Y, Z


def haar_unitary(k, rng):
    """Haar-random 2^k x 2^k unitary: QR of a complex Gaussian matrix with
    the phases of diag(R) divided out."""
    d = 1 << k
    z = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / np.sqrt(2.0)
    q, r = np.linalg.qr(z)
    ph = np.diag(r) / np.abs(np.diag(r))
    return q * ph[None, :]


def random_mixed_circuit(n, ngates, seed, kmax=5, max_ctrl=3):
    """Gates of every shape the engine sees: named 1-qubit gates, rotations,
    dense Haar gates on up to kmax qubits, with 0..max_ctrl controls."""
    rng = np.random.default_rng(seed)
    named = [H, X, Y, Z, S, T]
    gates = []
    for _ in range(ngates):
        kind = rng.integers(4)
        if kind == 0:
            m = named[int(rng.integers(len(named)))]
            k = 1
        elif kind == 1:
            m = [Rx, Ry, Rz][int(rng.integers(3))](float(rng.uniform(0, 4 * np.pi)))
            k = 1
        else:
            k = int(rng.integers(1, min(kmax, n) + 1))
            m = haar_unitary(k, rng)
        nc = int(rng.integers(0, min(max_ctrl, n - k) + 1))
        qs = [int(v) for v in rng.choice(n, size=k + nc, replace=False)]
        gates.append((m, tuple(qs[:k]), tuple(qs[k:])))
    return gates


def random_pauli_sum(nq, nterms, seed, with_identity=True, p_identity=0.5):
    rng = np.random.default_rng(seed)
    terms = []
    if with_identity:
        terms.append(([], float(rng.standard_normal())))
    for _ in range(nterms):
        term = []
        for q in range(nq):
            if rng.uniform() < p_identity:
                continue
            term.append((q, "XYZ"[int(rng.integers(3))]))
        terms.append((term, float(rng.standard_normal())))
    return terms


def run_circuit(sim, gates, run_each=False):
    for m, t, c in gates:
        sim.apply_controlled_gate(m, list(t), list(c))
        if run_each:
            sim.run()
    sim.run()


def allocate(sim, n):
    for q in range(n):
        sim.allocate_qubit(q)


def fma(a, b, c):
    """a*b + c with a single rounding (exact rational arithmetic, then the
    correctly rounded float): the value of C's fma()."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def norm2(z):
    """|z|^2 as the reference's std::norm compiles with FMA: fma(re, re, im*im)."""
    return fma(z.real, z.real, z.imag * z.imag)


def numpy_apply(psi, U, targets, ctrls, n):
    """FP64 reference for one controlled k-qubit gate, independent of every
    engine: the state as a tensor of n axes (axis a <-> bit n-1-a), the
    target axes moved to the front in matrix-bit order (targets[k-1] first),
    one NumPy matrix product, and the old values kept where a control is 0."""
    k = len(targets)
    axes = [n - 1 - q for q in reversed(targets)]
    t = np.moveaxis(np.asarray(psi, dtype=np.complex128).reshape([2] * n), axes, list(range(k)))
    shp = t.shape
    X = t.reshape(1 << k, -1)
    Y = np.asarray(U, dtype=np.complex128) @ X
    if ctrls:
        rest = [q for q in range(n - 1, -1, -1) if q not in targets]  # remaining axes, most significant first
        r = np.arange(X.shape[1])
        ok = np.ones(X.shape[1], dtype=bool)
        for c in ctrls:
            ok &= ((r >> (len(rest) - 1 - rest.index(c))) & 1).astype(bool)
        Y = np.where(ok[None, :], Y, X)
    return np.ascontiguousarray(np.moveaxis(Y.reshape(shp), list(range(k)), axes)).reshape(-1)
