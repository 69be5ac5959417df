"""Seeded synthetic workloads used by bench.py and the tests.

Gate matrices follow ProjectQ's definitions (projectq/ops/_gates.py: H :72,
X :89, Y :106, Z :123, S :136, T :155, Rx :276-281, Ry :290-295,
Rz :304-309).  A circuit is a list of (matrix, target ids, control ids);
qubit ids are 0..n-1, allocated in order, so id i sits at bit position i.
"""

from __future__ import annotations

import math

import numpy as np

SQ2 = 1.0 / math.sqrt(2.0)
H = np.array([[SQ2, SQ2], [SQ2, -SQ2]], dtype=np.complex128)
X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
Z = np.array([[1, 0], [0, -1]], dtype=np.complex128)
S = np.array([[1, 0], [0, 1j]], dtype=np.complex128)
T = np.array([[1, 0], [0, np.exp(1j * np.pi / 4)]], dtype=np.complex128)


def Rx(t):  # noqa: N802 (ProjectQ's gate names)
    c, s = math.cos(0.5 * t), math.sin(0.5 * t)
    return np.array([[c, -1j * s], [-1j * s, c]], dtype=np.complex128)


def Ry(t):  # noqa: N802
    c, s = math.cos(0.5 * t), math.sin(0.5 * t)
    return np.array([[c, -s], [s, c]], dtype=np.complex128)


def Rz(t):  # noqa: N802
    return np.array([[np.exp(-0.5j * t), 0], [0, np.exp(0.5j * t)]], dtype=np.complex128)


def layered_rotation_circuit(n=20, depth=20, seed=0):
    """Layered circuit: Rx, Ry, Rz on every qubit (angles U[0, 2pi) drawn in
    layer -> qubit -> gate order from numpy default_rng(seed)), then CNOT
    (i -> i+1) for i = 0, 2, ... on even layers and 1, 3, ... on odd ones."""
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0.0, 2.0 * np.pi, size=(depth, n, 3))
    gates = []
    for layer in range(depth):
        for q in range(n):
            gates.append((Rx(ang[layer, q, 0]), (q,), ()))
            gates.append((Ry(ang[layer, q, 1]), (q,), ()))
            gates.append((Rz(ang[layer, q, 2]), (q,), ()))
        for i in range(layer % 2, n - 1, 2):
            gates.append((X, (i + 1,), (i,)))
    return gates


RANDOM_GATE_KINDS = ("H", "T", "S", "Rx", "Ry", "Rz", "CNOT", "CZ", "Toffoli")


def random_gate_circuit(n=30, depth=40, per_layer=40, seed=0):
    """Random circuit: each layer has `per_layer` gates drawn uniformly from
    {H, T, S, Rx, Ry, Rz (theta ~ U[0, 2pi)), CNOT and CZ on a random pair,
    Toffoli on a random triple (2 controls)}, all on uniformly random qubits."""
    rng = np.random.default_rng(seed)
    gates = []
    for _ in range(depth):
        for _ in range(per_layer):
            kind = RANDOM_GATE_KINDS[int(rng.integers(len(RANDOM_GATE_KINDS)))]
            if kind in ("H", "T", "S"):
                q = int(rng.integers(n))
                gates.append(({"H": H, "T": T, "S": S}[kind], (q,), ()))
            elif kind in ("Rx", "Ry", "Rz"):
                q = int(rng.integers(n))
                t = float(rng.uniform(0.0, 2.0 * np.pi))
                gates.append(({"Rx": Rx, "Ry": Ry, "Rz": Rz}[kind](t), (q,), ()))
            elif kind in ("CNOT", "CZ"):
                c, t = (int(v) for v in rng.choice(n, size=2, replace=False))
                gates.append((X if kind == "CNOT" else Z, (t,), (c,)))
            else:
                c1, c2, t = (int(v) for v in rng.choice(n, size=3, replace=False))
                gates.append((X, (t,), (c1, c2)))
    return gates


def random_state(n, seed=0, dtype=np.complex128, chunk=1 << 24):
    """i.i.d. complex Gaussian amplitudes (numpy PCG64, `seed`), normalised.
    Generated in chunks so that 2^30-amplitude states fit host memory."""
    rng = np.random.default_rng(seed)
    N = 1 << n
    out = np.empty(N, dtype=dtype)
    nrm = 0.0
    for o in range(0, N, chunk):
        c = min(chunk, N - o)
        z = rng.standard_normal(c) + 1j * rng.standard_normal(c)
        nrm += float(np.vdot(z, z).real)
        out[o:o + c] = z
    s = 1.0 / math.sqrt(nrm)
    for o in range(0, N, chunk):
        out[o:o + chunk] *= s
    return out


def gate_bytes(nq, ctrl_count, bytes_per_amp):
    """Algorithmic HBM bytes of one gate: read + write of the 2^(N-c)
    amplitudes that satisfy the controls."""
    return 2 * (1 << (nq - ctrl_count)) * bytes_per_amp


def mt19937_uniform(seed, count):
    """The first `count` draws of std::uniform_real_distribution<double>(0, 1)
    over std::mt19937(seed) (libstdc++: generate_canonical from two 32-bit
    outputs), as the engine's measurement RNG produces them."""
    bg = np.random.MT19937()
    bg._legacy_seeding(int(seed))
    out = []
    for _ in range(count):
        x0, x1 = (int(v) for v in bg.random_raw(2))
        r = float(x0 + x1 * 2**32) / 2.0**64
        if r >= 1.0:
            r = math.nextafter(1.0, 0.0)
        out.append(r)
    return out


def random_pauli_hamiltonian(n, nterms=200, seed=0, p_identity=0.7):
    """`nterms` Pauli strings: each qubit I with probability p_identity and
    X, Y, Z with (1 - p_identity)/3 each; coefficients ~ N(0, 1).  Returned
    as [(term, coeff)] with term = [(qubit index, 'X'|'Y'|'Z'), ...]."""
    rng = np.random.default_rng(seed)
    q = (1.0 - p_identity) / 3.0
    terms = []
    for _ in range(nterms):
        ops = rng.choice(4, size=n, p=[p_identity, q, q, q])
        term = [(i, "XYZ"[o - 1]) for i, o in enumerate(ops) if o]
        terms.append((term, float(rng.standard_normal())))
    return terms
