"""The engine's host-side Pauli arithmetic (projectq_gb300/csrc/pauli.hpp),
checked on the CPU: the term form the expectation, Pauli-apply and
time-evolution kernels use (against products of 2x2 Pauli matrices in the
reference's factor order, simulator.hpp:538-550), the commutation test, a
term's exponential as a gate (against scipy's expm), and the Bessel
coefficients of the Chebyshev expansion (against scipy.special.jv and the
Jacobi-Anger identity)."""

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
SRC = HERE / "cpp" / "pauli_check.cpp"
HDR = HERE.parent / "projectq_gb300" / "csrc" / "pauli.hpp"
LIB = HERE.parent / "oracle" / "_build" / "libpauli_check.so"

PAULI = {
    "X": np.array([[0, 1], [1, 0]], dtype=np.complex128),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    "Z": np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


@pytest.fixture(scope="module")
def lib():
    LIB.parent.mkdir(parents=True, exist_ok=True)
    if not LIB.exists() or LIB.stat().st_mtime < max(SRC.stat().st_mtime, HDR.stat().st_mtime):
        subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", str(SRC), "-o", str(LIB)], check=True)
    lib = C.CDLL(str(LIB))
    lib.pauli_term.restype = C.c_int
    lib.pauli_term.argtypes = [C.POINTER(C.c_uint), C.c_char_p, C.c_int, C.POINTER(C.c_ulonglong),
                               C.POINTER(C.c_ulonglong), C.POINTER(C.c_int)]
    lib.paulis_commute.restype = C.c_int
    lib.paulis_commute.argtypes = [C.c_ulonglong] * 4
    lib.pauli_exp.restype = None
    lib.pauli_exp.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_double, C.c_double, C.c_double, C.c_double,
                              C.POINTER(C.c_double)]
    lib.bessel_orders.restype = C.c_int
    lib.bessel_orders.argtypes = [C.c_double, C.c_double, C.POINTER(C.c_double), C.c_int]
    return lib


def term(lib, factors):
    pos = (C.c_uint * max(1, len(factors)))(*[q for q, _ in factors])
    chars = "".join(p for _, p in factors).encode()
    x, z, ny = C.c_ulonglong(), C.c_ulonglong(), C.c_int()
    ok = lib.pauli_term(pos, chars, len(factors), C.byref(x), C.byref(z), C.byref(ny))
    return ok, x.value, z.value, ny.value


def dense_from_form(x, z, ny, n):
    """(P psi)_i = (-i)^ny (-1)^popcount(i & z) psi_{i ^ x}."""
    d = 1 << n
    m = np.zeros((d, d), dtype=np.complex128)
    for i in range(d):
        m[i, i ^ x] = (-1j) ** ny * (-1) ** bin(i & z).count("1")
    return m


def dense_product(factors, n):
    """F_last ... F_first, each factor a Pauli on bit q of the index."""
    m = np.eye(1 << n, dtype=np.complex128)
    for q, p in factors:
        ops = [np.eye(2)] * n
        ops[q] = PAULI[p]
        f = np.ones((1, 1))
        for k in reversed(range(n)):
            f = np.kron(f, ops[k])
        m = f @ m
    return m


def test_term_form_matches_factor_products(lib):
    rng = np.random.default_rng(0)
    n = 5
    for _ in range(300):
        nf = int(rng.integers(0, 7))
        factors = [(int(rng.integers(n)), "XYZ"[int(rng.integers(3))]) for _ in range(nf)]  # repeats allowed
        ok, x, z, ny = term(lib, factors)
        assert ok
        np.testing.assert_allclose(dense_from_form(x, z, ny, n), dense_product(factors, n), atol=1e-15)
    assert term(lib, [(0, "Q")])[0] == 0


def test_commutation(lib):
    rng = np.random.default_rng(1)
    n = 4
    for _ in range(300):
        a = [(q, "XYZ"[int(rng.integers(3))]) for q in range(n) if rng.uniform() < 0.6]
        b = [(q, "XYZ"[int(rng.integers(3))]) for q in range(n) if rng.uniform() < 0.6]
        _, xa, za, _ = term(lib, a)
        _, xb, zb, _ = term(lib, b)
        pa, pb = dense_product(a, n), dense_product(b, n)
        commutes = np.allclose(pa @ pb, pb @ pa)
        assert lib.paulis_commute(xa, za, xb, zb) == int(commutes)


def test_term_exponential_gate(lib):
    import scipy.linalg

    rng = np.random.default_rng(2)
    for _ in range(100):
        w = int(rng.integers(1, 6))
        factors = [(q, "XYZ"[int(rng.integers(3))]) for q in range(w)]
        _, x, z, ny = term(lib, factors)
        theta = float(rng.normal())
        a = np.cos(theta)
        b = -1j * np.sin(theta) * (-1j) ** ny
        out = np.zeros(2 * 4 ** w)
        lib.pauli_exp(w, x, z, a.real, 0.0, b.real, b.imag, out.ctypes.data_as(C.POINTER(C.c_double)))
        got = out.view(np.complex128).reshape(1 << w, 1 << w)
        want = scipy.linalg.expm(-1j * theta * dense_product(factors, w))
        np.testing.assert_allclose(got, want, atol=1e-14)


@pytest.mark.parametrize("x", [0.0, 1e-3, 0.5, 3.0, 20.0, 137.5, 1000.0, 5000.0])
def test_bessel_coefficients(lib, x):
    """Against mpmath (30 digits) at 40 orders where it converges (x <= 1000),
    and scipy.special.jv everywhere (scipy's own error grows to ~1e-14 at
    x = 1000)."""
    import scipy.special

    out = np.zeros(20000)
    n = lib.bessel_orders(x, 1e-16, out.ctypes.data_as(C.POINTER(C.c_double)), len(out))
    assert n > 0
    j = out[:n]
    k = np.arange(n)
    np.testing.assert_allclose(j, scipy.special.jv(k, x), atol=1e-15 * max(1.0, x / 10), rtol=0)
    if x <= 1000:
        mpmath = pytest.importorskip("mpmath")
        mpmath.mp.dps = 30
        ks = np.unique(np.linspace(0, n - 1, 40).astype(int))
        ref = np.array([float(mpmath.besselj(int(q), x)) for q in ks])
        assert np.max(np.abs(j[ks] - ref)) < 2e-15
    assert n - 1 >= x
    # truncation: the dropped tail is below the tolerance
    tail = scipy.special.jv(np.arange(n, n + 200), x)
    assert 2 * np.sum(np.abs(tail)) <= 1e-15
    # Jacobi-Anger at x * cos(phi): exp(-i x c) = J0 + 2 sum (-i)^k J_k T_k(c)
    for c in (-1.0, -0.3, 0.0, 0.7, 1.0):
        tk = np.cos(k * np.arccos(c))
        coef = np.where(k == 0, 1.0, 2.0) * (-1j) ** k * j
        assert abs(np.sum(coef * tk) - np.exp(-1j * x * c)) < 1e-12 * max(1.0, x / 100)
