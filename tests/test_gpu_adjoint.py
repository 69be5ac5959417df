"""Adjoint-method gradients (gsim_adjoint_gradient) against central finite
differences, the parameter-shift rule, the CPU oracle's energies, and through
torch.autograd.  Tolerances: relative 1e-5 of the gradient's max norm for
complex128 against finite differences (h = 1e-4); complex64 within 2e-4."""

import numpy as np
import pytest

from _backends import make
from _circuits import allocate
from projectq_gb300.adjoint import ParamCircuit, energy_and_gradient, expectation, hardware_efficient_ansatz
from projectq_gb300.workloads import H, X, random_pauli_hamiltonian

pytestmark = pytest.mark.gpu


def engine(n, prec="c128"):
    s = make("gpu", seed=1, precision=prec)
    allocate(s, n)
    return s


def oracle_energy(circ, theta, terms, n):
    o = make("oracle", seed=1)
    allocate(o, n)
    for m, t, c in zip(circ.matrices(theta), circ.target, circ.ctrls):
        o.apply_controlled_gate(m, [t], list(c))
    o.run()
    return o.get_expectation_value(terms, list(range(n)))


def mixed_circuit(n, rng):
    """Every gate kind, controls included, parameters shared between gates."""
    c = ParamCircuit()
    p = 0
    for q in range(n):
        c.gate(H, q)
    for layer in range(3):
        for q in range(n):
            kind = ["rx", "ry", "rz"][(q + layer) % 3]
            getattr(c, kind)(q, p)
            p += 1
        c.gate(X, (layer + 1) % n, ctrls=(layer % n,))
        c.rx(2, p, ctrls=(0,))
        c.rz(3, p + 1, ctrls=(1, 4))
        c.ph(1, p + 2)
        c.r(5, p + 3, ctrls=(2,))
        c.ry(0, 1)  # shares parameter 1
        p += 4
    return c, p


def test_gradient_matches_finite_differences_complex128():
    n = 8
    rng = np.random.default_rng(0)
    circ, npar = mixed_circuit(n, rng)
    theta = rng.uniform(-np.pi, np.pi, size=npar)
    terms = random_pauli_hamiltonian(n, 30, seed=1, p_identity=0.6)
    sim = engine(n)
    e, g = energy_and_gradient(sim, circ, theta, terms, range(n))
    assert e == pytest.approx(oracle_energy(circ, theta, terms, n), abs=1e-11)
    h = 1e-4
    fd = np.zeros(npar)
    for j in range(npar):
        tp, tm = theta.copy(), theta.copy()
        tp[j] += h
        tm[j] -= h
        fd[j] = (energy_and_gradient(sim, circ, tp, terms, range(n))[0]
                 - energy_and_gradient(sim, circ, tm, terms, range(n))[0]) / (2 * h)
    assert np.max(np.abs(g - fd)) <= 1e-5 * max(1.0, np.max(np.abs(fd)))


def test_gradient_matches_parameter_shift_and_oracle_fd():
    """Hardware-efficient ansatz (Ry, Rz + CNOT ladder), every parameter used
    once: the parameter-shift rule is exact; the CPU oracle's energies give an
    independent finite-difference check."""
    n, layers = 6, 3
    circ = hardware_efficient_ansatz(n, layers)
    rng = np.random.default_rng(3)
    theta = rng.uniform(-np.pi, np.pi, size=circ.nparams)
    terms = random_pauli_hamiltonian(n, 40, seed=2)
    sim = engine(n)
    e, g = energy_and_gradient(sim, circ, theta, terms, range(n))
    ps = np.zeros_like(g)
    fd = np.zeros_like(g)
    for j in range(circ.nparams):
        tp, tm = theta.copy(), theta.copy()
        tp[j] += np.pi / 2
        tm[j] -= np.pi / 2
        ps[j] = 0.5 * (energy_and_gradient(sim, circ, tp, terms, range(n))[0]
                       - energy_and_gradient(sim, circ, tm, terms, range(n))[0])
        tp, tm = theta.copy(), theta.copy()
        tp[j] += 1e-4
        tm[j] -= 1e-4
        fd[j] = (oracle_energy(circ, tp, terms, n) - oracle_energy(circ, tm, terms, n)) / 2e-4
    assert np.max(np.abs(g - ps)) < 1e-11
    assert np.max(np.abs(g - fd)) <= 1e-5 * max(1.0, np.max(np.abs(fd)))


@pytest.mark.parametrize("ckpt", [0, 7])
def test_complex64_gradient_close_to_complex128(ckpt):
    n, layers = 12, 6
    circ = hardware_efficient_ansatz(n, layers)
    theta = np.random.default_rng(5).uniform(-np.pi, np.pi, size=circ.nparams)
    terms = random_pauli_hamiltonian(n, 60, seed=4)
    e128, g128 = energy_and_gradient(engine(n, "c128"), circ, theta, terms, range(n))
    e64, g64 = energy_and_gradient(engine(n, "c64"), circ, theta, terms, range(n), checkpoint_every=ckpt)
    assert e64 == pytest.approx(e128, abs=2e-5)
    assert np.max(np.abs(g64 - g128)) <= 2e-4 * max(1.0, np.max(np.abs(g128)))


def test_engine_state_is_unchanged_and_torch_autograd():
    torch = pytest.importorskip("torch")
    n = 5
    circ = hardware_efficient_ansatz(n, 2)
    terms = random_pauli_hamiltonian(n, 20, seed=6)
    sim = engine(n)
    sim.apply_controlled_gate(H, [2], [])
    sim.run()
    before = sim.cheat()[1].copy()
    theta = torch.tensor(np.random.default_rng(7).uniform(-1, 1, size=circ.nparams), requires_grad=True)
    e = expectation(theta, sim, circ, terms, range(n))
    e.backward()
    _, g = energy_and_gradient(sim, circ, theta.detach().numpy(), terms, range(n))
    assert np.allclose(theta.grad.numpy(), g, atol=1e-13)
    assert np.array_equal(sim.cheat()[1], before)


def test_every_parameter_against_finite_differences_16_qubits():
    """The configured ansatz family at 16 qubits (6 layers: 192 parameters) and
    a 60-term Hamiltonian: the complex128 adjoint gradient against central
    finite differences (h = 1e-4) on every parameter, with the energies taken
    through the plain public path (set_wavefunction, apply_gates, run,
    get_expectation_value), and the energy against the CPU oracle.
    Tolerance: 1e-5 of the gradient's max norm (at least 1)."""
    n, layers = 16, 6
    circ = hardware_efficient_ansatz(n, layers)
    theta = np.random.default_rng(9).uniform(-np.pi, np.pi, size=circ.nparams)
    terms = random_pauli_hamiltonian(n, 60, seed=8)
    e, g = energy_and_gradient(engine(n), circ, theta, terms, range(n))
    assert e == pytest.approx(oracle_energy(circ, theta, terms, n), abs=1e-10)
    fsim = make("gpu", seed=1, precision="c128", fusion="staged")
    allocate(fsim, n)
    zero = np.zeros(1 << n, dtype=np.complex128)
    zero[0] = 1.0
    ids = list(range(n))

    def energy(th):
        fsim.set_wavefunction(zero, ids)
        fsim.apply_gates(circ.gates(th))
        fsim.run()
        return fsim.get_expectation_value(terms, ids)

    assert energy(theta) == pytest.approx(e, abs=1e-11)
    h = 1e-4
    fd = np.zeros(circ.nparams)
    for j in range(circ.nparams):
        tp, tm = theta.copy(), theta.copy()
        tp[j] += h
        tm[j] -= h
        fd[j] = (energy(tp) - energy(tm)) / (2 * h)
    assert np.max(np.abs(g - fd)) <= 1e-5 * max(1.0, np.max(np.abs(fd)))
