"""Adjoint-method gradients of <psi(theta)|H|psi(theta)> on the GB300 engine.

`ParamCircuit` lists gates on qubit ids (fixed 2x2 matrices and Rx, Ry, Rz,
Ph, R rotations bound to parameter indices, each with optional controls);
`energy_and_gradient` returns E(theta) and dE/dtheta for every parameter
from one forward pass and one reverse sweep on the device
(gsim_adjoint_gradient: two state vectors, gates un-applied, checkpoints of
the forward state every ~sqrt(#gates) in complex64).  `expectation` wraps it
in a torch.autograd.Function; PyTorch is used only for that wrapper.
"""

from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .simulator import _pauli_csr, _p, _u32, _ids

KINDS = {"fixed": 0, "Rx": 1, "Ry": 2, "Rz": 3, "Ph": 4, "R": 5}


class ParamCircuit:
    """Gates applied in order to the engine's current state."""

    def __init__(self):
        self.kind, self.target, self.ctrls, self.param, self.mats = [], [], [], [], []

    def _add(self, kind, target, param, ctrls, matrix=None):
        self.kind.append(KINDS[kind])
        self.target.append(int(target))
        self.ctrls.append(list(ctrls))
        self.param.append(-1 if param is None else int(param))
        m = np.zeros((2, 2), dtype=np.complex128) if matrix is None else np.asarray(matrix, dtype=np.complex128)
        if m.shape != (2, 2):
            raise ValueError("fixed gates are single-target 2x2 matrices (use controls for CNOT, Toffoli ...)")
        self.mats.append(m)
        return self

    def gate(self, matrix, target, ctrls=()):
        return self._add("fixed", target, None, ctrls, matrix)

    def rx(self, target, param, ctrls=()):
        return self._add("Rx", target, param, ctrls)

    def ry(self, target, param, ctrls=()):
        return self._add("Ry", target, param, ctrls)

    def rz(self, target, param, ctrls=()):
        return self._add("Rz", target, param, ctrls)

    def ph(self, target, param, ctrls=()):
        return self._add("Ph", target, param, ctrls)

    def r(self, target, param, ctrls=()):
        return self._add("R", target, param, ctrls)

    def __len__(self):
        return len(self.kind)

    @property
    def nparams(self):
        return max(self.param, default=-1) + 1

    def matrices(self, theta):
        """Each gate's 2x2 matrix at `theta` (ProjectQ's conventions)."""
        out = []
        for k, p, m in zip(self.kind, self.param, self.mats):
            if k == 0:
                out.append(m)
                continue
            t = float(theta[p])
            c, s = math.cos(0.5 * t), math.sin(0.5 * t)
            out.append({1: np.array([[c, -1j * s], [-1j * s, c]]), 2: np.array([[c, -s], [s, c]]),
                        3: np.diag([np.exp(-0.5j * t), np.exp(0.5j * t)]), 4: np.exp(1j * t) * np.eye(2),
                        5: np.diag([1.0, np.exp(1j * t)])}[k].astype(np.complex128))
        return out

    def gates(self, theta):
        """The circuit at `theta` as (2x2 matrix, [target], controls) gates for
        apply_controlled_gate: the plain forward path, without the adjoint."""
        return [(m, [t], list(c)) for m, t, c in zip(self.matrices(theta), self.target, self.ctrls)]

    def packed(self):
        off = np.zeros(len(self.kind) + 1, dtype=np.uint32)
        off[1:] = np.cumsum([len(c) for c in self.ctrls])
        ctrl = _u32([q for c in self.ctrls for q in _ids(c)])
        mats = np.ascontiguousarray(np.stack(self.mats) if self.mats else np.zeros((0, 2, 2)), dtype=np.complex128)
        return (np.ascontiguousarray(self.kind, dtype=np.uint8), _u32(self.target), off, ctrl,
                np.ascontiguousarray(self.param, dtype=np.int32), mats.reshape(-1).view(np.float64).copy())


def hardware_efficient_ansatz(n, layers):
    """`layers` x (Ry(theta), Rz(theta) on every qubit, then CNOT 0->1->...->n-1);
    parameters in layer -> qubit -> (Ry, Rz) order: 2 n layers in total."""
    from .workloads import X

    c = ParamCircuit()
    p = 0
    for _ in range(layers):
        for q in range(n):
            c.ry(q, p)
            c.rz(q, p + 1)
            p += 2
        for q in range(n - 1):
            c.gate(X, q + 1, ctrls=(q,))
    return c


def energy_and_gradient(sim, circuit, theta, terms, ids, checkpoint_every=None):
    """(E, dE/dtheta) for the Pauli sum `terms` (real coefficients) on qubits `ids`."""
    theta = np.ascontiguousarray(theta, dtype=np.float64).reshape(-1)
    if theta.size < circuit.nparams:
        raise ValueError("theta has fewer entries than the circuit's parameters")
    if checkpoint_every is None:
        checkpoint_every = int(math.ceil(math.sqrt(len(circuit)))) if sim.precision == "c64" else 0
    kind, target, off, ctrl, param, mats = circuit.packed()
    toff, q, pa, cs = _pauli_csr(terms, real=True)
    ida = _u32(_ids(ids))
    grad = np.zeros(theta.size, dtype=np.float64)
    e = C.c_double()
    api = sim._api
    rc = api.adjoint_gradient(sim._h, len(circuit), _p(kind, C.c_uint8), _p(target, C.c_uint32),
                              _p(off, C.c_uint32), _p(ctrl, C.c_uint32), _p(param, C.c_int32),
                              _p(mats, C.c_double), _p(theta, C.c_double), theta.size, _p(toff, C.c_uint32),
                              _p(q, C.c_uint32), _p(pa, C.c_uint8), _p(cs, C.c_double), len(toff) - 1,
                              _p(ida, C.c_uint32), len(ida), int(checkpoint_every), C.byref(e),
                              _p(grad, C.c_double))
    _lib.check(api, rc)
    return e.value, grad


def _autograd_function():
    import torch

    class AdjointExpectation(torch.autograd.Function):
        """E(theta) = <psi(theta)|H|psi(theta)>; backward uses the adjoint
        gradient computed in forward (one reverse sweep, no stored layers)."""

        @staticmethod
        def forward(ctx, theta, sim, circuit, terms, ids, checkpoint_every):
            th = theta.detach().to("cpu", torch.float64).numpy()
            e, g = energy_and_gradient(sim, circuit, th, terms, ids, checkpoint_every)
            ctx.save_for_backward(torch.from_numpy(g).to(device=theta.device, dtype=theta.dtype))
            return theta.new_tensor(e)

        @staticmethod
        def backward(ctx, grad_out):
            (g,) = ctx.saved_tensors
            return grad_out * g, None, None, None, None, None

    return AdjointExpectation


_FN = None


def expectation(theta, sim, circuit, terms, ids, checkpoint_every=None):
    """Differentiable E(theta) (a torch scalar) through torch.autograd."""
    global _FN
    if _FN is None:
        _FN = _autograd_function()
    return _FN.apply(theta, sim, circuit, terms, ids, checkpoint_every)
