"""UnitarySimulator on the GPU engine.

ProjectQ's ``projectq.backends.UnitarySimulator`` (backends/_unitary.py:64-285)
accumulates the unitary of a circuit as a dense 2^n x 2^n NumPy matrix and
multiplies it by a full 2^n x 2^n embedding of every gate
(``cache @ self._unitary``, _unitary.py:241-245): O(8^n) per gate.

Here the unitary lives on the GPU as the 2n-qubit vector vec(U), U[r, c] at
the amplitude whose "row" qubits hold r and whose "column" qubits hold c.  A
gate G on the row qubits maps vec(U) to vec(G U), i.e. it is an ordinary
controlled gate on the row qubits of that state, applied by the same
kernels and planners as the state-vector engine: O(4^n) per gate, many
gates per pass.  Allocating a qubit, U -> I2 (x) U (_unitary.py:197-201),
adds a row and a column qubit in |0> and maps that pair |00> -> |00> + |11>
with one exact 0/1 two-qubit matrix.

The class derives from ProjectQ's own UnitarySimulator and leaves it the
parts that do not touch the unitary's storage: command dispatch
(``receive``), availability, deallocation (the qubit-map shift), the
measurement command (its checks and LogicalQubitIDTag handling) and
``history``.  It replaces allocation, the gate branch (including the reset
into ``history`` on the first gate after a measurement or deallocation), the
flush (host state <- U @ state) and the sampling of a measurement, which is
vectorised here and picks the same outcome as the reference's loop for the
same ``random.random()`` draw (_unitary.py:248-285).
"""

from __future__ import annotations

import random
import warnings

import numpy as np

from .simulator import Simulator

try:  # ProjectQ's own class is the base; this module is only usable with ProjectQ installed
    from projectq.backends._unitary import UnitarySimulator as _ProjectQUnitarySimulator
    from projectq.ops import AllocateQubitGate, DeallocateQubitGate, FlushGate, MeasureGate
except ImportError:  # pragma: no cover - exercised only without ProjectQ
    _ProjectQUnitarySimulator = object
    _PROJECTQ = False
else:
    _PROJECTQ = True

# on (row bit 0, column bit 1): |00> -> |00> + |11>; the other columns act on
# amplitudes that are zero right after the two qubits were allocated
_PAIR = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [1, 0, 0, 1]], dtype=np.complex128)


class _DeviceUnitary:
    """vec(U) of an n-qubit unitary in a 2n-qubit engine state."""

    def __init__(self, nqubits, precision, api=None):
        self.precision = precision
        if api is None:
            self.sim = Simulator(1, precision=precision, fusion="staged")
        else:  # another library with the same C ABI (tests: the CPU oracle)
            self.sim = Simulator(1, _api=api)
        self.rows, self.cols = [], []  # engine ids of row / column qubit i
        for _ in range(nqubits):
            self.add_qubit()

    def add_qubit(self):
        """U -> I2 (x) U: the new qubit is the most significant row and column bit."""
        r, c = 2 * len(self.rows), 2 * len(self.rows) + 1
        self.sim.allocate_qubit(r)
        self.sim.allocate_qubit(c)
        self.sim.apply_controlled_gate(_PAIR, [r, c], [])
        self.rows.append(r)
        self.cols.append(c)

    def apply(self, matrix, targets, controls):
        """U <- G U for G acting on row qubits `targets` with `controls`."""
        self.sim.apply_controlled_gate(matrix, [self.rows[t] for t in targets], [self.rows[c] for c in controls])

    def matrix(self):
        """U as a NumPy matrix (complex128)."""
        n = len(self.rows)
        if n == 0:
            return np.ones((1, 1), dtype=np.complex128)
        mapping, vec = self.sim.cheat()
        rng = np.arange(1 << n, dtype=np.int64)
        ri = np.zeros(1 << n, dtype=np.int64)
        ci = np.zeros(1 << n, dtype=np.int64)
        for i in range(n):
            bit = (rng >> i) & 1
            ri |= bit << mapping[self.rows[i]]
            ci |= bit << mapping[self.cols[i]]
        return np.asarray(vec, dtype=np.complex128)[ri[:, None] + ci[None, :]]

    def close(self):
        self.sim.close()


class UnitarySimulator(_ProjectQUnitarySimulator):
    """Drop-in for projectq.backends.UnitarySimulator with the unitary on the GPU.

    Extra keyword: ``precision`` ("c128", the reference's complex, or "c64").
    """

    _RESET_WARNING = ("Processing of other gates after a qubit deallocation or measurement will reset the unitary,"
                      "previous unitary can be accessed in history")

    def __init__(self, precision="c128", _api=None):
        if not _PROJECTQ:
            raise ImportError("UnitarySimulator needs ProjectQ (projectq.backends.UnitarySimulator)")
        super().__init__()
        self._precision = precision
        self._api = _api
        self._dev = _DeviceUnitary(0, precision, _api)
        self._state = np.ones(1, dtype=np.complex128)

    @property
    def unitary(self):
        """The current unitary, downloaded from the device as a NumPy matrix."""
        return self._dev.matrix()

    def _flush(self):
        if self._is_flushed:
            return
        self._is_flushed = True
        self._state = self._dev.matrix() @ np.asarray(self._state, dtype=np.complex128)

    def _handle(self, cmd):
        gate = cmd.gate
        if isinstance(gate, AllocateQubitGate):
            self._allocate(cmd.qubits[0][0].id)
        elif isinstance(gate, (DeallocateQubitGate, MeasureGate, FlushGate)):
            super()._handle(cmd)  # the base class: map shift, measurement checks and tags, flush dispatch
        else:
            self._apply(cmd)

    def _allocate(self, qubit_id):
        # the newest qubit is the most significant bit of the unitary and state
        self._qubit_map[qubit_id] = self._num_qubits
        self._num_qubits += 1
        self._dev.add_qubit()
        state = np.asarray(self._state, dtype=np.complex128)
        self._state = np.concatenate([state, np.zeros_like(state)])

    def _restart(self):
        """After a measurement or deallocation: the unitary so far goes to
        history and a fresh identity starts on the current qubits, from |0...0>."""
        self._flush()
        warnings.warn(self._RESET_WARNING)
        self._history.append(self._dev.matrix())
        self._dev.close()
        self._dev = _DeviceUnitary(self._num_qubits, self._precision, self._api)
        self._state = np.zeros(1 << self._num_qubits, dtype=np.complex128)
        self._state[0] = 1.0
        self._is_valid = True

    def _apply(self, cmd):
        if not self._is_valid:
            self._restart()
        self._is_flushed = False
        pos = self._qubit_map
        self._dev.apply(np.asarray(cmd.gate.matrix, dtype=np.complex128),
                        [pos[qb.id] for qr in cmd.qubits for qb in qr], [pos[qb.id] for qb in cmd.control_qubits])

    def measure_qubits(self, ids):
        """Sample basis state i with probability |state_i|^2 (the draw is one
        random.random(); the running sum is NumPy's sequential cumsum, so the
        outcome equals the reference's element loop, including its draw of
        exactly 0.0 selecting index -1), then project and renormalise."""
        draw = random.random()
        state = np.array(self._state, dtype=np.complex128)
        probs = np.abs(state) ** 2
        running = np.cumsum(probs)
        if draw <= 0.0:
            pick = -1
        else:
            pick = min(int(np.searchsorted(running, draw, side="left")), state.size - 1)
        positions = [self._qubit_map[q] for q in ids]
        outcome = [bool((pick >> p) & 1) for p in positions]
        mask = sum(1 << p for p in positions)
        value = sum(int(o) << p for o, p in zip(outcome, positions))
        keep = (np.arange(state.size, dtype=np.int64) & mask) == value
        norm = np.cumsum(np.where(keep, probs, 0.0))[-1]
        state[~keep] = 0.0
        state *= 1.0 / np.sqrt(norm)
        self._state = state
        return outcome
