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

Everything else follows the reference class: the qubit map and its shift on
deallocation, validity and the reset into ``history`` (with the same
warning) on the first gate after a measurement or deallocation, the host
state vector updated as ``unitary @ state`` on flush, and measurement with
Python's ``random`` on that state (_unitary.py:248-285).
"""

from __future__ import annotations

import math
import random
import warnings
from copy import deepcopy

import numpy as np

from .simulator import Simulator

try:  # ProjectQ's engine base class; the class is only usable with ProjectQ installed
    from projectq.cengines import BasicEngine
    from projectq.meta import LogicalQubitIDTag, get_control_count, has_negative_control
    from projectq.ops import AllocateQubitGate, DeallocateQubitGate, FlushGate, MeasureGate
    from projectq.types import WeakQubitRef
except ImportError:  # pragma: no cover - exercised only without ProjectQ
    BasicEngine = object
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


class UnitarySimulator(BasicEngine):
    """Drop-in for projectq.backends.UnitarySimulator with the unitary on the GPU.

    Extra keyword: ``precision`` ("c128", the reference's complex, or "c64").
    """

    def __init__(self, precision="c128", _api=None):
        if not _PROJECTQ:
            raise ImportError("UnitarySimulator needs ProjectQ (projectq.cengines.BasicEngine)")
        super().__init__()
        self._precision = precision
        self._api = _api
        self._qubit_map = {}
        self._dev = _DeviceUnitary(0, precision, _api)
        self._num_qubits = 0
        self._is_valid = True
        self._is_flushed = False
        self._state = [1]
        self._history = []

    @property
    def unitary(self):
        """The current unitary (a copy), as _unitary.py:102-110."""
        return self._dev.matrix()

    @property
    def history(self):
        """Previous unitaries, one per reset after a measurement or deallocation."""
        return deepcopy(self._history)

    def is_available(self, cmd):
        """_unitary.py:124-149: arbitrarily controlled gates with a matrix."""
        if has_negative_control(cmd):
            return False
        if isinstance(cmd.gate, (AllocateQubitGate, DeallocateQubitGate, MeasureGate)):
            return True
        try:
            gate_mat = cmd.gate.matrix
            if len(gate_mat) > 2**6:
                warnings.warn(f"Potentially large matrix gate encountered! ({math.log2(len(gate_mat))} qubits)")
            return True
        except AttributeError:
            return False

    def receive(self, command_list):
        for cmd in command_list:
            self._handle(cmd)
        if not self.is_last_engine:
            self.send(command_list)

    def _flush(self):
        """_unitary.py:170-174: state <- unitary @ state, once per flush."""
        if not self._is_flushed:
            self._is_flushed = True
            self._state = self.unitary @ np.asarray(self._state, dtype=np.complex128)

    def _handle(self, cmd):
        """_unitary.py:176-246."""
        if isinstance(cmd.gate, AllocateQubitGate):
            self._qubit_map[cmd.qubits[0][0].id] = self._num_qubits
            self._num_qubits += 1
            self._dev.add_qubit()
            self._state = list(self._state) + [0] * len(self._state)

        elif isinstance(cmd.gate, DeallocateQubitGate):
            pos = self._qubit_map[cmd.qubits[0][0].id]
            self._qubit_map = {key: value - 1 if value > pos else value for key, value in self._qubit_map.items()}
            self._num_qubits -= 1
            self._is_valid = False

        elif isinstance(cmd.gate, MeasureGate):
            self._is_valid = False
            if not self._is_flushed:
                raise RuntimeError(
                    'Please make sure all previous gates are flushed before measurement so the state gets updated'
                )
            if get_control_count(cmd) != 0:
                raise ValueError('Cannot have control qubits with a measurement gate!')
            all_qubits = [qb for qr in cmd.qubits for qb in qr]
            measurements = self.measure_qubits([qb.id for qb in all_qubits])
            for qb, res in zip(all_qubits, measurements):
                for tag in cmd.tags:
                    if isinstance(tag, LogicalQubitIDTag):
                        qb = WeakQubitRef(qb.engine, tag.logical_qubit_id)
                        break
                self.main_engine.set_measurement_result(qb, res)

        elif isinstance(cmd.gate, FlushGate):
            self._flush()
        else:
            if not self._is_valid:
                self._flush()
                warnings.warn(
                    "Processing of other gates after a qubit deallocation or measurement will reset the unitary,"
                    "previous unitary can be accessed in history"
                )
                self._history.append(self.unitary)
                self._dev.close()
                self._dev = _DeviceUnitary(self._num_qubits, self._precision, self._api)
                self._state = np.array([1] + ([0] * (2**self._num_qubits - 1)), dtype=complex)
                self._is_valid = True
            self._is_flushed = False
            targets = [self._qubit_map[qb.id] for qr in cmd.qubits for qb in qr]
            controls = [self._qubit_map[qb.id] for qb in cmd.control_qubits]
            self._dev.apply(np.asarray(cmd.gate.matrix, dtype=np.complex128), targets, controls)

    def measure_qubits(self, ids):
        """_unitary.py:248-285: sample from the flushed host state, project, renormalise."""
        random_outcome = random.random()
        state = np.asarray(self._state, dtype=np.complex128)
        val = 0.0
        i_picked = 0
        while val < random_outcome and i_picked < len(state):
            val += np.abs(state[i_picked]) ** 2
            i_picked += 1
        i_picked -= 1
        pos = [self._qubit_map[ID] for ID in ids]
        res = [False] * len(pos)
        mask = 0
        val = 0
        for i, _pos in enumerate(pos):
            res[i] = ((i_picked >> _pos) & 1) == 1
            mask |= 1 << _pos
            val |= (res[i] & 1) << _pos
        nrm = 0.0
        for i, amp in enumerate(state):
            if (mask & i) != val:
                state[i] = 0.0
            else:
                nrm += np.abs(amp) ** 2
        state *= 1.0 / np.sqrt(nrm)
        self._state = state
        return res
