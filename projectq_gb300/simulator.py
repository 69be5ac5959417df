"""Python face of the GB300 engine: a drop-in for ProjectQ's native simulator.

`Simulator` has the method surface of the pybind11 class
``projectq.backends._sim._cppsim.Simulator`` (projectq/backends/_sim/
_cppsim.cpp:45-66): same names, same argument meaning, same return types and
the same exception classes (RuntimeError / ValueError / TypeError).  Plug it
into ProjectQ's Python backend exactly as the reference's tests do
(projectq/backends/_sim/_simulator_test.py:80-93)::

    from projectq.backends import Simulator
    from projectq_gb300 import Simulator as GB300Simulator
    sim = Simulator(gate_fusion=True)
    sim._simulator = GB300Simulator(seed)

Every method goes through the C ABI of include/gb300sim.h into
libgb300sim.so; there is no CPU fallback.
"""

from __future__ import annotations

import atexit
import ctypes as C
import numbers

import numpy as np

from . import _lib

_PRECISIONS = {"c128": _lib.GSIM_C128, "complex128": _lib.GSIM_C128, "c64": _lib.GSIM_C64,
               "complex64": _lib.GSIM_C64}
_FUSION = {"reference": _lib.GSIM_FUSION_REFERENCE, "none": _lib.GSIM_FUSION_NONE,
           "staged": _lib.GSIM_FUSION_STAGED, "learned": _lib.GSIM_FUSION_LEARNED}


_PENDING = []


def _release_pending():
    while _PENDING:
        api, h = _PENDING.pop()
        try:
            api.destroy(h)
        except Exception:  # pragma: no cover - interpreter shutdown
            pass


atexit.register(_release_pending)


def _u32(seq) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(seq, dtype=np.int64).astype(np.uint32, copy=False)
                                if len(seq) else np.zeros(0, dtype=np.uint32))


def _p(arr: np.ndarray, ctype):
    return arr.ctypes.data_as(C.POINTER(ctype))


def _bits(bits) -> np.ndarray:
    return np.ascontiguousarray([1 if bool(b) else 0 for b in bits], dtype=np.uint8)


def _ids(ids) -> list:
    out = []
    for i in ids:
        if type(i) is not int:  # plain ints skip the slower abstract-class checks
            if isinstance(i, bool) or not isinstance(i, numbers.Integral):
                raise TypeError("qubit ids must be integers")
            i = int(i)
        if i < 0 or i > 0xFFFFFFFF:
            raise TypeError("qubit ids must fit in an unsigned 32-bit integer")
        out.append(i)
    return out


def _real(c):
    """A real coefficient, or TypeError as pybind11's double caster raises."""
    if isinstance(c, (complex, np.complexfloating)):
        raise TypeError("incompatible function arguments: coefficient must be a real number")
    return float(c)


def _pauli_csr(terms, real: bool):
    """[(term, coeff)] with term = [(index, 'X'|'Y'|'Z'), ...] -> CSR arrays."""
    off = [0]
    qs, ps, cs = [], [], []
    for term, coeff in terms:
        for idx, op in term:
            op = op.decode() if isinstance(op, bytes) else op
            if op not in ("X", "Y", "Z"):
                raise ValueError(f"unknown Pauli operator {op!r}")
            qs.append(int(idx))
            ps.append(ord(op))
        off.append(len(qs))
        if real:
            cs.append(_real(coeff))
        else:
            c = complex(coeff)
            cs.extend([c.real, c.imag])
    return (np.ascontiguousarray(off, dtype=np.uint32), _u32(qs),
            np.ascontiguousarray(ps, dtype=np.uint8), np.ascontiguousarray(cs, dtype=np.float64))


class Simulator:
    """GB300 state-vector engine with the reference engine's method surface.

    Args:
        rnd_seed: seed of the engine's std::mt19937 (as the reference).
        precision: "c128" (default; the plain method, FP64 like the reference)
            or "c64" (complex64 storage with FP64 reductions).
        fusion: gate-fusion planner: "reference" (default; the reference's
            greedy 4..5-qubit rule), "none" or "staged".
    """

    def __init__(self, rnd_seed=1, *args, precision="c128", fusion="reference", _api=None, **kwargs):
        if isinstance(rnd_seed, bool) or not isinstance(rnd_seed, numbers.Integral):
            raise TypeError("Simulator(): seed must be an unsigned 32-bit integer")
        if rnd_seed < 0 or rnd_seed > 0xFFFFFFFF:
            raise TypeError("Simulator(): seed must be an unsigned 32-bit integer")
        _release_pending()
        self._api = _api if _api is not None else _lib.load()
        self._prec = _PRECISIONS[precision]
        h = C.c_void_p()
        self._check(self._api.create(int(rnd_seed), self._prec, C.byref(h)))
        self.__dict__["_hv"] = h
        if fusion != "reference":
            self.set_fusion(fusion)

    # -- plumbing -----------------------------------------------------------
    def _check(self, rc):
        _lib.check(self._api, rc)

    def close(self):
        """Free the engine's device memory now (the object is unusable after)."""
        h = self.__dict__.get("_hv")
        if h is not None and h.value:
            self._api.destroy(h)
        self.__dict__["_hv"] = None

    def __del__(self):
        # Deferred: in a reference cycle (ProjectQ's MainEngine <-> backend)
        # Python may finalize this object before MainEngine.__del__ flushes
        # through it, as pybind11 objects are only freed after all finalizers.
        # The handle is destroyed at the next construction, close() or exit.
        h = self.__dict__.get("_hv")
        if h is not None and h.value:
            _PENDING.append((self._api, h))

    @property
    def _h(self):
        """The engine handle; a closed engine raises here.  (A property: a
        __getattribute__ override would tax every attribute access of the
        per-gate path.)"""
        h = self.__dict__.get("_hv")
        if h is None:
            raise RuntimeError("the simulator engine has been closed")
        return h

    @property
    def precision(self) -> str:
        return "c64" if self._prec == _lib.GSIM_C64 else "c128"

    # -- the reference surface (_cppsim.cpp:45-66) ----------------------------
    def allocate_qubit(self, qubit_id):
        """simulator.hpp:55-74."""
        (qid,) = _ids([qubit_id])
        self._check(self._api.allocate_qubit(self._h, qid))

    def deallocate_qubit(self, qubit_id):
        """simulator.hpp:194-202."""
        (qid,) = _ids([qubit_id])
        self._check(self._api.deallocate_qubit(self._h, qid))

    def get_classical_value(self, qubit_id, tol=1.0e-12):
        """simulator.hpp:76-91."""
        (qid,) = _ids([qubit_id])
        out = C.c_int()
        self._check(self._api.get_classical_value(self._h, qid, float(tol), C.byref(out)))
        return bool(out.value)

    def is_classical(self, qubit_id, tol=1.0e-12):
        """simulator.hpp:93-108."""
        (qid,) = _ids([qubit_id])
        out = C.c_int()
        self._check(self._api.is_classical(self._h, qid, float(tol), C.byref(out)))
        return bool(out.value)

    def measure_qubits(self, ids):
        """simulator.hpp:145-192: one RNG draw; returns list[bool]."""
        ids = _u32(_ids(ids))
        out = np.zeros(len(ids), dtype=np.uint8)
        self._check(self._api.measure_qubits(self._h, _p(ids, C.c_uint32), len(ids), _p(out, C.c_uint8)))
        return [bool(v) for v in out]

    def measure_qubits_at(self, ids, rnd):
        """measure_qubits with the uniform draw `rnd` given instead of drawn."""
        ids = _u32(_ids(ids))
        out = np.zeros(len(ids), dtype=np.uint8)
        self._check(self._api.measure_qubits_at(self._h, _p(ids, C.c_uint32), len(ids), float(rnd),
                                                _p(out, C.c_uint8)))
        return [bool(v) for v in out]

    def apply_controlled_gate(self, m, ids, ctrl):
        """simulator.hpp:204-222: queue a controlled gate (fused, run lazily).

        Called once per gate by ProjectQ's Simulator._handle, so the argument
        packing is kept short: ids as ctypes arrays, the matrix by address."""
        ids = _ids(ids)
        ctrl = _ids(ctrl)
        mat = np.ascontiguousarray(m, dtype=np.complex128)
        k = len(ids)
        if mat.ndim != 2 or mat.shape != (1 << k, 1 << k):
            raise ValueError(f"apply_controlled_gate(): a {k}-qubit gate needs a {1 << k}x{1 << k} matrix")
        nc = len(ctrl)
        rc = self._api.apply_controlled_gate(self._h, mat.ctypes.data, k, (C.c_uint32 * k)(*ids),
                                             (C.c_uint32 * nc)(*ctrl) if nc else None, nc)
        if rc:
            self._check(rc)

    def run(self):
        """simulator.hpp:487-527: apply all pending gates."""
        self._check(self._api.run(self._h))

    def _regs(self, quregs):
        sizes = [len(r) for r in quregs]
        flat = [q for r in quregs for q in _ids(r)]
        return _u32(flat), _u32(sizes), len(sizes)

    def emulate_math(self, f, quregs, ctrl):
        """simulator.hpp:224-269 with a Python function of the register values.

        The reference calls `f` once per basis state (through the GIL,
        _cppsim.cpp:33-41); here `f` is tabulated once over every tuple of
        register values and the permutation runs on the GPU.
        """
        sizes = [len(r) for r in quregs]
        W = sum(sizes)
        if W > 26:
            raise ValueError("emulate_math(): at most 26 register qubits are supported")
        shifts = np.cumsum([0] + sizes[:-1]).tolist()
        masks = [(1 << s) - 1 for s in sizes]
        table = np.empty(1 << W, dtype=np.uint64)
        for x in range(1 << W):
            vals = [(x >> sh) & mk for sh, mk in zip(shifts, masks)]
            res = f(vals)
            y = 0
            for r, (sh, mk) in enumerate(zip(shifts, masks)):
                y |= (int(res[r]) & mk) << sh
            table[x] = y
        ids, sz, nr = self._regs(quregs)
        ctrl = _u32(_ids(ctrl))
        self._check(self._api.emulate_math_table(self._h, _p(table, C.c_uint64), _p(ids, C.c_uint32),
                                                 _p(sz, C.c_uint32), nr, _p(ctrl, C.c_uint32), len(ctrl)))

    def emulate_math_addConstant(self, a, quregs, ctrl):  # noqa: N802 (reference name)
        """simulator.hpp:272-276."""
        ids, sz, nr = self._regs(quregs)
        ctrl = _u32(_ids(ctrl))
        self._check(self._api.emulate_math_add_constant(self._h, int(a), _p(ids, C.c_uint32), _p(sz, C.c_uint32),
                                                        nr, _p(ctrl, C.c_uint32), len(ctrl)))

    def emulate_math_addConstantModN(self, a, N, quregs, ctrl):  # noqa: N802,N803
        """simulator.hpp:279-283."""
        ids, sz, nr = self._regs(quregs)
        ctrl = _u32(_ids(ctrl))
        self._check(self._api.emulate_math_add_constant_modn(self._h, int(a), int(N), _p(ids, C.c_uint32),
                                                             _p(sz, C.c_uint32), nr, _p(ctrl, C.c_uint32),
                                                             len(ctrl)))

    def emulate_math_multiplyByConstantModN(self, a, N, quregs, ctrl):  # noqa: N802,N803
        """simulator.hpp:286-290."""
        ids, sz, nr = self._regs(quregs)
        ctrl = _u32(_ids(ctrl))
        self._check(self._api.emulate_math_multiply_by_constant_modn(
            self._h, int(a), int(N), _p(ids, C.c_uint32), _p(sz, C.c_uint32), nr, _p(ctrl, C.c_uint32),
            len(ctrl)))

    def get_expectation_value(self, terms, ids):
        """simulator.hpp:292-322: sum_t c_t <psi|P_t|psi> (real c_t)."""
        off, q, pa, cs = _pauli_csr(terms, real=True)
        ida = _u32(_ids(ids))
        out = C.c_double()
        self._check(self._api.get_expectation_value(self._h, _p(off, C.c_uint32), _p(q, C.c_uint32),
                                                    _p(pa, C.c_uint8), _p(cs, C.c_double), len(off) - 1,
                                                    _p(ida, C.c_uint32), len(ida), C.byref(out)))
        return out.value

    def apply_qubit_operator(self, terms, ids):
        """simulator.hpp:324-350: psi <- sum_t c_t P_t psi (complex c_t)."""
        off, q, pa, cs = _pauli_csr(terms, real=False)
        ida = _u32(_ids(ids))
        self._check(self._api.apply_qubit_operator(self._h, _p(off, C.c_uint32), _p(q, C.c_uint32),
                                                   _p(pa, C.c_uint8), _p(cs, C.c_double), len(off) - 1,
                                                   _p(ida, C.c_uint32), len(ida)))

    def emulate_time_evolution(self, terms, time, ids, ctrl):
        """simulator.hpp:386-438: exp(-i t H); exactly as a product of term
        exponentials when the terms commute (set_time_evolution), else by the
        Taylor series (FP64)."""
        off, q, pa, cs = _pauli_csr(terms, real=True)
        ida = _u32(_ids(ids))
        ctrl = _u32(_ids(ctrl))
        self._check(self._api.emulate_time_evolution(self._h, _p(off, C.c_uint32), _p(q, C.c_uint32),
                                                     _p(pa, C.c_uint8), _p(cs, C.c_double), len(off) - 1,
                                                     float(time), _p(ida, C.c_uint32), len(ida),
                                                     _p(ctrl, C.c_uint32), len(ctrl)))

    def get_probability(self, bit_string, ids):
        """simulator.hpp:352-368."""
        bits = _bits(bit_string)
        ida = _u32(_ids(ids))
        out = C.c_double()
        self._check(self._api.get_probability(self._h, _p(bits, C.c_uint8), _p(ida, C.c_uint32), len(ida),
                                              C.byref(out)))
        return out.value

    def get_amplitude(self, bit_string, ids):
        """simulator.hpp:370-384."""
        bits = _bits(bit_string)
        ida = _u32(_ids(ids))
        if len(bits) < len(ida):
            bits = np.concatenate([bits, np.zeros(len(ida) - len(bits), dtype=np.uint8)])
        out = np.zeros(2, dtype=np.float64)
        self._check(self._api.get_amplitude(self._h, _p(bits, C.c_uint8), _p(ida, C.c_uint32), len(ida),
                                            _p(out, C.c_double)))
        return complex(out[0], out[1])

    def set_wavefunction(self, wavefunction, ordering):
        """simulator.hpp:440-454."""
        wf = np.asarray(wavefunction)
        if wf.dtype == np.complex64:
            dtype = _lib.GSIM_C64
        else:
            wf = wf.astype(np.complex128, copy=False)
            dtype = _lib.GSIM_C128
        wf = np.ascontiguousarray(wf.reshape(-1))
        ordv = _u32(_ids(ordering))
        self._check(self._api.set_wavefunction(self._h, wf.ctypes.data_as(C.c_void_p), dtype, wf.size,
                                               _p(ordv, C.c_uint32), len(ordv)))

    def collapse_wavefunction(self, ids, values):
        """simulator.hpp:456-485."""
        ida = _u32(_ids(ids))
        vals = _bits(values)
        self._check(self._api.collapse_wavefunction(self._h, _p(ida, C.c_uint32), len(ida), _p(vals, C.c_uint8),
                                                    len(vals)))

    def cheat(self, dtype=np.complex128):
        """simulator.hpp:529-532: (qubit id -> bit position, state vector).

        The state is a NumPy array (the reference returns a list copy).
        """
        n = C.c_uint32()
        self._check(self._api.num_qubits(self._h, C.byref(n)))
        nq = n.value
        ids = np.zeros(max(nq, 1), dtype=np.uint32)
        pos = np.zeros(max(nq, 1), dtype=np.uint32)
        self._check(self._api.get_mapping(self._h, _p(ids, C.c_uint32), _p(pos, C.c_uint32), nq))
        mapping = {int(i): int(p) for i, p in zip(ids[:nq], pos[:nq])}
        return mapping, self.get_state(dtype=dtype)

    # -- extensions (no reference counterpart) --------------------------------
    def get_state(self, offset=0, count=None, dtype=np.complex128):
        n = C.c_uint32()
        self._check(self._api.num_qubits(self._h, C.byref(n)))
        total = 1 << n.value
        count = total - offset if count is None else count
        dt = np.dtype(dtype)
        code = _lib.GSIM_C64 if dt == np.complex64 else _lib.GSIM_C128
        out = np.empty(count, dtype=np.complex64 if code == _lib.GSIM_C64 else np.complex128)
        self._check(self._api.get_state(self._h, out.ctypes.data_as(C.c_void_p), code, offset, count))
        return out

    def set_fusion(self, mode="reference", kmax=0):
        self._check(self._api.set_fusion(self._h, _FUSION[mode], int(kmax)))

    def set_tensor_cores(self, on=True, renorm=True):
        """Use tcgen05 tensor cores for fused complex64 gates of 4-7 targets;
        renorm restores each amplitude group's norm after a unitary gate."""
        self._check(self._api.set_tensor_cores(self._h, (1 if renorm else 2) if on else 0))

    def set_stage_kernel(self, mode="packed"):
        """Stage kernel of the "staged" planner: "packed" (default: complex64
        stages with a free tile bit run as amplitude pairs on packed f32x2
        arithmetic), "register" (register substages) or "pass" (one
        shared-memory pass per operation)."""
        modes = {"pass": 0, "register": 1, "packed": 2}
        if mode not in modes:
            raise ValueError(f"stage kernel must be one of {sorted(modes)}")
        self._check(self._api.set_stage_kernel(self._h, modes[mode]))

    def set_time_evolution(self, mode="exact"):
        """emulate_time_evolution: "exact" (default: the product of the terms'
        exponentials when they commute pairwise and avoid the controls, else the
        reference's Taylor series), "taylor" (always the series) or "chebyshev"
        (as "exact", with a Chebyshev expansion instead of the series for
        non-commuting terms: about |t| sum|c| + 40 applications of H instead of
        about 16 |t| sum|c|)."""
        modes = {"taylor": 0, "exact": 1, "chebyshev": 2}
        if mode not in modes:
            raise ValueError(f"time-evolution mode must be one of {sorted(modes)}")
        self._check(self._api.set_time_evolution(self._h, modes[mode]))

    def synchronize(self):
        self._check(self._api.synchronize(self._h))

    def set_upload_mode(self, mode="pull"):
        """set_wavefunction transfer: "pull" (default: the SMs read page-locked
        host memory, see pin_host; pageable arrays still use the copy engine)
        or "copy" (always the copy engine)."""
        self._check(self._api.set_upload_mode(self._h, {"copy": 0, "pull": 1}[mode]))

    def reserve(self, nqubits):
        self._check(self._api.reserve(self._h, int(nqubits)))

    def counters(self):
        out = np.zeros(7, dtype=np.uint64)
        self._check(self._api.get_counters(self._h, _p(out, C.c_uint64), 7))
        return {"logical_gates": int(out[0]), "gate_launches": int(out[1]), "gate_bytes": int(out[2]),
                "gate_passes": int(out[3]), "evolutions_exact": int(out[4]), "evolutions_taylor": int(out[5]),
                "evolutions_chebyshev": int(out[6])}

    def reset_counters(self):
        self._check(self._api.reset_counters(self._h))

    def apply_gates(self, gates):
        """Submit many gates in one call: [(matrix, target ids, control ids), ...],
        the same as apply_controlled_gate per gate, packed into flat arrays and
        queued by one gsim_apply_gates call (no per-gate ctypes round trip)."""
        gates = list(gates)
        if not gates:
            return
        nt = np.empty(len(gates), dtype=np.uint32)
        nc = np.empty(len(gates), dtype=np.uint32)
        qubits, mats = [], []
        for g, (m, t, c) in enumerate(gates):
            t, c = _ids(t), _ids(c)
            mat = np.asarray(m, dtype=np.complex128)
            if mat.ndim != 2 or mat.shape != (1 << len(t), 1 << len(t)):
                raise ValueError(f"apply_gates(): gate {g}: a {len(t)}-qubit gate needs a "
                                 f"{1 << len(t)}x{1 << len(t)} matrix")
            nt[g], nc[g] = len(t), len(c)
            qubits.extend(t)
            qubits.extend(c)
            mats.append(mat.reshape(-1))
        qa = _u32(qubits)
        ma = np.ascontiguousarray(np.concatenate(mats)).view(np.float64)
        failed = C.c_size_t()
        self._check(self._api.apply_gates(self._h, len(gates), _p(nt, C.c_uint32), _p(nc, C.c_uint32),
                                          _p(qa, C.c_uint32), _p(ma, C.c_double), C.byref(failed)))

    def cuda_array(self):
        """Zero-copy view of the flushed device state: an object with
        __cuda_array_interface__ (wrap it with torch.as_tensor(view,
        device="cuda") or cupy.asarray).  Valid until the qubit count changes."""
        ptr, n, dt = self.device_state()

        class _View:
            __cuda_array_interface__ = {
                "shape": (n,), "typestr": "<c8" if dt == "c64" else "<c16", "data": (ptr, False),
                "version": 3, "strides": None,
            }

        return _View()

    def device_state(self):
        """(device pointer, number of amplitudes, "c64"|"c128") of the flushed state."""
        ptr = C.c_void_p()
        n = C.c_size_t()
        dt = C.c_int()
        self._check(self._api.state_device_ptr(self._h, C.byref(ptr), C.byref(n), C.byref(dt)))
        return ptr.value, n.value, ("c64" if dt.value == _lib.GSIM_C64 else "c128")

    def compare(self, other):
        """(<self|other> as complex, max |self_i - other_i|), FP64 on the device."""
        out = np.zeros(3, dtype=np.float64)
        self._check(self._api.compare_states(self._h, other._h, _p(out, C.c_double)))
        return complex(out[0], out[1]), float(out[2])

    def timer_mark(self, slot):
        """Record CUDA event `slot` (0..15) on the engine's stream."""
        self._check(self._api.timer_mark(self._h, int(slot)))

    def timer_elapsed(self, a, b):
        """Milliseconds between events a and b (waits for b)."""
        ms = C.c_float()
        self._check(self._api.timer_elapsed(self._h, int(a), int(b), C.byref(ms)))
        return ms.value

    def profile(self, on=True):
        """Bracket every gate-kernel launch with CUDA events (see profile_records)."""
        self._check(self._api.profile_enable(self._h, 1 if on else 0))

    def profile_records(self, clear=True):
        """Per-launch records: dicts of kind, k, nctrl, nqubits, targets, bytes, ms, ngates."""
        n = C.c_size_t()
        self._check(self._api.profile_fetch(self._h, None, 0, C.byref(n)))
        buf = (_lib.LaunchRecord * max(1, n.value))()
        self._check(self._api.profile_fetch(self._h, buf, n.value, C.byref(n)))
        out = [{f: getattr(r, f) for f, _ in _lib.LaunchRecord._fields_ if f != "pad"} for r in buf[: n.value]]
        if clear:
            self._check(self._api.profile_clear(self._h))
        return out


def pin_host(array: np.ndarray):
    """Page-lock a NumPy array's memory (returns an object whose close()
    unpins it) so host<->device copies through the engine run at link speed."""
    api = _lib.load()
    ptr = array.ctypes.data_as(C.c_void_p)
    _lib.check(api, api.host_register(ptr, array.nbytes))

    class _Pin:
        def close(self_inner):
            if getattr(self_inner, "_done", False):
                return
            _lib.check(api, api.host_unregister(ptr))
            self_inner._done = True

    return _Pin()


def set_device(device: int):
    api = _lib.load()
    _lib.check(api, api.set_device(int(device)))
