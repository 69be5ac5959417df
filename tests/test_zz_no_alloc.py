"""The allocation-free probability entry point, checked against the regular
one on the GPU.

gsim_probability_noalloc serves callers that cannot allocate device memory
(for instance code whose device memory is owned by another allocator): it
takes a device state pointer and keeps its partial sums in a fixed
__device__ array instead of engine scratch.  This test calls it through the
C ABI on an engine's device state and compares it with
gsim_get_probability on the same state, for two calls in a row.  The file is
named to run last, after every other test.
"""

import ctypes as C

import numpy as np
import pytest

from _backends import make
from projectq_gb300 import _lib
from projectq_gb300.workloads import random_state

pytestmark = pytest.mark.gpu

TOL = {"c128": 1e-12, "c64": 5e-6}


@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("n,patterns", [
    # one block: summed subspaces below 2^14 amplitudes
    (16, [([3, 9, 0], [1, 0, 1]), ([15, 2], [0, 0])]),
    # many blocks: 2^21 and 2^19 amplitudes summed (128 and 32 blocks), so the
    # last-block reduction and the counter reset between calls are exercised
    (22, [([7], [1]), ([0, 21, 11], [0, 1, 1])]),
])
def test_probability_noalloc_matches_get_probability(prec, n, patterns):
    api = _lib.load()
    sim = make("gpu", seed=1, precision=prec)
    for q in range(n):
        sim.allocate_qubit(q)
    sim.set_wavefunction(random_state(n, seed=5), list(range(n)))
    ptr, length, dt = sim.device_state()
    assert length == 1 << n and dt == prec
    code = _lib.GSIM_C64 if prec == "c64" else _lib.GSIM_C128
    # two calls in a row, on different patterns; the scratch keeps the first
    # call's contents when the second one starts
    for ids, bits in patterns:
        mask = sum(1 << q for q in ids)
        value = sum(b << q for q, b in zip(ids, bits))
        out = C.c_double(-1.0)
        rc = api.probability_noalloc(C.c_void_p(ptr), code, n, mask, value, C.byref(out), None)
        _lib.check(api, rc)
        expected = sim.get_probability(bits, ids)
        assert out.value == pytest.approx(expected, abs=TOL[prec])
    sim.close()


def test_probability_noalloc_rejects_oversized_requests():
    api = _lib.load()
    sim = make("gpu", seed=1)
    sim.allocate_qubit(0)
    ptr, _, _ = sim.device_state()
    out = C.c_double()
    rc = api.probability_noalloc(C.c_void_p(ptr), _lib.GSIM_C128, 40, 0, 0, C.byref(out), None)
    assert rc == _lib.GSIM_ERR_LENGTH
    assert b"2^32" in api.last_error()
