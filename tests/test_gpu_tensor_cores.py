"""Fused 4- to 7-qubit gates on complex64 states through the tcgen05
tensor-core kernel (3xTF32, FP32 accumulation), against an FP64 NumPy
contraction of the same gates (tests/_circuits.py numpy_apply, independent of
the engine), and complex64 on CUDA cores against the same.  The gates are
Haar-random with targets spanning low and high bit positions, with and
without controls.  Sizes cover a partial tile (fewer than 128 groups), one
tile, and many tiles per CTA (the stage ring and both TMEM accumulators
wrap many times).  Tolerance: max |d psi| 5e-6 and 1 - F 1e-10."""

import numpy as np
import pytest

from _backends import make
from _circuits import allocate, haar_unitary, numpy_apply
from projectq_gb300.workloads import random_state

pytestmark = pytest.mark.gpu


def run(prec, tc, n, psi, gates):
    s = make("gpu", seed=1, precision=prec, fusion="staged")
    allocate(s, n)
    s.set_tensor_cores(tc)
    s.set_wavefunction(psi, list(range(n)))
    for U, t, c in gates:
        s.apply_controlled_gate(U, t, c)
    s.run()
    return s.cheat()[1]


@pytest.mark.parametrize("k,n", [(4, 12), (4, 16), (4, 24), (5, 13), (5, 15), (6, 15), (7, 15), (5, 24), (6, 23),
                                 (7, 22)])
def test_tensor_core_gates_match_fp64(k, n):
    rng = np.random.default_rng(40 + k + n)
    psi = random_state(n, seed=k)
    gates = []
    for trial in range(4):
        low = 0 if trial < 2 else int(rng.integers(0, 3))  # bit 0: the paired-load path
        high = int(rng.integers(n - 3, n))
        rest = [q for q in rng.permutation(n) if q not in (low, high)]
        targets = [low, high] + [int(q) for q in rest[: k - 2]]
        if trial % 2:
            targets = targets[::-1]  # the kernel sorts targets (and permutes U) itself
        ctrls = [int(q) for q in rest[k - 2: k - 2 + trial % 3]]
        gates.append((haar_unitary(k, rng), targets, ctrls))
    ref = np.asarray(psi, dtype=np.complex128)
    for U, t, c in gates:
        ref = numpy_apply(ref, U, t, c, n)
    tc = run("c64", True, n, psi, gates)
    cuda = run("c64", False, n, psi, gates)
    err = np.max(np.abs(tc - ref))
    fid = abs(np.vdot(ref, tc)) ** 2 / (np.vdot(ref, ref).real * np.vdot(tc, tc).real)
    assert err < 5e-6, err
    assert 1 - fid < 1e-10, 1 - fid
    assert np.max(np.abs(cuda - ref)) < 5e-6


def test_norm_restoration_of_unitary_gates():
    """The tensor cores' FP32 accumulation loses norm systematically (about
    1e-8 x 2^(k+1) per gate); the default mode restores each amplitude
    group's input norm after a unitary gate.  200 alternating U, U^dagger
    7-qubit gates: the norm drifts at least 5x less with the restoration, and
    the state returns to the start within 1 - F 1e-7 either way."""
    n = 16
    psi = random_state(n, seed=1)
    U = haar_unitary(7, np.random.default_rng(7))
    targets = [0, 3, 7, 11, 13, 14, 15]
    drift = {}
    for renorm in (True, False):
        s = make("gpu", seed=1, precision="c64", fusion="none")
        allocate(s, n)
        s.set_tensor_cores(True, renorm=renorm)
        s.set_wavefunction(psi, list(range(n)))
        for it in range(200):
            s.apply_controlled_gate(U if it % 2 == 0 else U.conj().T, targets, [])
        s.run()
        v = s.cheat()[1]
        nv = float(np.vdot(v, v).real)
        drift[renorm] = abs(1 - nv)
        assert 1 - abs(np.vdot(psi, v)) ** 2 / nv < 1e-7
    assert drift[True] < 3e-5, drift
    assert drift[True] * 5 < drift[False], drift
