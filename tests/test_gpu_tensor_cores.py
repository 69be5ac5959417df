"""Fused 4- to 7-qubit gates on complex64 states through the tcgen05
tensor-core kernel (3xTF32, FP32 accumulation), against the complex128 path
(FP64 arithmetic) and against complex64 on CUDA cores.  The gates are
Haar-random with targets spanning low and high bit positions, with and
without controls.  Sizes cover a partial tile (fewer than 128 groups), one
tile, and many tiles per CTA (the stage ring and both TMEM accumulators
wrap many times).  Tolerance: max |d psi| 5e-6 and 1 - F 1e-10."""

import numpy as np
import pytest

from _backends import make
from _circuits import allocate, haar_unitary
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
    ref = run("c128", False, n, psi, gates)
    tc = run("c64", True, n, psi, gates)
    cuda = run("c64", False, n, psi, gates)
    err = np.max(np.abs(tc - ref))
    fid = abs(np.vdot(ref, tc)) ** 2 / (np.vdot(ref, ref).real * np.vdot(tc, tc).real)
    assert err < 5e-6, err
    assert 1 - fid < 1e-10, 1 - fid
    assert np.max(np.abs(cuda - ref)) < 5e-6
