"""Gates with 6 and 7 target qubits (the shared-memory wide-gate kernel, and
the stage planner's route for non-diagonal gates wider than 2 targets),
checked against NumPy: gather every amplitude group, multiply by U, scatter.
Tolerances: complex128 1e-12, complex64 5e-6 (normalised states)."""

import numpy as np
import pytest

from _backends import make
from _circuits import allocate, haar_unitary
from projectq_gb300.workloads import random_state

pytestmark = pytest.mark.gpu


def np_apply(psi, n, U, targets, ctrls):
    k = len(targets)
    fixed = sorted(list(targets) + list(ctrls))
    free = [q for q in range(n) if q not in fixed]
    base = np.zeros(1 << len(free), dtype=np.int64)
    for i, q in enumerate(free):
        base |= ((np.arange(1 << len(free)) >> i) & 1) << q
    for c in ctrls:
        base |= 1 << c
    off = np.zeros(1 << k, dtype=np.int64)
    for j in range(1 << k):
        for l, t in enumerate(targets):
            if (j >> l) & 1:
                off[j] |= 1 << t
    idx = base[:, None] + off[None, :]
    out = psi.copy()
    out[idx] = psi[idx] @ U.T
    return out


@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("fusion", ["none", "staged"])
@pytest.mark.parametrize("k", [6, 7])
def test_wide_gate_matches_numpy(prec, fusion, k):
    n = 12
    rng = np.random.default_rng(k)
    psi = random_state(n, seed=k)
    ref = psi.copy()
    sim = make("gpu", seed=1, precision=prec, fusion="staged" if fusion == "staged" else "none")
    allocate(sim, n)
    sim.set_wavefunction(psi, list(range(n)))
    for trial in range(3):
        qs = [int(v) for v in rng.choice(n, size=k + 2, replace=False)]
        U = haar_unitary(k, rng)
        targets, ctrls = qs[:k], qs[k:k + trial % 3]
        ref = np_apply(ref, n, U, targets, ctrls)
        sim.apply_controlled_gate(U, targets, ctrls)
    sim.run()
    got = sim.cheat()[1]
    assert np.max(np.abs(got - ref)) < (1e-12 if prec == "c128" else 5e-6)


def test_reference_mode_keeps_the_five_qubit_limit():
    """The reference engine rejects fused gates wider than 5 qubits at run()
    (simulator.hpp:522); the reference planner mode keeps that behaviour."""
    sim = make("gpu", seed=1)
    allocate(sim, 8)
    sim.apply_controlled_gate(np.eye(64), list(range(6)), [])
    with pytest.raises(ValueError):
        sim.run()
