"""The UnitarySimulator logic (vec(U) in a 2n-qubit engine state, qubit map,
resets into history, flush and measurement) on the CPU oracle engine, against
ProjectQ's own UnitarySimulator (backends/_unitary.py) on the same circuits."""

import random
import warnings

import numpy as np
import pytest

from _backends import oracle_api, projectq_available

pytestmark = pytest.mark.skipif(not projectq_available(), reason="ProjectQ's Python layers are not installed")


def circuit(eng, qureg, rng, ngates):
    from projectq.meta import Control
    from projectq.ops import CNOT, H, Rx, Ry, Rz, T, Toffoli

    n = len(qureg)
    for _ in range(ngates):
        kind = int(rng.integers(6))
        a, b, c = (int(v) for v in rng.choice(n, 3, replace=False))
        th = float(rng.uniform(0, 2 * np.pi))
        if kind == 0:
            H | qureg[a]
        elif kind == 1:
            Rx(th) | qureg[a]
        elif kind == 2:
            CNOT | (qureg[a], qureg[b])
        elif kind == 3:
            Toffoli | (qureg[a], qureg[b], qureg[c])
        elif kind == 4:
            with Control(eng, qureg[b]):
                Ry(th) | qureg[a]
        else:
            T | qureg[a]
            Rz(th) | qureg[b]


def scenario(backend, seed):
    from projectq import MainEngine
    from projectq.ops import All, Measure

    rng = np.random.default_rng(seed)
    eng = MainEngine(backend=backend, engine_list=[])
    qureg = eng.allocate_qureg(5)
    circuit(eng, qureg, rng, 40)
    eng.flush()
    u1 = backend.unitary
    random.seed(seed)
    All(Measure) | qureg
    bits = [int(q) for q in qureg]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        circuit(eng, qureg, rng, 20)  # resets the unitary: the old one goes to history
    eng.flush()
    return u1, bits, backend.unitary, backend.history


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_unitary_simulator_matches_reference_class(seed):
    from projectq.backends import UnitarySimulator as RefUnitary

    from projectq_gb300.unitary import UnitarySimulator

    ours = scenario(UnitarySimulator(_api=oracle_api()), seed)
    ref = scenario(RefUnitary(), seed)
    assert np.max(np.abs(ours[0] - ref[0])) < 1e-12
    assert ours[1] == ref[1]
    assert np.max(np.abs(ours[2] - ref[2])) < 1e-12
    assert len(ours[3]) == len(ref[3]) == 1
    assert np.max(np.abs(ours[3][0] - ref[3][0])) < 1e-12


def test_reference_unitary_suite_on_the_oracle_engine():
    """ProjectQ's own UnitarySimulator tests (backends/_unitary_test.py) with
    projectq_gb300.unitary.UnitarySimulator in place of the reference class,
    its vec(U) held by the CPU oracle engine (the GPU run is in
    test_gpu_dropin.py)."""
    import _refsuite

    rc, passed, out = _refsuite.run("oracle", "c128", unitary=True)
    assert rc == 0, out[-6000:]
    assert passed >= 8
