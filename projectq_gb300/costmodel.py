"""Learned fusion cost model.

The engine can execute a flush of queued gates with three planners: the
shared-memory stage planner ("staged", the greedy default), the reference's
dense-cluster rule ("reference") and one pass per gate ("none").  Which is
fastest depends on the state size (a state that fits in L2 favours cheap
per-gate passes), the gate mix and the precision.  The cost model is a 2x64
ReLU MLP (hand-written CUDA forward/backward/Adam kernels, mlp.cu) that maps
the 16 plan features of gsim_plan_features to log(milliseconds); with
fusion="learned" the engine evaluates it for every planner at each flush and
runs the plan with the lowest prediction.

Workflow (on the GPU):
    python -m projectq_gb300.costmodel --collect 240 --train --evaluate 60 \
        --out projectq_gb300/data/cost_model.npz
which times random circuits of the learned-planner workload under each
planner (engine CUDA events), trains on the recorded timings and reports the
measured wall time of learned vs greedy planning on held-out circuits.
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import time
from pathlib import Path

import numpy as np

from . import _lib
from .simulator import Simulator
from .workloads import Rz, Rx, Ry, X, Z

F = 16
H = 64
MODES = {"staged": _lib.GSIM_FUSION_STAGED, "reference": _lib.GSIM_FUSION_REFERENCE, "none": _lib.GSIM_FUSION_NONE}
DATA = Path(__file__).resolve().parent / "data" / "cost_model.npz"


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class MLP:
    """The cost-model network on the GPU (gsim_mlp_*)."""

    def __init__(self, nin=F, hidden=H, seed=0, api=None):
        self.api = api or _lib.load()
        self.nin, self.hidden = nin, hidden
        h = C.c_void_p()
        _lib.check(self.api, self.api.mlp_create(nin, hidden, seed, C.byref(h)))
        self.h = h
        n = C.c_size_t()
        _lib.check(self.api, self.api.mlp_num_params(self.h, C.byref(n)))
        self.nparams = n.value

    def __del__(self):
        if getattr(self, "h", None) is not None:
            try:
                self.api.mlp_destroy(self.h)
            except Exception:  # pragma: no cover
                pass
            self.h = None

    @property
    def params(self):
        out = np.zeros(self.nparams, dtype=np.float32)
        _lib.check(self.api, self.api.mlp_get_params(self.h, _fp(out)))
        return out

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.nparams:
            raise ValueError("wrong number of parameters")
        _lib.check(self.api, self.api.mlp_set_params(self.h, _fp(p)))

    def predict(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, self.nin)
        out = np.zeros(X.shape[0], dtype=np.float32)
        _lib.check(self.api, self.api.mlp_predict(self.h, _fp(X), X.shape[0], _fp(out)))
        return out

    def gradient(self, X, y):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, self.nin)
        y = np.ascontiguousarray(y, dtype=np.float32).reshape(-1)
        g = np.zeros(self.nparams, dtype=np.float32)
        loss = C.c_double()
        _lib.check(self.api, self.api.mlp_gradient(self.h, _fp(X), _fp(y), X.shape[0], _fp(g), C.byref(loss)))
        return g, loss.value

    def train(self, X, y, epochs=2000, lr=3e-3):
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, self.nin)
        y = np.ascontiguousarray(y, dtype=np.float32).reshape(-1)
        loss = C.c_double()
        _lib.check(self.api, self.api.mlp_train(self.h, _fp(X), _fp(y), X.shape[0], int(epochs), float(lr),
                                                C.byref(loss)))
        return loss.value


def random_circuit(rng, n, depth):
    """The learned-planner workload: `depth` x n/2 gates, 50% single-qubit
    rotations, 30% CNOT/CZ, 10% Toffoli, 10% Rz with 1-3 controls, on
    uniformly random qubits (angles U[0, 2pi))."""
    gates = []
    for _ in range(depth * max(1, n // 2)):
        u = rng.uniform()
        if u < 0.5:
            g = (Rx, Ry, Rz)[int(rng.integers(3))](float(rng.uniform(0, 2 * np.pi)))
            gates.append((g, (int(rng.integers(n)),), ()))
        elif u < 0.8:
            c, t = (int(v) for v in rng.choice(n, 2, replace=False))
            gates.append((X if rng.uniform() < 0.5 else Z, (t,), (c,)))
        elif u < 0.9:
            a, b, t = (int(v) for v in rng.choice(n, 3, replace=False))
            gates.append((X, (t,), (a, b)))
        else:
            k = int(rng.integers(1, 4))
            qs = [int(v) for v in rng.choice(n, k + 1, replace=False)]
            gates.append((Rz(float(rng.uniform(0, 2 * np.pi))), (qs[0],), tuple(qs[1:])))
    return gates


def plan_features(sim, mode):
    out = np.zeros(F, dtype=np.float32)
    _lib.check(sim._api, sim._api.plan_features(sim._h, MODES[mode], _fp(out), F))
    return out


def features_for(n, gates, precision="c64"):
    """Plan features of `gates` on n qubits under every planner."""
    sim = Simulator(1, precision=precision, fusion="staged")
    for q in range(n):
        sim.allocate_qubit(q)
    for m, t, c in gates:
        sim.apply_controlled_gate(m, t, c)
    feats = {mode: plan_features(sim, mode) for mode in MODES}
    sim.close()
    return feats


def time_plan(n, gates, fusion, precision="c64", repeats=1, cost_model=None):
    """Device milliseconds to apply `gates` with the given planner (engine
    CUDA events around submission and flush; the best of `repeats`)."""
    sim = Simulator(1, precision=precision, fusion="staged")
    for q in range(n):
        sim.allocate_qubit(q)
    if fusion == "learned":
        install(sim, cost_model)
    sim.set_fusion(fusion)
    best = math.inf
    for _ in range(repeats + 1):
        sim.synchronize()
        sim.timer_mark(0)
        for m, t, c in gates:
            sim.apply_controlled_gate(m, t, c)
        sim.run()
        sim.timer_mark(1)
        ms = sim.timer_elapsed(0, 1)
        best = min(best, ms)
    choice = C.c_int(-1)
    sim._api.last_plan_choice(sim._h, C.byref(choice))
    sim.close()
    return best, choice.value


def install(sim, params):
    """Install cost-model weights (array or path) into an engine."""
    if params is None:
        params = load_params()
    p = np.ascontiguousarray(params, dtype=np.float32)
    _lib.check(sim._api, sim._api.set_cost_model(sim._h, F, H, _fp(p)))


def load_params(path=DATA):
    return np.load(path)["params"]


def collect(ncirc, seed=0, nmin=18, nmax=27, dmin=10, dmax=200):
    rng = np.random.default_rng(seed)
    X, y, meta = [], [], []
    for i in range(ncirc):
        n = int(rng.integers(nmin, nmax + 1))
        depth = int(rng.integers(dmin, dmax + 1))
        gates = random_circuit(rng, n, depth)
        feats = features_for(n, gates)
        for mode in MODES:
            ms, _ = time_plan(n, gates, mode)
            X.append(feats[mode])
            y.append(math.log(max(ms, 1e-3)))
            meta.append((i, n, depth, mode, ms))
    return np.array(X, dtype=np.float32), np.array(y, dtype=np.float32), meta


def evaluate(params, ncirc, seed=1, **kw):
    """Measured device time of learned vs greedy (staged) planning on held-out
    circuits; both plans apply the same gates."""
    rng = np.random.default_rng(seed)
    rows = []
    for _ in range(ncirc):
        n = int(rng.integers(kw.get("nmin", 18), kw.get("nmax", 27) + 1))
        depth = int(rng.integers(kw.get("dmin", 10), kw.get("dmax", 200) + 1))
        gates = random_circuit(rng, n, depth)
        t_greedy, _ = time_plan(n, gates, "staged")
        t_learned, choice = time_plan(n, gates, "learned", cost_model=params)
        rows.append({"n": n, "gates": len(gates), "greedy_ms": t_greedy, "learned_ms": t_learned, "choice": choice})
    g = sum(r["greedy_ms"] for r in rows)
    lrn = sum(r["learned_ms"] for r in rows)
    return {"circuits": ncirc, "greedy_ms": g, "learned_ms": lrn, "speedup": g / lrn, "rows": rows}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--collect", type=int, default=240)
    ap.add_argument("--train", action="store_true")
    ap.add_argument("--evaluate", type=int, default=0)
    ap.add_argument("--epochs", type=int, default=3000)
    ap.add_argument("--out", default=str(DATA))
    a = ap.parse_args()
    t0 = time.time()
    X, y, meta = collect(a.collect)
    report = {"samples": len(y), "collect_s": time.time() - t0}
    params = None
    if a.train:
        net = MLP(seed=0)
        n = len(y)
        idx = np.random.default_rng(0).permutation(n)
        cut = int(0.8 * n)
        tr, va = idx[:cut], idx[cut:]
        loss = net.train(X[tr], y[tr], epochs=a.epochs)
        pred = net.predict(X[va])
        report.update(train_mse=loss, val_mse=float(np.mean((pred - y[va]) ** 2)))
        params = net.params
        Path(a.out).parent.mkdir(parents=True, exist_ok=True)
        np.savez(a.out, params=params, X=X, y=y)
    if a.evaluate and params is not None:
        report["evaluation"] = evaluate(params, a.evaluate)
    print(json.dumps(report))


if __name__ == "__main__":
    main()
