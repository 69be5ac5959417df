"""Learned fusion cost model.

A 20 -> 64 -> 64 -> 1 ReLU MLP (hand-written CUDA forward / backward / Adam
kernels, mlp.cu) predicts log(milliseconds) of ONE kernel launch from 20
features of it (gsim_launch_features: kernel kind, targets k, controls,
lowest target bit, targets inside a 128-byte line, bytes, flops, stage
operations and substages, packed-pair stage kernel, state size, whether the
state fits in L2, precision, and for the steps of a non-commuting time
evolution, series or expansion and the number of terms).  It is trained on the per-launch timings the engine records with
its profiler while running random circuits under several planners (greedy
fixed-size clusters of width 2..7, one launch per gate, stage plans).

With fusion="learned" the engine sums the predictions over three candidate
plans of each flush -- the greedy fixed-size clusters of the reference's rule,
clusters whose boundaries the model chooses (a gate joins the open cluster
when the merged launch is predicted cheaper than two launches), and the
stage plan -- and runs the cheapest.  The greedy fixed-size fusion is the
fallback and the yardstick: `calibrate` measures wall time of learned against
greedy per state size on circuits not used for training, and the engine
runs learned plans only on the state sizes where they won
(gsim_set_learned_regimes); everywhere else, and with no model installed,
it runs the greedy fusion.

Workflow (on the GPU):
    python -m projectq_gb300.costmodel --collect 60 --train --calibrate 3 \
        --evaluate 24 --out projectq_gb300/data/cost_model.npz
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
from .workloads import Rz, Rx, Ry, X, Z, random_pauli_hamiltonian

F = 20
H = 64
DATA = Path(__file__).resolve().parent / "data" / "cost_model.npz"
# planners whose launches make up the training set: (fusion mode, kmax); the
# learned clusters reach 7 qubits in complex64 and 5 in complex128
COLLECT_PLANNERS = {
    "c64": [("staged", 0), ("none", 0)] + [("reference", k) for k in (2, 3, 4, 5, 6, 7)],
    "c128": [("staged", 0), ("none", 0)] + [("reference", k) for k in (2, 3, 4, 5)],
}
CHOICES = {_lib.GSIM_FUSION_REFERENCE: "greedy", _lib.GSIM_FUSION_STAGED: "staged",
           _lib.GSIM_FUSION_LEARNED: "model clusters"}


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


def blocked_circuit(rng, n, block, per_block):
    """A circuit with locality: for each block of `block` neighbouring qubits
    in turn, `per_block` gates inside the block (60% Rx/Ry/Rz, 40% CNOT).
    Whole blocks fit one tensor-core cluster of up to 7 qubits, so here the
    learned planner's own clusters compete with the stage plan."""
    gates = []
    for b0 in range(0, n - block + 1, block):
        for _ in range(per_block):
            if rng.uniform() < 0.6:
                q = int(rng.integers(b0, b0 + block))
                gates.append(((Rx, Ry, Rz)[int(rng.integers(3))](float(rng.uniform(0, 2 * np.pi))), (q,), ()))
            else:
                a, c = (int(v) for v in rng.choice(np.arange(b0, b0 + block), 2, replace=False))
                gates.append((X, (a,), (c,)))
    return gates


def launch_features(records, api=None):
    """Features (n x 20) of launch records (dicts of profile_records or
    LaunchRecord structs), computed by the engine's own gsim_launch_features."""
    api = api or _lib.load()
    n = len(records)
    buf = (_lib.LaunchRecord * max(1, n))()
    for i, r in enumerate(records):
        for f, _ in _lib.LaunchRecord._fields_:
            setattr(buf[i], f, r[f] if isinstance(r, dict) else getattr(r, f))
    out = np.zeros((max(1, n), F), dtype=np.float32)
    _lib.check(api, api.launch_features(buf, n, _fp(out), F))
    return out[:n]


def _new_sim(n, precision, fusion="staged", kmax=0):
    sim = Simulator(1, precision=precision, fusion="staged")
    for q in range(n):
        sim.allocate_qubit(q)
    sim.set_fusion(fusion, kmax)
    return sim


def record_launches(n, gates, fusion, kmax=0, precision="c64"):
    """Run `gates` once on n qubits with the given planner and return the
    engine's per-launch records (kind, k, controls, targets, bytes, ms...)."""
    sim = _new_sim(n, precision, fusion, kmax)
    sim.profile(True)
    sim.apply_gates(gates)
    sim.run()
    recs = sim.profile_records()
    sim.close()
    return recs


def record_evolution_launches(n, terms, t, mode, precision="c64"):
    """The step launches of one emulate_time_evolution of `terms` (Pauli
    terms with real coefficients, no identity) on an n-qubit |+...+> state,
    with the series ("taylor") or the expansion ("chebyshev")."""
    sim = _new_sim(n, precision, "staged")
    sim.set_time_evolution(mode)
    h = np.array([[1, 1], [1, -1]]) / np.sqrt(2.0)
    sim.apply_gates([(h, (q,), ()) for q in range(n)])
    sim.run()
    sim.profile(True)
    sim.emulate_time_evolution(terms, t, list(range(n)), [])
    recs = [r for r in sim.profile_records() if r["kind"] in (4, 5)]
    sim.close()
    return recs


def collect(ncirc, seed=0, nmin=18, nmax=30, dmin=10, dmax=120, precisions=("c64", "c128"), te_every=3,
            te_nmax=28, big=6):
    """Per-launch training set: features and log(ms) of every launch of
    `ncirc` random circuits, each run under every planner of COLLECT_PLANNERS;
    every `te_every`-th circuit also gives the step launches of a time
    evolution of a random 10-80-term Hamiltonian, by the series and by the
    expansion (short times: a step's cost does not depend on t, only the
    number of steps does); `big` more shallow complex64 circuits run on 31-32
    qubits so that the largest states are inside the training range."""
    rng = np.random.default_rng(seed)
    feats, ys = [], []

    def add(recs):
        if recs:
            feats.append(launch_features(recs))
            ys.append(np.log(np.maximum(np.array([r["ms"] for r in recs], dtype=np.float64), 1e-4)))

    for i in range(ncirc + big):
        n = int(rng.integers(nmin, nmax + 1))
        prec = precisions[i % len(precisions)]
        if prec == "c128":
            n = min(n, nmax - 1)
        depth = int(rng.integers(dmin, dmax + 1))
        if i >= ncirc:  # shallow circuits on the largest states, complex64
            n, prec, depth = int(rng.integers(31, 33)), "c64", int(rng.integers(dmin, 21))
        gates = random_circuit(rng, n, depth)
        for fusion, kmax in COLLECT_PLANNERS[prec]:
            add(record_launches(n, gates, fusion, kmax, prec))
        if te_every and i % te_every == 0:
            m = min(n, te_nmax)
            ham = random_pauli_hamiltonian(m, nterms=int(rng.integers(10, 81)), seed=int(rng.integers(1 << 30)))
            terms = [(tuple(tt), c) for tt, c in ham if tt]
            for mode in ("taylor", "chebyshev"):
                add(record_evolution_launches(m, terms, 0.05, mode, prec))
    return np.concatenate(feats), np.concatenate(ys).astype(np.float32)


def aggregate(X, y):
    """One sample per distinct feature vector (median log-time)."""
    keys, inv = np.unique(X, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    out = np.zeros(len(keys), dtype=np.float32)
    for j in range(len(keys)):
        out[j] = np.median(y[inv == j])
    return keys.astype(np.float32), out


def install(sim, params=None, regimes=None):
    """Install cost-model weights (default: the shipped model) and, when
    given (default: the shipped table for the engine's precision), the
    per-state-size regimes in which learned plans beat the greedy fusion."""
    if params is None or regimes is None:
        shipped = load()
        params = shipped["params"] if params is None else params
        if regimes is None:
            regimes = shipped["regimes_" + sim.precision]
    p = np.ascontiguousarray(params, dtype=np.float32).reshape(-1)
    want = H * F + H + H * H + H + H + 1
    if p.size != want:
        raise ValueError(f"cost model: {p.size} parameters, the {F} -> {H} -> {H} -> 1 network has {want} "
                         "(weights of another feature set: retrain with python -m projectq_gb300.costmodel)")
    _lib.check(sim._api, sim._api.set_cost_model(sim._h, F, H, _fp(p)))
    if regimes is not False:
        r = np.ascontiguousarray(regimes, dtype=np.uint8)
        _lib.check(sim._api, sim._api.set_learned_regimes(sim._h, r.ctypes.data_as(C.POINTER(C.c_uint8)), r.size))


def load(path=DATA):
    d = np.load(path)
    return {k: d[k] for k in d.files}


def load_params(path=DATA):
    return load(path)["params"]


def last_choice(sim):
    mode = C.c_int(-1)
    pred = np.zeros(3, dtype=np.float64)
    _lib.check(sim._api, sim._api.last_plan_choice(sim._h, C.byref(mode), pred.ctypes.data_as(C.POINTER(C.c_double))))
    return mode.value, pred


def wall_time(n, gates, fusion, precision="c64", params=None, regimes=None, tail=None, keep=False, parts=None):
    """Host wall time (s) of submitting `gates`, flushing and synchronising
    on a fresh n-qubit engine (allocation excluded), with `tail` (a Pauli
    Hamiltonian and time) applied as emulate_time_evolution after the gates.
    With a dict `parts`, parts["gates_s"] receives the time up to the end of
    the circuit (before the tail)."""
    sim = _new_sim(n, precision)
    if fusion == "learned":
        install(sim, params, regimes)
    sim.set_fusion(fusion)
    sim.synchronize()
    t0 = time.perf_counter()
    sim.apply_gates(gates)
    if parts is not None:
        sim.run()
        sim.synchronize()
        parts["gates_s"] = time.perf_counter() - t0
    if tail is not None:
        terms, t = tail
        sim.emulate_time_evolution(terms, t, list(range(n)), [])
    sim.run()
    sim.synchronize()
    dt = time.perf_counter() - t0
    choice = last_choice(sim)[0] if fusion == "learned" else None
    if parts is not None and tail is not None:
        parts["tail_method"] = "chebyshev" if sim.counters()["evolutions_chebyshev"] else "taylor"
    if keep:
        return dt, choice, sim
    sim.close()
    return dt, choice


TAIL_NMAX = 30  # the evolution's three complex128 vectors take 3 x 16 GiB at 30 qubits (192 GiB at 32)


def _stream(rng, n, dmin, dmax, p_tail=0.1):
    depth = int(rng.integers(dmin, dmax + 1))
    gates = random_circuit(rng, n, depth)
    tail = None
    if rng.uniform() < p_tail and n <= TAIL_NMAX:
        ham = random_pauli_hamiltonian(n, nterms=50, seed=int(rng.integers(1 << 30)))
        terms = [(tuple(t), c) for t, c in ham if t]
        tail = (terms, float(rng.uniform(0, 1)))
    return gates, tail


def calibrate(params, per_size=3, sizes=range(18, 33), precisions=("c64", "c128"), seed=7, dmin=10, dmax=120):
    """The yardstick: per state size, total wall time of learned against greedy
    fixed-size fusion on `per_size` random circuits (not the training ones);
    returns {precision: uint8[65]} with 1 where learned was faster."""
    out = {}
    rng = np.random.default_rng(seed)
    for prec in precisions:
        allowed = np.zeros(65, dtype=np.uint8)
        for n in sizes:
            if prec == "c128" and n > 30:
                continue
            tg = tl = 0.0
            for _ in range(per_size):
                gates, _ = _stream(rng, n, dmin, dmax, p_tail=0.0)
                tg += wall_time(n, gates, "reference", prec)[0]
                tl += wall_time(n, gates, "learned", prec, params, regimes=np.ones(65, np.uint8))[0]
            allowed[n] = 1 if tl < tg else 0
        out[prec] = allowed
    return out


def evaluate(params, regimes, ncirc, seed=1, nmin=20, nmax=32, dmin=10, dmax=200, precision="c64",
             with_staged=True, fidelity=True):
    """A stream of `ncirc` random circuits (random_circuit; 10% end with the time
    evolution of a 50-term Pauli Hamiltonian): wall time with the learned
    planner against the greedy fixed-size fusion (and the stage planner), and
    1 - F between the learned and the greedy final states.  The totals
    include the time evolutions, which every planner runs the same way (the
    Taylor series of a non-commuting Hamiltonian); the *_gates_s totals are
    the circuits alone, the part the planner decides."""
    rng = np.random.default_rng(seed)
    rows = []
    for _ in range(ncirc):
        n = int(rng.integers(nmin, nmax + 1))
        gates, tail = _stream(rng, n, dmin, dmax)
        pg, pl = {}, {}
        tg, _, sg = wall_time(n, gates, "reference", precision, tail=tail, keep=True, parts=pg)
        tl, choice, sl = wall_time(n, gates, "learned", precision, params, regimes, tail=tail, keep=True, parts=pl)
        row = {"n": n, "gates": len(gates), "tail": tail is not None, "greedy_s": tg, "learned_s": tl,
               "greedy_gates_s": pg["gates_s"], "learned_gates_s": pl["gates_s"],
               "choice": CHOICES.get(choice, str(choice))}
        if tail is not None:
            row["tail_method"] = pl.get("tail_method")
        if fidelity:
            ip, err = sg.compare(sl)
            n1, n2 = sg.compare(sg)[0].real, sl.compare(sl)[0].real
            row["one_minus_fidelity"] = max(0.0, 1.0 - abs(ip) ** 2 / (n1 * n2))
            row["max_abs_err"] = err
        sg.close()
        sl.close()
        if with_staged:
            ps = {}
            row["staged_s"] = wall_time(n, gates, "staged", precision, tail=tail, parts=ps)[0]
            row["staged_gates_s"] = ps["gates_s"]
        rows.append(row)
    res = {"circuits": ncirc, "precision": precision, "with_time_evolution": sum(r["tail"] for r in rows)}
    for k in ("greedy_s", "learned_s", "greedy_gates_s", "learned_gates_s") + (
            ("staged_s", "staged_gates_s") if with_staged else ()):
        res[k] = sum(r[k] for r in rows)
    res["speedup_vs_greedy"] = res["greedy_s"] / res["learned_s"]
    res["gates_speedup_vs_greedy"] = res["greedy_gates_s"] / res["learned_gates_s"]
    if with_staged:
        res["speedup_vs_staged"] = res["staged_s"] / res["learned_s"]
        res["gates_speedup_vs_staged"] = res["staged_gates_s"] / res["learned_gates_s"]
    if fidelity:
        res["max_one_minus_fidelity"] = max(r["one_minus_fidelity"] for r in rows)
    res["rows"] = rows
    return res


def evaluate_blocked(params, regimes, sizes=(26, 28, 30), blocks=((7, 40), (6, 30), (5, 20)), seed=3,
                     precision="c64"):
    """Wall time of the learned planner against the stage plan and the greedy
    fixed-size fusion on block-local circuits (best of two runs each)."""
    rows = []
    for n in sizes:
        for block, per in blocks:
            gates = blocked_circuit(np.random.default_rng(seed * 1000 + n * 10 + block), n, block, per)
            row = {"n": n, "block": block, "gates": len(gates)}
            for mode in ("reference", "staged", "learned"):
                best, choice = math.inf, None
                for _ in range(2):
                    t, ch = wall_time(n, gates, mode, precision, params, regimes)
                    best = min(best, t)
                    choice = ch if ch is not None else choice
                row[("greedy" if mode == "reference" else mode) + "_s"] = best
                if mode == "learned":
                    row["choice"] = CHOICES.get(choice, str(choice))
            rows.append(row)
    tot = {k: sum(r[k] for r in rows) for k in ("greedy_s", "staged_s", "learned_s")}
    return {"circuits": len(rows), **tot, "speedup_vs_greedy": tot["greedy_s"] / tot["learned_s"],
            "speedup_vs_staged": tot["staged_s"] / tot["learned_s"], "rows": rows}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--collect", type=int, default=60)
    ap.add_argument("--train", action="store_true")
    ap.add_argument("--epochs", type=int, default=4000)
    ap.add_argument("--calibrate", type=int, default=0, help="circuits per state size for the calibration against greedy fusion")
    ap.add_argument("--evaluate", type=int, default=0)
    ap.add_argument("--out", default=str(DATA))
    a = ap.parse_args()
    t0 = time.time()
    X, y = collect(a.collect)
    Xu, yu = aggregate(X, y)
    report = {"launches": int(len(y)), "distinct": int(len(yu)), "collect_s": time.time() - t0}
    if a.train:
        net = MLP(seed=0)
        idx = np.random.default_rng(0).permutation(len(yu))
        cut = int(0.85 * len(yu))
        tr, va = idx[:cut], idx[cut:]
        loss = net.train(Xu[tr], yu[tr], epochs=a.epochs)
        pred = net.predict(Xu[va])
        report.update(train_mse=loss, val_mse=float(np.mean((pred - yu[va]) ** 2)))
        params = net.params
        regimes = {"c64": np.ones(65, np.uint8), "c128": np.ones(65, np.uint8)}
        if a.calibrate:
            t1 = time.time()
            regimes = calibrate(params, per_size=a.calibrate)
            report["calibrate_s"] = time.time() - t1
            report["learned_sizes"] = {p: [int(i) for i in np.nonzero(r)[0]] for p, r in regimes.items()}
        Path(a.out).parent.mkdir(parents=True, exist_ok=True)
        np.savez(a.out, params=params, regimes_c64=regimes["c64"], regimes_c128=regimes["c128"])
        if a.evaluate:
            ev = evaluate(params, regimes["c64"], a.evaluate)
            ev.pop("rows")
            report["evaluation"] = ev
    print(json.dumps(report))


if __name__ == "__main__":
    main()
