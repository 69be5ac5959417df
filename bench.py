#!/usr/bin/env python3
"""Benchmark: 30-qubit random circuit on one GB300 — gates/s and HBM GB/s of
the complex64 engine (FP64 reductions) next to the complex128 plain path.

Workload (one "step"): the depth-40 random circuit of 30 qubits with 40 gates
per layer over {H, T, S, Rx, Ry, Rz, CNOT, CZ, Toffoli} (seeded, numpy PCG64
seed 0) applied to the device-resident state (8 GiB complex64; the complex128
arm holds 16 GiB).  The initial state is i.i.d. complex Gaussian, normalised.
Inputs are larger than L2 (129 MB), so no cache flush is needed between steps.

Reported:
  value     logical gates/s of the complex64 engine (device-resident state,
            CUDA events on the engine's stream, max over ranks);
  e2e       the same metric through the reference-facing Python API
            (Simulator.set_wavefunction from pinned host memory, one
            apply_controlled_gate call per gate, run, and a host read of
            <Z0 Z1 + X5 X6> and a measurement) — host<->device copies inside;
  c128      the complex128 plain path on the same circuit and GPU;
  fidelity  1 - |<psi_c128|psi_c64>|^2 and max |d psi| after one circuit;
  roofline  the dominant gate kernel's achieved algorithmic HBM GB/s
            (bytes per launch / per-launch CUDA-event time) vs the measured
            copy bandwidth in MEASURED_PEAKS.json;
  cpu_baseline  the CPU oracle (a restatement of the reference engine, OpenMP
            on all host cores) on a bounded sample of the same circuit.

`--impl reference` times that CPU implementation alone on the same metric.
Multi-GPU: the path runs as independent replicas (one per rank).
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "30q circuit gates/s & HBM GB/s: c64+FP64-reduce vs c128 on GB300 at 1-F<=1e-6"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--depth", type=int, default=40)
    ap.add_argument("--per-layer", type=int, default=40)
    ap.add_argument("--fusion", default="staged", choices=["staged", "reference", "none"])
    ap.add_argument("--stage-kernel", default="packed", choices=["packed", "register", "pass"],
                    help="stage kernel of the staged planner (complex64 packed pairs by default)")
    ap.add_argument("--c128-steps", type=int, default=None,
                    help="timed steps of the complex128 arm (default: --steps, at most 5: 5.5 s each at 30 qubits)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-gates", type=int, default=100, help="gates in each mode of the CPU baseline sample")
    ap.add_argument("--ref-gates", type=int, default=8,
                    help="--impl reference: gates per timed window (per step, in each mode)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--check-qubits", type=int, default=26,
                    help="qubits of the accuracy check against the CPU reference engine (0: skip)")
    ap.add_argument("--only", choices=["c64", "c128"], default=None,
                    help="profiling mode: time one precision only (no accuracy, e2e or CPU legs)")
    ap.add_argument("--init", choices=["random", "zero"], default="random",
                    help="initial state; kernel times do not depend on the amplitudes")
    ap.add_argument("--workload", choices=["circuit", "fused", "adjoint", "learned", "gates", "evolution"],
                    default="circuit",
                    help="circuit: the 30-qubit headline; fused: k=5..7 dense gates at 32 qubits on tensor "
                         "cores; adjoint: energy + gradient of a 960-parameter ansatz at 24 qubits; learned: "
                         "learned vs greedy fusion planning on random circuits; gates: HBM bandwidth of the "
                         "single-gate kernels (one pass per gate); evolution: QAOA-style time evolution of "
                         "commuting Hamiltonians, exact product vs Taylor series, and a non-commuting one, "
                         "Chebyshev expansion vs Taylor series")
    ap.add_argument("--ngates", type=int, default=60, help="fused workload: gates per step")
    ap.add_argument("--fd-params", type=int, default=0,
                    help="adjoint workload: parameters checked by finite differences (0: every parameter)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


KERNEL_KINDS = ["dense_gate", "stage", "wide_gate", "tensor_core_gate"]
# DRAM bytes (read + write) per amplitude of one stage-kernel launch, from the
# ncu capture of the 26-qubit complex64 circuit on the packed-pair kernel
# (537.50 MB read + 475.22 MB written per launch over 2^26 amplitudes);
# traffic grows with the state size, so a 30-qubit launch moves 2^30 times this.
NCU_TRAFFIC_PER_AMP = {(1, 1): (537.502976e6 + 475.218944e6) / 2 ** 26}
NCU_TRAFFIC_SOURCE = "profiles/stage_pk_kernel_c64_26q_ncu.md, scaled from 2^26 to 2^nq amplitudes"


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        return dist, world, rank, local
    return None, 1, 0, 0


def allreduce_max(dist, x):
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ---------------------------------------------------------------------------
def apply_circuit(sim, gates):
    for m, t, c in gates:
        sim.apply_controlled_gate(m, t, c)
    sim.run()


def timed_steps(sim, gates, steps, warmup, dist, profile_kernel=True):
    for _ in range(warmup):
        apply_circuit(sim, gates)
    sim.synchronize()
    sim.reset_counters()
    barrier(dist)
    sim.synchronize()
    sim.profile(profile_kernel)
    sim.timer_mark(0)
    for _ in range(steps):
        apply_circuit(sim, gates)
    sim.timer_mark(1)
    ms = sim.timer_elapsed(0, 1)
    sim.synchronize()
    barrier(dist)
    recs = sim.profile_records() if profile_kernel else []
    sim.profile(False)
    return ms, sim.counters(), recs


def dominant_kernel(recs):
    """Group launches by kernel kind and width; the group with the most time."""
    groups = {}
    for r in recs:
        key = (r["kind"], r["k"], r["precision"])
        g = groups.setdefault(key, {"launches": 0, "ms": 0.0, "bytes": 0})
        g["launches"] += 1
        g["ms"] += r["ms"]
        g["bytes"] += r["bytes"]
    if not groups:
        return None, {}
    key = max(groups, key=lambda k: groups[k]["ms"])
    return key, groups


class CpuEngine:
    """The CPU implementation timed as the baseline: the reference engine
    itself, built from ProjectQ's own simulator.hpp with the flags of its
    setup.py (oracle/_ref/libref_sim_setup.so, made by oracle/build_ref.sh),
    with all host threads (OMP_NUM_THREADS = cores, OMP_PROC_BIND=spread);
    the oracle port (oracle/oracle_sim.cpp) only where that build is absent.
    One engine of `nq` qubits is allocated once (|0...0>; its kernels' times
    do not depend on the amplitudes) and then runs windows of the circuit in
    the reference's two modes: one run() per gate (ProjectQ's Simulator with
    gate_fusion=False, the default) and one run() per window (gate_fusion=True,
    the greedy fusion of simulator.hpp:204-222)."""

    def __init__(self, nq):
        sys.path.insert(0, str(ROOT / "tests"))
        from _backends import make, ref_setup_api

        self.cores = os.cpu_count() or 1
        if ref_setup_api() is not None:
            self.kind, self.sim = "reference", make("ref_setup", seed=0)
            self.what = "reference engine (simulator.hpp) built with setup.py's flags"
        else:
            self.kind, self.sim = "port", make("oracle", seed=0)
            self.sim.set_fusion("reference")
            self.what = "oracle port (reference build absent)"
        self.nq = nq
        t0 = time.perf_counter()
        for q in range(nq):
            self.sim.allocate_qubit(q)
        self.setup_seconds = time.perf_counter() - t0

    def window(self, gates, start, count):
        return [gates[(start + i) % len(gates)] for i in range(count)]

    def time_per_gate(self, sample):
        t0 = time.perf_counter()
        for m, t, c in sample:
            self.sim.apply_controlled_gate(m, t, c)
            self.sim.run()
        return time.perf_counter() - t0

    def time_fused(self, sample):
        t0 = time.perf_counter()
        for m, t, c in sample:
            self.sim.apply_controlled_gate(m, t, c)
        self.sim.run()
        return time.perf_counter() - t0

    def close(self):
        self.sim.close()


def set_omp_env():
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    os.environ.setdefault("OMP_PROC_BIND", "spread")


def cpu_nq(nq):
    """The baseline's state size: the workload's, unless host memory cannot
    hold its complex128 state (plus the reallocation of the last allocate)."""
    if host_memory_gib() and host_memory_gib() < 3 * (1 << nq) * 16 / 2**30 + 8:
        return 26
    return nq


def cpu_baseline(gates, nq, ngates):
    """One bounded sample at full width: the first `ngates` gates with one
    run() per gate, and the next `ngates` with the reference's fusion."""
    eng = CpuEngine(nq)
    per_gate = eng.time_per_gate(eng.window(gates, 0, ngates))
    fused = eng.time_fused(eng.window(gates, ngates, ngates))
    eng.close()
    best = min(per_gate, fused)
    nbytes = sum(2 * (1 << (nq - len(c))) * 16 for _, _, c in gates[:ngates])
    return {"value": ngates / best, "unit": "gates/s", "cores": eng.cores, "kind": eng.kind,
            "sample": f"{eng.what}, {nq} qubits complex128: gates 0-{ngates - 1} of the circuit with one run() per "
                      f"gate ({ngates / per_gate:.3f} gates/s) and gates {ngates}-{2 * ngates - 1} with the "
                      f"reference's gate fusion ({ngates / fused:.3f} gates/s); value = the faster mode",
            "per_gate_gates_per_s": ngates / per_gate, "fused_gates_per_s": ngates / fused,
            "hbm_like_gbs_per_gate_mode": nbytes / per_gate / 1e9, "seconds": per_gate + fused}


def host_memory_gib():
    try:
        return os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES") / 2**30
    except Exception:
        return 0.0


def run_reference(a):
    """--impl reference: the reference's CPU engine on this machine's host
    cores, on the same 30-qubit circuit.  Every step times a window of
    `--ref-gates` consecutive gates (the windows advance through the circuit,
    so K steps time K x window gates) in both of the reference's modes; the
    value is the faster mode's gates/s over the timed steps."""
    from projectq_gb300.workloads import random_gate_circuit

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    set_omp_env()
    gates = random_gate_circuit(a.qubits, a.depth, a.per_layer, seed=0)
    nq = cpu_nq(a.qubits)
    eng = CpuEngine(nq)
    S = a.ref_gates
    for i in range(a.warmup):
        eng.time_per_gate(eng.window(gates, i * S, S))
    tg, tf = [], []
    for i in range(a.warmup, a.warmup + a.steps):
        tg.append(eng.time_per_gate(eng.window(gates, i * S, S)))
        tf.append(eng.time_fused(eng.window(gates, i * S, S)))
    eng.close()
    vg, vf = S * a.steps / sum(tg), S * a.steps / sum(tf)
    v = max(vg, vf)
    mode = "one run() per gate" if vg >= vf else "gate fusion"
    sample = (f"{eng.what}, {nq} qubits complex128, {a.steps} windows of {S} consecutive gates "
              f"({S * a.steps} gates timed per mode): one run() per gate {vg:.3f} gates/s, gate fusion "
              f"{vf:.3f} gates/s; value = {mode}")
    print(json.dumps({
        "metric": METRIC, "impl": "reference", "value": v, "unit": "gates/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1000.0 * S / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic", "config": {"workload": f"random circuit, {nq} qubits, depth {a.depth}, "
                                                    f"{a.per_layer} gates/layer ({S}-gate window per step)",
                                        "qubits": nq},
        "cpu_baseline": {"value": v, "unit": "gates/s", "cores": eng.cores, "kind": eng.kind, "sample": sample},
        "modes": {"per_gate_run": vg, "gate_fusion": vf},
        "e2e": {"value": v, "unit": "gates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def accuracy_vs_reference(nq, depth, per_layer, fusion):
    """The headline circuit family at `nq` qubits (the same generator and
    seeds, i.i.d. complex Gaussian initial state) on the GPU in complex64 and
    complex128 with the bench's planner, and on the CPU in the reference
    engine itself (oracle/_ref/libref_sim.so: ProjectQ's simulator.hpp with
    its own greedy fusion; the oracle port where that build is absent).
    Returns 1 - F and max |d psi| of each GPU state against the CPU one."""
    sys.path.insert(0, str(ROOT / "tests"))
    from _backends import make, ref_api
    from projectq_gb300 import Simulator
    from projectq_gb300.workloads import random_gate_circuit, random_state

    gates = random_gate_circuit(nq, depth, per_layer, seed=0)
    psi0 = random_state(nq, seed=0, dtype=np.complex128)
    ids = list(range(nq))
    kind = "reference engine (simulator.hpp), its own gate fusion" if ref_api() is not None else "oracle port"
    cpu = make("ref" if ref_api() is not None else "oracle", seed=0)
    for q in ids:
        cpu.allocate_qubit(q)
    cpu.set_wavefunction(psi0, ids)
    t0 = time.perf_counter()
    apply_circuit(cpu, gates)
    cpu_seconds = time.perf_counter() - t0
    ref = cpu.cheat()[1]
    cpu.close()
    nref = float(np.vdot(ref, ref).real)
    out = {"qubits": nq, "gates": len(gates), "reference": kind, "cpu_seconds": cpu_seconds}
    for prec in ("c64", "c128"):
        sim = Simulator(1, precision=prec, fusion=fusion)
        for q in ids:
            sim.allocate_qubit(q)
        sim.set_wavefunction(psi0.astype(np.complex64) if prec == "c64" else psi0, ids)
        apply_circuit(sim, gates)
        st = sim.cheat()[1]
        sim.close()
        ip = np.vdot(ref, st)
        out[prec] = {"one_minus_fidelity": float(1.0 - abs(ip) ** 2 / (nref * float(np.vdot(st, st).real))),
                     "max_abs_err": float(np.max(np.abs(st - ref)))}
        del st
    return out


def run_only(a):
    """Profiling mode: the circuit on one precision, from |0...0> or psi0."""
    from projectq_gb300 import Simulator
    from projectq_gb300.workloads import random_gate_circuit, random_state

    gates = random_gate_circuit(a.qubits, a.depth, a.per_layer, seed=0)
    sim = Simulator(1, precision=a.only, fusion=a.fusion)
    sim.set_stage_kernel(a.stage_kernel)
    for q in range(a.qubits):
        sim.allocate_qubit(q)
    if a.init == "random":
        sim.set_wavefunction(random_state(a.qubits, seed=0, dtype=np.complex64), list(range(a.qubits)))
    ms, cnt, recs = timed_steps(sim, gates, a.steps, a.warmup, None)
    key, groups = dominant_kernel(recs)
    print(json.dumps({"mode": "only", "precision": a.only, "qubits": a.qubits, "ms_per_step": ms / max(1, a.steps),
                      "gates_per_s": len(gates) * a.steps / (ms * 1e-3), "counters": cnt,
                      "kernel_groups": {f"kind{k[0]}_k{k[1]}_p{k[2]}": v for k, v in groups.items()}}), flush=True)


def sampled_group_check(sim, nq, haar_unitary, rng, k=7, ngroups=16):
    """Apply H to every qubit (so no amplitude is zero), then one Haar k-qubit
    gate with a target below 5; read 16 random amplitude groups before and
    after it and compare with the FP64 product U x on the host."""
    from projectq_gb300.workloads import H

    for q in range(nq):
        sim.apply_controlled_gate(H, [q], [])
    sim.run()
    low = int(rng.integers(0, 5))
    rest = [int(q) for q in rng.permutation(nq) if q != low]
    targets = [low] + rest[: k - 1]
    U = haar_unitary(k, rng)
    ids = list(range(nq))

    def amp(index):
        return sim.get_amplitude([(index >> q) & 1 for q in range(nq)], ids)

    offs = [sum(((j >> l) & 1) << targets[l] for l in range(k)) for j in range(1 << k)]
    tmask = sum(1 << t for t in targets)
    bases = []
    while len(bases) < ngroups:
        b = int(rng.integers(0, 1 << nq)) & ~tmask
        if b not in bases:
            bases.append(b)
    xs = [np.array([amp(b + o) for o in offs], dtype=np.complex128) for b in bases]
    sim.apply_controlled_gate(U, targets, [])
    sim.run()
    err, scale = 0.0, 0.0
    for b, x in zip(bases, xs):
        y = np.array([amp(b + o) for o in offs], dtype=np.complex128)
        ref = U @ x
        err = max(err, float(np.max(np.abs(y - ref))))
        scale = max(scale, float(np.max(np.abs(ref))))
    return {"qubits": nq, "k": k, "groups": ngroups, "max_abs_err": err, "max_abs_err_relative": err / scale}


def run_fused(a):
    """Dense Haar-random k-qubit gates, k uniform in {5, 6, 7}, on a 32-qubit
    complex64 state (32 GiB); targets always include a qubit below 5 and one
    above 25.  All run on the tcgen05 tensor-core kernel (3xTF32, FP32
    accumulation).  Error: the same kind of gates at 24 qubits against the
    complex128 path (FP64 arithmetic)."""
    sys.path.insert(0, str(ROOT / "tests"))
    from _circuits import haar_unitary
    from projectq_gb300 import Simulator
    from projectq_gb300.workloads import random_state

    def gates_for(n, count, seed):
        rng = np.random.default_rng(seed)
        out = []
        for _ in range(count):
            k = int(rng.integers(5, 8))
            low, high = int(rng.integers(0, 5)), int(rng.integers(n - 6, n))
            rest = [int(q) for q in rng.permutation(n) if q not in (low, high)]
            out.append((haar_unitary(k, rng), [low, high] + rest[: k - 2], []))
        return out

    nq = 32 if a.qubits == 30 else a.qubits
    gates = gates_for(nq, a.ngates, 0)
    sim = Simulator(1, precision="c64", fusion="staged")
    for q in range(nq):
        sim.allocate_qubit(q)
    with ClockSampler(0) as clk:
        ms, cnt, recs = timed_steps(sim, gates, a.steps, a.warmup, None)
    key, groups = dominant_kernel(recs)
    # the same gates without the per-group norm restoration (tensor-core mode 2)
    sim.set_tensor_cores(True, renorm=False)
    ms_nr, _, recs_nr = timed_steps(sim, gates, a.steps, 1, None)
    _, groups_nr = dominant_kernel(recs_nr)
    sim.set_tensor_cores(True)
    flops = sum(8.0 * 2 ** nq * 2 ** len(t) for _, t, _ in gates) * a.steps
    # accuracy at 24 qubits against complex128 (FP64 arithmetic)
    small = gates_for(24, 30, 1)
    res = {}
    for prec in ("c64", "c128"):
        s = Simulator(1, precision=prec, fusion="staged")
        for q in range(24):
            s.allocate_qubit(q)
        s.set_wavefunction(random_state(24, seed=3), list(range(24)))
        for m, t, c in small:
            s.apply_controlled_gate(m, t, c)
        s.run()
        res[prec] = s
    ip, maxerr = res["c128"].compare(res["c64"])
    n1 = res["c128"].compare(res["c128"])[0].real
    n2 = res["c64"].compare(res["c64"])[0].real
    for s_ in res.values():
        s_.close()
    # sampled check at full width: one more k = 7 gate on the spread-out state,
    # 16 random groups read before and after and compared with an FP64 product
    sampled = sampled_group_check(sim, nq, haar_unitary, np.random.default_rng(5))
    print(json.dumps({"workload": "fused k=5..7 dense gates", "qubits": nq, "gates_per_step": len(gates),
                      "ms_per_step": ms / a.steps, "gates_per_s": len(gates) * a.steps / (ms * 1e-3),
                      "algorithmic_tflops": flops / (ms * 1e-3) / 1e12,
                      "hbm_gbs": cnt["gate_bytes"] / (ms * 1e-3) / 1e9,
                      "accuracy_24q_30gates": {"one_minus_fidelity": 1 - abs(ip) ** 2 / (n1 * n2), "max_abs_err": maxerr},
                      "accuracy_sampled_full_width": sampled,
                      "without_norm_restoration": {
                          "ms_per_step": ms_nr / a.steps,
                          "kernel_groups": {f"kind{k[0]}_k{k[1]}_p{k[2]}": v for k, v in groups_nr.items()}},
                      "kernel_groups": {f"kind{k[0]}_k{k[1]}_p{k[2]}": v for k, v in groups.items()},
                      "clocks": clk.summary()}), flush=True)


def run_gates(a):
    """Single-gate kernels, one launch per gate (fusion "none"), on a 30-qubit
    state: for each (precision, gate kind) the achieved HBM bandwidth
    (algorithmic bytes / CUDA-event time per launch, mean over launches) as a
    fraction of the measured copy bandwidth.  Targets cycle over every bit
    position, so low (in-vector) and high (strided) targets are both timed."""
    from projectq_gb300 import Simulator
    from projectq_gb300.workloads import H, Rx, T, X

    nq = a.qubits
    peak, _ = measured_peak()
    out = {}
    cases = {
        "1q_dense(H)": lambda q, n: (H, [q], []),
        "1q_rx": lambda q, n: (Rx(0.3), [q], []),
        "1q_diag(T)": lambda q, n: (T, [q], []),
        "cnot": lambda q, n: (X, [q], [(q + 7) % n]),
        "2q_dense": lambda q, n: (np.kron(Rx(0.2), H), [q, (q + 11) % n], []),
        "3q_dense": lambda q, n: (np.kron(np.kron(Rx(0.2), H), Rx(0.5)), [q, (q + 11) % n, (q + 19) % n], []),
        "4q_dense": lambda q, n: (haar4, [q, (q + 7) % n, (q + 13) % n, (q + 23) % n], []),
    }
    haar4 = np.linalg.qr(np.random.default_rng(4).standard_normal((16, 16))
                         + 1j * np.random.default_rng(5).standard_normal((16, 16)))[0]
    wide = {  # with the tensor cores off: the CUDA-core kernels (4 qubits: dense, 7: wide), with FLOP rates
        "4q_dense_cuda_cores": lambda q, n: (haar4, [q, (q + 7) % n, (q + 13) % n, (q + 23) % n], []),
        "7q_dense_cuda_cores": lambda q, n: (haar7, [(q + 4 * i) % n for i in range(7)], []),
    }
    haar7 = np.linalg.qr(np.random.default_rng(7).standard_normal((128, 128))
                         + 1j * np.random.default_rng(8).standard_normal((128, 128)))[0]
    for prec in ("c64", "c128"):
        sim = Simulator(1, precision=prec, fusion="none")
        for q in range(nq):
            sim.allocate_qubit(q)
        for name, mk in cases.items():
            gates = [mk(q, nq) for q in range(nq)]
            ms, cnt, recs = timed_steps(sim, gates, max(1, a.steps), max(1, a.warmup), None)
            gbs = [r["bytes"] / (r["ms"] * 1e-3) / 1e9 for r in recs if r["ms"] > 0]
            mean = float(np.mean(gbs)) if gbs else 0.0
            out[f"{prec}/{name}"] = {"launches": len(recs), "gbs_mean": round(mean, 1), "gbs_min": round(min(gbs), 1),
                                     "frac_of_peak": round(mean / peak, 3)}
        sim.set_tensor_cores(False)
        for name, mk in wide.items():
            gates = [mk(q, nq) for q in range(0, nq, 5)]
            ms, cnt, recs = timed_steps(sim, gates, 1, 1, None)
            per = [r["ms"] for r in recs if r["ms"] > 0]
            kq = len(gates[0][1])
            tflops = 8.0 * 2 ** nq * 2 ** kq / (np.mean(per) * 1e-3) / 1e12 if per else 0.0
            gbs = 2 * 2 ** nq * (8 if prec == "c64" else 16) / (np.mean(per) * 1e-3) / 1e9 if per else 0.0
            out[f"{prec}/{name}"] = {"launches": len(recs), "ms_mean": round(float(np.mean(per)), 3),
                                     "algorithmic_tflops": round(tflops, 2), "frac_of_peak": round(gbs / peak, 3)}
        sim.close()
    print(json.dumps({"workload": "single-gate kernels, one pass per gate", "qubits": nq, "peak_gbs": peak,
                      "kernels": out}), flush=True)


def public_energy(sim, circ, theta, terms, zero):
    """E(theta) through the plain public path, independent of the adjoint
    kernels: set_wavefunction(|0...0>), the circuit's gates through
    apply_gates + run (the stage planner), then get_expectation_value."""
    ids = list(range(zero.size.bit_length() - 1))
    sim.set_wavefunction(zero, ids)
    sim.apply_gates(circ.gates(theta))
    sim.run()
    return sim.get_expectation_value(terms, ids)


def run_adjoint(a):
    """Energy and gradient of the hardware-efficient ansatz (20 layers of Ry,
    Rz on each qubit + CNOT ladder: 960 parameters at 24 qubits) for a
    200-term random Pauli Hamiltonian, by one adjoint sweep.  Checked (c128):
    against central finite differences (h = 1e-4) on EVERY parameter, with
    energies from the plain public path (public_energy: 1920 evaluations);
    against the parameter-shift rule on 8 parameters; and the energy against
    the reference engine itself on the CPU (simulator.hpp's
    get_expectation_value, oracle/_ref/libref_sim.so; the oracle port where
    that build is absent).  Plus a batch of 16 parameter sets with 4, 8, 12
    and 20 layers (complex64).  --fd-params limits the finite differences to
    that many evenly spaced parameters (0: all)."""
    sys.path.insert(0, str(ROOT / "tests"))
    from _backends import make, ref_api
    from projectq_gb300 import Simulator
    from projectq_gb300.adjoint import energy_and_gradient, hardware_efficient_ansatz
    from projectq_gb300.simulator import pin_host
    from projectq_gb300.workloads import random_pauli_hamiltonian

    nq = 24 if a.qubits == 30 else a.qubits
    circ = hardware_efficient_ansatz(nq, 20)
    terms = random_pauli_hamiltonian(nq, 200, seed=0)
    theta = np.random.default_rng(0).uniform(-np.pi, np.pi, size=circ.nparams)
    out = {"workload": "adjoint gradient", "qubits": nq, "parameters": circ.nparams, "terms": len(terms)}
    for prec in ("c128", "c64"):
        sim = Simulator(1, precision=prec)
        for q in range(nq):
            sim.allocate_qubit(q)
        for _ in range(max(1, a.warmup)):
            energy_and_gradient(sim, circ, theta, terms, range(nq))
        t0 = time.perf_counter()
        for _ in range(a.steps):
            e, g = energy_and_gradient(sim, circ, theta, terms, range(nq))
        dt = (time.perf_counter() - t0) / a.steps
        rec = {"seconds_per_gradient": dt, "energy": e}
        if prec == "c128":
            h = 1e-4
            # central finite differences on every parameter, energies through the public path
            fsim = Simulator(1, precision="c128", fusion="staged")
            for q in range(nq):
                fsim.allocate_qubit(q)
            zero = np.zeros(1 << nq, dtype=np.complex128)
            zero[0] = 1.0
            pin = pin_host(zero)
            e_pub = public_energy(fsim, circ, theta, terms, zero)
            idx = (np.arange(circ.nparams) if a.fd_params == 0
                   else np.linspace(0, circ.nparams - 1, a.fd_params).astype(int))
            t0 = time.perf_counter()
            fd = np.empty(idx.size)
            for i, j in enumerate(idx):
                tp, tm = theta.copy(), theta.copy()
                tp[j] += h
                tm[j] -= h
                fd[i] = (public_energy(fsim, circ, tp, terms, zero) - public_energy(fsim, circ, tm, terms, zero)) / (2 * h)
            fd_seconds = time.perf_counter() - t0
            pin.close()
            fsim.close()
            err = np.abs(g[idx] - fd)
            scale = max(1.0, float(np.max(np.abs(fd))))
            rec["finite_differences"] = {
                "h": h, "parameters_checked": int(idx.size), "energies": int(2 * idx.size),
                "energy_path": "set_wavefunction + apply_gates + run + get_expectation_value (stage planner)",
                "fd_all_max_rel_err": float(np.max(err)) / scale, "max_abs_err": float(np.max(err)),
                "median_abs_err": float(np.median(err)), "max_abs_fd": float(np.max(np.abs(fd))),
                "seconds": fd_seconds, "energy_public_path_minus_adjoint": e_pub - e}
            # parameter shift (exact for exp(-i theta P / 2)): (E(t + pi/2) - E(t - pi/2)) / 2
            pidx = np.linspace(0, circ.nparams - 1, 8).astype(int)
            ps = []
            for j in pidx:
                tp, tm = theta.copy(), theta.copy()
                tp[j] += np.pi / 2
                tm[j] -= np.pi / 2
                ps.append((energy_and_gradient(sim, circ, tp, terms, range(nq))[0]
                           - energy_and_gradient(sim, circ, tm, terms, range(nq))[0]) / 2)
            rec["param_shift_max_abs_err"] = float(np.max(np.abs(g[pidx] - np.array(ps))))
            # the energy on the CPU reference engine (FP64, its own fusion)
            kind = "reference engine (simulator.hpp)" if ref_api() is not None else "oracle port"
            cpu = make("ref" if ref_api() is not None else "oracle", seed=1)
            for q in range(nq):
                cpu.allocate_qubit(q)
            t0 = time.perf_counter()
            apply_circuit(cpu, circ.gates(theta))
            e_cpu = cpu.get_expectation_value(terms, list(range(nq)))
            cpu.close()
            rec["energy_vs_cpu_reference"] = {"reference": kind, "energy": e_cpu, "abs_err": abs(e - e_cpu),
                                              "seconds": time.perf_counter() - t0}
            g128, e128 = g, e
        else:
            rec["max_abs_diff_vs_c128"] = float(np.max(np.abs(g - g128)))
            rec["energy_abs_diff_vs_c128"] = abs(e - e128)
            rec["energy_abs_err_vs_cpu_reference"] = abs(e - out["c128"]["energy_vs_cpu_reference"]["energy"])
            # a batch of 16 parameter sets, 4 each of 4, 8, 12 and 20 layers
            rng = np.random.default_rng(1)
            batch = []
            for layers in (4, 8, 12, 20):
                c = hardware_efficient_ansatz(nq, layers)
                for _ in range(4):
                    batch.append((c, rng.uniform(-np.pi, np.pi, size=c.nparams)))
            t0 = time.perf_counter()
            for c, th in batch:
                energy_and_gradient(sim, c, th, terms, range(nq))
            rec["batch16_seconds"] = time.perf_counter() - t0
            rec["batch16_parameters"] = int(sum(c.nparams for c, _ in batch))
        sim.close()
        out[prec] = rec
    print(json.dumps(out), flush=True)


def run_learned(a):
    """Learned fusion planner on a stream of random circuits (qubits uniform
    in 20..32 complex64, depth 10..200, the gate mix of
    costmodel.random_circuit, 10% ending with the time evolution of a 50-term
    Pauli Hamiltonian, on states of up to 30 qubits): host wall time with the shipped cost model against the greedy
    fixed-size fusion and the stage planner, the evolution method the learned
    planner chose for each tail, and 1 - F of the learned result against the
    greedy one;
    then the same comparison on block-local circuits (26-30 qubits), where the
    model's own tensor-core clusters compete with the stage plan."""
    from projectq_gb300 import costmodel

    shipped = costmodel.load()
    res = costmodel.evaluate(shipped["params"], shipped["regimes_c64"], ncirc=a.ngates, seed=11)
    choices, tails = {}, {}
    for r in res["rows"]:
        choices[r["choice"]] = choices.get(r["choice"], 0) + 1
        if r.get("tail"):
            tails[r["tail_method"]] = tails.get(r["tail_method"], 0) + 1
    rows = res.pop("rows")
    tail_rows = [r for r in rows if r.get("tail")]
    res["time_evolution"] = {
        "learned_methods": tails,
        "greedy_s": sum(r["greedy_s"] - r["greedy_gates_s"] for r in tail_rows),
        "learned_s": sum(r["learned_s"] - r["learned_gates_s"] for r in tail_rows),
        "staged_s": sum(r["staged_s"] - r["staged_gates_s"] for r in tail_rows) if tail_rows and "staged_s" in tail_rows[0]
        else None}
    blk = costmodel.evaluate_blocked(shipped["params"], shipped["regimes_c64"])
    blk_rows = blk.pop("rows")

    def rnd(r):
        return {k: (round(v, 5) if isinstance(v, float) else v) for k, v in r.items()}

    print(json.dumps({"workload": "learned fusion planner vs greedy fixed-size fusion", **res, "choices": choices,
                      "per_circuit": [rnd(r) for r in rows],
                      "local_block_circuits": {**rnd(blk), "per_circuit": [rnd(r) for r in blk_rows]}}), flush=True)


def run_evolution(a):
    """Time evolution of commuting Hamiltonians through emulate_time_evolution:
    p = 4 QAOA-style layers (a ring Ising cost Hamiltonian, 2n + 1 terms, then
    the transverse mixer sum_i X_i, n terms) from |+>^n.  The exact product of
    the terms' exponentials (the default) at 30 qubits in both precisions, and
    against the Taylor series (complex128) at 24 qubits with the fidelity
    between the two."""
    from projectq_gb300 import Simulator

    def ising(n, rng):
        terms = [([], 0.7)]
        for i in range(n):
            terms.append(([(i, "Z"), ((i + 1) % n, "Z")] if i + 1 < n else [(0, "Z"), (i, "Z")],
                          float(rng.uniform(0.5, 1.5))))
            terms.append(([(i, "Z")], float(rng.uniform(-1, 1))))
        return terms

    had = np.array([[1, 1], [1, -1]]) / np.sqrt(2)

    def qaoa(sim, n, mode, layers=4):
        rng = np.random.default_rng(0)
        cost, mixer = ising(n, rng), [([(i, "X")], 1.0) for i in range(n)]
        sim.set_time_evolution(mode)
        for q in range(n):
            sim.apply_controlled_gate(had, [q], [])
        sim.run()
        sim.synchronize()
        sim.reset_counters()
        t0 = time.perf_counter()
        for layer in range(layers):
            sim.emulate_time_evolution(cost, 0.3 + 0.1 * layer, list(range(n)), [])
            sim.emulate_time_evolution(mixer, 0.5 - 0.1 * layer, list(range(n)), [])
        sim.synchronize()
        return (time.perf_counter() - t0) / (2 * layers), sim.counters()

    def engine(n, prec):
        sim = Simulator(1, precision=prec, fusion="staged")
        for q in range(n):
            sim.allocate_qubit(q)
        return sim

    out = {"workload": "QAOA-style time evolution, commuting Hamiltonians", "layers": 4}
    nq = a.qubits
    for prec in ("c64", "c128"):
        sim = engine(nq, prec)
        for _ in range(max(1, a.warmup)):
            qaoa(sim, nq, "exact", layers=1)
        dt, c = qaoa(sim, nq, "exact")
        out[f"exact_{prec}_{nq}q"] = {"seconds_per_evolution": dt, "gate_passes": c["gate_passes"],
                                      "terms_per_layer": 3 * nq + 1}
        sim.close()
    n2 = min(24, nq)
    res = {}
    for mode in ("exact", "taylor"):
        sim = engine(n2, "c128")
        qaoa(sim, n2, mode, layers=1)
        dt, c = qaoa(sim, n2, mode)
        res[mode] = (dt, sim.cheat()[1])
        out[f"{mode}_c128_{n2}q"] = {"seconds_per_evolution": dt, "gate_passes": c["gate_passes"]}
        sim.close()
    a_, b_ = res["exact"][1], res["taylor"][1]
    out[f"speedup_exact_vs_taylor_{n2}q"] = res["taylor"][0] / res["exact"][0]
    out[f"one_minus_fidelity_exact_vs_taylor_{n2}q"] = float(
        1 - abs(np.vdot(b_, a_)) ** 2 / (np.vdot(a_, a_).real * np.vdot(b_, b_).real))
    # a non-commuting 50-term random Pauli Hamiltonian (the learned-planner
    # workload's time evolution): Taylor series against the Chebyshev expansion
    from projectq_gb300.workloads import random_pauli_hamiltonian

    ham = [(tuple(t), c) for t, c in random_pauli_hamiltonian(n2, nterms=50, seed=7)]
    res = {}
    for mode in ("taylor", "chebyshev"):
        sim = engine(n2, "c128")
        sim.set_time_evolution(mode)
        for q in range(n2):
            sim.apply_controlled_gate(had, [q], [])
        sim.run()
        sim.synchronize()
        t0 = time.perf_counter()
        sim.emulate_time_evolution(ham, 0.5, list(range(n2)), [])
        sim.synchronize()
        res[mode] = (time.perf_counter() - t0, sim.cheat()[1])
        sim.close()
    a_, b_ = res["chebyshev"][1], res["taylor"][1]
    out[f"noncommuting_50_terms_{n2}q"] = {
        "t": 0.5, "sum_abs_coeffs": float(sum(abs(c) for t, c in ham if t)),
        "taylor_seconds": res["taylor"][0], "chebyshev_seconds": res["chebyshev"][0],
        "speedup": res["taylor"][0] / res["chebyshev"][0],
        "max_abs_diff": float(np.max(np.abs(a_ - b_)))}
    print(json.dumps(out), flush=True)


def main():
    a = parse()
    set_omp_env()
    if a.impl == "reference":
        run_reference(a)
        return
    if a.only:
        run_only(a)
        return
    if a.workload != "circuit":
        {"fused": run_fused, "adjoint": run_adjoint, "learned": run_learned, "gates": run_gates,
         "evolution": run_evolution}[a.workload](a)
        return
    dist, world, rank, local = dist_init()
    from projectq_gb300 import Simulator
    from projectq_gb300.simulator import pin_host, set_device
    from projectq_gb300.workloads import random_gate_circuit, random_state

    set_device(local)
    nq = a.qubits
    gates = random_gate_circuit(nq, a.depth, a.per_layer, seed=0)
    G = len(gates)
    psi0 = random_state(nq, seed=0, dtype=np.complex64)
    h2d_bytes = int(psi0.nbytes)
    ids = list(range(nq))

    # --- accuracy: one circuit from psi0 on both precisions ------------------
    s64 = Simulator(1, precision="c64", fusion=a.fusion)
    s64.set_stage_kernel(a.stage_kernel)
    for q in ids:
        s64.allocate_qubit(q)
    s64.set_wavefunction(psi0, ids)
    s128 = Simulator(1, precision="c128", fusion=a.fusion)
    for q in ids:
        s128.allocate_qubit(q)
    s128.set_wavefunction(psi0.astype(np.complex128), ids)
    apply_circuit(s64, gates)
    apply_circuit(s128, gates)
    ip, maxerr = s128.compare(s64)
    n128 = s128.compare(s128)[0].real
    n64 = s64.compare(s64)[0].real
    one_minus_f = 1.0 - abs(ip) ** 2 / (n128 * n64)

    # --- timed: complex64 ------------------------------------------------------
    with ClockSampler(local) as clk:
        ms64, cnt64, recs = timed_steps(s64, gates, a.steps, a.warmup, dist)
    ms64 = allreduce_max(dist, ms64)
    key, groups = dominant_kernel(recs)
    # --- timed: complex128 -----------------------------------------------------
    k128 = a.c128_steps if a.c128_steps is not None else max(1, min(a.steps, 5))
    ms128, cnt128, _ = timed_steps(s128, gates, k128, max(1, min(a.warmup, 3)), dist, profile_kernel=False)
    ms128 = allreduce_max(dist, ms128)
    del s128

    # --- e2e through the Python API, host buffers ------------------------------
    pin = pin_host(psi0)
    e2e_times = []
    zz = [([(0, "Z"), (1, "Z")], 1.0), ([(5, "X"), (6, "X")], 1.0)]
    e2e_sim = s64
    phases = []
    for i in range(a.e2e_steps + 1):
        e2e_sim.synchronize()
        t0 = time.perf_counter()
        e2e_sim.set_wavefunction(psi0, ids)
        t1 = time.perf_counter()
        apply_circuit(e2e_sim, gates)
        t2 = time.perf_counter()
        ev = e2e_sim.get_expectation_value(zz, ids)
        bits = e2e_sim.measure_qubits(ids)
        t3 = time.perf_counter()
        dt = t3 - t0
        if i > 0:  # the first call pays one-time host page-locking costs
            e2e_times.append(dt)
            phases.append((t1 - t0, t2 - t1, t3 - t2))
    pin.close()
    e2e = allreduce_max(dist, statistics.median(e2e_times))

    # --- CPU legs (rank 0, N = 1 only): baseline, and accuracy at check size -
    cpu = None
    vs_ref = None
    if rank == 0 and world == 1 and not a.no_cpu:
        del psi0, pin
        s64.close()
        try:
            cpu = cpu_baseline(gates, cpu_nq(nq), a.cpu_gates)
        except Exception as exc:  # pragma: no cover - host memory
            cpu = {"value": None, "unit": "gates/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {exc}"}
        if a.check_qubits:
            vs_ref = accuracy_vs_reference(a.check_qubits, a.depth, a.per_layer, a.fusion)

    if rank != 0:
        return
    peak, peak_src = measured_peak()
    kern = {}
    for r in recs:  # per kernel (kind, precision), all widths together
        kg = kern.setdefault((r["kind"], r["precision"]), {"launches": 0, "ms": 0.0, "bytes": 0})
        kg["launches"] += 1
        kg["ms"] += r["ms"]
        kg["bytes"] += r["bytes"]
    roofline = None
    if kern:
        kkey = max(kern, key=lambda k: kern[k]["ms"])
        g = kern[kkey]
        avg_bytes = g["bytes"] / g["launches"]
        avg_ms = g["ms"] / g["launches"]
        achieved = avg_bytes / (avg_ms * 1e-3) / 1e9
        per_amp = NCU_TRAFFIC_PER_AMP.get((kkey[0], kkey[1]))
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "traffic": per_amp * 2 ** nq if per_amp else None,
                    "traffic_source": NCU_TRAFFIC_SOURCE if per_amp else None, "peak_source": peak_src,
                    "kernel": {"kind": KERNEL_KINDS[kkey[0]], "precision": "c64" if kkey[1] == 1 else "c128",
                               "launches": g["launches"], "bytes_per_launch": avg_bytes, "ms_per_launch": avg_ms,
                               "share": g["ms"] / max(1e-9, sum(x["ms"] for x in kern.values()))},
                    "gates_per_launch": G * a.steps / max(1, g["launches"]),
                    "note": "achieved = algorithmic bytes per launch / mean per-launch CUDA-event time; a stage "
                            "launch applies gates_per_launch gates in one pass over the state"}
    value = world * G * a.steps / (ms64 * 1e-3)
    v128 = world * G * k128 / (ms128 * 1e-3)
    out = {
        "metric": METRIC, "value": value, "unit": "gates/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms64 / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": {"workload": f"random circuit, {nq} qubits, depth {a.depth}, {a.per_layer} gates/layer "
                               f"({G} gates), complex64 state (FP64 reductions) vs complex128",
                   "qubits": nq, "gates_per_step": G, "fusion": a.fusion,
                   "l2": "inputs larger than L2 (state 8 GiB c64 / 16 GiB c128); no flush",
                   "parallelism": f"replicas x{world}"},
        "hbm_gbs": cnt64["gate_bytes"] / (ms64 * 1e-3) / 1e9,
        "c128": {"value": v128, "unit": "gates/s", "ms_per_step": ms128 / k128, "steps": k128,
                 "hbm_gbs": cnt128["gate_bytes"] / (ms128 * 1e-3) / 1e9},
        "c64_over_c128": value / v128,
        "accuracy": {"one_minus_fidelity": one_minus_f, "max_abs_err": maxerr, "reference": "engine c128 path",
                     "vs_reference": vs_ref},
        "e2e": {"value": world * G / e2e, "unit": "gates/s", "h2d_bytes_per_step": h2d_bytes,
                "d2h_bytes_per_step": 8 + nq, "seconds_per_step": e2e,
                "phase_seconds_median": {k: statistics.median(p[j] for p in phases)
                                         for j, k in enumerate(("upload", "submit_and_launch", "device_expectation_measure"))},
                "path": "Simulator.set_wavefunction (pinned host c64) + apply_controlled_gate per gate + run "
                        "+ get_expectation_value + measure_qubits"},
        "gpu_launches": cnt64["gate_launches"],
        "passes_per_step": cnt64["gate_passes"] / a.steps,
        "roofline": roofline,
        "cpu_baseline": cpu and {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "clocks": clk.summary(),
        "kernel_groups": {f"kind{k[0]}_k{k[1]}_p{k[2]}": v for k, v in groups.items()},
        "expectation_z0z1_x5x6": ev, "measured": int(sum(b << i for i, b in enumerate(bits))),
    }
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
