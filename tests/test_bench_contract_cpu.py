"""bench.py's reference arm on the CPU, at a small size: one JSON line with the
keys the benchmark contract names (metric, value, unit, steps, warmup,
higher_is_better, scaling, dtype, data, config, cpu_baseline, e2e with zero
copy bytes, impl = "reference"), timed on the reference engine built from its
own sources with setup.py's flags where that build exists (else the oracle
port); and a rank other than 0 prints nothing."""

import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _run(extra_env=None):
    env = dict(os.environ)
    env.update(extra_env or {})
    cmd = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--qubits", "14", "--steps", "1",
           "--warmup", "3", "--ref-gates", "8"]
    return subprocess.run(cmd, cwd=str(ROOT), env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_json_line():
    res = _run()
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["steps"] == 1 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["value"] > 0 and d["unit"] == "gates/s"
    want = "reference" if (ROOT / "oracle" / "_ref" / "libref_sim_setup.so").exists() else "port"
    assert d["cpu_baseline"]["kind"] == want and d["cpu_baseline"]["value"] == d["value"]
    assert set(d["modes"]) == {"per_gate_run", "gate_fusion"}
    assert d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "gates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["qubits"] == 14


def test_reference_arm_other_ranks_print_nothing():
    res = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert res.returncode == 0, res.stderr[-2000:]
    assert res.stdout.strip() == ""
