"""bench.py --impl reference: the CPU arm runs without a GPU, so its JSON
line is checked here against the keys the benchmark contract names."""
from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def run_bench(*args: str, env_extra: dict | None = None) -> subprocess.CompletedProcess:
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, "bench.py", *args], cwd=ROOT, env=env, capture_output=True, text=True,
                          timeout=600)


def test_reference_arm_prints_one_contract_line(oracle):
    done = run_bench("--impl", "reference", "--steps", "1", "--warmup", "0")
    assert done.returncode == 0, done.stderr[-2000:]
    lines = [line for line in done.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    out = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e", "gpu_launches"):
        assert key in out, key
    assert out["impl"] == "reference" and out["value"] > 0 and out["steps"] == 1
    assert out["higher_is_better"] is True and out["gpu_launches"] == 0
    assert out["config"]["workload"] == "dam_break_1m" and out["config"]["particles"] == 1 << 20
    base = out["cpu_baseline"]
    assert base["kind"] == "port" and base["cores"] >= 1 and base["value"] == out["value"]
    assert out["e2e"] == {"value": out["value"], "unit": out["unit"], "h2d_bytes_per_step": 0,
                          "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    done = run_bench("--impl", "reference", "--steps", "1", "--warmup", "0",
                     env_extra={"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert done.returncode == 0, done.stderr[-2000:]
    assert not [line for line in done.stdout.splitlines() if line.startswith("{")]
