"""bench.py --impl reference on the CPU: the reference arm times the oracle
(the FP64 restatement of the reference) on a whole step of the workload and
prints one JSON line with the contract's keys; under torchrun only rank 0
runs and prints, the other ranks exit 0 without work."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run(env_extra, *args):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args],
                          capture_output=True, text=True, env=env, timeout=900, cwd=ROOT)


def test_reference_arm_json_line():
    r = run({}, "--steps", "1", "--warmup", "0")
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "config",
              "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and "whole" in cb["sample"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert abs(line["e2e"]["value"] - line["value"]) < 1e-9


def test_reference_arm_other_ranks_exit_quietly():
    r = run({"RANK": "1", "WORLD_SIZE": "2"}, "--steps", "1", "--warmup", "0")
    assert r.returncode == 0 and r.stdout.strip() == ""
