"""bench.py's reference arm runs on the host cores only (the FP64 oracle
port), so its output line is checked here without a GPU: one JSON line with
the keys the benchmark line carries, and no output from ranks other than 0."""

import json
import os
import subprocess
import sys

from conftest import ROOT

ARGS = ["--impl", "reference", "--steps", "2", "--warmup", "3", "--ref-points", "2"]


def _run(env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *ARGS], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_one_contract_line():
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["steps"] == 2 and line["warmup"] == 3 and line["n_gpus"] == 1
    assert line["higher_is_better"] is True and line["vs_baseline"] is None
    assert line["config"]["workload"] == "tof13-64x64x48"
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["unit"] == line["unit"] and cb["sample"].startswith("2 of the workload's 3270 scatter points")
    assert cb["statistic"] == "mean over steps"
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
