"""bench.py's reference arm on the CPU: the JSON line's contract.

`bench.py --impl reference` times the oracle (the C restatement of the
reference step) on the host cores and prints one JSON line with the same
metric, unit and config as the GPU arm; under a multi-rank launch only rank 0
works and prints.  Run on the 32^3 dam break so it stays short (its sampling
budget is 10 s).
"""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--workload", "dam32",
                        "--steps", "1", "--warmup", "1"], cwd=REPO, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_reference_arm_line():
    lines = _run({"RANK": "0", "WORLD_SIZE": "1"})
    assert len(lines) == 1
    d = json.loads(lines[0])
    import bench
    assert d["metric"] == bench.METRIC and d["impl"] == "reference"
    assert d["unit"] == "steps/s" and d["higher_is_better"] is True and d["value"] > 0
    assert abs(d["ms_per_step"] - 1000.0 / d["value"]) < 1e-6 * d["ms_per_step"]
    assert d["steps"] == 1 and d["warmup"] == 1 and d["n_gpus"] == 1 and d["vs_baseline"] is None
    assert d["config"]["workload"] == "dam32" and d["config"]["grid"] == [32, 32, 32]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert isinstance(cb["sample"], str) and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_nonzero_rank_is_silent():
    assert _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}) == []
