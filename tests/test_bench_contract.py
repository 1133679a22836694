"""The benchmark's reference arm on CPU: its one JSON line and the keys a reader of it needs.

The reference arm times the reference's CPU Monte-Carlo (the oracle, a bit-exact restatement
of its node graph) on the host cores, so it runs here without a GPU; the GPU arm is covered
by the GPU tests and the benchmark run itself.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(*args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, env=e,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_one_line_with_the_contract_keys():
    p = run_bench("--impl", "reference", "--steps", "2", "--warmup", "1", "--cpu-sample-paths", "1024")
    assert p.returncode == 0, p.stderr
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["metric"] == "path-steps/sec" and line["unit"] == "path-steps/s"
    assert line["higher_is_better"] is True and line["steps"] == 2 and line["warmup"] == 1
    assert line["config"]["workload"] == "heston_vanilla_grid" and line["config"]["paths"] == 1 << 20
    assert line["value"] > 0 and line["ms_per_step"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == (os.cpu_count() or 1) and cb["value"] == line["value"]
    assert "1024 paths" in cb["sample"]
    assert cb["one_core"]["cores"] == 1 and cb["one_core"]["value"] > 0
    e = line["e2e"]
    assert e["value"] == line["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_runs_on_rank_zero_only():
    p = run_bench("--impl", "reference", "--steps", "1", "--warmup", "0", "--cpu-sample-paths", "1024",
                  env={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""
