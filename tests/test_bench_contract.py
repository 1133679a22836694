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
    p = run_bench("--impl", "reference", "--steps", "2", "--warmup", "1", "--paths", "1024")
    assert p.returncode == 0, p.stderr
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["metric"] == "path-steps/sec" and line["unit"] == "path-steps/s"
    assert line["higher_is_better"] is True and line["steps"] == 2 and line["warmup"] == 1
    assert line["config"]["workload"] == "heston_vanilla_grid" and line["config"]["paths"] == 1024
    assert line["value"] > 0 and line["ms_per_step"] > 0
    # the timed steps are the whole workload: ms_per_step is what the timed region took per step
    assert line["steps"] * line["ms_per_step"] <= 1e3 * line["wall_s_timed_region"] * 1.001
    assert abs(line["value"] - 1024 * 504 / (line["ms_per_step"] * 1e-3)) <= 1e-6 * line["value"]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == (os.cpu_count() or 1) and cb["value"] == line["value"]
    assert "1024 paths" in cb["sample"]
    assert cb["one_core"]["cores"] == 1 and cb["one_core"]["value"] > 0
    e = line["e2e"]
    assert e["value"] == line["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_runs_on_rank_zero_only():
    p = run_bench("--impl", "reference", "--steps", "1", "--warmup", "0", "--paths", "1024",
                  env={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""


def test_clock_summary_counts_samples_from_the_mark_and_reports_throttling():
    """The bench's clocks record: nvidia-smi CSV samples from the start of the timed region,
    median SM clock, and every throttle reason seen active."""
    sys.path.insert(0, ROOT)
    import bench
    c = bench.Clocks(0)
    c.lines = ["0, 1200, 2070, 300.0, 0x0, Not Active, Not Active, Not Active, Not Active",  # before the region
               "0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active",
               "0, 2055, 2070, 1100.2, 0x4, Not Active, Not Active, Not Active, Active",
               "not a sample"]
    s = c.summary(since=1)
    assert s["samples"] == 2 and s["sm_mhz"] == 2062.5 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    assert c.summary()["sm_mhz"] == 2055.0                      # the idle sample counts without a mark
    c.lines.append("0, 1900, 2070, 1300.0, 0x40, Not Active, Active, Not Active, Not Active")
    assert c.summary(since=1)["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert bench.Clocks(0).summary()["reasons"] == ["unsampled"]
