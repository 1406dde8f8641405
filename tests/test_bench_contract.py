"""The JSON line of bench.py's reference arm (the oracle on the host cores,
no GPU needed) for every path carries the keys of the benchmark contract."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config")


def run(*extra):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "2", "--warmup", "1", *extra],
                         capture_output=True, text=True, check=True, timeout=600, cwd=ROOT)
    return json.loads(out.stdout.strip().splitlines()[-1])


def check(line):
    for k in KEYS:
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert set(("value", "unit", "sample")) <= set(cb)
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_headline():
    """The default sediment arm: the reference algorithm over the headline's
    window (a column sample of the 2048 x 2048 workload, brought to the
    window's start day untimed)."""
    line = run("--start-day", "0.25", "--ref-columns", "24")
    check(line)
    assert line["unit"] == "column-steps/s"
    cfg = line["config"]
    assert cfg["workload"] == "surrogate_2048x2048" and cfg["columns"] == 2936778
    assert cfg["simulated_days_timed"] == "0.250..0.333"
    assert "of 2936778 active columns" in line["cpu_baseline"]["sample"]


def test_reference_arm_sediment_plain():
    line = run("--solver", "plain", "--cpu-columns", "32")
    check(line)
    assert line["unit"] == "column-steps/s" and line["config"]["workload"] == "plain_gpu_256x256"
    # the host beside the all-core figure, and the same window on one core
    cb = line["cpu_baseline"]
    assert cb["host"]["nproc"] >= 1 and cb["host"]["machine"]
    assert cb["one_core"]["value"] > 0 and cb["one_core"]["unit"] == "column-steps/s"


def test_reference_arm_pelagic():
    line = run("--path", "pelagic", "--pel-cpu-columns", "256")
    check(line)
    assert line["unit"] == "column-runs/s" and line["config"]["model"] == "gotm_npzd"


def test_reference_arm_coupling():
    line = run("--path", "coupling", "--cpl-cpu-seconds", "0.5")
    check(line)
    assert line["unit"] == "columns/s" and line["config"]["mode"] == "CPL_AS_RUN"
    assert line["config"]["columns"] == 1024 * 1024
