"""bench.py's one-line JSON contract, through its reference arm (the OpenMP
C++ restatement of the step on the host cores, which runs without a GPU) on
the small cantilever workload: the keys, their types and the values the
reference arm fixes (impl, zero host-device bytes, its cpu_baseline)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_reference_arm(*extra):
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--workload", "cantilever", "--steps", "2",
           "--warmup", "1", *extra]
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_prints_the_contract_line():
    d = run_reference_arm()
    assert d["impl"] == "reference"
    assert isinstance(d["metric"], str) and d["metric"]
    assert d["unit"] == "steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert abs(d["value"] - 1000.0 / d["ms_per_step"]) <= 1e-6 * d["value"]
    assert d["n_gpus"] == 1 and d["steps"] == 2 and d["warmup"] == 1
    assert d["scaling"] in ("weak", "strong")
    assert d["vs_baseline"] is None
    assert d["dtype"] == "f32" and d["data"] == "synthetic"
    assert d["config"]["workload"].startswith("cantilever")
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["cores"] >= 1 and cb["kind"] in ("port", "reference") and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
