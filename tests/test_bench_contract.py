"""bench.py's JSON contract, checked on its reference arm (the oracle on the
host cores, no GPU): one JSON line with the metric, unit and direction of
the GPU arm, a positive value, the CPU-baseline description and an e2e
object with no host-device copies."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "histories/s" and d["higher_is_better"] is True
    assert d["metric"].startswith("histories/s")
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] >= 3
    assert d["n_gpus"] == 1 and d["dtype"] == "f64"
    assert "workload" in d["config"] and "lattice" in d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert "sample" in cb
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
