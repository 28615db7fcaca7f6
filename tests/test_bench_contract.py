"""bench.py's reference arm on the CPU: one JSON line with the keys the
measurement contract names (the GPU arm is exercised on a GPU)."""

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e")


# the horizon case runs on a 64^3 volume: the find's cost does not depend on it
@pytest.mark.parametrize("workload,extra", [("teukolsky", []), ("puncture", []), ("puncture_axi", []),
                                            ("horizon", ["--n", "64"])])
def test_reference_arm_line(workload, extra):
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", workload, "--steps", "1",
                          "--warmup", "1", *extra], cwd=ROOT, capture_output=True, text=True, timeout=600,
                         check=True)
    lines = [line for line in out.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in KEYS:
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["higher_is_better"] is True and d["dtype"] == "f64"
    assert "workload" in d["config"]
    cpu = d["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["cores"] >= 1 and cpu["value"] == d["value"] and cpu["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
