"""bench.py's reference arm (the CPU restatement of the reference's search on a bounded sample)
prints one JSON line with the keys the benchmark contract asks for.  No GPU needed."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_one_contract_line():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
           "--warmup", "1", "--cpu-scale", "0.005", "--cpu-seconds", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT, timeout=600, check=True)
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout
    out = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in out, key
    assert out["impl"] == "reference" and out["unit"] == "reads/s" and out["value"] > 0
    assert out["config"]["workload"] == "250Mbp_L100_20x_t55" and out["config"]["index"] == "U64"
    cb = out["cpu_baseline"]
    assert set(cb) >= {"value", "unit", "cores", "kind", "sample"} and cb["kind"] == "port"
    assert cb["value"] == out["value"] and cb["cores"] >= 1
    assert out["e2e"] == {"value": out["value"], "unit": "reads/s", "h2d_bytes_per_step": 0,
                          "d2h_bytes_per_step": 0}
