"""bench.py --impl reference on CPU: the reference arm times the CPU restatement of the iteration on
the host cores and prints one JSON line with the contract's keys (metric and unit as our arm, a
cpu_baseline describing the run, an e2e with no host-device copies)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config",
                          "siam_b10_nk3_16", "--steps", "1", "--warmup", "0"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["unit"] == "s/iteration" and line["higher_is_better"] is False
    assert line["value"] > 0 and line["steps"] == 1
    assert line["config"]["name"] == "siam_b10_nk3_16" and "SIAM" in line["config"]["workload"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "s/iteration", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
