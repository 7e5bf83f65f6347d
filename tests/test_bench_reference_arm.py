"""The benchmark's reference arm on the CPU: it times the CPU restatement of
the reference on the named workload, prints the contract's JSON line (with
its cpu_baseline and e2e blocks), and maps nothing of the engine: no
liblbm_gb300.so in the process.  No GPU is needed."""

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

DRIVER = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--workload", "box64_p16_f64",
            "--steps", "2", "--warmup", "1"]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("ENGINE_MAPPED=" + str("liblbm_gb300" in maps))
"""


def test_reference_arm_line_and_isolation(oracle_mod):
    r = subprocess.run([sys.executable, "-c", DRIVER], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert lines[-1] == "ENGINE_MAPPED=False"
    line = json.loads(lines[-2])
    assert line["impl"] == "reference" and line["metric"] == "MLUPS" and line["value"] > 0
    assert line["steps"] == 2 and line["config"]["workload"] == "box64_p16_f64"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
