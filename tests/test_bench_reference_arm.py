"""`bench.py --impl reference` (the reference's host path restated by the oracle) runs without a
GPU: it prints one JSON line with the default arm's metric, unit and workload, a cpu_baseline
describing the run and an e2e object with no host-device copies, and libtt.so never loads in its
process. It builds the full 2M-triangle terrain, so this test takes about half a minute."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

_RUN = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit as e:
    if e.code not in (0, None):
        raise
print("LIBTT_LOADED" if "libtt.so" in open("/proc/self/maps").read() else "LIBTT_ABSENT")
"""


def test_reference_arm_runs_on_the_host_alone():
    pr = subprocess.run([sys.executable, "-c", _RUN], capture_output=True, text=True, timeout=900, cwd=ROOT,
                        env={**os.environ, "PYTHONPATH": str(ROOT)})
    assert pr.returncode == 0, pr.stderr[-3000:]
    lines = pr.stdout.strip().splitlines()
    assert lines[-1] == "LIBTT_ABSENT"
    line = json.loads([l for l in lines if l.startswith("{")][-1])
    sys.path.insert(0, str(ROOT))
    import bench
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["higher_is_better"] is True and line["value"] > 0 and line["steps"] == 1 and line["warmup"] >= 3
    assert "2,097,152 tris" in line["config"]["workload"]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"] and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
