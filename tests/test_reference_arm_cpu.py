"""The reference arm of bench.py (the CPU restatement of the reference's hot
path) run for real on a small workload: one JSON line with the contract's
keys, the same metric as the GPU arm, and no part of libsu2g loaded."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--D", "120", "--nspin1", "2", "--steps", "2", "--warmup", "1"]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit as e:
    assert not e.code, e.code
print("LOADED_LIBSU2G", "libsu2g" in open("/proc/self/maps").read())
"""


def test_reference_arm_line_without_libsu2g():
    r = subprocess.run([sys.executable, "-c", SCRIPT], cwd=REPO, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["metric"].startswith("H_eff*psi TFLOP/s")
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["same_config"] is True
    assert "LOADED_LIBSU2G False" in r.stdout
