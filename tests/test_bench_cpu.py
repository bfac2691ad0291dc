"""bench.py's reference arm on the CPU: it times the reference's CPU step
(the reference compiled in place where its sources are present, else the
oracle's C restatement) and must not load the CUDA library, so that its
numbers are independent of the code under test.  Run in a fresh process:
the other CPU tests load libfipi_gb300.so into this one."""
import json
import subprocess
import sys
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent

_PROBE = r"""
import contextlib, io, json, runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--workload", "t16", "--steps", "2", "--warmup", "3"]
out = io.StringIO()
with contextlib.redirect_stdout(out):
    try:
        runpy.run_path("bench.py", run_name="__main__")
    except SystemExit as e:
        if e.code not in (0, None):
            raise
with open("/proc/self/maps") as f:
    maps = f.read()
print(json.dumps({"lines": out.getvalue().strip().splitlines(), "cuda_library_loaded": "libfipi_gb300" in maps}))
"""


def test_reference_arm_loads_no_cuda_library():
    r = subprocess.run([sys.executable, "-c", _PROBE], cwd=REPO, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert not res["cuda_library_loaded"]
    line = json.loads(res["lines"][-1])
    assert line["impl"] == "reference"
    assert line["unit"] == "steps/s" and line["value"] > 0
    assert line["config"]["workload"] == "t16"
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
