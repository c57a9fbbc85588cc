"""bench.py's reference arm on CPU: the oracle port of validate.cu's step on
host threads, printing the contract's JSON line, without loading the
product library."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
import sys, json, io, contextlib
sys.argv = ["bench.py", "--impl", "reference", "--scale", "12", "--steps", "3", "--warmup", "1",
            "--ref-threads", "2"]
import bench
buf = io.StringIO()
with contextlib.redirect_stdout(buf):
    rc = bench.main()
maps = open("/proc/self/maps").read()
print(json.dumps({"rc": rc, "line": buf.getvalue().strip().splitlines()[-1],
                  "libmg": "libmg.so" in maps, "pkg": "multigraph_gb300" in sys.modules}))
"""


def test_reference_arm_line_and_no_product_library():
    out = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    res = json.loads(out.stdout.strip().splitlines()[-1])
    assert res["rc"] == 0
    assert not res["libmg"] and not res["pkg"]
    line = json.loads(res["line"])
    assert line["impl"] == "reference" and line["metric"] == "GTEPS" and line["value"] > 0
    assert line["steps"] == 4 and line["cpu_baseline"]["cores"] == 2   # 3 steps over 2 threads: 2 each
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["ne"] > 0 and line["higher_is_better"] is True
