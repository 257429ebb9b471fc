"""`bench.py --impl reference` on the CPU: the reference arm's JSON line and
its isolation from the package.

The arm times the oracle's restatement of QCalculator::calQ inside BKW3D's
RK4 step (BKW.h:480-510) on the host's cores.  It must load nothing of this
build (no import of the package, so no libedb.so), and its line must carry the
same metric and unit as the GPU arm, a `cpu_baseline` describing the run, and
an `e2e` with zero host-device bytes.  One RK4 step over one solve per host
thread, no warm-up: a few seconds here.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import json, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"]
import bench
rc = bench.main()
loaded = sorted(m for m in sys.modules if m.startswith("entropydecreaseboltzmann_gb300"))
print("ARM_RESULT " + json.dumps({"rc": rc, "loaded": loaded,
                                  "metric": bench.METRIC, "unit": bench.UNIT}))
"""


def test_reference_arm_line_and_isolation():
    env = dict(os.environ)
    env.pop("RANK", None)
    env.pop("WORLD_SIZE", None)
    p = subprocess.run([sys.executable, "-c", SCRIPT], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    line = json.loads(lines[0])
    res = json.loads(next(ln for ln in p.stdout.splitlines()
                          if ln.startswith("ARM_RESULT "))[len("ARM_RESULT "):])
    assert res["rc"] in (0, None)
    assert res["loaded"] == [], res["loaded"]  # nothing of this build was imported
    assert line["impl"] == "reference"
    assert line["metric"] == res["metric"] and line["unit"] == res["unit"]
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] == 0
    assert line["ms_per_step"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert cb["value"] == line["value"] and cb["unit"] == line["unit"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert "workload" in line["config"]
