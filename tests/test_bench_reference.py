"""bench.py --impl reference on the host (no GPU): the reference arm times the
reference's shaders compiled for the host, loads only the oracle's
libraries (never the product library), and reports the GPU arm's metric and
workload config with no host-device traffic."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_runs_the_compiled_reference_only():
    if not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libasuna_ref.so")):
        pytest.skip("the reference's shaders are not built here (oracle/build_oracle.py)")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1", "--ref-budget", "4", "--ref-seconds", "2"],
                         cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([l for l in out.stdout.splitlines() if l.startswith("{")][-1])
    assert line["impl"] == "reference" and line["metric"] == "Mrays/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "reference" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["libraries"] and all(p.startswith("oracle/") for p in line["libraries"])
    assert not any("libasuna_rt" in p for p in line["libraries"])
    # the GPU arm reports the same workload config (its launch choices go in "run")
    sys.path.insert(0, ROOT)
    import bench

    shot = type("Shot", (), {"width": 1920, "height": 1080})()
    assert line["config"] == bench.workload_config(shot)
    assert line["config"]["triangles"] == 20971526 and "run" not in line
