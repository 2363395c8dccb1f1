"""The reference arm of bench.py (`--impl reference`) for the load-time and query workloads: the
oracle's restatement timed on the host cores, one JSON line with the contract's keys and the
workload, metric and unit of the GPU arm.  Runs on the CPU (no GPU involved)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"}


def _line(config: int) -> dict:
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", str(config),
                        "--steps", "2", "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


@pytest.mark.parametrize("config, metric, unit, workload", [
    (7, "triangles_per_second", "triangles/s", "blas_build_atrium_249k_triangles"),
    (8, "poses_per_second", "poses/s", "pose_22_bones_65536_requests"),
])
def test_reference_arm_line(config, metric, unit, workload):
    d = _line(config)
    assert KEYS <= set(d), KEYS - set(d)
    assert d["impl"] == "reference" and d["metric"] == metric and d["unit"] == unit
    assert d["config"]["workload"] == workload
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 3 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert {"value", "unit", "cores", "kind", "sample"} <= set(cb) and cb["kind"] == "port" and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
