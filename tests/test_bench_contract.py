"""The JSON line bench.py prints: every key of its contract, for the reference arm (host cores,
runs anywhere) and, on a GPU, for a reduced native run."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BASE_KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
             "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline"}


def run_bench(*args, timeout=900):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, capture_output=True,
                       text=True, timeout=timeout)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_line():
    d = run_bench("--impl", "reference", "--steps", "1", "--warmup", "3")
    assert d["impl"] == "reference"
    assert BASE_KEYS <= set(d)
    assert d["unit"] == "MLUPS" and d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert {"value", "unit", "cores", "kind", "sample"} <= set(cb)
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in d["config"]


@pytest.mark.gpu
def test_native_line_reduced():
    d = run_bench("--steps", "2", "--warmup", "3", "--no-cpu", "--forms", "", "--serving", "off", "--no-configs",
                  "--e2e-steps", "1", "--nz", "64")
    assert BASE_KEYS <= set(d) and "impl" not in d
    assert d["value"] > 0 and d["unit"] == "MLUPS" and d["scaling"] == "weak" and d["dtype"] == "f32"
    rf = d["roofline"]
    assert {"bound", "achieved", "peak", "unit", "frac", "traffic"} <= set(rf)
    assert rf["bound"] == "hbm" and rf["unit"] == "GB/s" and 0 < rf["frac"] == pytest.approx(rf["achieved"] / rf["peak"])
    e = d["e2e"]
    assert {"value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"} <= set(e)
    assert e["value"] > 0 and e["h2d_bytes_per_step"] == e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] == d["steps"]  # one fused launch per step
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= set(d["clocks"])
    assert d["checks"]["nonfinite"] == 0 and d["checks"]["status"] == 0
    assert "x64 " in d["config"]["workload"]


def test_serving_bound_arithmetic():
    """The cases/s ceiling of a request stream at the plain kernel's per-request times: the makespan
    of the best preemptive one-at-a-time schedule with those release times."""
    import bench
    reqs = [{"t": 0.0}, {"t": 1.0}, {"t": 2.0}]
    # work-bound: everything released early, 7 s of work
    b = bench.serving_bound(reqs, [5.0, 1.0, 1.0])
    assert abs(b["makespan_s"] - 7.0) < 1e-12 and abs(b["cases_per_s"] - 3 / 7.0) < 1e-12
    # release-bound: the last request arrives late, after the rest is done
    reqs2 = [{"t": 0.0}, {"t": 1.0}, {"t": 10.0}]
    b2 = bench.serving_bound(reqs2, [1.0, 1.0, 0.5])
    assert abs(b2["makespan_s"] - 10.5) < 1e-12
    # order of the list does not matter (sorted by release time)
    b3 = bench.serving_bound(list(reversed(reqs2)), [0.5, 1.0, 1.0])
    assert abs(b3["makespan_s"] - 10.5) < 1e-12
