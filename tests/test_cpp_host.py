"""The C++ host layer (include/mbcg_lbm.hpp): a driver using the reference's own host API names
compiles against the C ABI and gives the same fields as the Python case API."""
import json
import os
import subprocess

import numpy as np
import pytest

import mbcg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build_driver(tmp_path):
    exe = os.path.join(str(tmp_path), "drive")
    cmd = ["g++", "-std=c++17", "-O2", f"-I{os.path.join(ROOT, 'include')}", f"-I{CUDA}/include",
           os.path.join(ROOT, "tests", "cpp", "drive_reference_api.cpp"), "-o", exe,
           f"-L{os.path.dirname(mbcg.LIB_PATH)}", "-lmbcg", f"-Wl,-rpath,{os.path.dirname(mbcg.LIB_PATH)}",
           f"-L{CUDA}/lib64", "-lcudart"]
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.skipif(not os.path.exists(mbcg.LIB_PATH), reason="libmbcg.so not built")
def test_driver_compiles(tmp_path):
    assert os.path.exists(build_driver(tmp_path))


@pytest.mark.gpu
def test_reference_api_driver_matches_case_api(tmp_path):
    exe = build_driver(tmp_path)
    out = json.loads(subprocess.run([exe, "20"], check=True, capture_output=True, text=True).stdout)
    p = mbcg.reference_jet_params(34, 30, 26, q=27, tau=0.8, sigma=0.05, beta=0.7, radius=5.0)
    with mbcg.Case(p) as c:
        c.init()
        c.step(20)
        s = c.copy_out().astype(np.float64)
    sums = [s[f, 1:-1, :, 1:-1].sum() for f in range(11)]
    assert out["mlups"] > 0
    # The driver's split launches on the reference's dense layout run the plain-load kernel,
    # the case API the TMA kernel: separate compilations that may fuse different multiply-add
    # pairs, so per-field sums agree to FP32 round-off relative to the field's magnitude (sums
    # of the velocity fields cancel to ~1e-7 and carry no relative precision of their own).
    for a, b, m in zip(out["sums"], sums, out["abs_sums"]):
        assert abs(a - b) <= 1e-5 * m + 1e-12, (out["sums"], sums)


@pytest.mark.gpu
def test_jet_breakup_sampler_records_statistics(tmp_path):
    """JetBreakupSampler (include/mbcg_lbm.hpp) in the reference-style loop: one CSV row every 5
    steps from step 5, the injected jet attached to the inlet and advancing."""
    exe = build_driver(tmp_path)
    csv = os.path.join(str(tmp_path), "stats", "jet.csv")
    subprocess.run([exe, "40", csv], check=True, capture_output=True, text=True)
    rows = [line.split(",") for line in open(csv).read().strip().splitlines()]
    head, data = rows[0], rows[1:]
    assert head[:4] == ["step", "penetration", "regions", "detached"]
    steps = [int(r[0]) for r in data]
    assert steps == list(range(5, 41, 5))
    pen = [float(r[1]) for r in data]
    assert all(b >= a for a, b in zip(pen, pen[1:])) and pen[-1] > pen[0] >= 1
    for r in data:
        regions, detached, largest = int(r[2]), int(r[3]), int(r[5])
        assert regions >= 1 and 0 <= detached < regions and largest > 0
