"""include/mbcg_operators.cuh (the reference's lattice and operator surface with run-time
parameters) against the reference's own headers: tests/cpp/ops_eval.cpp evaluates every operator
and case functor on seeded inputs, compiled once against the reference (the golden outputs in
tests/golden/ref_ops_q{27,19}.npz, made by tests/golden/make_golden.py) and here against this
library's header.  FP32, no multiply-add contraction on either side: bit-exact."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def build(tmp_path, q):
    exe = os.path.join(str(tmp_path), f"ops_eval_q{q}")
    cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", f"-I{os.path.join(ROOT, 'include')}",
           os.path.join(ROOT, "tests", "cpp", "ops_eval.cpp"), "-o", exe]
    if q == 19:
        cmd.insert(1, "-DMBCG_D3Q19")
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.parametrize("q", [27, 19])
def test_operators_match_the_reference_headers(tmp_path, q):
    z = np.load(os.path.join(GOLD, f"ref_ops_q{q}.npz"))
    meta = json.loads(str(z["params"]))
    exe = build(tmp_path, q)
    fi, fo = os.path.join(str(tmp_path), "in.raw"), os.path.join(str(tmp_path), "out.raw")
    z["inputs"].astype(np.float32).tofile(fi)
    args = [str(meta[k]) for k in ("nx", "ny", "nz", "tau", "sigma", "beta", "jet_radius", "jet_velocity",
                                   "bubble_radius", "rti_amplitude", "rti_width", "q")]
    subprocess.run([exe, fi, fo] + args, check=True)
    got = np.fromfile(fo, dtype=np.float32)
    ref = z["outputs"]
    assert got.shape == ref.shape
    bad = np.flatnonzero(got.view(np.uint32) != ref.view(np.uint32))
    assert bad.size == 0, f"{bad.size} values differ, first at {bad[:8]}: {got[bad[:4]]} vs {ref[bad[:4]]}"


def test_operators_compile_for_the_gpu(tmp_path):
    """The header is __host__ __device__: a kernel using it compiles for sm_103a."""
    src = os.path.join(str(tmp_path), "k.cu")
    with open(src, "w") as f:
        f.write('#include "mbcg_operators.cuh"\n'
                "using namespace mbcg::ops;\n"
                "__global__ void k(float* out, OpParams<float> p) {\n"
                "  float s = 0.f;\n"
                "  constexpr_for<0, LbmStencil::q>([&](auto I) {\n"
                "    constexpr label_t i = decltype(I)::value;\n"
                "    s += fpost<i>(1.f, 0.01f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, p);\n"
                "  });\n"
                "  constexpr_for<0, D3Q19::q>([&](auto I) {\n"
                "    s += Omega2<decltype(I)::value, D3Q19>(0.1f, 0.f, 0.f, 0.1f, 0.01f);\n"
                "  });\n"
                "  out[threadIdx.x] = s;\n"
                "}\n")
    nvcc = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "--expt-relaxed-constexpr",
                    f"-I{os.path.join(ROOT, 'include')}", "-c", src, "-o", src + ".o"], check=True)


def test_operator_invariants(tmp_path):
    """tests/cpp/invariants.cpp, in FP64 for D3Q27 and D3Q19: the weights sum to 1 and B to 1/3;
    sum_i w_i cos2rule_i = cs^2 (cos2rule omits 1/|c_i|^2); Omega2 has zero sum and zero first
    moment above |F| = 1e-4; the recolouring terms cancel over c_i and -c_i."""
    exe = os.path.join(str(tmp_path), "invariants")
    subprocess.run(["g++", "-std=c++20", "-O2", f"-I{os.path.join(ROOT, 'include')}",
                    os.path.join(ROOT, "tests", "cpp", "invariants.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout
