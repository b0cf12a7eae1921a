"""Generate the golden fixtures in this folder from the reference itself.

Run where the reference sources are mounted (they are compiled, unmodified, into host
shared objects by oracle/Makefile `shim`; see oracle/ref_shim.cpp):

    python tests/golden/make_golden.py

Each fixture is an .npz with the case parameters (JSON), the input state and the
reference's output states, all in the reference's dense layout (11, nz, ny, nx).  The
fixtures pin both the CPU oracle (tests/test_oracle_golden.py) and the CUDA library
(tests/test_gpu_parity.py) on machines where the reference is absent.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle_lib as ol  # noqa: E402
import mbcg  # noqa: E402


def random_mixed_state(p: mbcg.Params, seed: int, dtype) -> np.ndarray:
    """Seeded state with both colours everywhere (every node is an interface node),
    non-zero velocity and non-equilibrium moments: exercises every term of the step."""
    rng = np.random.default_rng(seed)
    s = np.zeros((11,) + p.shape)
    s[0] = rng.uniform(0.05, 1.0, p.shape)
    s[1] = rng.uniform(0.05, 1.0, p.shape)
    s[2:5] = rng.uniform(-0.05, 0.05, (3,) + p.shape)
    s[5:11] = rng.uniform(-2e-3, 2e-3, (6,) + p.shape)
    return s.astype(dtype)


def save(name: str, p: mbcg.Params, **arrays):
    meta = json.dumps(p.describe())
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, params=np.array(meta), **arrays)
    print("wrote", path, {k: v.shape for k, v in arrays.items()})


def jet_fixture(q: int):
    """Reference jet case (jet along y) from its own initial condition: states at steps
    1, 10 and 100 of main.cu's loop."""
    p = mbcg.reference_jet_params(18, 14, 12, q=q, tau=0.8, sigma=0.05, beta=0.7, radius=3.0, velocity=0.05)
    sh = ol.Shim(f"golden_jet{q}", p, "float")
    a = sh.init("jet")
    out = {"init": a.copy()}
    cur = a.copy()
    nxt = a.copy()
    for n in range(1, 101):
        sh.lib.ref_step(ol._ptrs(cur), ol._ptrs(nxt), 1, 1)
        cur, nxt = nxt, cur
        if n in (1, 10, 100):
            out[f"step{n}"] = cur.copy()
    save(f"ref_jet_q{q}", p, **out)


def defaults_fixture():
    """The reference exactly as shipped (tau = 1, sigma = 0.1, beta = 0.9, jet radius 12,
    velocity 0.05, D3Q27) on a 32 x 24 x 32 lattice: 20 steps."""
    p = mbcg.reference_jet_params(32, 24, 32, q=27, tau=1.0, sigma=0.1, beta=0.9, radius=12.0)
    sh = ol.Shim("golden_defaults", p, "float")
    a = sh.init("jet")
    cur, nxt = a.copy(), a.copy()
    for _ in range(20):
        sh.lib.ref_step(ol._ptrs(cur), ol._ptrs(nxt), 1, 1)
        cur, nxt = nxt, cur
    save("ref_defaults_q27", p, init=a, step20=cur)


def random_fixture(q: int):
    """One RCS + boundary step from a random mixed state, in FP32 and in FP64."""
    p = mbcg.reference_jet_params(12, 10, 9, q=q, tau=0.7, sigma=0.05, beta=0.7, radius=3.0)
    out = {}
    for real, dt in (("float", np.float32), ("double", np.float64)):
        sh = ol.Shim(f"golden_rand{q}_{real}", p, real)
        a = random_mixed_state(p, 1000 + q, dt)
        out[f"in_{real}"] = a
        out[f"out_{real}"] = sh.step(a.copy(), 1, 1, b=a.copy())
        out[f"rcs_{real}"] = sh.step(a.copy(), 1, 0, b=a.copy())
    save(f"ref_random_q{q}", p, **out)


def ic_fixture():
    """Initial-condition functors of the bubble and RTI cases (bubbleIn.cuh, rtiIn.cuh)."""
    p = mbcg.reference_jet_params(20, 18, 16, q=27)
    p.bubble_radius = 5.0
    p.rti_amplitude = 2.0
    p.rti_width = 3.0
    sh = ol.Shim("golden_ic", p, "float")
    save("ref_ic", p, bubble=sh.init("bubble"), rti=sh.init("rti"))


def vti_state(p: mbcg.Params) -> np.ndarray:
    """Seeded FP32 state with values of many magnitudes and both signs, every one exactly
    representable (small integers times powers of two and a decimal scale, formed in float32);
    the periodic ghost layers of x and y hold the images of the opposite fluid layer, as the
    library keeps them."""
    rng = np.random.default_rng(77)
    s = np.zeros((11,) + p.shape, dtype=np.float32)
    scale = [np.float32(v) for v in (1.0, 1e-3, 1e-7, 3.5e2, 1e-20)]
    for f in range(11):
        ints = rng.integers(-100000, 100000, p.shape).astype(np.float32) * np.float32(2.0 ** -12)
        s[f] = ints * scale[f % len(scale)]
    s[:, :, :, 0] = s[:, :, :, p.nx - 2]
    s[:, :, :, p.nx - 1] = s[:, :, :, 1]
    s[:, :, 0, :] = s[:, :, p.ny - 2, :]
    s[:, :, p.ny - 1, :] = s[:, :, 1, :]
    return s


def vti_fixture():
    """The reference's own VTI writer (io/vtiWriter.cuh, write_vti) on a seeded state: the bytes
    the library's ASCII writer must reproduce."""
    import subprocess
    import tempfile
    p = mbcg.bubble_params(5, q=19)  # 7 x 7 x 7 lattice, periodic
    p.nx, p.ny, p.nz = 9, 7, 6
    p.ic = mbcg.IC_NONE
    s = vti_state(p)
    defs = " ".join(ol.shim_defs(p, "float"))
    subprocess.run(["make", "-s", "-C", ol.ORACLE_DIR, "vti", "TAG=golden", f"DEFS={defs}",
                    f"REF_ROOT={ol.REF_ROOT}"], check=True)
    with tempfile.TemporaryDirectory() as d:
        raw = os.path.join(d, "in.raw")
        s[0:5].astype(np.float32).tofile(raw)
        out = os.path.join(HERE, "ref_vti_ascii.vti")
        subprocess.run([os.path.join(ol.REF_DIR, "ref_vti_golden"), raw, out], check=True, capture_output=True)
    save("ref_vti_state", p, state=s)
    print("wrote", out)


OPS_LATTICE = dict(nx=9, ny=8, nz=7)


def ops_params(q: int) -> mbcg.Params:
    """The configuration the operator fixtures are evaluated at (a reference-expressible jet
    along y on a 9 x 8 x 7 lattice)."""
    p = mbcg.reference_jet_params(OPS_LATTICE["nx"], OPS_LATTICE["ny"], OPS_LATTICE["nz"], q=q, tau=0.8,
                                  sigma=0.05, beta=0.7, radius=2.0, velocity=0.05)
    p.bubble_radius = 2.5
    p.rti_amplitude = 1.0
    p.rti_width = 1.5
    return p


def ops_inputs(p: mbcg.Params, seed: int = 5) -> np.ndarray:
    """Seeded float32 inputs of tests/cpp/ops_eval.cpp: 32 samples of (rho, u, Pi, F, rhor, rhob),
    with the force vectors spanning both sides of the |F| = 1e-4 cut-off, then two lattice states."""
    rng = np.random.default_rng(seed)
    ns = 32
    smp = np.zeros((ns, 15))
    smp[:, 0] = rng.uniform(0.8, 1.2, ns)
    smp[:, 1:4] = rng.uniform(-0.06, 0.06, (ns, 3))
    smp[:, 4:10] = rng.uniform(-3e-3, 3e-3, (ns, 6))
    mag = 10.0 ** rng.uniform(-6, -1, ns)
    smp[:, 10:13] = rng.normal(size=(ns, 3)) * mag[:, None]
    smp[:, 13] = rng.uniform(0.0, 1.0, ns)
    smp[:, 14] = rng.uniform(0.0, 1.0, ns)
    smp[0, 13] = 0.0  # a pure blue node
    states = [random_mixed_state(p, seed + 1 + i, np.float32) for i in range(2)]
    return np.concatenate([smp.astype(np.float32).ravel()] + [s.ravel() for s in states])


def ops_fixture(q: int):
    """The reference's own operator headers evaluated by tests/cpp/ops_eval.cpp (-DOPS_REFERENCE)
    on seeded inputs: what include/mbcg_operators.cuh must reproduce bit for bit."""
    import subprocess
    import tempfile
    p = ops_params(q)
    inp = ops_inputs(p)
    tag = f"ops{q}"
    defs = " ".join(ol.shim_defs(p, "float"))
    subprocess.run(["make", "-s", "-C", ol.ORACLE_DIR, "ops", f"TAG={tag}", f"DEFS={defs}",
                    f"REF_ROOT={ol.REF_ROOT}"], check=True)
    with tempfile.TemporaryDirectory() as d:
        fi, fo = os.path.join(d, "in.raw"), os.path.join(d, "out.raw")
        inp.tofile(fi)
        subprocess.run([os.path.join(ol.REF_DIR, f"ops_ref_{tag}"), fi, fo], check=True)
        out = np.fromfile(fo, dtype=np.float32)
    save(f"ref_ops_q{q}", p, inputs=inp, outputs=out)


def main():
    if not ol.reference_available():
        raise SystemExit("reference sources not found; set MBCG_REF_ROOT")
    if len(sys.argv) > 1 and sys.argv[1] == "vti":
        vti_fixture()
        return
    if len(sys.argv) > 1 and sys.argv[1] == "ops":
        for q in (27, 19):
            ops_fixture(q)
        return
    for q in (27, 19):
        jet_fixture(q)
        random_fixture(q)
    defaults_fixture()
    ic_fixture()
    vti_fixture()
    for q in (27, 19):
        ops_fixture(q)


if __name__ == "__main__":
    main()
