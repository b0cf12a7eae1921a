"""The reference's own CUDA kernels (kernels.cu, unmodified, compiled for sm_103a into
oracle/_ref/*.cubin by __graft_entry__.build() where the reference sources are mounted; the
cubins travel with the working tree to the GPU) run on the GPU beside this library, from the
same initial state, for every moment group (each colour density, the velocity field and the
stress field):

* the jet fixture's small lattice at steps 1, 10, 100, also against the reference's host build;
* the jet configuration's physics (tau 0.51, sigma 1e-3, beta 0.7, inlet radius 16, u 0.05) on a
  64 x 128 x 64 fluid box at step 100, also against the FP64 oracle;
* the full jet lattice, 256 x 1024 x 256 fluid nodes (258 x 1026 x 258, jet along y), at step 100;
* timing: the reference kernel on the 256 x 1024 x 256 jet and at the bubble's and the
  Rayleigh-Taylor case's sizes, beside this library on the same lattices (printed; run with -s).

Gate (relative L2 per group): 1e-5, or, for a group where the reference's own FP32 CUDA result
is further than 1e-5 from the FP64 oracle (the stress field: Pi = A - rho/3 - rho u u cancels
most of the digits of the second moment A), 3x that distance.  This library must then be within
the gate both of the reference's CUDA result and of the FP64 oracle.

A missing cubin fails the test (it is never skipped on a GPU).
"""
import ctypes
import os

import numpy as np
import pytest

import mbcg
import oracle_lib as ol
from gpu_util import GROUPS, group_errors, load_fixture, written_nodes
from ref_cuda import REF, RefKernels

pytestmark = pytest.mark.gpu


def _cubin(tag):
    path = os.path.join(REF, f"ref_{tag}.cubin")
    if not os.path.exists(path):
        pytest.fail(f"reference cubin {path} missing: run __graft_entry__.build() where the reference "
                    f"sources are mounted (MBCG_REF_ROOT) and ship oracle/_ref with the tree")
    return path


GATE = 1e-5


def gates_from(e_ref_vs_fp64: dict) -> dict:
    """Per-group gate: 1e-5, or 3x the reference CUDA build's own distance from the FP64 oracle."""
    return {k: max(GATE, 3.0 * v) for k, v in e_ref_vs_fp64.items()}


def assert_within(e: dict, gate: dict, what: str):
    for k in ("rhor", "rhob", "u", "Pi"):
        assert e[k] <= gate[k], f"{what} {k}: {e[k]:.3e} > {gate[k]:.3e} (all: {e})"


@pytest.mark.parametrize("q", [27, 19])
def test_reference_cuda_matches_host_build_and_library(q):
    p, z = load_fixture(f"ref_jet_q{q}")
    k = RefKernels(_cubin(f"jet_q{q}"), (p.nx, p.ny, p.nz))
    a, b = k.state(z["init"]), k.state(z["init"])
    idx = written_nodes(p)
    o64 = z["init"].astype(np.float64)
    with mbcg.Case(p) as c:
        c.copy_in(z["init"])
        done = 0
        for n in (1, 10, 100):
            for _ in range(n - done):
                k.step(a, b)
                a, b = b, a
            c.step(n - done)
            o64 = ol.oracle_run(p, o64, n - done, first_step=done + 1)
            done = n
            ref_gpu = k.host(a)
            ours = c.copy_out()
            e_host = group_errors(ref_gpu, z[f"step{n}"], idx)   # reference CUDA vs reference host
            gate = gates_from(group_errors(ref_gpu, o64, idx))    # reference CUDA vs FP64 oracle
            assert_within(e_host, gate, f"q{q} step {n} reference CUDA vs host build")
            assert_within(group_errors(ours, ref_gpu, idx), gate, f"q{q} step {n} library vs reference CUDA")
            assert_within(group_errors(ours, o64, idx), gate, f"q{q} step {n} library vs FP64 oracle")
            assert e_host["rhor"] < GATE and e_host["rhob"] < GATE, (n, e_host)


def _torch_group_errors(got, ref):
    """Relative L2 per group of two lists of 11 device tensors (float64 accumulation)."""
    import torch
    out = {}
    for name, fs in GROUPS.items():
        num = sum(float(torch.sum((got[f].double() - ref[f].double()) ** 2)) for f in fs)
        den = sum(float(torch.sum(ref[f].double() ** 2)) for f in fs)
        out[name] = (num ** 0.5) / (den ** 0.5) if den > 0 else num ** 0.5
    return out


def _run_pair(tag, p, steps):
    """The reference kernel and this library from the same initial state (this library's initial
    condition, copied into both), `steps` steps each; returns (reference, library) states on the
    host, restricted to the nodes a step writes."""
    k = RefKernels(_cubin(tag), (p.nx, p.ny, p.nz))
    with mbcg.Case(p) as c:
        c.init()
        init = c.copy_out()
        a, b = k.state(init), k.state(init)
        for _ in range(steps):
            k.step(a, b)
            a, b = b, a
        c.step(steps)
        ours = c.copy_out()
        assert c.status() == 0
    ref = k.host(a)
    del a, b
    return init, ref, ours


# the jet configuration's physics (reference semantics: jet along y, convective outlet, blue jet)
JET_PHYS = dict(q=27, tau=0.51, sigma=1e-3, beta=0.7, radius=16.0, velocity=0.05)


@pytest.fixture(scope="module")
def jet_physics_gate():
    """64 x 128 x 64 fluid nodes with the jet configuration's physics, 100 steps: the reference
    CUDA build against the FP64 oracle gives the per-group gate; this library must meet it against
    both."""
    p = mbcg.reference_jet_params(66, 130, 66, **JET_PHYS)
    init, ref, ours = _run_pair("jet66x130", p, 100)
    o64 = ol.oracle_run(p, init.astype(np.float64), 100)
    idx = written_nodes(p)
    e_ref = group_errors(ref, o64, idx)
    gate = gates_from(e_ref)
    e_ours = group_errors(ours, o64, idx)
    e_pair = group_errors(ours, ref, idx)
    print(f"\njet physics 64x128x64, 100 steps: reference CUDA vs FP64 {e_ref}\n  library vs FP64 {e_ours}"
          f"\n  library vs reference CUDA {e_pair}")
    return gate, e_ours, e_pair


def test_reference_cuda_jet_physics_reduced(jet_physics_gate):
    gate, e_ours, e_pair = jet_physics_gate
    assert_within(e_ours, gate, "jet physics 64x128x64: library vs FP64 oracle")
    assert_within(e_pair, gate, "jet physics 64x128x64: library vs reference CUDA")


def test_reference_cuda_jet_256x1024x256_100_steps():
    """The full jet lattice (258 x 1026 x 258, jet along y), 100 steps, every group, against the
    reference's CUDA build and the FP64 oracle.  Disturbances travel at most one node per step
    from the inlet (the ambient rest state is a fixed point, bit for bit), so after 100 steps the
    lattice beyond row 101 is still the initial state, and the FP64 oracle on a lattice cut at
    row 113 (258 x 114 x 258, its outlet still at rest at step 100) gives the FP64 result of the
    full lattice on rows 0..104, where the comparison with the oracle is made."""
    import torch
    p = mbcg.reference_jet_params(258, 1026, 258, **JET_PHYS)
    pc = mbcg.reference_jet_params(258, 114, 258, **JET_PHYS)
    k = RefKernels(_cubin("jet256"), (p.nx, p.ny, p.nz))
    with mbcg.Case(p) as c:
        c.init()
        init = c.copy_out()
        a, b = k.state(init), k.state(init)
        for _ in range(100):
            k.step(a, b)
            a, b = b, a
        c.step(100)
        ours = c.copy_out()
        assert c.status() == 0
    ref = k.host(a)
    del a, b
    torch.cuda.empty_cache()
    # the cut lattice starts from the same state: the full lattice's first 114 rows (row 113, its
    # outlet ghost, is ambient rest like every row beyond the inlet)
    o64 = ol.oracle_run(pc, np.ascontiguousarray(init[:, :, :114, :]).astype(np.float64), 100)
    idx = (slice(None), slice(1, -1), slice(0, 105), slice(1, -1))  # periodic x / z fluid nodes, rows 0..104
    e_ref = group_errors(ref[idx], o64[idx])
    gate = gates_from(e_ref)
    e_ours = group_errors(ours[idx], o64[idx])
    e_pair = group_errors(ours, ref, written_nodes(p))
    moved = float(np.abs(ours[:, :, 110:-1, :] - init[:, :, 110:-1, :]).max())
    print(f"\njet 256x1024x256 step 100: reference CUDA vs FP64 {e_ref}\n  library vs FP64 {e_ours}"
          f"\n  library vs reference CUDA (whole lattice) {e_pair}\n  largest change beyond row 110: {moved:.3e}")
    assert e_ours["rhor"] <= GATE and e_ours["rhob"] <= GATE, e_ours
    assert_within(e_ours, gate, "jet 256x1024x256 step 100: library vs FP64 oracle")
    assert_within(e_pair, gate, "jet 256x1024x256 step 100: library vs reference CUDA")


REF_TIMING = {
    # tag: (lattice, q, steps) -- the jet (256 x 1024 x 256 fluid nodes), and the reference kernel at
    # the bubble's (64^3, D3Q19) and the Rayleigh-Taylor case's (128 x 512 x 128, D3Q27) sizes
    "jet256": ((258, 1026, 258), 27, 20),
    "box64_q19": ((66, 66, 66), 19, 200),
    "box128x512_q27": ((130, 514, 130), 27, 50),
}


@pytest.mark.parametrize("tag", sorted(REF_TIMING))
def test_reference_cuda_timing(tag):
    """Prints the reference kernel's MLUPS at each configuration's size and this library's on the
    same lattice (no assertion on speed)."""
    import torch
    (NX, NY, NZ), q, steps = REF_TIMING[tag]
    k = RefKernels(_cubin(tag), (NX, NY, NZ))
    p = mbcg.reference_jet_params(NX, NY, NZ, q=q, tau=0.51, sigma=1e-3, beta=0.7, radius=16.0)
    lib = mbcg.Library.get()
    a = [torch.zeros(NX * NY * NZ, device="cuda") for _ in range(11)]
    m = mbcg.moments_from_tensors(a, NX)
    lib.check(lib.mbcg_init_moments(ctypes.byref(p), ctypes.byref(m), None), "init")
    b = [t.clone() for t in a]
    for i in range(3):
        k.step(a, b)
        a, b = b, a
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for i in range(steps):
        k.step(a, b)
        a, b = b, a
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / steps
    nodes = (NX - 2) * (NY - 2) * (NZ - 2)
    mlups = nodes / ms / 1e3
    with mbcg.Case(p) as c:
        c.init()
        c.step(3)
        torch.cuda.synchronize()
        s.record()
        c.step(steps)
        e.record()
        torch.cuda.synchronize()
        ms_ours = s.elapsed_time(e) / steps
    print(f"\nreference RCSKernel + JetBoundaryConditions, {tag} ({NX - 2}x{NY - 2}x{NZ - 2} fluid nodes, D3Q{q}): "
          f"{ms:.3f} ms/step, {mlups:.0f} MLUPS; this library on the same lattice {nodes / ms_ours / 1e3:.0f} MLUPS")
    assert mlups > 0
