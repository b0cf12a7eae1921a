"""The reference's own CUDA kernels (kernels.cu, unmodified, compiled for sm_103a into
oracle/_ref/*.cubin by __graft_entry__.build() where the reference sources are mounted) run on
the GPU beside this library.

* parity: the reference's RCSKernel + JetBoundaryConditions from the golden jet fixture's
  initial state agree with the reference's host build (the fixture) and with libmbcg.so;
* timing: the reference kernel on the 256 x 1024 x 256 jet and at the bubble's and the Rayleigh-Taylor
  case's sizes, beside this library on the same lattices (printed; run with -s).

Skipped when the cubins are absent (the reference sources are not available everywhere).
"""
import ctypes
import os

import numpy as np
import pytest

import mbcg
import oracle_lib as ol
from gpu_util import group_errors, load_fixture, written_nodes

pytestmark = pytest.mark.gpu
REF = os.path.join(ol.ORACLE_DIR, "_ref")
RCS = b"_Z9RCSKernel13MomentsDeviceS_"
JBC = b"_Z21JetBoundaryConditions13MomentsDeviceS_"


class RefKernels:
    """RCSKernel / JetBoundaryConditions of one reference configuration, via the driver API."""

    def __init__(self, cubin: str, dims):
        import torch
        torch.zeros(1, device="cuda")
        self.torch = torch
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.mod = ctypes.c_void_p()
        self._ck(self.cu.cuModuleLoad(ctypes.byref(self.mod), cubin.encode()), "cuModuleLoad")
        self.rcs, self.jbc = ctypes.c_void_p(), ctypes.c_void_p()
        self._ck(self.cu.cuModuleGetFunction(ctypes.byref(self.rcs), self.mod, RCS), "RCSKernel")
        self._ck(self.cu.cuModuleGetFunction(ctypes.byref(self.jbc), self.mod, JBC), "JetBoundaryConditions")
        self.NX, self.NY, self.NZ = dims

    @staticmethod
    def _ck(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: CUDA driver error {rc}")

    def state(self, host: np.ndarray):
        return [self.torch.from_numpy(np.ascontiguousarray(host[f]).ravel()).cuda() for f in range(11)]

    @staticmethod
    def struct(fields):
        return (ctypes.c_void_p * 11)(*[t.data_ptr() for t in fields])

    def step(self, a, b):
        """main.cu:41-45 without the swap: RCSKernel(A, B), JetBoundaryConditions(B, A)."""
        sa, sb = self.struct(a), self.struct(b)
        kp = (ctypes.c_void_p * 2)(ctypes.addressof(sa), ctypes.addressof(sb))
        # block 32x4x2 (compile.sh:34-36), grid ceil(N / block) (utilities/cudaConfig.cuh:34-43)
        self._ck(self.cu.cuLaunchKernel(self.rcs, (self.NX + 31) // 32, (self.NY + 3) // 4, (self.NZ + 1) // 2,
                                        32, 4, 2, 0, None, kp, None), "RCSKernel launch")
        kb = (ctypes.c_void_p * 2)(ctypes.addressof(sb), ctypes.addressof(sa))
        # 2-D x/z launch (utilities/cudaConfig.cuh:48-61)
        self._ck(self.cu.cuLaunchKernel(self.jbc, (self.NX + 31) // 32, (self.NZ + 3) // 4, 1, 32, 4, 1, 0, None,
                                        kb, None), "JetBoundaryConditions launch")

    def host(self, fields):
        self.torch.cuda.synchronize()
        return np.stack([t.cpu().numpy().reshape(self.NZ, self.NY, self.NX) for t in fields])


def _cubin(tag):
    path = os.path.join(REF, f"ref_{tag}.cubin")
    if not os.path.exists(path):
        pytest.skip(f"reference cubin {path} not built here (reference sources absent)")
    return path


@pytest.mark.parametrize("q", [27, 19])
def test_reference_cuda_matches_host_build_and_library(q):
    p, z = load_fixture(f"ref_jet_q{q}")
    k = RefKernels(_cubin(f"jet_q{q}"), (p.nx, p.ny, p.nz))
    a, b = k.state(z["init"]), k.state(z["init"])
    idx = written_nodes(p)
    with mbcg.Case(p) as c:
        c.copy_in(z["init"])
        done = 0
        for n in (1, 10, 100):
            for _ in range(n - done):
                k.step(a, b)
                a, b = b, a
            c.step(n - done)
            done = n
            ref_gpu = k.host(a)
            ours = c.copy_out()
            e_host = group_errors(ref_gpu, z[f"step{n}"], idx)   # reference CUDA vs reference host
            e_ours = group_errors(ours, ref_gpu, idx)             # this library vs reference CUDA
            assert e_host["rhor"] < 1e-5 and e_host["rhob"] < 1e-5, (n, e_host)
            assert e_ours["rhor"] < 1e-5 and e_ours["rhob"] < 1e-5, (n, e_ours)


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
