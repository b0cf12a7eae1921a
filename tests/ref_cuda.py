"""The reference's own CUDA kernels, RCSKernel and JetBoundaryConditions (kernels.cu:102-131,
unmodified, compiled for sm_103a into oracle/_ref/ref_<tag>.cubin by oracle/Makefile `cubin`
with one configuration's constants), launched through the CUDA driver API on torch tensors.

Test and baseline infrastructure: the parity tests run it beside the library, and bench.py
times it as the reference CUDA baseline.  Nothing in the library uses it.
"""
import ctypes
import os

import numpy as np

import oracle_lib as ol

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




def cubin_path(tag: str) -> str:
    return os.path.join(REF, f"ref_{tag}.cubin")
