"""Test-side access to the CPU oracle (oracle/mbcg_oracle.cpp) and, where the reference
sources are present, to the reference parity shims (oracle/ref_shim.cpp).

The oracle is the checker: it is loaded only by tests, __graft_entry__.smoke() and the
bench's CPU legs, never by the product path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "lightweight-mb-color-gradient-lbm_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)

import mbcg  # noqa: E402

ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "_build", "liboracle.so")
REF_DIR = os.path.join(ORACLE_DIR, "_ref")
# the reference checkout: MBCG_REF_ROOT, else a "reference" folder beside this repository
REF_ROOT = os.environ.get("MBCG_REF_ROOT", os.path.join(os.path.dirname(ROOT), "reference"))

_VP = ctypes.c_void_p
_oracle = None


def build_oracle() -> str:
    src = os.path.join(ORACLE_DIR, "mbcg_oracle.cpp")
    if not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    return ORACLE_SO


def oracle():
    global _oracle
    if _oracle is None:
        lib = ctypes.CDLL(build_oracle())
        lib.oracle_step.restype = ctypes.c_int
        lib.oracle_step.argtypes = [ctypes.POINTER(mbcg.Params), ctypes.c_int, _VP * 11, _VP * 11,
                                    ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.oracle_init.restype = ctypes.c_int
        lib.oracle_init.argtypes = [ctypes.POINTER(mbcg.Params), ctypes.c_int, _VP * 11]
        lib.oracle_noise.restype = ctypes.c_double
        lib.oracle_noise.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_uint64, ctypes.c_int]
        _oracle = lib
    return _oracle


def _ptrs(state: np.ndarray):
    assert state.flags["C_CONTIGUOUS"] and state.shape[0] == 11
    return (_VP * 11)(*[state[f].ctypes.data for f in range(11)])


def empty_state(p: mbcg.Params, dtype=np.float64) -> np.ndarray:
    return np.zeros((11,) + p.shape, dtype=dtype)


def oracle_init(p: mbcg.Params, dtype=np.float64) -> np.ndarray:
    s = empty_state(p, dtype)
    rc = oracle().oracle_init(ctypes.byref(p), s.itemsize, _ptrs(s))
    assert rc == 0
    return s


def oracle_step(p: mbcg.Params, a: np.ndarray, step: int, do_rcs=True, do_bc=True, threads=None,
                b: np.ndarray = None, reference_cost: bool = False) -> np.ndarray:
    """One step A -> B (B starts as a copy of A so ghost layers carry over, as the
    reference's ping-pong buffers do after the first steps).  reference_cost: recompute each
    source's colour gradient for every direction, as the reference does (same results; the
    timed CPU baseline), instead of once per node."""
    if b is None:
        b = a.copy()
    threads = threads or os.cpu_count() or 1
    rcs = (2 if reference_cost else 1) if do_rcs else 0
    rc = oracle().oracle_step(ctypes.byref(p), a.itemsize, _ptrs(a), _ptrs(b), int(step), rcs,
                              int(do_bc), int(threads))
    assert rc == 0
    return b


def oracle_run(p: mbcg.Params, a: np.ndarray, nsteps: int, first_step: int = 1, threads=None) -> np.ndarray:
    """nsteps steps with A/B ping-pong (main.cu:38-55); returns the final state."""
    b = a.copy()
    for n in range(nsteps):
        rc = oracle().oracle_step(ctypes.byref(p), a.itemsize, _ptrs(a), _ptrs(b), int(first_step + n), 1, 1,
                                  int(threads or os.cpu_count() or 1))
        assert rc == 0
        a, b = b, a
    return a


def oracle_noise(seed: int, step: int, node: int, comp: int) -> float:
    return oracle().oracle_noise(seed, step, node, comp)


# --------------------------------------------------------------------------- reference shims
def reference_available() -> bool:
    return os.path.exists(os.path.join(REF_ROOT, "lbm.cuh"))


def shim_defs(p: mbcg.Params, real: str = "float") -> list:
    """-D flags that compile the reference's constants for a reference-expressible case."""
    defs = [f"-DREF_NX={p.nx}", f"-DREF_NY={p.ny}", f"-DREF_NZ={p.nz}", f"-DREF_TAU={p.tau!r}",
            f"-DREF_SIGMA={p.sigma!r}", f"-DREF_BETA={p.beta!r}", f"-DREF_JET_RADIUS={p.jet_radius!r}",
            f"-DREF_JET_VELOCITY={p.jet_velocity!r}", f"-DREF_BUBBLE_RADIUS={p.bubble_radius!r}",
            f"-DREF_RTI_AMPLITUDE={p.rti_amplitude!r}", f"-DREF_RTI_WIDTH={p.rti_width!r}",
            f"-DREF_REAL={real}"]
    if p.q == 19:
        defs.append("-DLBM_D3Q19")
    return defs


def build_shim(tag: str, p: mbcg.Params, real: str = "float") -> str:
    out = os.path.join(REF_DIR, f"libref_{tag}.so")
    defs = " ".join(shim_defs(p, real))
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "shim", f"TAG={tag}", f"DEFS={defs}",
                    f"REF_ROOT={REF_ROOT}"], check=True)
    return out


class Shim:
    """The reference's own device functions compiled for the host (one configuration)."""

    def __init__(self, tag: str, p: mbcg.Params, real: str = "float"):
        self.p = p
        self.lib = ctypes.CDLL(build_shim(tag, p, real))
        self.dtype = np.float32 if real == "float" else np.float64
        for fn in ("ref_init_jet", "ref_init_bubble", "ref_init_rti"):
            getattr(self.lib, fn).argtypes = [_VP * 11]
            getattr(self.lib, fn).restype = None
        self.lib.ref_step.argtypes = [_VP * 11, _VP * 11, ctypes.c_int, ctypes.c_int]
        self.lib.ref_step.restype = None
        assert self.lib.ref_q() == p.q

    def init(self, kind: str) -> np.ndarray:
        s = np.zeros((11,) + self.p.shape, dtype=self.dtype)
        getattr(self.lib, f"ref_init_{kind}")(_ptrs(s))
        return s

    def step(self, a: np.ndarray, do_rcs=True, do_bc=True, b=None) -> np.ndarray:
        if b is None:
            b = a.copy()
        self.lib.ref_step(_ptrs(a), _ptrs(b), int(do_rcs), int(do_bc))
        return b

    def run(self, a: np.ndarray, nsteps: int) -> np.ndarray:
        b = a.copy()
        for _ in range(nsteps):
            self.lib.ref_step(_ptrs(a), _ptrs(b), 1, 1)
            a, b = b, a
        return a


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.linalg.norm(a - b)
    n = np.linalg.norm(b)
    return float(d / n) if n > 0 else float(d)


def fluid(state: np.ndarray) -> np.ndarray:
    """View of the fluid nodes (drop the ghost frame) of an (11, nz, ny, nx) state."""
    return state[:, 1:-1, 1:-1, 1:-1]
