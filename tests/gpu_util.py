"""Shared helpers of the GPU tests: run the CUDA library and the oracle on the same case."""
from __future__ import annotations

import json
import os

import numpy as np

import mbcg
import oracle_lib as ol

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load_fixture(name):
    z = np.load(os.path.join(GOLD, f"{name}.npz"))
    meta = json.loads(str(z["params"]))
    p = mbcg.default_params()
    for k, v in meta.items():
        if isinstance(v, list):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(p, k, v)
    return p, z


def written_nodes(p: mbcg.Params):
    """Index of the nodes a step writes: fluid nodes plus, on an inlet/outlet axis, the
    ghost layers (with interior transverse coordinates)."""
    sl = []
    for a, n in zip((2, 1, 0), (p.nz, p.ny, p.nx)):
        sl.append(slice(0, n) if p.bc[a] == mbcg.BC_INOUT else slice(1, n - 1))
    return (slice(None),) + tuple(sl)


def field_errors(got: np.ndarray, ref: np.ndarray, idx=None):
    if idx is not None:
        got, ref = got[idx], ref[idx]
    return [ol.rel_l2(got[f], ref[f]) for f in range(11)]


GROUPS = {"rhor": [0], "rhob": [1], "u": [2, 3, 4], "Pi": [5, 6, 7, 8, 9, 10]}


def group_errors(got: np.ndarray, ref: np.ndarray, idx=None) -> dict:
    """Relative L2 error per moment group: each colour density, the velocity vector field
    and the non-equilibrium stress tensor field (components pooled, so a component that is
    identically zero in the reference does not make the metric ill-conditioned)."""
    if idx is not None:
        got, ref = got[idx], ref[idx]
    return {k: ol.rel_l2(got[v], ref[v]) for k, v in GROUPS.items()}


def assert_fp32_parity(got: np.ndarray, ref64: np.ndarray, ref32: np.ndarray, idx, gate: float = 1e-5,
                       slack: float = 3.0, what: str = ""):
    """The CUDA result must be within `gate` relative L2 of the FP64 oracle, or at least as
    close to it as the reference's FP32 arithmetic is (times `slack`), for every group."""
    eg = group_errors(got, ref64, idx)
    er = group_errors(ref32, ref64, idx)
    for k in GROUPS:
        lim = max(gate, slack * er[k])
        assert eg[k] <= lim, f"{what} {k}: gpu-vs-fp64 {eg[k]:.3e} > {lim:.3e} (fp32-vs-fp64 {er[k]:.3e})"
    return eg, er


def gpu_run(p: mbcg.Params, state: np.ndarray, nsteps: int, env=None) -> np.ndarray:
    old = {}
    for k, v in (env or {}).items():
        old[k] = os.environ.get(k)
        os.environ[k] = v
    try:
        with mbcg.Case(p) as c:
            c.copy_in(state.astype(np.float32))
            c.step(nsteps)
            return c.copy_out()
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def gpu_from_ic(p: mbcg.Params, nsteps: int) -> np.ndarray:
    with mbcg.Case(p) as c:
        c.init()
        c.step(nsteps)
        return c.copy_out()
