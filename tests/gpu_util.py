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
