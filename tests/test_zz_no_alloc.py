"""The allocation-free diagnostics entry point, mbcg_diagnostics_static().

It exists for callers that cannot allocate device memory where they need conservation numbers
(every byte reserved for resident states, or a framework allocator owning the GPU), so it keeps
its partial sums in a fixed array inside the library.  Checked through the C ABI against the
case-handle entry point mbcg_diagnostics(), on two calls in a row with the state changing in
between (the shared array must not carry anything from the previous call).  This file is named
to be collected last.
"""
import ctypes

import numpy as np
import pytest

import mbcg

pytestmark = pytest.mark.gpu


def _static_diag(lib, params, view):
    d = mbcg.Diag()
    rc = lib.mbcg_diagnostics_static(ctypes.byref(params), ctypes.byref(view), ctypes.byref(d), None)
    lib.check(rc, "mbcg_diagnostics_static")
    return d.as_dict()


def _close(a, b):
    for k in ("mass_r", "mass_b", "p_in", "p_out", "dp"):
        assert abs(a[k] - b[k]) <= 1e-12 * (abs(b[k]) + 1e-30) + 1e-14, (k, a[k], b[k])
    for i in range(3):
        scale = abs(a["mass_r"]) + abs(a["mass_b"])
        assert abs(a["momentum"][i] - b["momentum"][i]) <= 1e-12 * scale, ("momentum", i)
    assert a["nonfinite"] == b["nonfinite"] and a["nodes"] == b["nodes"]


@pytest.mark.parametrize("precision", [mbcg.FP32, mbcg.FP16, mbcg.BF16])
def test_static_diagnostics_match_case_diagnostics(precision):
    lib = mbcg.Library.get()
    p = mbcg.bubble_params(40, q=27, radius=10.0, precision=precision)
    with mbcg.Case(p) as c:
        c.init()
        c.step(5)
        for call in range(2):
            a, _ = c.fields()
            got = _static_diag(lib, c.params, a)
            want = c.diagnostics()
            _close(got, want)
            assert got["nodes"] == p.active_nodes() and got["mass_r"] > 0
            c.step(7)  # change the state between the two calls


def test_static_diagnostics_reject_oversized_lattice():
    lib = mbcg.Library.get()
    p = mbcg.jet_params(512, 512, 1024)          # 268M fluid nodes, above the fixed capacity
    view = mbcg.Moments()
    for i in range(mbcg.NFIELDS):
        view.f[i] = 256 * (i + 1)                # never dereferenced: rejected before any launch
    view.pitch = p.nx
    view.precision = p.precision
    d = mbcg.Diag()
    rc = lib.mbcg_diagnostics_static(ctypes.byref(p), ctypes.byref(view), ctypes.byref(d), None)
    assert rc != 0
    assert b"at most" in lib.mbcg_last_error()
