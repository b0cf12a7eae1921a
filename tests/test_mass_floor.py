"""The phase-mass floor of FP32 state storage on the 64^3 D3Q19 bubble (conservative Omega2),
10^4 steps: the FP64 oracle's arithmetic with the state rounded to FP32 after every step.  This
separates what FP32 storage costs from what FP32 arithmetic costs (the GPU's phase drift,
tests/test_gpu_diagnostics.py).  Measured on 6 host threads (about 27 min): red +6.9e-7,
blue +8.6e-8.  Opt-in: MBCG_LONG=1.
"""
import os

import numpy as np
import pytest

import mbcg
import oracle_lib as ol

pytestmark = pytest.mark.skipif(not os.environ.get("MBCG_LONG"), reason="opt-in (MBCG_LONG=1): ~30 min of host time")


def test_fp32_storage_mass_floor():
    p = mbcg.bubble_params(64, q=19, conservative=True)
    a = ol.oracle_init(p, np.float64).astype(np.float32).astype(np.float64)
    m0 = [a[f, 1:-1, 1:-1, 1:-1].sum() for f in (0, 1)]
    b = a.copy()
    for n in range(10000):
        ol.oracle_step(p, a, n + 1, b=b)
        a, b = b, a
        a[...] = a.astype(np.float32)  # FP32 storage
    drift = [(a[f, 1:-1, 1:-1, 1:-1].sum() - m0[f]) / m0[f] for f in (0, 1)]
    print(f"\nFP32-storage floor over 10^4 steps: red {drift[0]:+.3e}, blue {drift[1]:+.3e}")
    assert abs(drift[0]) < 1e-6 and abs(drift[1]) < 1e-6
