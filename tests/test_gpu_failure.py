"""Failure reporting of the fused step, made without faulting the GPU.

* Bounded waits: every wait of the step for a staged plane gives up after a cycle limit and the
  tile drains its in-flight copies before it exits.  The parameter field wait_test_cycles makes
  the first wait of every tile wait on a barrier that nothing completes, with a short limit, so
  that the wait runs out: the call returns and mbcg_status reports 1.  The real copies complete, so
  the drain completes and the context stays usable for the next case (in general a non-zero
  status marks the context as poisoned, because the drain is itself bounded).
* Non-finite states: a state seeded on the host with one node of zero (FP32) or negative (16-bit
  forms) density and one node
  with a NaN velocity is counted by the diagnostics (2 nodes), and one step carries the NaN into
  every destination of that node's populations (IEEE arithmetic: nothing in the step addresses
  memory by a field value, so a bad value spreads but never faults).
"""
import numpy as np
import pytest

import mbcg
import oracle_lib as ol
from gpu_util import assert_fp32_parity, written_nodes

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_reports():
    p = mbcg.reference_jet_params(34, 26, 22, q=27, tau=0.8, sigma=0.05, beta=0.7, radius=4.0)
    p.wait_test_cycles = 200000  # about 0.1 ms of SM clock per tile
    with mbcg.Case(p) as c:
        c.init()
        c.step(1)
        assert c.status() == 1  # a wait gave up (the tile drained its in-flight copies)
        assert c.status() == 0  # mbcg_status clears the word
    # the context is usable: the same case without the hook meets the parity gate
    p.wait_test_cycles = 0
    a0 = ol.oracle_init(p, np.float64)
    ref64 = ol.oracle_run(p, a0.copy(), 5)
    ref32 = ol.oracle_run(p, a0.astype(np.float32), 5)
    with mbcg.Case(p) as c:
        c.copy_in(a0.astype(np.float32))
        c.step(5)
        got = c.copy_out()
        assert c.status() == 0
    assert_fp32_parity(got, ref64, ref32, written_nodes(p), what="after a bounded-wait failure")


@pytest.mark.parametrize("precision", [mbcg.FP32, mbcg.FP16])
def test_bad_nodes_are_reported(precision):
    p = mbcg.bubble_params(16, q=19, radius=4.0, precision=precision)
    a = ol.oracle_init(p, np.float64).astype(np.float32)
    # one node with a non-physical density: zero in FP32; in the 16-bit forms the stored slot is the
    # scaled deviation from the nominal density, which decodes a zero density to ~1e-8 > 0, so a
    # negative density stands in for it there
    bad_rho = 0.0 if precision == mbcg.FP32 else -0.25
    a[0, 8, 7, 9] = bad_rho  # rhor and rhob
    a[1, 8, 7, 9] = bad_rho
    a[2, 4, 11, 5] = np.nan  # ux of another node
    with mbcg.Case(p) as c:
        c.copy_in(a)
        d0 = c.diagnostics()
        c.step(1)
        d1 = c.diagnostics()
        assert c.status() == 0  # no wait gave up: bad data is not a stall
    assert d0["nonfinite"] == 2, d0
    assert d1["nonfinite"] >= 19, d1  # the NaN node's 19 destinations (itself included)
