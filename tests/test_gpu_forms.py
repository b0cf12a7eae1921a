"""FP16 / BF16 moment storage (scaled deviations, FP32 arithmetic) against the FP64 oracle on a
reduced jet with the jet configuration's physics (tau 0.51, sigma 1e-3, 1% inlet noise)."""
import os

import numpy as np
import pytest

import mbcg
import oracle_lib as ol
from gpu_util import assert_fp32_parity, group_errors, written_nodes

pytestmark = pytest.mark.gpu


def jet(precision):
    return mbcg.jet_params(48, 48, 96, q=27, diameter=16.0, precision=precision)


@pytest.fixture(scope="module")
def oracle_states():
    p = jet(mbcg.FP32)
    a = ol.oracle_init(p, np.float64)
    s100 = ol.oracle_run(p, a.copy(), 100)
    s1000 = ol.oracle_run(p, s100.copy(), 900, first_step=101)
    f100 = ol.oracle_run(p, a.astype(np.float32), 100)
    return p, a, s100, s1000, f100


def test_fp32_form_vs_fp64(oracle_states):
    p, a, s100, s1000, f100 = oracle_states
    with mbcg.Case(p) as c:
        c.copy_in(a.astype(np.float32))
        c.step(100)
        got = c.copy_out()
    assert_fp32_parity(got, s100, f100, written_nodes(p), what="fp32 jet")


# FP16 / BF16 bounds: what the scaled-deviation forms with stochastically rounded stores reach
# (relative L2 against the FP64 oracle, per colour density, velocity field and stress field;
# measured at 100 steps FP16 1.5e-4, 9.8e-6, 6.4e-4, 3.6e-3 and BF16 1.1e-3, 6.9e-5, 5.1e-3,
# 2.9e-2; at 1000 steps FP16 4.0e-4, 7.4e-5, 9.6e-4, 6.7e-3 and BF16 3.4e-3, 6.3e-4, 7.5e-3,
# 5.4e-2).  Rounded to nearest instead, the slowly changing jet is rounded the same way every
# step and the errors add up: FP16 rhor reached 1.05e-3 and BF16 rhor 3.7e-2 at 1000 steps.
# The FP16 target of 1e-3 holds for the densities and the velocity at 100 and 1000 steps; the
# stress field misses it: the 16-bit velocity's rounding alone puts 3.3e-3 into Pi, and no
# 16-bit encoding found gets below 1.4e-3 (tests/test_form_floor.py, the FP64 oracle with the
# stored state round-tripped through the encodings).
FORM_TARGET = 1e-3
@pytest.mark.parametrize("prec,tol100,tol1000", [
    (mbcg.FP16, {"rhor": 5e-4, "rhob": 5e-5, "u": 1e-3, "Pi": 5e-3}, {"rhor": 1e-3, "rhob": 2e-4, "u": 1e-3, "Pi": 1.5e-2}),
    (mbcg.BF16, {"rhor": 5e-3, "rhob": 5e-4, "u": 1e-2, "Pi": 5e-2}, {"rhor": 1e-2, "rhob": 2e-3, "u": 2e-2, "Pi": 0.15})])
def test_storage_form_error_vs_fp64(oracle_states, prec, tol100, tol1000):
    p32, a, s100, s1000, _ = oracle_states
    p = jet(prec)
    idx = written_nodes(p)
    with mbcg.Case(p) as c:
        c.copy_in(a.astype(np.float32))
        c.step(100)
        e100 = group_errors(c.copy_out(), s100, idx)
        c.step(900)
        e1000 = group_errors(c.copy_out(), s1000, idx)
        d = c.diagnostics()
    name = {mbcg.FP32: "fp32", mbcg.FP16: "fp16", mbcg.BF16: "bf16"}[prec]
    print(f"\n{name}: step 100 {e100}  step 1000 {e1000}")
    assert d["nonfinite"] == 0
    for k in ("rhor", "rhob", "u", "Pi"):
        assert e100[k] < tol100[k], (name, k, e100)
        assert e1000[k] < tol1000[k], (name, k, e1000)
    if prec == mbcg.FP16:
        for k in ("rhor", "rhob", "u"):
            assert e100[k] < FORM_TARGET and e1000[k] < FORM_TARGET, (k, e100, e1000)
        if not (e100["Pi"] < FORM_TARGET and e1000["Pi"] < FORM_TARGET):
            pytest.xfail(f"FP16 stress field {e100['Pi']:.1e} (100 steps) / {e1000['Pi']:.1e} (1000 steps) above "
                         f"the 1e-3 target: the 16-bit velocity's rounding enters Pi through rho u u")


def test_stochastic_rounding_is_reproducible():
    """The 16-bit stores round stochastically from a counter-based stream keyed by (seed, step,
    node): two runs agree bit for bit, a run with another seed does not (restarts continuing
    bit for bit are tests/test_gpu_io.py's checkpoint tests)."""
    p = jet(mbcg.FP16)
    outs = []
    for _ in range(2):
        with mbcg.Case(p) as c:
            c.init()
            c.step(30)
            outs.append(c.copy_out())
    assert np.array_equal(outs[0], outs[1])
    q = mbcg.jet_params(48, 48, 96, q=27, diameter=16.0, precision=mbcg.FP16)
    q.seed = p.seed + 1
    with mbcg.Case(q) as c:
        c.init()
        c.step(30)
        other = c.copy_out()
    # another seed draws other roundings (and other inlet noise): the states differ
    assert not np.array_equal(outs[0], other)


@pytest.mark.parametrize("prec", [mbcg.FP32, mbcg.FP16, mbcg.BF16])
def test_pinned_and_pageable_copies_agree(prec):
    """Pinned host fields are read and written by the device directly (one kernel with the layout
    conversion); pageable ones go through staged copies.  Both paths give the same bits, in and
    out, on an odd-sized lattice."""
    torch = pytest.importorskip("torch")
    p = mbcg.jet_params(37, 29, 23, q=27, diameter=9.0, precision=prec)
    shape = (mbcg.NFIELDS,) + p.shape
    with mbcg.Case(p) as c:
        c.init()
        c.step(3)
        pageable_out = c.copy_out()
        pinned_out = torch.empty(shape, dtype=torch.float32, pin_memory=True)
        c.copy_out(out=pinned_out.numpy())
        assert np.array_equal(pageable_out, pinned_out.numpy())
        state = pageable_out.copy()
    # the same state in through each path, one step, out through the pageable path
    outs = []
    for pinned in (False, True):
        with mbcg.Case(p) as c:
            if pinned:
                src = torch.empty(shape, dtype=torch.float32, pin_memory=True)
                src.numpy()[...] = state
                c.copy_in(src.numpy())
            else:
                c.copy_in(state)
            c.step(2)
            outs.append(c.copy_out())
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("prec", [mbcg.FP32, mbcg.FP16])
@pytest.mark.parametrize("nsteps", [1, 2])
def test_run_host_matches_sequential_calls(prec, nsteps):
    """mbcg_run_host overlaps the transfers of consecutive host states; its results are those of
    copy_in; step; copy_out for every state, bit for bit, and the step counter advances alike."""
    torch = pytest.importorskip("torch")
    p = mbcg.jet_params(33, 27, 21, q=27, diameter=9.0, precision=prec)
    shape = (mbcg.NFIELDS,) + p.shape
    states = []
    with mbcg.Case(p) as c:
        c.init()
        for _ in range(4):
            c.step(3)
            states.append(c.copy_out())
    want = []
    with mbcg.Case(p) as c:
        for s_ in states:
            c.copy_in(s_)
            c.step(nsteps)
            want.append(c.copy_out())
        steps_seq = mbcg.Library.get().mbcg_steps_done(c.handle)
    for pinned in (True, False):
        if pinned:
            ins = [torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy() for _ in states]
            outs = [torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy() for _ in states]
            for a, s_ in zip(ins, states):
                a[...] = s_
        else:
            ins = [s_.copy() for s_ in states]
            outs = [np.empty(shape, dtype=np.float32) for _ in states]
        with mbcg.Case(p) as c:
            c.run_host(ins, outs, nsteps)
            assert mbcg.Library.get().mbcg_steps_done(c.handle) == steps_seq
            last = c.copy_out()
        for j in range(len(states)):
            assert np.array_equal(outs[j], want[j]), f"state {j} (pinned={pinned})"
        assert np.array_equal(last, want[-1])


def test_run_host_edge_cases():
    """count 0 changes nothing; nsteps 0 is copy_in + copy_out (a round trip of the state)."""
    p = mbcg.jet_params(20, 18, 16, q=19, diameter=6.0)
    with mbcg.Case(p) as c:
        c.init()
        c.step(2)
        before = c.copy_out()
        c.run_host([], [], 1)
        assert np.array_equal(c.copy_out(), before)
        assert mbcg.Library.get().mbcg_steps_done(c.handle) == 2
        out = np.empty_like(before)
        c.run_host([before], [out], 0)
        assert np.array_equal(out, before)
        assert mbcg.Library.get().mbcg_steps_done(c.handle) == 2
        with pytest.raises(mbcg.MbcgError):
            c.run_host([before], [out], -1)


@pytest.mark.skipif(not os.environ.get("MBCG_LONG"), reason="10^4-step FP64 oracle run (~6 min of host CPU): set MBCG_LONG=1")
def test_forms_error_at_10k_steps():
    """Field error against the FP64 oracle after 10^4 steps (the jet above): FP32 stays at its
    100-step level; the 16-bit forms, stochastically rounded, grow like a random walk (measured
    FP32 2.2e-5, 1.4e-5, 1.1e-5, 1.7e-4; FP16 3.1e-2, 1.9e-2, 3.9e-3, 5.4e-2; BF16 0.22, 0.14,
    2.5e-2, 0.42)."""
    p = jet(mbcg.FP32)
    a = ol.oracle_init(p, np.float64)
    ref = ol.oracle_run(p, a.copy(), 10000)
    idx = written_nodes(p)
    bounds = {mbcg.FP32: {"rhor": 5e-5, "rhob": 5e-5, "u": 3e-5, "Pi": 5e-4},
              mbcg.FP16: {"rhor": 6e-2, "rhob": 4e-2, "u": 1e-2, "Pi": 0.1},
              mbcg.BF16: {"rhor": 0.45, "rhob": 0.3, "u": 6e-2, "Pi": 0.8}}
    for prec, tol in bounds.items():
        with mbcg.Case(jet(prec)) as c:
            c.copy_in(a.astype(np.float32))
            c.step(10000)
            e = group_errors(c.copy_out(), ref, idx)
        print(f"\n{prec}: step 10000 {e}")
        for k, v in tol.items():
            assert e[k] < v, (prec, k, e)
