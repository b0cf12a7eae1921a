"""The accuracy floor of 16-bit moment storage, measured with the FP64 oracle on the host.

The FP64 oracle steps the reduced jet of tests/test_gpu_forms.py (48 x 48 x 96, D3Q27, the jet
configuration's physics) and after every step the stored state is round-tripped through a
16-bit encoding with stochastic rounding, restated here in numpy; the result is compared with
the plain FP64 oracle (relative L2 per group, as in the GPU tests).

* The FP16 form of the library (density deviation, colour complement, velocity and stress as
  scaled FP16 slots) gives a stress-field error of ~3.6e-3 after 100 steps, the GPU's figure.
  Rounding one slot group at a time shows where it comes from: the velocity ~3.3e-3, the
  density deviation ~1.5e-3, the stress slots themselves ~4e-4, the colour slot ~5e-5.
* The best encoding found that still fits 16 bits per moment (the density deviation as 16-bit
  fixed point over +-0.02, the velocity as one shared exponent with three 14-bit mantissas in
  its 48 bits) still leaves ~1.4e-3 at 100 steps (2.8e-3 at 1000 steps, opt-in MBCG_LONG=1):
  the 1e-3 stress target is out of reach of 16-bit slots, whatever their encoding.
"""
import os

import numpy as np
import pytest

import mbcg
import oracle_lib as ol
from gpu_util import group_errors, written_nodes


def sr_fp16(x, rng):
    """Stochastic rounding to the FP16 grid (up with probability equal to the distance from the
    lower neighbour in ulps), as the kernel's cvt.rs stores do."""
    x = np.asarray(x, np.float64)
    h = x.astype(np.float16)
    hd = h.astype(np.float64)
    up = hd < x
    lo = np.where(up, hd, np.nextafter(h, np.float16(-np.inf)).astype(np.float64))
    hi = np.where(up, np.nextafter(h, np.float16(np.inf)).astype(np.float64), hd)
    span = hi - lo
    p = np.where(span > 0, (x - lo) / np.where(span > 0, span, 1.0), 0.0)
    return np.where(hd == x, x, np.where(rng.random(x.shape) < p, hi, lo))


def sr_fixed(x, step, rng):
    q = x / step
    f = np.floor(q)
    return (f + (rng.random(x.shape) < (q - f))) * step


def roundtrip(a, p, enc, rng):
    """Store and reload every node through the encoding `enc` (a dict of slot group -> rule);
    groups without a rule are kept exact."""
    f = a.copy()
    rr, rb = f[0], f[1]
    with np.errstate(invalid="ignore", divide="ignore"):
        rho = rr + rb
        c = np.where(rr >= rb, 2.0 * rb / rho, -(2.0 * rr / rho))      # colour complement slot
        if enc.get("c") == "fp16":
            c = sr_fp16(c, rng)
        phi = np.copysign(1.0 - np.abs(c), c)
        nominal = 0.5 * (p.rho_r0 + p.rho_b0) + phi * 0.5 * (p.rho_r0 - p.rho_b0)
        dev = (rho - nominal) / p.rho_scale
        if enc.get("rho") == "fp16":
            dev = sr_fp16(dev, rng)
        elif enc.get("rho") == "fixed":                                  # +-0.02 in 65536 steps
            R = 0.02 / p.rho_scale
            inr = np.abs(dev) <= R
            dev = np.where(inr, sr_fixed(np.clip(dev, -R, R), 2.0 * R / 65536.0, rng), dev)
        rho_r = nominal + p.rho_scale * dev
        minor = 0.5 * rho_r * np.abs(c)
        red_major = ~np.signbit(c)
        live = np.isfinite(c)                                           # nodes outside hold zeros
        f[0] = np.where(live, np.where(red_major, rho_r - minor, minor), rr)
        f[1] = np.where(live, np.where(red_major, minor, rho_r - minor), rb)
    u = f[2:5] / p.u_ref
    if enc.get("u") == "fp16":
        u = sr_fp16(u, rng)
    elif enc.get("u") == "shared14":                                    # one exponent, 3 x 14 bits
        m = np.max(np.abs(u), axis=0)
        e = np.ceil(np.log2(np.where(m > 0, m, 1e-30)))
        u = sr_fixed(u, (2.0 ** (e - 13))[None], rng)
    f[2:5] = u * p.u_ref
    if enc.get("pi") == "fp16":
        f[5:11] = sr_fp16(f[5:11] / p.pi_scale, rng) * p.pi_scale
    return f


FP16_FORM = {"c": "fp16", "rho": "fp16", "u": "fp16", "pi": "fp16"}
BEST_16BIT = {"c": "fp16", "rho": "fixed", "u": "shared14", "pi": "fp16"}


@pytest.fixture(scope="module")
def jet_case():
    p = mbcg.jet_params(48, 48, 96, q=27, diameter=16.0, precision=mbcg.FP16)
    p64 = mbcg.jet_params(48, 48, 96, q=27, diameter=16.0)
    a0 = ol.oracle_init(p64, np.float64)
    return p, p64, a0, written_nodes(p64), {}


def emulate(jet_case, enc, nsteps, seed=11):
    p, p64, a0, idx, refs = jet_case
    if nsteps not in refs:
        refs[nsteps] = ol.oracle_run(p64, a0.copy(), nsteps)
    rng = np.random.default_rng(seed)
    a = roundtrip(a0.copy(), p, enc, rng)
    for n in range(nsteps):
        a = ol.oracle_run(p64, a, 1, first_step=1 + n)
        a = roundtrip(a, p, enc, rng)
    return group_errors(a, refs[nsteps], idx)


def test_fp16_form_stress_error(jet_case):
    e = emulate(jet_case, FP16_FORM, 100)
    assert 2e-3 < e["Pi"] < 6e-3, e                 # the GPU's FP16 form: 3.6e-3
    assert e["rhor"] < 1e-3 and e["u"] < 1e-3, e


@pytest.mark.skipif(not os.environ.get("MBCG_LONG"), reason="opt-in (MBCG_LONG=1): ~1 min of host time")
def test_fp16_form_stress_error_sources(jet_case):
    e = emulate(jet_case, FP16_FORM, 100)
    e_u = emulate(jet_case, {"u": "fp16"}, 100)
    e_pi = emulate(jet_case, {"pi": "fp16"}, 100)
    assert e_u["Pi"] > 0.5 * e["Pi"], (e_u, e)     # the velocity slots carry most of it
    assert e_pi["Pi"] < 0.25 * e["Pi"], (e_pi, e)  # the stress slots themselves little


@pytest.mark.parametrize("nsteps", [100] + ([1000] if os.environ.get("MBCG_LONG") else []))
def test_best_16bit_encoding_still_misses_the_stress_target(jet_case, nsteps):
    e = emulate(jet_case, BEST_16BIT, nsteps)
    print(f"\nbest 16-bit encoding, {nsteps} steps: {e}")
    assert e["Pi"] > 1e-3, e
