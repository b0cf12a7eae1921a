"""The colour split of the populations, restated on the host in IEEE FP32 (numpy), without a GPU.

Each source node sends its populations g_i = W_i (rho + sm_i) (W_i the integer D3Q19 weights
12 / 2 / 1, S = 36; sm_i the part without the density, which sums to zero over the directions) and
the red share of each.  Formed as aR g_i with aR = fl(rr / rho), a source's red populations sum to
S aR rho (+ the roundings of g and of the products): the quotient's rounding error, times S rho,
is emitted as red mass.  In a near-steady state that error repeats step after step (the stored
densities change by an ulp or so, which barely moves the quotient's rounding), so over ~10^5
interface nodes the red phase of the 64^3 bubble drifted by 7e-6 in 10^4 steps.  Formed as
W_i (rr + aR sm_i), the step kernel's form on interface warps, the same populations sum to
S rr + aR sum(W_i sm_i) in exact arithmetic: the quotient's rounding has dropped out.  The GPU
test of the consequence is the 10^4-step mass gate in tests/test_gpu_diagnostics.py.
"""
import numpy as np

# D3Q19 directions and integer weights (w_i * 36)
C = np.array([(0, 0, 0)] + [(x, y, z) for x in (-1, 0, 1) for y in (-1, 0, 1) for z in (-1, 0, 1)
                            if 0 < x * x + y * y + z * z <= 2], dtype=np.float64)
W = np.array([12.0 if (c ** 2).sum() == 0 else (2.0 if (c ** 2).sum() == 1 else 1.0) for c in C])


def bubble_sources(n=200_000, seed=7, uscale=1e-4):
    """Interface sources of a tanh bubble with a Laplace pressure: colour fraction over (0, 1),
    density 1 + 1.7e-3 inside and 1 - 1.4e-4 outside, small velocities."""
    rng = np.random.default_rng(seed)
    phi = -np.tanh(rng.uniform(-3.0, 3.0, n))        # +1 inside (red)
    rho = 1.0 + 1.7e-3 * 0.5 * (1.0 + phi) - 1.4e-4 * 0.5 * (1.0 - phi)
    rr = (0.5 * (1.0 + phi) * rho).astype(np.float32)
    rb = (0.5 * (1.0 - phi) * rho).astype(np.float32)
    u = (uscale * rng.standard_normal((n, 3))).astype(np.float32)
    return rr, rb, u


def small_parts(rho, u):
    """sm_i = rho (c.u / cs2 + (c.u)^2 / (2 cs4) - u.u / (2 cs2)) in FP32 (cs2 = 1/3)."""
    cu = (u @ C.T.astype(np.float32)).astype(np.float32)
    uu = (u ** 2).sum(axis=1, dtype=np.float32)[:, None]
    sm = rho[:, None] * (np.float32(3.0) * cu + np.float32(4.5) * cu * cu - np.float32(1.5) * uu)
    return sm.astype(np.float32)


def colour_fraction(rr, rb):
    rho = (rr + rb).astype(np.float32)
    return rho, (rr / rho).astype(np.float32)  # correctly rounded quotient


def fma32(a, b, c):
    """fl32(a * b + c): the product of two FP32 values is exact in FP64."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def emitted_red32(rr, rb, u, exact):
    """A source's red populations formed in FP32, summed exactly (FP64)."""
    rho, aR = colour_fraction(rr, rb)
    sm = small_parts(rho, u)
    Wf = W.astype(np.float32)[None, :]
    if exact:
        red = Wf * fma32(aR[:, None], sm, np.broadcast_to(rr[:, None], sm.shape))
    else:
        red = aR[:, None] * (Wf * (rho[:, None] + sm))
    return red.astype(np.float32).astype(np.float64).sum(axis=1)


def test_weights_sum_to_S():
    assert W.sum() == 36.0 and len(C) == 19
    assert np.allclose((W[:, None] * C).sum(axis=0), 0.0)


def test_exact_split_does_not_carry_the_colour_fraction_rounding():
    """Evaluated exactly (FP64) from the FP32 inputs: moving aR by one ulp moves the direct split's
    emitted red mass by S rho ulp, the exact split's only by ulp * sum(W_i sm_i)."""
    rr, rb, u = bubble_sources()
    rho, aR = colour_fraction(rr, rb)
    sm = small_parts(rho, u).astype(np.float64)
    aR2 = np.nextafter(aR, np.float32(2.0))
    g = W[None, :] * (rho.astype(np.float64)[:, None] + sm)

    def direct(a):
        return a.astype(np.float64) * g.sum(axis=1)

    def exact(a):
        return (W[None, :] * (rr.astype(np.float64)[:, None] + a.astype(np.float64)[:, None] * sm)).sum(axis=1)

    d_direct = np.abs(direct(aR2) - direct(aR))
    d_exact = np.abs(exact(aR2) - exact(aR))
    assert np.all(d_direct > 30.0 * np.spacing(aR).astype(np.float64))
    assert d_exact.max() < 1e-4 * d_direct.min()
    # and the exact split emits S rr up to aR sum(W_i sm_i), which vanishes with the small parts
    resid = exact(aR) - 36.0 * rr.astype(np.float64)
    assert np.allclose(resid, aR.astype(np.float64) * (W[None, :] * sm).sum(axis=1), rtol=0, atol=1e-12)


def test_one_ulp_changes_leave_the_quotient_rounding_correlated():
    """Why the rounding repeats from step to step: nudging the stored colour densities by one ulp
    (what a slowly changing state does, or a +-1-ulp dither) moves rr / rho by almost exactly an
    ulp near rho = 1, so the quotient's rounding error stays correlated with the old one."""
    rr, rb, _ = bubble_sources()

    def qerr(r, b):
        rho, aR = colour_fraction(r, b)
        return aR.astype(np.float64) * rho.astype(np.float64) - r.astype(np.float64)

    e0 = qerr(rr, rb)
    e1 = qerr(np.nextafter(rr, np.float32(2.0)), rb)
    e2 = qerr(np.nextafter(rr, np.float32(2.0)), np.nextafter(rb, np.float32(2.0)))
    assert np.corrcoef(e0, e1)[0, 1] > 0.5
    assert np.corrcoef(e0, e2)[0, 1] > 0.4


def test_fp32_emission_error_is_smaller_with_the_exact_split():
    """In FP32 the exact split's per-source emission error (S rr against the formed red
    populations) is well under half the direct split's, from near-static to jet-like velocities."""
    for uscale in (1e-5, 1e-3):
        rr, rb, u = bubble_sources(uscale=uscale)
        ref = 36.0 * rr.astype(np.float64)
        direct = emitted_red32(rr, rb, u, exact=False) - ref
        exact = emitted_red32(rr, rb, u, exact=True) - ref
        rms_d, rms_e = np.sqrt((direct ** 2).mean()), np.sqrt((exact ** 2).mean())
        assert rms_e < 0.5 * rms_d, (uscale, rms_e, rms_d)
