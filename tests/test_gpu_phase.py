"""In-situ phase statistics (mbcg_phase_statistics) against numpy on synthetic states with known
answers, and on running cases."""
import numpy as np
import pytest

import mbcg
from gpu_util import gpu_from_ic

pytestmark = pytest.mark.gpu


def balls_state(p, centres, radii):
    """Blue everywhere, sharp red balls (periodic distances on the fluid nodes)."""
    s = np.zeros((11,) + p.shape, dtype=np.float32)
    s[1] = 1.0
    nf = np.array([p.nz - 2, p.ny - 2, p.nx - 2])
    zz, yy, xx = np.meshgrid(np.arange(1, p.nz - 1), np.arange(1, p.ny - 1), np.arange(1, p.nx - 1), indexing="ij")
    red = np.zeros(tuple(nf), dtype=bool)
    for (cx, cy, cz), r in zip(centres, radii):
        d = [np.abs(xx - cx), np.abs(yy - cy), np.abs(zz - cz)]
        d = [np.minimum(di, L - di) for di, L in zip(d, nf[::-1])]
        red |= d[0] ** 2 + d[1] ** 2 + d[2] ** 2 <= r * r
    s[0, 1:-1, 1:-1, 1:-1] = red
    s[1, 1:-1, 1:-1, 1:-1] = ~red
    return s, red


def expected(red):
    phi = np.where(red, 1.0, -1.0)
    g2 = np.zeros_like(phi)
    for ax in range(3):
        g2 += ((np.roll(phi, -1, ax) - np.roll(phi, 1, ax)) / 2.0) ** 2
    area = 0.5 * np.sqrt(g2).sum()
    zz, yy, xx = np.nonzero(red)
    return area, red.sum(), (xx.mean() + 1, yy.mean() + 1, zz.mean() + 1)


@pytest.mark.parametrize("prec", [mbcg.FP32, mbcg.FP16])
def test_statistics_of_known_balls(prec):
    p = mbcg.bubble_params(40, q=19, precision=prec)
    p.nx, p.ny, p.nz = 42, 38, 34
    p.ic = mbcg.IC_NONE
    # three disjoint balls, the third wrapping across the periodic x boundary
    state, red = balls_state(p, [(12, 12, 10), (28, 26, 22), (2, 10, 25)], [5.0, 7.0, 4.0])
    with mbcg.Case(p) as c:
        c.copy_in(state)
        st = c.phase_statistics(components=True)
    area, vol, cen = expected(red)
    assert st["status"] == 0
    assert st["volume_tracked"] == vol and st["volume_other"] == red.size - vol
    assert st["interface_nodes"] == 0  # sharp interfaces: no mixed node
    assert abs(st["interface_area"] - area) <= 1e-9 * area
    assert np.allclose(st["centroid"], cen, rtol=0, atol=1e-9)
    assert st["penetration"] == -1.0
    assert st["components"] == 3
    sizes = []
    for (cx, cy, cz), r in zip([(12, 12, 10), (28, 26, 22), (2, 10, 25)], [5.0, 7.0, 4.0]):
        _, single = balls_state(p, [(cx, cy, cz)], [r])
        sizes.append(int(single.sum()))
    assert st["largest_component"] == max(sizes)
    assert st["detached"] == 3 and st["detached_volume"] == vol


def test_diffuse_bubble_area():
    """A tanh bubble of radius R and width w: |grad phi| / 2 is a sech^2 kernel of variance
    pi^2 w^2 / 12 around the sphere, so its volume integral is 4 pi (R^2 + pi^2 w^2 / 12); the
    discrete sum must match that within 1 %."""
    R, w = 12.0, 3.0
    p = mbcg.bubble_params(48, q=27, radius=R, width=w)
    with mbcg.Case(p) as c:
        c.init()
        st = c.phase_statistics(components=True)
    area = 4 * np.pi * (R * R + np.pi ** 2 * w * w / 12)
    assert abs(st["interface_area"] / area - 1) < 0.01, (st, area)
    assert st["interface_nodes"] > 0 and st["components"] == 1 and st["detached"] == 1
    assert np.allclose(st["centroid"], [p.bubble_center[0]] * 3, atol=0.05)


def test_jet_penetration_grows():
    p = mbcg.jet_params(34, 34, 120, q=19, diameter=12.0, velocity=0.08)
    pens = []
    with mbcg.Case(p) as c:
        c.init()
        for _ in range(4):
            c.step(60)
            st = c.phase_statistics(components=True)
            pens.append(st["penetration"])
            # the injected jet stays attached to the inlet layer
            assert st["components"] >= 1 and st["largest_component"] > 0 and st["status"] == 0
            assert st["detached"] <= st["components"] - 1
    assert pens[0] > 1 and all(b >= a for a, b in zip(pens, pens[1:])) and pens[-1] > pens[0], pens
