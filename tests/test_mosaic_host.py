"""Host-side mosaic logic: pointing lattice, mosaic placement, the combine formula."""
import math

import numpy as np


def test_hex_lattice_is_centred_and_hexagonal():
    from sde_gb300.synth import hex_pointings
    p = hex_pointings(49, 1.0)
    assert p.shape == (49, 2)
    assert np.allclose(p.mean(axis=0), 0.0)
    d = np.sqrt(((p[:, None, :] - p[None, :, :]) ** 2).sum(-1))
    d[d == 0] = np.inf
    assert np.allclose(d.min(axis=1), 1.0)  # nearest neighbour at one spacing


def test_config4_is_seeded_and_in_range():
    from sde_gb300 import synth
    a, c = synth.config4(n_point=5, nvis_range=(2e3, 2e4))
    b, _ = synth.config4(n_point=5, nvis_range=(2e3, 2e4))
    for x, y in zip(a, b):
        assert x["imsize"] == y["imsize"] and np.array_equal(x["vis"], y["vis"])
        assert 2000 <= len(x["u"]) <= 20000
        assert x["imsize"] in (256, 512, 1024, 2048)


def test_layout_holds_every_image():
    from sde_gb300.mosaic import mosaic_layout
    cell = math.radians(2.0 / 3600)
    offs = [(0.0, 0.0), (0.01, 0.0), (-0.004, 0.006)]
    sizes = [256, 2048, 512]
    mnx, mny, cx, cy, fw = mosaic_layout(offs, sizes, cell, math.radians(0.5))
    for (l, m), n, x, y in zip(offs, sizes, cx, cy):
        cen = (n + 1) // 2
        assert 1 <= x - cen + 1 and x - cen + n <= mnx
        assert 1 <= y - cen + 1 and y - cen + n <= mny
    # x runs against l, y along m
    assert cx[1] < cx[0] and cy[2] > cy[0]
    assert abs(fw[0] - math.radians(0.5) / cell) < 1e-3


def test_combine_of_one_pointing_is_its_image_where_sensitive():
    from sde_gb300.mosaic import combine_host
    rng = np.random.default_rng(1)
    im = rng.normal(size=(64, 64)).astype(np.float32)
    lay = dict(mnx=64, mny=64, cx=np.array([32]), cy=np.array([32]), fwhm_px=np.array([20.0]),
               wt=np.array([3.0]), clip=0.1)
    out = combine_host([im], lay)
    yy, xx = np.mgrid[0:64, 0:64]
    pb = np.exp(-4 * math.log(2) / 400.0 * ((xx - 31) ** 2 + (yy - 31) ** 2))
    m = pb ** 2 > 0.1
    assert np.allclose(out[m], im[m] / pb[m], rtol=1e-6, atol=1e-6)
    assert np.all(out[~m] == 0)
