"""Batched imaging of many plans (mosaic pointings) against the single-plan path.

A batch images every pointing with one persistent gridding launch, batched FFTs and a CUDA
graph; each image must equal what the single-plan entry points (uvmap, sde_plan_grid +
sde_image_from_grid) give for that pointing, within the bar every dirty-image test here
holds: 1e-5 of the image peak inside the CRDNHALF window (the grid correction amplifies
FP32 summation-order differences towards the image corners, where 5e-3 is allowed).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _window(n):
    lo = n // 4 + 1
    length = min(3 * n // 4 - 1 - lo + 1, n // 2 - 1)
    return slice(lo - 1, lo - 1 + length)


def _close(a, b, tol_in=1e-5, tol_all=5e-3):
    w = _window(a.shape[0])
    peak = np.abs(b).max()
    assert np.abs(a - b)[w, w].max() / peak < tol_in
    assert np.abs(a - b).max() / peak < tol_all


@pytest.fixture(scope="module")
def pointings():
    from sde_gb300 import synth
    p, c = synth.config4(n_point=6, nvis_range=(3e3, 3e4), size_range=(256, 512))
    return p, c


def test_batch_equals_single_plan_path(gpu_ctx, pointings):
    from sde_gb300.imaging import Geom, uvmap
    from sde_gb300.mosaic import Mosaic
    pts, c = pointings
    ctx = gpu_ctx
    m = Mosaic(ctx, pts, c["cell_arcsec"])
    m.dirty(graph=False)
    batched = [m.read(i) for i in range(m.n)]
    psfs = [m.read(i, 1) for i in range(m.n)]
    torch = ctx.torch
    for i in (0, 3, 5):
        p = pts[i]
        g = Geom(p["imsize"], c["cell_arcsec"])
        t = {k: ctx.tensor(p[k], torch.float32) for k in ("u", "v", "w", "wt")}
        t["vis"] = ctx.tensor(np.asarray(p["vis"], np.complex64).view(np.float32), torch.float32)
        r = uvmap(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"], rmode="UNIFORM")
        ctx.sync()
        _close(batched[i], r["dirty"].cpu().numpy())
        # the batch keeps the PSF unnormalised; uvmap divides it by its peak
        _close(psfs[i] / m.peak(i), r["psf"].cpu().numpy())
        r["plan"].close()
    m.close()


def test_batch_large_images_equal_single_plan_path(gpu_ctx):
    """Pointings of 1024^2 to 4096^2: the batched column pass through TMA (several grids of
    one shape per launch) and the row-pair c2r pass, against the single-plan path."""
    from sde_gb300 import synth
    from sde_gb300.imaging import Geom, uvmap
    from sde_gb300.mosaic import Mosaic
    pts, c = synth.config4(n_point=7, seed=synth.SEED_BASE + 5, nvis_range=(2e4, 6e4),
                           size_range=(1024, 4096))
    sizes = [p["imsize"] for p in pts]
    assert {1024, 2048, 4096} <= set(sizes) and sizes.count(2048) >= 2
    ctx = gpu_ctx
    m = Mosaic(ctx, pts, c["cell_arcsec"])
    m.dirty(graph=True)
    m.dirty(graph=True)  # the captured graph
    torch = ctx.torch
    seen = set()
    for i, p in enumerate(pts):
        if p["imsize"] in seen:
            continue
        seen.add(p["imsize"])
        g = Geom(p["imsize"], c["cell_arcsec"])
        t = {k: ctx.tensor(p[k], torch.float32) for k in ("u", "v", "w", "wt")}
        t["vis"] = ctx.tensor(np.asarray(p["vis"], np.complex64).view(np.float32), torch.float32)
        r = uvmap(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"], rmode="UNIFORM")
        ctx.sync()
        _close(m.read(i), r["dirty"].cpu().numpy())
        r["plan"].close()
    m.close()


def test_batch_graph_and_loop_agree(gpu_ctx, pointings):
    from sde_gb300.mosaic import Mosaic
    pts, c = pointings
    m = Mosaic(gpu_ctx, pts, c["cell_arcsec"])
    m.dirty(graph=False)
    eager = [m.read(i) for i in range(m.n)] + [m.read(-1)]
    for _ in range(3):  # eager run, capture + launch, replay
        m.dirty(graph=True)
    assert m.graph_nodes > 0
    graph = [m.read(i) for i in range(m.n)] + [m.read(-1)]
    m.dirty_loop()
    loop = [m.read(i) for i in range(m.n)] + [m.read(-1)]
    for a, b, c_ in zip(eager[:-1], graph[:-1], loop[:-1]):
        _close(b, a)
        _close(c_, a)
    mpk = np.abs(eager[-1]).max()
    assert np.abs(graph[-1] - eager[-1]).max() / mpk < 1e-3
    assert np.abs(loop[-1] - eager[-1]).max() / mpk < 1e-3
    m.close()


def test_mosaic_combine_matches_formula(gpu_ctx, pointings):
    from sde_gb300.mosaic import Mosaic, combine_host
    pts, c = pointings
    m = Mosaic(gpu_ctx, pts, c["cell_arcsec"])
    m.dirty(graph=False)
    imgs = [m.read(i) for i in range(m.n)]
    dev = m.read(-1)
    host = combine_host(imgs, m.layout)
    assert np.abs(dev - host).max() <= 1e-4 * np.abs(host).max()
    m.close()


def test_point_source_lands_on_one_mosaic_pixel(gpu_ctx):
    """A single 1 Jy source seen by four overlapping pointings: every pointing's image peaks
    on the same mosaic pixel, the one the source's (l, m) maps to."""
    from sde_gb300 import synth
    from sde_gb300.mosaic import Mosaic, mosaic_layout
    c = dict(synth.CONFIG4)
    a2r = math.radians(1.0 / 3600.0)
    cell = 4.0 * a2r
    fwhm = c["fwhm_arcmin"] * 60 * a2r
    pos = synth.y_array(27, 2500.0, 3)
    u, v, w = synth.uvw_tracks(pos, 40.0, 6.0, 600.0, [1.4e9])
    src = (3.0 * 60 * a2r, -2.0 * 60 * a2r)
    offs = [(0.0, 0.0), (6 * 60 * a2r, 0.0), (0.0, -5 * 60 * a2r), (5 * 60 * a2r, -4 * 60 * a2r)]
    pts = []
    for (l0, m0) in offs:
        dl, dm = src[0] - l0, src[1] - m0
        vis = synth.visibilities(u, v, [1.0], [dl], [dm], 0.0, 1)
        pts.append(dict(u=u, v=v, w=w, vis=vis, wt=np.ones(len(u), np.float32), imsize=256,
                        l0=l0, m0=m0, pb_fwhm_rad=fwhm))
    m = Mosaic(gpu_ctx, pts, 4.0, rmode="UNIFORM")
    m.dirty(graph=False)
    mnx, mny, cx, cy, _ = mosaic_layout(offs, [256] * 4, cell, fwhm)
    want = (int(cy[0] - 1 + round(src[1] / cell)), int(cx[0] - 1 - round(src[0] / cell)))
    for i in range(4):
        im = m.read(i)
        iy, ix = np.unravel_index(np.argmax(im), im.shape)
        cen = (256 + 1) // 2 - 1
        got = (int(cy[i] - 1 + iy - cen), int(cx[i] - 1 + ix - cen))
        assert abs(got[0] - want[0]) <= 1 and abs(got[1] - want[1]) <= 1, (i, got, want)
    mos = m.read(-1)
    iy, ix = np.unravel_index(np.argmax(mos), mos.shape)
    assert abs(iy - want[0]) <= 1 and abs(ix - want[1]) <= 1
    m.close()


def test_bucket_sizes_do_not_change_the_image(gpu_ctx, obs_small):
    from sde_gb300.imaging import Geom, uvmap
    ctx = gpu_ctx
    torch = ctx.torch
    o = obs_small
    g = Geom(o["imsize"], o["cell"], vdec=o["vdec"])
    out = []
    for opts in (None, (2048, 16), (1024, 4)):
        t = {k: ctx.tensor(o[k], torch.float32) for k in ("u", "v", "w", "wt")}
        t["vis"] = ctx.tensor(np.asarray(o["vis"], np.complex64).view(np.float32), torch.float32)
        from sde_gb300 import imaging
        ctx.weights(g, t["u"], t["v"], t["w"], t["wt"], rmode="UNIFORM")
        plan = imaging.Plan(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"], opts=opts)
        grid = ctx.grid_buffer(g)
        img = ctx.image_buffer(g)
        plan.grid(grid)
        ctx.image_from_grid(g, grid, img)
        ctx.sync()
        out.append(img.cpu().numpy())
        plan.close()
    _close(out[1], out[0])
    _close(out[2], out[0])


def test_autotune_picks_a_candidate_and_caches(gpu_ctx, pointings):
    from sde_gb300 import mosaic
    pts, c = pointings
    cands = [(8192, 64), (2048, 16)]
    r = mosaic.autotune(gpu_ctx, pts, c["cell_arcsec"], candidates=cands, reps=2)
    assert r["best"] in cands and len(r["table"]) == 2
    assert mosaic.autotune(gpu_ctx, pts, c["cell_arcsec"], candidates=cands) is r
