"""Dirty-image error against the FP64 oracle on dense uv coverage.

TEST INFRASTRUCTURE (a checker): used by tests/test_gpu_precision.py and by bench.py's
precision legs; the product package never imports it.

The uv coverage of the large single field (27 antennas, 8 h x 10 s x 64 channels) imaged
on a small grid puts tens to thousands of visibilities in each cell, where the way cell sums
are formed decides the error.  GRDH2D adds every visibility into its cell in REAL
(grd/grdh2d.f:177-187): once a cell's running sum is 1e5-1e6 times a single contribution,
each addition rounds away a large part of that contribution.  The GPU path sums at most a
chunk of visibilities in registers, the chunks of a work item in the shared tile, and the
work items in the raw grid with TwoSum-compensated adds (sde_ctx_set_compensated); FP64 is
used for coordinates, phase rotation and the grid-correction taper only.

study() reports, for one such case, max |image - FP64 oracle image| over the CRDNHALF
window and over the whole image, as a fraction of the FP64 image peak, for the GPU path
with and without compensation and for the reference's own FP32 arithmetic (oracle/).
"""
import math

import numpy as np

from oracle import oracle as O
from sde_gb300 import synth
from sde_gb300._abi import lib
from sde_gb300.imaging import Geom, uvmap


def dense_case(stride=8, n_src=20, seed_offset=0):
    """Every stride-th visibility of the large single field's uv coverage, with a seeded
    sky of n_src point sources."""
    (u, v, w), seed = synth.config2_uvw(n_chan=64)
    u, v, w = u[::stride].copy(), v[::stride].copy(), w[::stride].copy()
    flux, l, m = synth.point_sky(200, 512 * 4.0, seed + seed_offset)
    vis = synth.visibilities(u, v, flux[:n_src], l[:n_src], m[:n_src], 1e-3, seed)
    return u, v, w, np.asarray(vis, np.complex64), np.ones(len(u), np.float32)


def _window(n):
    lo = n // 4 + 1
    length = min(3 * n // 4 - 1 - lo + 1, n // 2 - 1)
    return slice(lo - 1, lo - 1 + length)


def study(ctx, data, imsize=512, cell=4.0, vdec=40.0, reference=True):
    """Errors vs the FP64 oracle (natural weights, uvmap normalisation by the PSF peak)."""
    O.lib()
    torch = ctx.torch
    u, v, w, vis, wt = data
    g = Geom(imsize, cell, vdec=vdec)
    out = {"nvis": int(len(u)), "imsize": imsize, "cell_arcsec": cell}
    imgs = {}
    for comp in (True, False):
        lib().sde_ctx_set_compensated(ctx.h, int(comp))
        t = {k: ctx.tensor(x, torch.float32) for k, x in (("u", u), ("v", v), ("w", w), ("wt", wt))}
        t["vis"] = ctx.tensor(vis.view(np.float32), torch.float32)
        r = uvmap(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"], weighting=False)
        ctx.sync()
        imgs["compensated" if comp else "plain_fp32"] = r["dirty"].cpu().numpy().astype(np.float64)
        r["plan"].close()
    lib().sde_ctx_set_compensated(ctx.h, 1)
    p = O.params(imsize, cell, fov=1.0, rmode="NONE", vdec=vdec)
    og = O.geom(p)
    d64 = O.uvmap_image64(og, u, v, w, vis, wt, False)
    p64 = O.uvmap_image64(og, u, v, w, vis, wt, True)
    d64 /= p64.max()
    if reference:
        d32, *_ = O.uvmap(p, u, v, w, vis, wt)
        imgs["reference_fp32"] = d32.astype(np.float64)
    W = _window(imsize)
    pk = np.abs(d64).max()
    for k, im in imgs.items():
        out[k] = {"window": float(np.abs(im - d64)[W, W].max() / pk),
                  "image": float(np.abs(im - d64).max() / pk)}
    # cell occupancy of the case (gridding cells of the half plane)
    du = 1.0 / (imsize * math.radians(cell / 3600.0))
    iu = np.abs(np.rint(u / du)).astype(np.int64)
    iv = np.rint(np.where(u < 0, -v, v) / du).astype(np.int64)
    _, cnt = np.unique(iv * 100003 + iu, return_counts=True)
    out["vis_per_cell"] = {"mean": float(cnt.mean()), "max": int(cnt.max())}
    return out
