"""Mosaic imaging over libsdegpu batches, and the sort-bucket autotuner.

task/mosclean.f images the pointings of a mosaic one after another and forms the linear
mosaic sum_i SUMWT_i PB_i I_i / sum_i SUMWT_i PB_i^2 (task/mosclean.f:413-432, ARRLC with
the pointing weight SUMWT, IMGPB 'APPLY' for the primary beam).  Here each pointing is
weighted and planned on the device and the whole set is imaged by one sde_batch: one
persistent gridding launch over all pointings' work items, batched FFTs per image size,
the PSF-peak normalisation of uvmap and the primary-beam-weighted combine, captured in one
CUDA graph and replayed.  Mosaic.dirty_loop() produces the same images through the
single-plan entry points, one pointing at a time.

autotune() picks the plans' sort-bucket sizes (visibilities per work item and per chunk)
for a given set of pointings by timing the batched pass with each candidate.
"""
import ctypes as C
import math

import numpy as np

from . import _abi
from ._abi import check, lib
from .imaging import Geom, Plan, _ptr


def mosaic_layout(offsets, sizes, cell_rad, fwhm_rad):
    """Mosaic size and placement for pointings at (l, m) offsets (radians) with square
    images of the given sizes.  Pixel x runs against l (RA increases to the left, as the
    images uvmap makes), y along m.  Returns (mnx, mny, cx, cy, fwhm_px) with cx, cy the
    1-based mosaic pixel of each image's centre pixel (n+1)//2."""
    offs = np.asarray(offsets, np.float64).reshape(-1, 2)
    sizes = np.asarray(sizes, np.int64)
    px = np.rint(-offs[:, 0] / cell_rad).astype(np.int64)
    py = np.rint(offs[:, 1] / cell_rad).astype(np.int64)
    half = (sizes + 1) // 2
    x0 = int((px - half).min()) - 1
    y0 = int((py - half).min()) - 1
    x1 = int((px + sizes - half).max()) + 1
    y1 = int((py + sizes - half).max()) + 1
    mnx, mny = x1 - x0 + 1, y1 - y0 + 1
    cx = (px - x0 + 1).astype(np.int32)
    cy = (py - y0 + 1).astype(np.int32)
    fwhm_px = np.full(len(sizes), fwhm_rad / cell_rad, np.float32)
    return int(mnx), int(mny), cx, cy, fwhm_px


class Mosaic:
    """All pointings of a mosaic resident on the device and imaged as one batch."""

    def __init__(self, ctx, pointings, cell_arcsec, rmode="UNIFORM", opts=None, clip=0.1,
                 mosaic=True):
        torch = ctx.torch
        self.ctx = ctx
        self.n = len(pointings)
        self.cell_rad = math.radians(cell_arcsec / 3600.0)
        self.geoms, self.plans, self.sumwt = [], [], []
        self._keep = []
        for p in pointings:
            g = Geom(p["imsize"], cell_arcsec)
            u = ctx.tensor(p["u"], torch.float32)
            v = ctx.tensor(p["v"], torch.float32)
            w = ctx.tensor(p["w"], torch.float32)
            vis = ctx.tensor(np.asarray(p["vis"], np.complex64).view(np.float32), torch.float32)
            wt = ctx.tensor(p["wt"], torch.float32)
            if rmode is not None:
                ctx.weights(g, u, v, w, wt, rmode=rmode)
            self.geoms.append(g)
            self.plans.append(Plan(ctx, g, u, v, w, vis, wt, opts=opts))
            self.sumwt.append(float(wt.clamp(min=0).sum().item()))
            self._keep.append((u, v, w, vis, wt))
        self.nvis = sum(pl.nvis for pl in self.plans)
        hp = (C.c_void_p * self.n)(*[pl.h.value for pl in self.plans])
        nx = (C.c_int * self.n)(*[g.nx for g in self.geoms])
        ny = (C.c_int * self.n)(*[g.ny for g in self.geoms])
        h = C.c_void_p()
        check(lib().sde_batch_create(ctx.h, self.n, hp, nx, ny, C.byref(h)), "sde_batch_create")
        self.h = h
        self.layout = None
        if mosaic:
            mnx, mny, cx, cy, fw = mosaic_layout([(p["l0"], p["m0"]) for p in pointings],
                                                 [g.nx for g in self.geoms], self.cell_rad,
                                                 pointings[0]["pb_fwhm_rad"])
            wts = np.asarray(self.sumwt, np.float32)
            check(lib().sde_batch_set_mosaic(self.h, mnx, mny, cx.ctypes.data_as(C.c_void_p),
                                             cy.ctypes.data_as(C.c_void_p),
                                             fw.ctypes.data_as(C.c_void_p),
                                             wts.ctypes.data_as(C.c_void_p), float(clip)),
                  "sde_batch_set_mosaic")
            self.layout = dict(mnx=mnx, mny=mny, cx=cx, cy=cy, fwhm_px=fw, wt=wts, clip=clip)
        check(lib().sde_batch_psf(self.h), "sde_batch_psf")

    def dirty(self, graph=True):
        check(lib().sde_batch_dirty(self.h, int(graph)), "sde_batch_dirty")

    def dirty_loop(self):
        check(lib().sde_batch_dirty_loop(self.h), "sde_batch_dirty_loop")

    @property
    def graph_nodes(self):
        return lib().sde_batch_graph_nodes(self.h)

    @property
    def nbytes(self):
        return lib().sde_batch_bytes(self.h)

    def read(self, i=-1, which=0):
        """Host copy: i = -1 the mosaic; else plan i's dirty image (which=0) or PSF (1)."""
        if i == -1:
            shape = (self.layout["mny"], self.layout["mnx"])
        else:
            shape = (self.geoms[i].ny, self.geoms[i].nx)
        out = np.empty(shape, np.float32)
        check(lib().sde_batch_read(self.h, i, which, out.ctypes.data_as(C.c_void_p), out.size),
              "sde_batch_read")
        return out

    def peak(self, i):
        out = np.empty(1, np.float32)
        check(lib().sde_batch_read(self.h, i, 2, out.ctypes.data_as(C.c_void_p), 1), "sde_batch_read")
        return float(out[0])

    def close(self):
        if getattr(self, "h", None) and self.ctx.h:
            lib().sde_batch_destroy(self.h)
        self.h = None
        for p in self.plans:
            p.close()
        self.plans = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def combine_host(images, layout):
    """The linear mosaic on the host (numpy, float64 sums): the formula the device combine
    evaluates, for checking it."""
    mnx, mny = layout["mnx"], layout["mny"]
    num = np.zeros((mny, mnx))
    den = np.zeros((mny, mnx))
    for im, cx, cy, fw, wt in zip(images, layout["cx"], layout["cy"], layout["fwhm_px"], layout["wt"]):
        ny, nx = im.shape
        cenx, ceny = (nx + 1) // 2 - 1, (ny + 1) // 2 - 1
        yy, xx = np.mgrid[0:ny, 0:nx]
        pb = np.exp(-4.0 * math.log(2.0) / float(fw) ** 2 * ((xx - cenx) ** 2 + (yy - ceny) ** 2))
        mx = cx - 1 + xx - cenx
        my = cy - 1 + yy - ceny
        ok = (mx >= 0) & (mx < mnx) & (my >= 0) & (my < mny)
        np.add.at(num, (my[ok], mx[ok]), float(wt) * pb[ok] * im[ok])
        np.add.at(den, (my[ok], mx[ok]), float(wt) * pb[ok] ** 2)
    out = np.zeros_like(num)
    m = (den > 0) & (den > layout["clip"] * den.max())
    out[m] = num[m] / den[m]
    return out


# ---- autotuner ---------------------------------------------------------------------------
CANDIDATES = [(8192, 64), (4096, 64), (16384, 64), (8192, 32), (4096, 32), (2048, 32),
              (8192, 128), (16384, 128)]
_CACHE = {}


def tune_key(pointings):
    """Cache key: pointing count, image sizes and total visibilities (to 1 significant bit)."""
    nv = sum(len(p["u"]) for p in pointings)
    return (len(pointings), tuple(sorted(int(p["imsize"]) for p in pointings)),
            int(round(math.log2(max(nv, 1)))))


def autotune(ctx, pointings, cell_arcsec, candidates=None, reps=5, rmode="UNIFORM"):
    """Time the batched dirty pass (graph replay) for each (item_max, chunk_max) candidate;
    return dict(best=(item_max, chunk_max), ms=..., table=[((im, cm), ms), ...]).  Results
    are cached per tune_key for the life of the process."""
    key = tune_key(pointings)
    if key in _CACHE:
        return _CACHE[key]
    torch = ctx.torch
    table = []
    for cand in candidates or CANDIDATES:
        m = Mosaic(ctx, pointings, cell_arcsec, rmode=rmode, opts=cand, mosaic=False)
        m.dirty(graph=True)
        m.dirty(graph=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(ctx.stream)
        for _ in range(reps):
            m.dirty(graph=True)
        e1.record(ctx.stream)
        torch.cuda.synchronize()
        table.append((tuple(cand), e0.elapsed_time(e1) / reps))
        m.close()
    best = min(table, key=lambda t: t[1])
    res = dict(best=best[0], ms=best[1], table=table, key=key)
    _CACHE[key] = res
    return res
