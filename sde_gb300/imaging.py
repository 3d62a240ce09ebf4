"""Host-side mirror of the SDE task flow for the imaging hot path, over libsdegpu.

  make_geom   IMGMAKE + FFTCONJA/FFTCONJ + VISGRID scalars (img/imgmake.f, fft/fftconja.f,
              fft/fftconj.f, vis/visgrid.f:148-153) in the reference's REAL arithmetic
  crdshift    the FP64 phase-centre rotation matrix (crd/crdshift.f:95-160)
  Context     one device + stream (torch's current stream) + the library context
  Plan        a device-resident, tile-sorted visibility set (sde_plan)
  uvmap       weighting -> PSF -> dirty, PSF-peak normalised (task/uvmap.f:212-491)
  vismodel    grid-correct -> r2c FFT -> degrid (task/vismodel.f:70-74)
  hogbom      PIX2DRCL on the CRDNHALF window (task/clean.f:150-207, img/imgclean.f:186)
  major_cycle grid residual -> dirty -> CLEAN -> model -> degrid -> residual

Device memory is torch tensors (plumbing only); every computation runs in libsdegpu's
CUDA kernels.  Images are [ny][nx] float32, grids [nv][pitch] complex64.
"""
import ctypes as C
import math

import numpy as np

from . import _abi
from ._abi import check, lib

RMODES = {"UNIFORM": 0, "NORM": 1, "ABS": 2, "AZ-NORM": 3, "NONE": 4}


def fftpwr2(i):
    """fft/fftpwr2.f:30-39 (next power of two, via NINT(LOG(I)/LOG(2)))."""
    if i < 1:
        return 1
    lg = int(np.round(np.float32(np.log(np.float32(i))) / np.float32(np.log(np.float32(2.0)))))
    p = 2 ** lg
    while p < i:
        p *= 2
    return p


def crdshift(vra, vdec, ira, idec, vrota3=0.0):
    """SHIFT(3,3) column-major, crd/crdshift.f:95-160 (FP64, same operation order)."""
    dtor = 4.0 * math.atan(1.0) / 180.0
    rao, deco, ra, dec = dtor * vra, dtor * vdec, dtor * ira, dtor * idec
    T = [[0.0] * 3 for _ in range(3)]
    T[0][0] = math.cos(ra - rao)
    T[1][0] = math.sin(ra - rao) * math.sin(deco)
    T[2][0] = -math.sin(ra - rao) * math.cos(deco)
    T[0][1] = -math.sin(ra - rao) * math.sin(dec)
    T[1][1] = math.cos(ra - rao) * math.sin(dec) * math.sin(deco) + math.cos(dec) * math.cos(deco)
    T[2][1] = -math.cos(ra - rao) * math.cos(deco) * math.sin(dec) + math.cos(dec) * math.sin(deco)
    T[0][2] = math.sin(ra - rao) * math.cos(dec)
    T[1][2] = -math.cos(ra - rao) * math.sin(deco) * math.cos(dec) + math.sin(dec) * math.cos(deco)
    T[2][2] = math.cos(ra - rao) * math.cos(dec) * math.cos(deco) + math.sin(dec) * math.sin(deco)
    rota = float(np.float32(dtor * vrota3))
    s = np.zeros(9, np.float64)
    if rota != 0.0:
        R = [[math.cos(rota), math.sin(rota), 0.0], [-math.sin(rota), math.cos(rota), 0.0],
             [0.0, 0.0, 1.0]]
        S = [[0.0] * 3 for _ in range(3)]
        for j in range(3):
            for i in range(3):
                acc = 0.0
                for k in range(3):
                    acc = acc + T[k][j] * R[i][k]
                S[i][j] = acc
        for j in range(3):
            for i in range(3):
                acc = 0.0
                for k in range(3):
                    acc = acc + R[j][k] * S[i][k]
                s[i + 3 * j] = acc
    else:
        for j in range(3):
            for i in range(3):
                s[i + 3 * j] = T[i][j]
    return s


class Geom:
    """Image + half-plane grid geometry of one imaging job."""

    def __init__(self, imsize, cellsize, vra=0.0, vdec=40.0, shift=(0.0, 0.0), fov=1.0):
        f32 = np.float32
        PI = f32(3.141592654)
        D2R = f32(PI / f32(180.0))
        n = int(imsize)
        delt_ra = -f32(cellsize) / f32(3600.0)
        delt_dec = f32(cellsize) / f32(3600.0)
        self.nx = self.ny = n
        self.fnu = fftpwr2(n)
        self.nu = self.fnu // 2 + 1
        self.nv = fftpwr2(n)
        cdelt_u = f32(1.0) / (D2R * (f32(fftpwr2(n)) * delt_ra))
        cdelt_v = f32(1.0) / (D2R * (f32(fftpwr2(n)) * delt_dec))
        self.cdelt_u, self.cdelt_v = cdelt_u, cdelt_v
        self.deltx, self.delty = float(delt_ra), float(delt_dec)  # image CDELT, degrees
        self.uscale = f32(1.0) / cdelt_u
        self.vscale = f32(1.0) / cdelt_v
        self.wuscale = f32(fov) / cdelt_u  # GRDUWT: WTFOV / CDELT (grd/grduwt.f:115)
        self.wvscale = f32(fov) / cdelt_v
        self.uorigin = 1
        self.vorigin = int(np.round(f32((self.nv + 1) // 2)))
        self.cenx = self.ceny = float((n + 1) // 2)
        ira = vra + float(f32(shift[0]) / f32(3600.0))
        idec = vdec + float(f32(shift[1]) / f32(3600.0))
        self.shift = crdshift(vra, vdec, ira, idec)
        self.cellsize, self.vra, self.vdec, self.shift_arcsec, self.fov = cellsize, vra, vdec, tuple(shift), fov
        self.pitch = lib().sde_grid_pitch(self.nu)

    def spec(self):
        s = _abi.GridSpec()
        s.nu, s.nv = self.nu, self.nv
        s.uscale, s.uoffset, s.vscale, s.voffset = float(self.uscale), 0.0, float(self.vscale), 0.0
        s.uorigin, s.vorigin, s.supp, s.osamp = self.uorigin, self.vorigin, 3, 128
        s.shift = (C.c_double * 9)(*self.shift)
        return s

    def window(self):
        """CRDNHALF's inner window, 0-based [lo, hi) per axis (crd/crdnhalf.f:39-52)."""
        lo = self.nx // 4 + 1
        length = min(3 * self.nx // 4 - 1 - lo + 1, self.nx // 2 - 1)
        return lo - 1, lo - 1 + length


def _torch():
    import torch
    return torch


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class Context:
    """A libsdegpu context bound to torch's current CUDA stream."""

    def __init__(self, device=0, stream=None):
        """stream: a torch.cuda.Stream for the library's work (default: the current one)."""
        torch = _torch()
        self.torch = torch
        self.device = torch.device("cuda", device)
        torch.cuda.set_device(self.device)
        h = C.c_void_p()
        check(lib().sde_ctx_create(C.byref(h), device), "sde_ctx_create")
        self.h = h
        import weakref
        self._plans = weakref.WeakSet()  # closed before the context goes away
        self.stream = stream if stream is not None else torch.cuda.current_stream(self.device)
        check(lib().sde_ctx_set_stream(h, C.c_void_p(self.stream.cuda_stream)), "set_stream")

    def close(self):
        if self.h:
            for p in list(self._plans):
                p.close()
            lib().sde_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        check(lib().sde_ctx_sync(self.h), "sde_ctx_sync")

    def tensor(self, a, dtype=None):
        t = self.torch.as_tensor(np.ascontiguousarray(a))
        if dtype is not None:
            t = t.to(dtype)
        return t.to(self.device)

    def empty(self, shape, dtype):
        return self.torch.empty(shape, dtype=dtype, device=self.device)

    def zeros(self, shape, dtype):
        return self.torch.zeros(shape, dtype=dtype, device=self.device)

    # -- kernels ---------------------------------------------------------------------------
    def weights(self, geom, u, v, w, wt, rmode="UNIFORM", robust=(0.0, 0.0, 0.0), ds=0.0,
                gwt=None, newwt=None):
        """GRDUWT2D / GRDRUW2D on device arrays; newwt defaults to wt (in place)."""
        st = _abi.WStats()
        rob = (C.c_float * 3)(*[float(x) for x in (list(robust) + [0.0] * 3)[:3]])
        out = wt if newwt is None else newwt
        check(lib().sde_weights(self.h, RMODES[rmode], rob, float(ds), _ptr(wt), _ptr(u), _ptr(v),
                                _ptr(w), int(wt.numel()), float(geom.wuscale), 0.0,
                                float(geom.wvscale), 0.0, geom.uorigin, geom.vorigin, geom.nu,
                                geom.nv, geom.shift.ctypes.data_as(C.c_void_p), _ptr(out),
                                _ptr(gwt), C.byref(st)), "sde_weights")
        return st

    def grid_buffer(self, geom):
        return self.zeros((geom.nv, geom.pitch), self.torch.complex64)

    def image_buffer(self, geom):
        return self.empty((geom.ny, geom.nx), self.torch.float32)

    def image_from_grid(self, geom, grid, image, correct=True, scale_dev=None):
        check(lib().sde_image_from_grid(self.h, _ptr(grid), geom.pitch, geom.nx, geom.ny, geom.fnu,
                                        geom.nv, int(correct), _ptr(scale_dev), _ptr(image)),
              "sde_image_from_grid")
        return image

    def grid_from_image(self, geom, image, grid, correct=True):
        check(lib().sde_grid_from_image(self.h, _ptr(image), geom.nx, geom.ny, geom.fnu, geom.nv,
                                        int(correct), _ptr(grid), geom.pitch),
              "sde_grid_from_image")
        return grid

    def image_max(self, image, out):
        check(lib().sde_image_max(self.h, _ptr(image), int(image.numel()), _ptr(out)), "image_max")
        return out

    def scale_by_inverse(self, image, maxv):
        check(lib().sde_image_scale_by_inverse(self.h, _ptr(image), int(image.numel()), _ptr(maxv)),
              "scale_by_inverse")

    def hogbom(self, drt, psf, niter, gain, flux=0.0, box=None, bsub=1, tflux=0.0,
               cancel_flag=None):
        torch = self.torch
        ny, nx = drt.shape
        pny, pnx = psf.shape
        n = max(abs(niter), 1)
        cln = self.zeros((ny, nx), torch.float32)
        res = self.empty((ny, nx), torch.float32)
        cflux = self.zeros(n, torch.float32)
        cx = self.zeros(n, torch.int32)
        cy = self.zeros(n, torch.int32)
        r = _abi.CleanResult()
        rc = lib().sde_hogbom(self.h, _ptr(drt), _ptr(psf), _ptr(box), nx, ny, pnx, pny,
                              float(gain), int(niter), int(bsub), float(flux), float(tflux),
                              _ptr(cln), _ptr(res), _ptr(cflux), _ptr(cx), _ptr(cy), cancel_flag,
                              C.byref(r))
        if rc not in (_abi.SDE_OK, _abi.SDE_ECANCELLED):
            check(rc, "sde_hogbom")
        return dict(cln=cln, res=res, cflux=cflux, cx=cx, cy=cy, ansub=r.ansub,
                    maxres=r.maxres, tflux=r.tflux, cancelled=rc == _abi.SDE_ECANCELLED)


class Plan:
    """Device-resident, tile-sorted visibilities of one job (sde_plan)."""

    def __init__(self, ctx, geom, u, v, w, vis, wt, opts=None):
        """opts: (item_max, chunk_max) sort-bucket sizes, None for the defaults."""
        self.ctx, self.geom = ctx, geom
        self.nvis_in = int(wt.numel())
        h = C.c_void_p()
        spec = geom.spec()
        if opts is None:
            check(lib().sde_plan_create(ctx.h, C.byref(spec), self.nvis_in, _ptr(u), _ptr(v),
                                        _ptr(w), _ptr(vis), _ptr(wt), _abi.SDE_DEVICE,
                                        C.byref(h)), "sde_plan_create")
        else:
            o = _abi.PlanOpts(int(opts[0]), int(opts[1]))
            check(lib().sde_plan_create_opts(ctx.h, C.byref(spec), self.nvis_in, _ptr(u), _ptr(v),
                                             _ptr(w), _ptr(vis), _ptr(wt), _abi.SDE_DEVICE,
                                             C.byref(o), C.byref(h)), "sde_plan_create_opts")
        self.h = h
        ctx._plans.add(self)

    def close(self):
        if self.h and self.ctx.h:
            lib().sde_plan_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nvis(self):
        return lib().sde_plan_nvis(self.h)

    @property
    def nbytes(self):
        return lib().sde_plan_bytes(self.h)

    def grid(self, out, psf=False):
        sw = C.c_float()
        check(lib().sde_plan_grid(self.h, _abi.SDE_GRID_PSF if psf else _abi.SDE_GRID_VIS,
                                  _ptr(out), self.geom.pitch, C.byref(sw)), "sde_plan_grid")
        return sw.value

    def image(self, image, grid=None, psf=False, correct=True, scale_dev=None, sumwt=False):
        """Dirty image (or PSF) of the plan into image (sde_plan_image: GRDH2D then FFTR2D's
        inverse with PIXCOR2D's correction, divided by scale_dev[0] if given; the finalize
        runs inside the column pass).  grid, if given, receives the column-transformed grid.
        Returns GRDH2D's SUMWT when sumwt (a synchronisation), else None."""
        sw = C.c_float() if sumwt else None
        check(lib().sde_plan_image(self.h, _abi.SDE_GRID_PSF if psf else _abi.SDE_GRID_VIS,
                                   self.geom.nx, self.geom.ny, int(correct),
                                   None if scale_dev is None else _ptr(scale_dev), _ptr(image),
                                   None if grid is None else _ptr(grid), self.geom.pitch,
                                   C.byref(sw) if sumwt else None), "sde_plan_image")
        return sw.value if sumwt else None

    def grid_async(self, out, psf=False):
        check(lib().sde_plan_grid(self.h, _abi.SDE_GRID_PSF if psf else _abi.SDE_GRID_VIS,
                                  _ptr(out), self.geom.pitch, None), "sde_plan_grid")

    def degrid_residual(self, grid):
        check(lib().sde_plan_degrid_residual(self.h, _ptr(grid), self.geom.pitch), "degrid_residual")

    def reset_residual(self):
        check(lib().sde_plan_reset_residual(self.h), "reset_residual")

    def degrid(self, grid, vis_out, wt_out):
        nb = C.c_int64()
        check(lib().sde_plan_degrid(self.h, _ptr(grid), self.geom.pitch, _ptr(vis_out),
                                    _ptr(wt_out), _abi.SDE_DEVICE, C.byref(nb)), "sde_plan_degrid")
        return nb.value

    def residual(self, out):
        check(lib().sde_plan_get_residual(self.h, _ptr(out), _abi.SDE_DEVICE), "get_residual")
        return out

    def set_vis(self, vis):
        check(lib().sde_plan_set_vis(self.h, _ptr(vis), _abi.SDE_DEVICE), "set_vis")


def uvmap(ctx, geom, u, v, w, vis, wt, rmode="UNIFORM", robust=(0.0, 0.0, 0.0), ds=0.0,
          weighting=True):
    """task/uvmap.f: weighting (FOV != 0) -> PSF -> dirty, both divided by the PSF peak.
    Inputs are device tensors; wt is reweighted in place.  Returns dict of device tensors."""
    torch = ctx.torch
    wst = None
    if weighting:
        wst = ctx.weights(geom, u, v, w, wt, rmode=rmode, robust=robust, ds=ds)
    plan = Plan(ctx, geom, u, v, w, vis, wt)
    grid = ctx.grid_buffer(geom)
    psf = ctx.image_buffer(geom)
    dirty = ctx.image_buffer(geom)
    maxpsf = ctx.zeros(1, torch.float32)
    sumwt = plan.image(psf, grid, psf=True, sumwt=True)
    ctx.image_max(psf, maxpsf)
    ctx.scale_by_inverse(psf, maxpsf)
    plan.image(dirty, grid, scale_dev=maxpsf)
    return dict(dirty=dirty, psf=psf, maxpsf=maxpsf, sumwt=sumwt, plan=plan, wstats=wst,
                grid=grid)


def vismodel(ctx, geom, plan, image, vis_out, wt_out):
    """task/vismodel.f:71-73: IMGGRIDC CORRECT -> IMGFFT (r2c) -> VISDEGRI (GRDDEH2D)."""
    grid = ctx.grid_buffer(geom)
    ctx.grid_from_image(geom, image, grid)
    return plan.degrid(grid, vis_out, wt_out)


def image_double(ctx, image, rpix_x, rpix_y):
    """IMGDOUBL (sde_image_double): the image padded to FFTPWR2 of twice each axis, its
    reference pixel moved to about the centre.  Returns (padded image, new rpix_x, rpix_y)."""
    ny, nx = int(image.shape[0]), int(image.shape[1])
    px = fftpwr2(2 * nx) if nx > 1 else 1
    py = fftpwr2(2 * ny) if ny > 1 else 1
    out = ctx.empty((py, px), ctx.torch.float32)
    rp = (C.c_float * 2)()
    check(lib().sde_image_double(ctx.h, _ptr(image), nx, ny, float(rpix_x), float(rpix_y), _ptr(out),
                                 px, py, rp), "sde_image_double")
    return out, rp[0], rp[1]


def padded_geom(geom):
    """The grid geometry IMGTOVIS degrids from (img/imgtovis.f:60-63): FFTCONJA of the image
    padded by IMGDOUBL -- FFTPWR2(2N) pixels at the same cell size, so the uv cells are half
    as large; with uvmap's reference pixel (N+1)/2 the padded one is P/2, this geometry's
    centre."""
    return Geom(fftpwr2(2 * geom.nx), geom.cellsize, vra=geom.vra, vdec=geom.vdec,
                shift=geom.shift_arcsec, fov=geom.fov)


def imgtovis(ctx, geom, plan_padded, image, vis_out, wt_out):
    """img/imgtovis.f:55-84 for a 2-D model image of geom (reference pixel (N+1)/2): IMGDOUBL,
    then IMGGRIDC CORRECT, IMGFFT and VISDEGRI on the padded image's grid.  plan_padded is a
    Plan built on padded_geom(geom) (once per job, like the degrid plan of a major cycle)."""
    pg = plan_padded.geom
    pad, rx, ry = image_double(ctx, image, geom.cenx, geom.ceny)
    if (rx, ry) != (pg.cenx, pg.ceny):
        raise ValueError("imgtovis: the padded reference pixel (%g, %g) is not the padded grid's "
                         "centre (%g, %g)" % (rx, ry, pg.cenx, pg.ceny))
    grid = ctx.grid_buffer(pg)
    ctx.grid_from_image(pg, pad, grid)
    return plan_padded.degrid(grid, vis_out, wt_out)


def components_image(ctx, geom, cln_window):
    """Place a CLEAN window's component image back in a full-size image."""
    lo, hi = geom.window()
    img = ctx.zeros((geom.ny, geom.nx), ctx.torch.float32)
    img[lo:hi, lo:hi] = cln_window
    return img


def hogbom(ctx, geom, dirty, psf, niter, gain=0.1, flux=0.0):
    """task/clean.f HOGBOM path: CRDNHALF window of the dirty image, full PSF."""
    lo, hi = geom.window()
    drt = dirty[lo:hi, lo:hi].contiguous()
    return ctx.hogbom(drt, psf, niter, gain, flux)


def weights_ungridded(ctx, geom, u, v, w, wt, rmode="NORM", robust=0.0, ds=0.0, wtfov=1.0, nbu=0, nbv=0):
    """uvmap's slow weighting (GRDURUWT with GRDURUW2, sde_weights_ungridded) on host arrays:
    the weighting plane's cell (IDELT) is the gridding plane's 1/uscale, 1/vscale.  Returns
    (newwt, stats dict)."""
    n = len(wt)
    f32 = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
    u, v, w, wt = f32(u), f32(v), f32(w), f32(wt)
    newwt = np.empty(n, np.float32)
    st = _abi.UruwtStats()
    rob = (C.c_float * 3)(float(robust), 0.0, 0.0)
    shift = np.ascontiguousarray(geom.shift, np.float64)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    check(lib().sde_weights_ungridded(ctx.h, n, p(u), p(v), p(w), p(wt), float(1.0 / geom.uscale),
                                      float(1.0 / geom.vscale), float(wtfov),
                                      {"NORM": 1, "ABS": 2, "NONE": 3}[rmode], rob, float(ds), p(shift),
                                      int(nbu), int(nbv), p(newwt), C.byref(st)), "sde_weights_ungridded")
    return newwt, {k: getattr(st, k) for k, _ in st._fields_}


def model_image(ctx, comps, nx, ny, refx, deltx, refy, delty, image=None):
    """MODIMG2D (sde_model_image): comps = [(type, flux, ra, dec, bmaj, bmin, bpa), ...] with
    offsets/axes in arcsec and the position angle in degrees, added into image (a zeroed
    device image by default); deltx/delty arcsec per pixel."""
    if image is None:
        image = ctx.zeros((ny, nx), ctx.torch.float32)
    n = len(comps)
    types = "".join(str(c[0])[:4].ljust(4) for c in comps).encode()
    cols = [np.ascontiguousarray([float(c[j]) for c in comps], np.float32) for j in range(1, 7)]
    ptr = [a.ctypes.data_as(C.c_void_p) for a in cols]
    check(lib().sde_model_image(ctx.h, n, types, *ptr, nx, ny, float(refx), float(deltx), float(refy),
                                float(delty), _ptr(image)), "sde_model_image")
    return image


def dft_image(ctx, u, v, vis, wt, nx, ny, refx, deltx, refy, delty, dirty=True, psf=True):
    """VISDFT3D (2-D) on device tensors (sde_dft_image): dict(dirty, psf) [ny][nx]."""
    torch = ctx.torch
    out = {"dirty": ctx.empty((ny, nx), torch.float32) if dirty else None,
           "psf": ctx.empty((ny, nx), torch.float32) if psf else None}
    check(lib().sde_dft_image(ctx.h, int(wt.numel()), _ptr(u), _ptr(v), _ptr(vis), _ptr(wt), nx, ny,
                              float(refx), float(deltx), float(refy), float(delty),
                              _ptr(out["dirty"]), _ptr(out["psf"])), "sde_dft_image")
    return out


def dft_vis(ctx, image, refx, deltx, refy, delty, u, v, wt, vis):
    """IMGDFT2D on device tensors (sde_dft_vis): vis (complex64) updated where wt > 0."""
    ny, nx = int(image.shape[0]), int(image.shape[1])
    check(lib().sde_dft_vis(ctx.h, _ptr(image), nx, ny, float(refx), float(deltx), float(refy),
                            float(delty), int(wt.numel()), _ptr(u), _ptr(v), _ptr(wt), _ptr(vis)),
          "sde_dft_vis")
    return vis


def uvmap_dft(ctx, geom, u, v, vis, wt):
    """uvmap with DFT = T (task/uvmap.f:416-418): VISDFT into the image geometry (CDELT =
    -/+ CELLSIZE/3600, CRPIX = (N+1)/2), normalised by the sum of weights."""
    return dft_image(ctx, u, v, vis, wt, geom.nx, geom.ny, geom.cenx, geom.deltx, geom.ceny,
                     geom.delty)


def clark(ctx, dirty, psf, niter=100, gain=0.1, flux=0.0, numcl=32768, bpatch=128, box=None,
          comp=None, biter=1):
    """task/clean.f CLARK path with IMGCCLEA (sde_clark): N x N dirty image and PSF (device
    tensors) -> components and residual over CRDHALF's N/2 window, the component list, and
    the per-major-cycle trace (ANL, ANITER, MAXRES, TFLUX).  The defaults are clean.inf's."""
    torch = ctx.torch
    n = int(dirty.shape[0])
    w = n // 2
    if comp is None:
        comp = ctx.zeros((w, w), torch.float32)
    resid = ctx.empty((w, w), torch.float32)
    cl = ctx.zeros(niter, torch.float32)
    cx = ctx.zeros(niter, torch.int32)
    cy = ctx.zeros(niter, torch.int32)
    p = _abi.ClarkParams(int(niter), float(gain), float(flux), int(numcl), int(bpatch), int(biter))
    r = _abi.ClarkResult()
    check(lib().sde_clark(ctx.h, _ptr(dirty), _ptr(psf), n, _ptr(box), C.byref(p), _ptr(comp),
                          _ptr(resid), _ptr(cl), _ptr(cx), _ptr(cy), C.byref(r)), "sde_clark")
    out = dict(comp=comp, resid=resid, cl=cl, cx=cx, cy=cy)
    out.update({k: getattr(r, k) for k, _ in r._fields_ if not k.startswith("t_")})
    nc = min(r.ncycles, 64)
    out["trace"] = [(r.t_anl[i], r.t_aniter[i], r.t_maxres[i], r.t_tflux[i]) for i in range(nc)]
    return out


class MajorCycle:
    """One CLEAN major cycle as the reference composes it (task/mosclean.f:227-364):
    grid the residual -> dirty image -> Hogbom minor cycle -> model image -> degrid ->
    residual = observed - model.  Everything stays on the device."""

    def __init__(self, ctx, geom, plan, maxpsf, psf):
        self.ctx, self.geom, self.plan = ctx, geom, plan
        self.maxpsf, self.psf = maxpsf, psf
        self.grid = ctx.grid_buffer(geom)
        self.mgrid = ctx.grid_buffer(geom)
        self.dirty = ctx.image_buffer(geom)
        self.model = ctx.zeros((geom.ny, geom.nx), ctx.torch.float32)

    def grid_step(self):
        self.plan.image(self.dirty, self.grid, scale_dev=self.maxpsf)
        return self.dirty

    def degrid_step(self, model_image):
        self.ctx.grid_from_image(self.geom, model_image, self.mgrid)
        self.plan.degrid_residual(self.mgrid)

    def run(self, niter, gain=0.1, flux=0.0):
        self.grid_step()
        r = hogbom(self.ctx, self.geom, self.dirty, self.psf, niter, gain, flux)
        self.model += components_image(self.ctx, self.geom, r["cln"])
        self.degrid_step(self.model)
        return r
