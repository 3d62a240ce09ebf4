"""ctypes bindings for the CPU oracle (oracle/sde_oracle.c).

TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs
import this module.  The product package (sde_gb300) never imports it.

Every wrapper takes/returns numpy arrays in the reference's layouts: images [ny][nx]
float32 (Fortran IMAGE(NX,NY) column-major == C row-major [NY][NX]), grids [nv][nu]
complex64, visibilities complex64, coordinates float32 wavelengths.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
c64p = np.ctypeslib.ndpointer(np.complex64, flags="C_CONTIGUOUS")
c128p = np.ctypeslib.ndpointer(np.complex128, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")

RMODES = {"NONE": 0, "NORM": 1, "ABS": 2, "AZ-NORM": 3}


class UvmapParams(C.Structure):
    _fields_ = [("imsize", C.c_int), ("cellsize", C.c_float), ("fov", C.c_float),
                ("rmode", C.c_int), ("robust", C.c_float * 3), ("ds", C.c_float),
                ("vra", C.c_double), ("vdec", C.c_double),
                ("shift_ra", C.c_float), ("shift_dec", C.c_float)]


class Geom(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("fnu", C.c_int), ("nu", C.c_int),
                ("nv", C.c_int), ("uscale", C.c_float), ("vscale", C.c_float),
                ("uorigin", C.c_int), ("vorigin", C.c_int), ("cenx", C.c_float),
                ("ceny", C.c_float), ("shift", C.c_double * 9)]


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(
                os.path.join(_HERE, "sde_oracle.c")):
            build()
        L = C.CDLL(_LIB)
        L.orc_grdsf.restype = C.c_double
        L.orc_grdsf.argtypes = [C.c_double]
        L.orc_fftpwr2.restype = C.c_int
        L.orc_grdcf.argtypes = [C.c_int, f32p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.orc_grdccf.argtypes = [C.c_int, f32p, C.c_int]
        L.orc_crdshift.argtypes = [C.c_double] * 4 + [C.c_float, f64p]
        common = [f32p, f32p, f32p, f32p, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                  C.c_int, C.c_int]
        L.orc_grduwt2d.argtypes = common + [f32p, f32p, C.c_int, C.c_int, f64p,
                                            C.POINTER(C.c_int)]
        L.orc_grdruw2d.argtypes = common + [f32p, f32p, C.c_int, C.c_int, f64p, C.c_char_p,
                                            f32p, C.c_float, C.POINTER(C.c_int),
                                            C.POINTER(C.c_double), C.POINTER(C.c_double),
                                            C.POINTER(C.c_float)]
        L.orc_grdh2d.argtypes = [c64p, f32p, f32p, f32p, f32p, C.c_int, C.c_float, C.c_float,
                                 C.c_float, C.c_float, C.c_int, C.c_int, c64p, C.c_int, C.c_int,
                                 C.c_int, f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_int, f64p,
                                 C.POINTER(C.c_float), C.POINTER(C.c_double)]
        L.orc_grddeh2d.argtypes = [c64p, f32p, f32p, f32p, f32p, C.c_int, C.c_float, C.c_float,
                                   C.c_float, C.c_float, C.c_int, C.c_int, c64p, C.c_int,
                                   C.c_int, f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_int,
                                   f64p, C.POINTER(C.c_int)]
        L.orc_fftr2d.argtypes = [f32p, c64p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_fftx.argtypes = [c64p, c64p, C.c_int, C.c_int]
        L.orc_pixcor2d.argtypes = [f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_int, f32p,
                                   C.c_float, C.c_float]
        L.orc_pixisama.restype = C.c_int
        L.orc_pixisama.argtypes = [C.c_int, f32p, C.c_int]
        L.orc_pix2drcl.argtypes = [f32p, f32p, f32p, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_float, C.c_int, C.c_int, C.c_float, f32p, f32p,
                                   C.POINTER(C.c_int), C.POINTER(C.c_float),
                                   C.POINTER(C.c_float), f32p, i32p, i32p]
        L.orc_visdft2d.restype = C.c_int
        L.orc_visdft2d.argtypes = [c64p, C.c_int, f32p, f32p, f32p, f32p, f32p, C.c_int, C.c_int,
                                   C.c_float, C.c_float, C.c_float, C.c_float]
        L.orc_imgdft2d.argtypes = [f32p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                   c64p, C.c_int, f32p, f32p, f32p]
        L.orc64_visdft2d.restype = C.c_int
        L.orc64_visdft2d.argtypes = [c64p, C.c_int, f32p, f32p, f32p, f64p, f64p, C.c_int, C.c_int,
                                     C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc64_imgdft2d.argtypes = [f32p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                     C.c_double, c128p, C.c_int, f32p, f32p, f32p]
        L.orc_grduruwt.restype = C.c_int
        L.orc_grduruwt.argtypes = [f32p, f32p, f32p, f32p, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int,
                                   C.c_float, C.c_float, f64p, C.c_int, C.c_int, f32p, f64p]
        L.orc_grdh23d.restype = C.c_int
        L.orc_grdh23d.argtypes = [c64p, f32p, f32p, f32p, f32p, C.c_int, C.c_float, C.c_float, C.c_float,
                                  C.c_float, C.c_int, C.c_int, c64p, C.c_int, C.c_int, C.c_int, f32p, C.c_int,
                                  C.c_int, f32p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, f64p,
                                  C.POINTER(C.c_float)]
        L.orc_grddeh23.restype = C.c_int
        L.orc_grddeh23.argtypes = [c64p, f32p, f32p, f32p, f32p, C.c_int, C.c_float, C.c_float, C.c_float,
                                   C.c_float, C.c_int, C.c_int, c64p, C.c_int, C.c_int, f32p, C.c_int, C.c_int,
                                   f32p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, f64p]
        L.orc_grdqh2d.restype = C.c_int
        L.orc_grdqh2d.argtypes = [c64p, f32p, f32p, f32p, f32p, C.c_int, C.c_float, C.c_float, C.c_float,
                                  C.c_float, C.c_int, C.c_int, c64p, C.c_int, C.c_int, C.c_int, f64p,
                                  C.POINTER(C.c_float)]
        L.orc_modimg2d.restype = C.c_int
        L.orc_modimg2d.argtypes = [C.c_int, i32p, f32p, f32p, f32p, f32p, f32p, f32p, f32p, C.c_int,
                                   C.c_int, C.c_float, C.c_float, C.c_float, C.c_float]
        L.orc_clark.restype = C.c_int
        L.orc_clark.argtypes = [f32p, f32p, C.c_int, C.c_void_p, C.POINTER(ClarkParams), f32p, f32p,
                                f32p, i32p, i32p, C.POINTER(ClarkResult)]
        L.orc_make_geom.argtypes = [C.POINTER(UvmapParams), C.POINTER(Geom)]
        L.orc_uvmap.argtypes = [C.POINTER(UvmapParams), C.c_int, f32p, f32p, f32p, c64p, f32p,
                                f32p, f32p, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_vismodel.argtypes = [C.POINTER(UvmapParams), C.c_int, f32p, f32p, f32p, c64p,
                                   f32p, f32p]
        L.orc64_uvmap_image.argtypes = [C.POINTER(Geom), C.c_int, f32p, f32p, f32p, c64p, f32p,
                                        C.c_int, f64p]
        L.orc_point_vis_mt.argtypes = [C.c_int64, f32p, f32p, C.c_int, f64p, f64p, f64p, c64p, C.c_int]
        L.orc_grdh2d_acc.argtypes = [c64p, f32p, f32p, f32p, f32p, C.c_int, C.c_int, C.c_float, C.c_float,
                                     C.c_float, C.c_float, C.c_int, C.c_int, c64p, C.c_int, C.c_int,
                                     C.c_int, f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_int, f64p,
                                     C.POINTER(C.c_float), C.POINTER(C.c_double)]
        L.orc_grdh2d_end.restype = C.c_int
        L.orc_grdh2d_end.argtypes = [c64p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double]
        L.orc_imgdoubl.argtypes = [f32p, C.c_int, C.c_int, C.c_float, C.c_float, f32p, C.POINTER(C.c_int),
                                   C.POINTER(C.c_int), C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_imgtovis.argtypes = [C.POINTER(UvmapParams), C.c_int, f32p, f32p, f32p, c64p, f32p, f32p]
        L.orc64_uvmap_image_mt.argtypes = [C.POINTER(Geom), C.c_int, f32p, f32p, f32p, c64p,
                                           f32p, C.c_int, f64p, C.c_int]
        L.orc64_fftr2d_inv.argtypes = [c128p, f64p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc64_dft_image.argtypes = [C.POINTER(Geom), C.c_int, f32p, f32p, c64p, f32p,
                                      C.c_int, f64p]
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.complex64)


def params(imsize, cellsize, fov=1.0, rmode="NONE", robust=(0.0, 0.0, 0.0), ds=0.0,
           vra=0.0, vdec=40.0, shift=(0.0, 0.0)):
    p = UvmapParams()
    p.imsize, p.cellsize, p.fov, p.rmode = imsize, cellsize, fov, RMODES[rmode]
    p.robust = (C.c_float * 3)(*robust)
    p.ds, p.vra, p.vdec = ds, vra, vdec
    p.shift_ra, p.shift_dec = shift
    return p


def geom(p):
    g = Geom()
    lib().orc_make_geom(C.byref(p), C.byref(g))
    return g


def grdcf():
    cf = np.zeros(1 + 8 * 129, np.float32)
    s, o = C.c_int(), C.c_int()
    lib().orc_grdcf(1, cf, C.byref(s), C.byref(o))
    return cf, s.value, o.value


def grdccf(ccflen):
    ccf = np.zeros(ccflen, np.float32)
    lib().orc_grdccf(1, ccf, ccflen)
    return ccf


def crdshift(vra, vdec, ira, idec, rota=0.0):
    s = np.zeros(9, np.float64)
    lib().orc_crdshift(vra, vdec, ira, idec, rota, s)
    return s


def grduwt2d(wt, u, v, w, uscale, vscale, uorigin, vorigin, nu, nv, shift,
             uoffset=0.0, voffset=0.0):
    wt = _f32(wt)
    newwt = np.empty_like(wt)
    gwt = np.zeros((nv, nu), np.float32)
    nd = C.c_int()
    lib().orc_grduwt2d(wt, _f32(u), _f32(v), _f32(w), len(wt), uscale, uoffset, vscale,
                       voffset, uorigin, vorigin, newwt, gwt, nu, nv,
                       np.ascontiguousarray(shift, np.float64), C.byref(nd))
    return newwt, gwt, nd.value


def grdruw2d(wt, u, v, w, uscale, vscale, uorigin, vorigin, nu, nv, shift, rmode,
             robust, ds=0.0, uoffset=0.0, voffset=0.0):
    wt = _f32(wt)
    newwt = np.empty_like(wt)
    gwt = np.zeros((nv, nu), np.float32)
    nd, sw, slw, f2 = C.c_int(), C.c_double(), C.c_double(), C.c_float()
    rc = lib().orc_grdruw2d(wt, _f32(u), _f32(v), _f32(w), len(wt), uscale, uoffset, vscale,
                            voffset, uorigin, vorigin, newwt, gwt, nu, nv,
                            np.ascontiguousarray(shift, np.float64), rmode.encode(),
                            _f32(list(robust) + [0.0] * (3 - len(robust))), ds, C.byref(nd),
                            C.byref(sw), C.byref(slw), C.byref(f2))
    return rc, newwt, gwt, nd.value, sw.value, slw.value, f2.value


def grdh2d(vis, wt, u, v, w, uscale, vscale, uorigin, vorigin, nu, nv, shift, psf=False,
           cf=None, supp=3, osamp=128, uoffset=0.0, voffset=0.0):
    if cf is None:
        cf, supp, osamp = grdcf()
    gvis = np.zeros((nv, nu), np.complex64)
    sw, lsw = C.c_float(), C.c_double()
    rc = lib().orc_grdh2d(_c64(vis), _f32(wt), _f32(u), _f32(v), _f32(w), len(wt), uscale,
                          uoffset, vscale, voffset, uorigin, vorigin, gvis, int(psf), nu, nv,
                          cf, supp, osamp, cf, supp, osamp,
                          np.ascontiguousarray(shift, np.float64), C.byref(sw), C.byref(lsw))
    return rc, gvis, sw.value, lsw.value


def grddeh2d(vis, wt, u, v, w, uscale, vscale, uorigin, vorigin, gvis, shift, cf=None,
             supp=3, osamp=128, uoffset=0.0, voffset=0.0):
    """Returns (vis_out, wt_out, nbad); inputs are not modified."""
    if cf is None:
        cf, supp, osamp = grdcf()
    vis = _c64(vis).copy()
    wt = _f32(wt).copy()
    nv, nu = gvis.shape
    nb = C.c_int()
    lib().orc_grddeh2d(vis, wt, _f32(u), _f32(v), _f32(w), len(wt), uscale, uoffset, vscale,
                       voffset, uorigin, vorigin, _c64(gvis), nu, nv, cf, supp, osamp, cf,
                       supp, osamp, np.ascontiguousarray(shift, np.float64), C.byref(nb))
    return vis, wt, nb.value


def fftr2d(nx, ny, fnu, nv, direction, rarray=None, xarray=None):
    """DIR=-1: xarray [nv][fnu/2+1] -> image [ny][nx]; DIR=+1: image -> grid."""
    nu = fnu // 2 + 1
    r = np.zeros((ny, nx), np.float32) if rarray is None else _f32(rarray).copy()
    x = np.zeros((nv, nu), np.complex64) if xarray is None else _c64(xarray).copy()
    lib().orc_fftr2d(r, x, nx, ny, fnu, nv, direction)
    return r, x


def fftx(x, isig):
    x = _c64(x).copy()
    wk = np.zeros_like(x)
    lib().orc_fftx(x, wk, len(x), isig)
    return x


def pixcor2d(img, ccf, cenx, ceny, correct=True):
    img = _f32(img)
    out = np.empty_like(img)
    ny, nx = img.shape
    lib().orc_pixcor2d(img, nx, ny, _f32(ccf), len(ccf), int(correct), out, cenx, ceny)
    return out


def pixisama(a):
    a = _f32(a).ravel()
    return lib().orc_pixisama(len(a), a, 1)


def pix2drcl(drt, psf, box, gain, nsub, bsub=1, flux=0.0, tflux=0.0):
    drt, psf, box = _f32(drt), _f32(psf), _f32(box)
    ny, nx = drt.shape
    pny, pnx = psf.shape
    cln = np.zeros_like(drt)
    res = np.zeros_like(drt)
    n = abs(nsub)
    cflux = np.zeros(max(n, 1), np.float32)
    cx = np.zeros(max(n, 1), np.int32)
    cy = np.zeros(max(n, 1), np.int32)
    ansub, maxres, tf = C.c_int(), C.c_float(), C.c_float(tflux)
    lib().orc_pix2drcl(drt, psf, box, nx, ny, pnx, pny, gain, nsub, bsub, flux, cln, res,
                       C.byref(ansub), C.byref(maxres), C.byref(tf), cflux, cx, cy)
    return dict(cln=cln, res=res, ansub=ansub.value, maxres=maxres.value, tflux=tf.value,
                cflux=cflux, cx=cx, cy=cy)


class ClarkParams(C.Structure):
    _fields_ = [("niter", C.c_int), ("gain", C.c_float), ("flux", C.c_float), ("numcl", C.c_int),
                ("bpatch", C.c_int)]


class ClarkResult(C.Structure):
    _fields_ = [("aniter", C.c_int), ("ncycles", C.c_int), ("window", C.c_int), ("blc", C.c_int),
                ("last_anl", C.c_int), ("maxres", C.c_float), ("tflux", C.c_float),
                ("extside", C.c_float), ("last_slim", C.c_float),
                ("t_anl", C.c_int * 64), ("t_aniter", C.c_int * 64),
                ("t_maxres", C.c_float * 64), ("t_tflux", C.c_float * 64)]


def clark(dirty, psf, niter=100, gain=0.1, flux=0.0, numcl=32768, bpatch=128, box=None):
    """Clark CLEAN of an N x N dirty image (task/clean.f CLARK branch + img/imgcclea.f).
    Returns dict(comp, resid (window w x w), cl, cx, cy, rc, and the result fields)."""
    dirty, psf = _f32(dirty), _f32(psf)
    n = dirty.shape[0]
    w = n // 2
    comp = np.zeros((w, w), np.float32)
    resid = np.zeros((w, w), np.float32)
    cl = np.zeros(niter, np.float32)
    cx = np.zeros(niter, np.int32)
    cy = np.zeros(niter, np.int32)
    p = ClarkParams(niter, gain, flux, numcl, bpatch)
    r = ClarkResult()
    boxp = None
    if box is not None:
        box = _f32(box)
        boxp = box.ctypes.data_as(C.c_void_p)
    rc = lib().orc_clark(dirty, psf, n, boxp, C.byref(p), comp, resid, cl, cx, cy, C.byref(r))
    out = dict(comp=comp, resid=resid, cl=cl, cx=cx, cy=cy, rc=rc)
    out.update({k: getattr(r, k) for k, _ in r._fields_ if not k.startswith("t_")})
    nc = min(r.ncycles, 64)
    out["trace"] = [(r.t_anl[i], r.t_aniter[i], r.t_maxres[i], r.t_tflux[i]) for i in range(nc)]
    return out


def visdft2d(vis, wt, u, v, nx, ny, refx, deltx, refy, delty, fp64=False):
    """VISDFT3D (2-D): (image, psf, rc); fp64 = exact phases in double."""
    vis, wt, u, v = _c64(vis), _f32(wt), _f32(u), _f32(v)
    dt = np.float64 if fp64 else np.float32
    img = np.zeros((ny, nx), dt)
    psf = np.zeros((ny, nx), dt)
    f = lib().orc64_visdft2d if fp64 else lib().orc_visdft2d
    rc = f(vis, len(wt), wt, u, v, img, psf, nx, ny, refx, deltx, refy, delty)
    return img, psf, rc


def imgdft2d(image, refx, deltx, refy, delty, wt, u, v, vis_in=None, fp64=False):
    """IMGDFT2D: visibilities of a model image; points with WT <= 0 keep vis_in."""
    image, wt, u, v = _f32(image), _f32(wt), _f32(u), _f32(v)
    ny, nx = image.shape
    if fp64:
        vis = np.zeros(len(wt), np.complex128) if vis_in is None else np.asarray(vis_in, np.complex128).copy()
        lib().orc64_imgdft2d(image, nx, ny, refx, deltx, refy, delty, vis, len(wt), wt, u, v)
    else:
        vis = np.zeros(len(wt), np.complex64) if vis_in is None else _c64(vis_in).copy()
        lib().orc_imgdft2d(image, nx, ny, refx, deltx, refy, delty, vis, len(wt), wt, u, v)
    return vis


def grdqh2d(vis, wt, u, v, w, g, psf=False):
    """GRDQH2D with the geometry g (orc_geom): (grid [nv][nu] complex64, sumwt, rc)."""
    grid = np.zeros((g.nv, g.nu), np.complex64)
    sw = C.c_float()
    shift = np.ascontiguousarray(np.array(list(g.shift), np.float64))
    rc = lib().orc_grdqh2d(_c64(vis), _f32(wt), _f32(u), _f32(v), _f32(w), len(wt), g.uscale, 0.0, g.vscale, 0.0,
                           g.uorigin, g.vorigin, grid, int(psf), g.nu, g.nv, shift, C.byref(sw))
    return grid, sw.value, rc


def grduruwt(u, v, w, wt, idelt_u, idelt_v, shift, wtfov=1.0, rmode="NORM", robust=0.0, ds=0.0, nbu=0, nbv=0):
    """GRDURUWT/GRDURUW2: (newwt, rc, stats dict)."""
    newwt = np.zeros(len(wt), np.float32)
    st = np.zeros(7, np.float64)
    rc = lib().orc_grduruwt(_f32(u), _f32(v), _f32(w), _f32(wt), len(wt), idelt_u, idelt_v, wtfov,
                            {"NORM": 1, "ABS": 2, "NONE": 3}[rmode], robust, ds,
                            np.ascontiguousarray(shift, np.float64), nbu, nbv, newwt, st)
    keys = ("nbu", "nbv", "ndrop", "nsel", "uradius", "vradius", "f2")
    return newwt, rc, dict(zip(keys, st.tolist()))


def grdh23d(vis, wt, u, v, w, g, cf, nz, cellz, refz, psf=False):
    """GRDH23D with geometry g and the SF table cf: (grid [nz][nv][nu] complex64, sumwt, rc)."""
    grid = np.zeros((nz, g.nv, g.nu), np.complex64)
    sw = C.c_float()
    shift = np.ascontiguousarray(np.array(list(g.shift), np.float64))
    rc = lib().orc_grdh23d(_c64(vis), _f32(wt), _f32(u), _f32(v), _f32(w), len(wt), g.uscale, 0.0, g.vscale, 0.0,
                           g.uorigin, g.vorigin, grid, int(psf), g.nu, g.nv, _f32(cf), 3, 128, _f32(cf), 3, 128,
                           nz, cellz, refz, shift, C.byref(sw))
    return grid, sw.value, rc


def grddeh23(vis, wt, u, v, w, g, cf, grid, cellz, refz):
    """GRDDEH23: (vis, wt, nbad) with the model cube grid [nz][nv][nu]."""
    vis = _c64(vis).copy()
    wt = _f32(wt).copy()
    shift = np.ascontiguousarray(np.array(list(g.shift), np.float64))
    nz = grid.shape[0]
    nbad = lib().orc_grddeh23(vis, wt, _f32(u), _f32(v), _f32(w), len(wt), g.uscale, 0.0, g.vscale, 0.0, g.uorigin,
                              g.vorigin, np.ascontiguousarray(grid, np.complex64), g.nu, g.nv, _f32(cf), 3, 128,
                              _f32(cf), 3, 128, nz, cellz, refz, shift)
    return vis, wt, nbad


MODEL_TYPES = ["POIN", "GAUS", "DISK", "RECT", "SPHE", "SHEL", "PLOR"]


def modimg2d(comps, nx, ny, refx, deltx, refy, delty, image=None):
    """comps: list of (type, flux, ra, dec, bmaj, bmin, bpa), offsets/sizes in arcsec.
    Returns (image, rc)."""
    img = np.zeros((ny, nx), np.float32) if image is None else _f32(image).copy()
    col = lambda j: np.array([c[j] for c in comps], np.float32)  # noqa: E731
    types = np.array([MODEL_TYPES.index(c[0][:4]) for c in comps], np.int32)
    rc = lib().orc_modimg2d(len(comps), types, col(1), col(2), col(3), col(4), col(5), col(6), img, nx, ny,
                            refx, deltx, refy, delty)
    return img, rc


def uvmap(p, u, v, w, vis, wt):
    """Returns (dirty, psf, wt_after_weighting, maxpsf, sumwt, rc)."""
    wt = _f32(wt).copy()
    dirty = np.zeros((p.imsize, p.imsize), np.float32)
    psf = np.zeros_like(dirty)
    mx, sw = C.c_float(), C.c_float()
    rc = lib().orc_uvmap(C.byref(p), len(wt), _f32(u), _f32(v), _f32(w), _c64(vis), wt, dirty,
                         psf, C.byref(mx), C.byref(sw))
    return dirty, psf, wt, mx.value, sw.value, rc


def vismodel(p, u, v, w, vis, wt, image):
    vis = _c64(vis).copy()
    wt = _f32(wt).copy()
    lib().orc_vismodel(C.byref(p), len(wt), _f32(u), _f32(v), _f32(w), vis, wt, _f32(image))
    return vis, wt


def imgdoubl(img, rpix_x, rpix_y):
    """IMGDOUBL/PIXRPAD: (padded image [py][px], new rpix_x, new rpix_y)."""
    img = _f32(img)
    ny, nx = img.shape
    pn = [max(1, fftpwr2_host(2 * nx)) if nx > 1 else 1, max(1, fftpwr2_host(2 * ny)) if ny > 1 else 1]
    out = np.zeros((pn[1], pn[0]), np.float32)
    px, py, rx, ry = C.c_int(), C.c_int(), C.c_float(), C.c_float()
    lib().orc_imgdoubl(img, nx, ny, rpix_x, rpix_y, out, C.byref(px), C.byref(py), C.byref(rx), C.byref(ry))
    assert (px.value, py.value) == (pn[0], pn[1])
    return out, rx.value, ry.value


def fftpwr2_host(i):
    return lib().orc_fftpwr2(int(i))


def imgtovis(p, u, v, w, vis, wt, image):
    """IMGTOVIS: the model image padded (IMGDOUBL) and degridded from the padded grid."""
    vis = _c64(vis).copy()
    wt = _f32(wt).copy()
    lib().orc_imgtovis(C.byref(p), len(wt), _f32(u), _f32(v), _f32(w), vis, wt, _f32(image))
    return vis, wt


def uvmap_image64(g, u, v, w, vis, wt, psf):
    img = np.zeros((g.ny, g.nx), np.float64)
    lib().orc64_uvmap_image(C.byref(g), len(wt), _f32(u), _f32(v), _f32(w), _c64(vis),
                            _f32(wt), int(psf), img)
    return img


def point_vis(u, v, flux, l, m, nthreads=None):
    """sum_k S_k exp(+2 pi i (u l_k + v m_k)) in double -> complex64, on host threads."""
    nthreads = nthreads or max(1, min(os.cpu_count() or 1, 64))
    u, v = _f32(u), _f32(v)
    out = np.empty(len(u), np.complex64)
    f64 = lambda a: np.ascontiguousarray(a, np.float64)  # noqa: E731
    lib().orc_point_vis_mt(len(u), u, v, len(flux), f64(flux), f64(l), f64(m), out, int(nthreads))
    return out


class Grdh2dParts:
    """GRDH2D over consecutive visibility ranges (orc_grdh2d_acc / orc_grdh2d_end): the grid
    equals one orc_grdh2d call over all of them."""

    def __init__(self, g, cf=None, psf=False):
        if cf is None:
            cf, _, _ = grdcf()
        self.g, self.cf, self.psf = g, cf, int(psf)
        self.grid = np.zeros((g.nv, g.nu), np.complex64)
        self.sw, self.lsw = C.c_float(0.0), C.c_double(0.0)
        self.shift = np.ascontiguousarray(np.array(list(g.shift)), np.float64)

    def add(self, vis, wt, u, v, w, i0, i1):
        g = self.g
        lib().orc_grdh2d_acc(_c64(vis), _f32(wt), _f32(u), _f32(v), _f32(w), int(i0), int(i1),
                             g.uscale, 0.0, g.vscale, 0.0, g.uorigin, g.vorigin, self.grid,
                             self.psf, g.nu, g.nv, self.cf, 3, 128, self.cf, 3, 128, self.shift,
                             C.byref(self.sw), C.byref(self.lsw))

    def end(self):
        g = self.g
        return lib().orc_grdh2d_end(self.grid, g.nu, g.nv, g.uorigin, g.vorigin, 3, self.lsw.value)


def uvmap_image64_mt(g, u, v, w, vis, wt, psf, nthreads=None):
    """uvmap_image64 on host threads (the same grid; used at full benchmark sizes)."""
    nthreads = nthreads or max(1, min(os.cpu_count() or 1, 64))
    img = np.zeros((g.ny, g.nx), np.float64)
    lib().orc64_uvmap_image_mt(C.byref(g), len(wt), _f32(u), _f32(v), _f32(w), _c64(vis),
                               _f32(wt), int(psf), img, int(nthreads))
    return img


def fftr2d_inv64(xarray, nx, ny, fnu, nv):
    img = np.zeros((ny, nx), np.float64)
    lib().orc64_fftr2d_inv(np.ascontiguousarray(xarray, np.complex128), img, nx, ny, fnu, nv)
    return img


def dft_image64(g, u, v, vis, wt, psf):
    img = np.zeros((g.ny, g.nx), np.float64)
    lib().orc64_dft_image(C.byref(g), len(wt), _f32(u), _f32(v), _c64(vis), _f32(wt),
                          int(psf), img)
    return img
