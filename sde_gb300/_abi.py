"""ctypes declarations of libsdegpu's C ABI (include/sde_gpu.h).

The library is built in-tree (sde_gb300/_lib/libsdegpu.so).  Loading it never touches the
GPU; a missing library is an error, never a silent fallback.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libsdegpu.so")

SDE_OK, SDE_EINVAL, SDE_ENOMEM, SDE_ECUDA, SDE_ENOWEIGHT = 0, 1, 2, 3, 4
SDE_ETIMEDOUT, SDE_EBADMODE, SDE_ENODEV, SDE_ECANCELLED = 5, 6, 7, 8
SDE_HOST, SDE_DEVICE = 0, 1
SDE_GRID_VIS, SDE_GRID_PSF = 0, 1

_NAMES = {0: "SDE_OK", 1: "SDE_EINVAL", 2: "SDE_ENOMEM", 3: "SDE_ECUDA", 4: "SDE_ENOWEIGHT",
          5: "SDE_ETIMEDOUT", 6: "SDE_EBADMODE", 7: "SDE_ENODEV", 8: "SDE_ECANCELLED"}


class SdeError(RuntimeError):
    def __init__(self, code, where, text):
        super().__init__("%s failed: %s (%s)" % (where, _NAMES.get(code, code), text))
        self.code = code


class GridSpec(C.Structure):
    _fields_ = [("nu", C.c_int), ("nv", C.c_int), ("uscale", C.c_float), ("uoffset", C.c_float),
                ("vscale", C.c_float), ("voffset", C.c_float), ("uorigin", C.c_int),
                ("vorigin", C.c_int), ("supp", C.c_int), ("osamp", C.c_int),
                ("shift", C.c_double * 9)]


class WStats(C.Structure):
    _fields_ = [("ndrop", C.c_int64), ("sumwt", C.c_double), ("sumlocwt", C.c_double),
                ("f2", C.c_float), ("d2", C.c_float)]


class PlanOpts(C.Structure):
    _fields_ = [("item_max", C.c_int), ("chunk_max", C.c_int)]


class UvmapArgs(C.Structure):
    _fields_ = [("spec", GridSpec), ("nx", C.c_int), ("ny", C.c_int), ("rmode", C.c_int),
                ("robust", C.c_float * 3), ("ds", C.c_float), ("wuscale", C.c_float),
                ("wvscale", C.c_float), ("out_where", C.c_int)]


class UvmapResult(C.Structure):
    _fields_ = [("psf_peak", C.c_float), ("sumwt", C.c_float), ("ngrid", C.c_int64),
                ("ndrop", C.c_int64)]


class CleanResult(C.Structure):
    _fields_ = [("ansub", C.c_int), ("maxres", C.c_float), ("tflux", C.c_float)]


class SysiCommon(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("error", "msgwidth", "sysdebug", "sysmon", "sysintrp",
                                        "sysmsg", "syspar")]


P = C.c_void_p
I = C.c_int
I64 = C.c_int64
F = C.c_float


class ClarkParams(C.Structure):
    """sde_clark_params of include/sde_gpu.h."""
    _fields_ = [("niter", C.c_int), ("gain", C.c_float), ("flux", C.c_float), ("numcl", C.c_int),
                ("bpatch", C.c_int), ("biter", C.c_int)]


class ClarkResult(C.Structure):
    """sde_clark_result of include/sde_gpu.h."""
    _fields_ = [("aniter", C.c_int), ("ncycles", C.c_int), ("window", C.c_int), ("blc", C.c_int),
                ("last_anl", C.c_int), ("maxres", C.c_float), ("tflux", C.c_float),
                ("extside", C.c_float), ("last_slim", C.c_float),
                ("t_anl", C.c_int * 64), ("t_aniter", C.c_int * 64),
                ("t_maxres", C.c_float * 64), ("t_tflux", C.c_float * 64)]


class UruwtStats(C.Structure):
    """sde_uruwt_stats of include/sde_gpu.h."""
    _fields_ = [("nbu", C.c_int), ("nbv", C.c_int), ("ndrop", C.c_int64), ("nsel", C.c_int64),
                ("uradius", C.c_float), ("vradius", C.c_float), ("f2", C.c_float), ("d2", C.c_float),
                ("sumlocwt", C.c_double)]


class UvfitsDesc(C.Structure):
    """sde_uvfits_desc of include/sde_gpu.h."""
    _fields_ = [("ngroups", C.c_int64), ("ngroups_in_file", C.c_int64), ("npar", C.c_int),
                ("bitpix", C.c_int), ("ncomplex", C.c_int), ("nstokes", C.c_int),
                ("iquv", C.c_int), ("uvw_scaled", C.c_int), ("freq", C.c_double),
                ("ra", C.c_double), ("dec", C.c_double)]

# (name, restype, argtypes) of every exported function declared in include/sde_gpu.h
SIGNATURES = [
    ("sde_last_error", C.c_char_p, []),
    ("sde_version", I, []),
    ("sde_ctx_create", I, [C.POINTER(P), I]),
    ("sde_ctx_destroy", I, [P]),
    ("sde_ctx_sync", I, [P]),
    ("sde_ctx_stream", P, [P]),
    ("sde_ctx_set_stream", I, [P, P]),
    ("sde_ctx_bytes_in_use", I64, [P]),
    ("sde_ctx_profile", I, [P, I]),
    ("sde_ctx_kernel_stats", I, [P, C.c_char_p, C.POINTER(C.c_double), C.POINTER(I64)]),
    ("sde_ctx_reset_stats", I, [P]),
    ("sde_ctx_launches", I64, [P]),
    ("sde_ctx_set_compensated", I, [P, I]),
    ("sde_weights", I, [P, I, P, F, P, P, P, P, I64, F, F, F, F, I, I, I, I, P, P, P,
                        C.POINTER(WStats)]),
    ("sde_plan_create", I, [P, C.POINTER(GridSpec), I64, P, P, P, P, P, I, C.POINTER(P)]),
    ("sde_plan_create_opts", I, [P, C.POINTER(GridSpec), I64, P, P, P, P, P, I,
                                 C.POINTER(PlanOpts), C.POINTER(P)]),
    ("sde_plan_destroy", I, [P]),
    ("sde_plan_nvis", I64, [P]),
    ("sde_plan_bytes", I64, [P]),
    ("sde_plan_stats", I, [P, C.POINTER(I64), C.POINTER(I64), C.POINTER(I64)]),
    ("sde_plan_set_vis", I, [P, P, I]),
    ("sde_grid_pitch", I, [I]),
    ("sde_plan_grid", I, [P, I, P, I, C.POINTER(F)]),
    ("sde_plan_image", I, [P, I, I, I, I, P, P, P, I, C.POINTER(F)]),
    ("sde_plan_degrid_residual", I, [P, P, I]),
    ("sde_plan_reset_residual", I, [P]),
    ("sde_plan_degrid", I, [P, P, I, P, P, I, C.POINTER(I64)]),
    ("sde_plan_get_residual", I, [P, P, I]),
    ("sde_image_from_grid", I, [P, P, I, I, I, I, I, I, P, P]),
    ("sde_grid_from_image", I, [P, P, I, I, I, I, I, P, I]),
    ("sde_image_max", I, [P, P, I64, P]),
    ("sde_image_scale_by_inverse", I, [P, P, I64, P]),
    ("sde_hogbom", I, [P, P, P, P, I, I, I, I, F, I, I, F, F, P, P, P, P, P, P,
                       C.POINTER(CleanResult)]),
    ("sde_isamax", I, [P, P, I64, C.POINTER(I64)]),
    ("sde_hogbom_noalloc", I, [P, P, P, P, I, I, I, I, F, I, I, F, F, P, P, P, P, P, P,
                               C.POINTER(CleanResult)]),
    ("sde_uvmap", I, [P, C.POINTER(UvmapArgs), I64, P, P, P, P, P, I, P, P,
                      C.POINTER(UvmapResult)]),
    ("sde_batch_create", I, [P, I, P, P, P, C.POINTER(P)]),
    ("sde_batch_destroy", I, [P]),
    ("sde_batch_bytes", I64, [P]),
    ("sde_batch_psf", I, [P]),
    ("sde_batch_set_mosaic", I, [P, I, I, P, P, P, P, F]),
    ("sde_batch_dirty", I, [P, I]),
    ("sde_batch_dirty_loop", I, [P]),
    ("sde_batch_graph_nodes", I, [P]),
    ("sde_batch_image", I, [P, I, I, C.POINTER(P)]),
    ("sde_batch_read", I, [P, I, I, P, I64]),
    ("sde_weights_ungridded", I, [P, I64, P, P, P, P, F, F, F, I, P, F, P, I, I, P,
                                  C.POINTER(UruwtStats)]),
    ("sde_grid_box", I, [P, I64, P, P, P, P, P, F, F, F, F, I, I, I, I, I, P, P, I, C.POINTER(F)]),
    ("sde_model_image", I, [P, I, C.c_char_p, P, P, P, P, P, P, I, I, F, F, F, F, P]),
    ("sde_image_double", I, [P, P, I, I, F, F, P, I, I, C.POINTER(F)]),
    ("sde_dft_image", I, [P, I64, P, P, P, P, I, I, C.c_double, C.c_double, C.c_double,
                          C.c_double, P, P]),
    ("sde_dft_vis", I, [P, P, I, I, C.c_double, C.c_double, C.c_double, C.c_double, I64, P, P,
                        P, P]),
    ("sde_clark", I, [P, P, P, I, P, C.POINTER(ClarkParams), P, P, P, P, P,
                      C.POINTER(ClarkResult)]),
    ("sde_uvfits_open", I, [C.c_char_p, C.POINTER(P)]),
    ("sde_uvfits_describe", I, [P, C.POINTER(UvfitsDesc)]),
    ("sde_uvfits_read", I, [P, P, I, P, P, P, P, P, I, C.POINTER(I64)]),
    ("sde_uvfits_close", I, [P]),
    ("sde_shim_cache_stats", I, [C.POINTER(I64), C.POINTER(I64)]),
    ("sde_shim_cache_clear", I, []),
    # Fortran-77 drop-in layer (all arguments by reference)
    ("grdh2d_", None, [P] * 24),
    ("grddeh2d_", None, [P] * 22),
    ("grdqh2d_", None, [P] * 18),
    ("grdh23d_", None, [P] * 27),
    ("grddeh23_", None, [P] * 25),
    ("grduwt2d_", None, [P] * 16),
    ("grdruw2d_", None, [P] * 19 + [C.c_size_t]),
    ("fftr2d_", None, [P] * 10),
    ("pixcor2d_", None, [P] * 9 + [C.c_size_t]),
    ("pix2drcl_", None, [P] * 19),
    ("pixisama_", I, [P, P, P]),
    ("grdsf_", C.c_double, [P]),
    ("grdcf_", None, [P, P, P, P, C.c_size_t]),
    ("grdccf_", None, [P, P, P, C.c_size_t]),
    ("errrepor_", None, [P, P, P, C.c_size_t, C.c_size_t, C.c_size_t]),
    ("msgput_", None, [P, P, C.c_size_t, C.c_size_t]),
]
DATA_SYMBOLS = ["sysi_"]

_lib = None


def lib():
    """Load libsdegpu.so (building it first if it is missing or stale)."""
    global _lib
    if _lib is None:
        from . import build as _build
        path = _build.build()
        L = C.CDLL(path)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error():
    t = lib().sde_last_error()
    return t.decode() if t else ""


def check(rc, where):
    if rc != SDE_OK:
        raise SdeError(rc, where, last_error())
    return rc


def sysi():
    return SysiCommon.in_dll(lib(), "sysi_")
