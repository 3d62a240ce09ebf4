"""Visibilities from FITS random-groups files (VISGET's FTS branch, vis/visget.f:60-68)
through libsdegpu's loader: the file is read in chunks into pinned memory, copied to the
device and decoded there (sde_uvfits_* in include/sde_gpu.h).

    with UVFits("3C10UV.FTS") as f:
        d = f.read(ctx, "I")        # device tensors u, v, w, vis (complex64), wt
        out = imaging.uvmap(ctx, Geom(128, 12.0, vra=f.desc["ra"], vdec=f.desc["dec"]),
                            d["u"], d["v"], d["w"], d["vis"], d["wt"], rmode="NONE")
"""
import ctypes as C

import numpy as np

from . import _abi
from ._abi import check, lib


class UVFits:
    """One random-groups file: header parsed at construction (no GPU needed), groups read
    by read()."""

    def __init__(self, path):
        h = C.c_void_p()
        check(lib().sde_uvfits_open(str(path).encode(), C.byref(h)), "sde_uvfits_open")
        self.h = h
        d = _abi.UvfitsDesc()
        check(lib().sde_uvfits_describe(self.h, C.byref(d)), "sde_uvfits_describe")
        self.desc = {k: getattr(d, k) for k, _ in d._fields_}

    def read(self, ctx, stokes="I", device=True):
        """u, v, w, vis, wt of one Stokes parameter ('I', 'V', 'Q' or 'U') as device tensors
        (device=True) or numpy arrays, plus nread (groups the file held)."""
        n = int(self.desc["ngroups"])
        if device:
            torch = ctx.torch
            out = {k: ctx.empty(n, torch.float32) for k in ("u", "v", "w", "wt")}
            out["vis"] = ctx.empty(n, torch.complex64)
            ptr = {k: C.c_void_p(t.data_ptr()) for k, t in out.items()}
            where = 1
        else:
            out = {k: np.empty(n, np.float32) for k in ("u", "v", "w", "wt")}
            out["vis"] = np.empty(n, np.complex64)
            ptr = {k: a.ctypes.data_as(C.c_void_p) for k, a in out.items()}
            where = 0
        nread = C.c_int64()
        check(lib().sde_uvfits_read(ctx.h, self.h, ord(stokes), ptr["u"], ptr["v"], ptr["w"],
                                    ptr["vis"], ptr["wt"], where, C.byref(nread)),
              "sde_uvfits_read")
        m = int(nread.value)
        out = {k: a[:m] for k, a in out.items()}
        out["nread"] = m
        return out

    def close(self):
        if self.h:
            lib().sde_uvfits_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
