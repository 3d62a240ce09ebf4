"""The drop-ins' host copies: the same GRDH2D / GRDDEH2D calls on the same data held in
ordinary (pageable) arrays, in pageable arrays whose start is not 16-byte aligned, and in
page-locked arrays give the same results.  Arrays of 256 KB and more in pageable memory are
moved by a copy kernel where the device reads and writes pageable host memory directly; the
others by the CUDA copy.  The degridded visibilities are compared bit for bit (each is
computed independently); the grids within 1e-6 of their peak (the gridder's atomic
additions may add in a different order from call to call)."""
import ctypes as C

import numpy as np
import pytest

from conftest import small_obs

pytestmark = pytest.mark.gpu

P = C.c_void_p
I = lambda x: C.byref(C.c_int(int(x)))
F = lambda x: C.byref(C.c_float(float(x)))


def _p(a):
    return a.ctypes.data_as(P)


def _held(kind, a, torch):
    """a copy of a in the given kind of host memory"""
    a = np.ascontiguousarray(a)
    if kind == "pageable":
        return a.copy()
    if kind == "offset":  # one element past an aligned start
        b = np.empty(a.size + 1, a.dtype)[1:].reshape(a.shape)
        b[...] = a
        return b
    t = torch.empty(a.shape, dtype=getattr(torch, a.dtype.name), pin_memory=True)
    b = t.numpy()
    b[...] = a
    return b


def test_pageable_offset_and_pinned_arrays_agree(orc):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sde_gb300 import _abi
    L = _abi.lib()
    _abi.sysi().error = 0
    o = small_obs(imsize=256, cell=2.0, ntime=400, seed=21)
    n = len(o["wt"])
    assert 4 * n >= 256 * 1024  # the 1-D arrays take the copy kernel where they are pageable
    p = orc.params(o["imsize"], o["cell"], fov=1.0, rmode="NONE", vdec=o["vdec"])
    g = orc.geom(p)
    assert 8 * g.nu * g.nv >= 256 * 1024  # and so does the grid
    cf, _, _ = orc.grdcf()
    shift = np.ascontiguousarray(list(g.shift), np.float64)
    rng = np.random.default_rng(5)
    model = (rng.normal(size=(g.nv, g.nu)) + 1j * rng.normal(size=(g.nv, g.nu))).astype(np.complex64)
    grids, degr = {}, {}
    for kind in ("pageable", "offset", "pinned"):
        u, v, w = (_held(kind, np.asarray(o[k], np.float32), torch) for k in ("u", "v", "w"))
        vis = _held(kind, np.asarray(o["vis"], np.complex64), torch)
        wt = _held(kind, np.asarray(o["wt"], np.float32), torch)
        gvis = _held(kind, np.zeros((g.nv, g.nu), np.complex64), torch)
        sw = C.c_float()
        L.grdh2d_(_p(vis), _p(wt), _p(u), _p(v), _p(w), I(n), F(g.uscale), F(0), F(g.vscale), F(0),
                  I(g.uorigin), I(g.vorigin), _p(gvis), I(0), I(g.nu), I(g.nv), _p(cf), I(3), I(128),
                  _p(cf), I(3), I(128), _p(shift), C.byref(sw))
        assert _abi.sysi().error == 0
        grids[kind] = np.array(gvis)
        mg = _held(kind, model, torch)
        dvis = _held(kind, np.zeros(n, np.complex64), torch)
        dwt = _held(kind, np.asarray(o["wt"], np.float32), torch)
        L.grddeh2d_(_p(dvis), _p(dwt), _p(u), _p(v), _p(w), I(n), F(g.uscale), F(0), F(g.vscale),
                    F(0), I(g.uorigin), I(g.vorigin), _p(mg), I(g.nu), I(g.nv), _p(cf), I(3),
                    I(128), _p(cf), I(3), I(128), _p(shift))
        assert _abi.sysi().error == 0
        degr[kind] = (np.array(dvis), np.array(dwt))
    ref = grids["pinned"]
    peak = np.abs(ref).max()
    assert peak > 0
    for kind in ("pageable", "offset"):
        assert np.abs(grids[kind] - ref).max() <= 1e-6 * peak, kind
        assert np.array_equal(degr[kind][0].view(np.uint32), degr["pinned"][0].view(np.uint32)), kind
        assert np.array_equal(degr[kind][1].view(np.uint32), degr["pinned"][1].view(np.uint32)), kind
    assert np.abs(degr["pinned"][0]).max() > 0
