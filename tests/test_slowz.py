"""Slow-Z gridding and degridding (GRDH23D, grd/grdh23d.f; GRDDEH23, grd/grddeh23.f), the
routines VISGRID and VISDEGRI call for N----SIN third axes, through the drop-ins grdh23d_ /
grddeh23_ against the oracle's restatements.

The slow-Z oracle is pinned on the 2-D one: with one plane and no plane rotation GRDH23D has
GRDH2D's window, fold, shift and normalisation, and GRDDEH23 GRDDEH2D's main branch; the
2-D routines keep the rotated coordinates, cells and weight sums in DOUBLE where the slow-Z
ones use REAL (grd/grdh2d.f:85-87, grd/grdh23d.f:72), which moves some visibilities by one
oversampled tap, so that pin holds to 1e-3 of the peak (a wrong fold or shift is O(1)).
GRDH23D normalises by LSUMWT, a REAL sum over every tap of every plane (NVIS x 49 x NZ
adds), whose own rounding is ~1e-4..1e-3; the GPU sums it in double.  So the GPU grid is the
oracle's times one scale factor within that rounding, and after that factor the two agree to
1e-5 of the peak (atomic sums in no fixed order).  Degridded visibilities, summed per
visibility in the reference's order, agree to 1e-6 of the largest, with identical WT."""
import ctypes as C

import numpy as np
import pytest

from conftest import small_obs

P = C.c_void_p
I = lambda x: C.byref(C.c_int(int(x)))  # noqa: E731
F = lambda x: C.byref(C.c_float(float(x)))  # noqa: E731
NZ, CELLZ, REFZ = 4, 0.02, 2.5


def _p(a):
    return a.ctypes.data_as(P)


@pytest.fixture(scope="module")
def case(orc):
    o = small_obs(imsize=128, cell=4.0, ntime=24, jitter=True, flag_frac=0.05, shift=(20.0, -10.0))
    p = orc.params(o["imsize"], o["cell"], fov=1.0, rmode="NONE", vdec=o["vdec"], shift=o["shift"])
    g = orc.geom(p)
    cf, _, _ = orc.grdcf()
    return o, g, cf


def test_oracle_slowz_one_plane_is_the_2d_gridder(orc, case):
    o, g, cf = case
    g3, sw3, rc = orc.grdh23d(o["vis"], o["wt"], o["u"], o["v"], o["w"], g, cf, 1, 0.0, 1.0)
    assert rc == 0
    rc2, g2, sw2, _ = orc.grdh2d(o["vis"], o["wt"], o["u"], o["v"], o["w"], g.uscale, g.vscale, g.uorigin,
                                 g.vorigin, g.nu, g.nv, np.array(list(g.shift)))
    assert rc2 == 0
    pk = np.abs(g2).max()
    assert np.abs(g3[0] - g2).max() / pk < 1e-3
    assert abs(sw3 - sw2) / sw2 < 1e-6
    v3, w3, nb3 = orc.grddeh23(o["vis"], o["wt"], o["u"], o["v"], o["w"], g, cf, g2[None], 0.0, 1.0)
    v2, w2, nb2 = orc.grddeh2d(o["vis"], o["wt"], o["u"], o["v"], o["w"], g.uscale, g.vscale, g.uorigin,
                               g.vorigin, g2, np.array(list(g.shift)))
    main = np.abs(np.asarray(o["u"]) * g.uscale) > 4  # away from the u = 0 axis both take the plain window
    assert np.abs(v3[main] - v2[main]).max() / np.abs(v2).max() < 1e-3


def _grdh23d(L, o, g, cf, psf=False, nz=NZ):
    from sde_gb300 import _abi
    vis = np.ascontiguousarray(o["vis"], np.complex64)
    wt = np.ascontiguousarray(o["wt"], np.float32)
    gvis = np.zeros((nz, g.nv, g.nu), np.complex64)
    sw = C.c_float()
    shift = np.ascontiguousarray(list(g.shift), np.float64)
    _abi.sysi().error = 0
    L.grdh23d_(_p(vis), _p(wt), _p(o["u"]), _p(o["v"]), _p(o["w"]), I(len(wt)), F(g.uscale), F(0), F(g.vscale),
               F(0), I(g.uorigin), I(g.vorigin), _p(gvis), I(int(psf)), I(g.nu), I(g.nv), _p(cf), I(3), I(128),
               _p(cf), I(3), I(128), I(nz), F(CELLZ), F(REFZ), _p(shift), C.byref(sw))
    return gvis, sw.value, _abi.sysi().error


def _grddeh23(L, o, g, cf, grid):
    from sde_gb300 import _abi
    vis = np.ascontiguousarray(o["vis"], np.complex64).copy()
    wt = np.ascontiguousarray(o["wt"], np.float32).copy()
    shift = np.ascontiguousarray(list(g.shift), np.float64)
    grid = np.ascontiguousarray(grid, np.complex64)
    _abi.sysi().error = 0
    L.grddeh23_(_p(vis), _p(wt), _p(o["u"]), _p(o["v"]), _p(o["w"]), I(len(wt)), F(g.uscale), F(0), F(g.vscale),
                F(0), I(g.uorigin), I(g.vorigin), _p(grid), I(g.nu), I(g.nv), _p(cf), I(3), I(128), _p(cf), I(3),
                I(128), I(grid.shape[0]), F(CELLZ), F(REFZ), _p(shift))
    return vis, wt, _abi.sysi().error


@pytest.mark.gpu
def test_gpu_grdh23d_and_grddeh23_match_oracle(orc, case):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sde_gb300 import _abi
    L = _abi.lib()
    o, g, cf = case
    for psf in (False, True):
        got, sw, err = _grdh23d(L, o, g, cf, psf=psf)
        ref, rsw, rc = orc.grdh23d(o["vis"], o["wt"], o["u"], o["v"], o["w"], g, cf, NZ, CELLZ, REFZ, psf=psf)
        assert err == 0 and rc == 0
        r64, g64 = ref.astype(np.complex128), got.astype(np.complex128)
        k = (np.vdot(r64, g64) / np.vdot(r64, r64)).real  # GPU = k * oracle
        assert abs(k - 1.0) < 3e-3
        assert np.abs(g64 / k - r64).max() / np.abs(r64).max() < 1e-5
        assert abs(sw - rsw) / rsw < 1e-5
    model, _, _ = orc.grdh23d(o["vis"], o["wt"], o["u"], o["v"], o["w"], g, cf, NZ, CELLZ, REFZ)
    gv, gw, err = _grddeh23(L, o, g, cf, model)
    rv, rw, nbad = orc.grddeh23(o["vis"], o["wt"], o["u"], o["v"], o["w"], g, cf, model, CELLZ, REFZ)
    assert err == 0
    assert np.array_equal(np.sign(gw), np.sign(rw)) and np.array_equal(np.abs(gw), np.abs(rw))
    assert np.abs(gv - rv).max() / np.abs(rv).max() < 1e-6
