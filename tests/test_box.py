"""GRDQH2D, VISGRID's gridder for the 'BOX' gridding function (grd/grdqh2d.f,
vis/visgrid.f:154-158), through the drop-in grdqh2d_ (every argument by reference, host
arrays) against the oracle's restatement.  Cells receive their visibilities through atomic
adds in no fixed order, and the weight sums (LSUMWT, SUMWT) are formed in double where the
reference adds in REAL one visibility at a time; so grids agree to 1e-5 of the grid peak
(the bar of the GRDH2D drop-in), SUMWT to 1e-5, and the PSF grid of unit weights exactly."""
import ctypes as C

import numpy as np
import pytest

from conftest import small_obs

P = C.c_void_p
I = lambda x: C.byref(C.c_int(int(x)))  # noqa: E731
F = lambda x: C.byref(C.c_float(float(x)))  # noqa: E731


def _p(a):
    return a.ctypes.data_as(P)


@pytest.fixture(scope="module")
def cases(orc):
    out = []
    for kw in (dict(imsize=128, cell=4.0, ntime=24, jitter=True, flag_frac=0.05),
               dict(imsize=256, cell=2.0, ntime=48, shift=(30.0, -45.0))):
        o = small_obs(**kw)
        p = orc.params(o["imsize"], o["cell"], fov=1.0, rmode="NONE", vdec=o["vdec"], shift=o["shift"])
        out.append((o, orc.geom(p)))
    return out


def test_oracle_box_gridding(orc, cases):
    o, g = cases[0]
    grid, sw, rc = orc.grdqh2d(o["vis"], o["wt"], o["u"], o["v"], o["w"], g, psf=True)
    assert rc == 0
    good = o["wt"] > 0
    assert abs(sw - float(o["wt"][good].sum(dtype=np.float64))) / sw < 1e-5
    assert np.all(grid[:, -1] == 0)  # the shifted-out column
    # the u = 0 column is Hermitian about VORIGIN after the fold (column UORIGIN after the shift)
    col = grid[:, g.uorigin - 1]
    vz = g.vorigin - 1
    for off in range(1, 20):
        assert col[vz - off] == np.conj(col[vz + off])
    wt0 = -np.ones_like(o["wt"])
    assert orc.grdqh2d(o["vis"], wt0, o["u"], o["v"], o["w"], g)[2] == -1


def _grdqh2d(L, o, g, psf=False, wt=None):
    from sde_gb300 import _abi
    vis = np.ascontiguousarray(o["vis"], np.complex64)
    wt = np.ascontiguousarray(o["wt"] if wt is None else wt, np.float32)
    gvis = np.zeros((g.nv, g.nu), np.complex64)
    sw = C.c_float()
    shift = np.ascontiguousarray(list(g.shift), np.float64)
    _abi.sysi().error = 0
    L.grdqh2d_(_p(vis), _p(wt), _p(o["u"]), _p(o["v"]), _p(o["w"]), I(len(wt)), F(g.uscale), F(0),
               F(g.vscale), F(0), I(g.uorigin), I(g.vorigin), _p(gvis), I(int(psf)), I(g.nu), I(g.nv),
               _p(shift), C.byref(sw))
    return gvis, sw.value, _abi.sysi().error


@pytest.mark.gpu
@pytest.mark.parametrize("which", [0, 1])
def test_gpu_grdqh2d_matches_oracle(orc, cases, which):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sde_gb300 import _abi
    L = _abi.lib()
    o, g = cases[which]
    for psf in (False, True):
        got, sw, err = _grdqh2d(L, o, g, psf=psf)
        ref, rsw, rc = orc.grdqh2d(o["vis"], o["wt"], o["u"], o["v"], o["w"], g, psf=psf)
        assert err == 0 and rc == 0
        pk = np.abs(ref).max()
        assert np.abs(got - ref).max() / pk < 1e-5
        assert abs(sw - rsw) / rsw < 1e-5
        if psf and which == 1:  # unit weights: every cell sum is an exact small integer
            assert np.array_equal(got, ref)


@pytest.mark.gpu
def test_gpu_grdqh2d_no_weight(cases):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sde_gb300 import _abi
    L = _abi.lib()
    o, g = cases[0]
    _, _, err = _grdqh2d(L, o, g, wt=-np.ones_like(o["wt"]))
    assert err != 0
    _abi.sysi().error = 0
