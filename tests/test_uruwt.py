"""Ungridded robust weighting (uvmap's slow weighting: GRDURUWT, grd/grduruwt.f, with
GRDURUW2, grd/grduruw2.f).  The GPU search walks the same bin plane of linked lists as the
reference (built on the host in its order) and sums in its order, so the local weight sums
and the new weights equal the oracle's bit for bit (NORM's F2 comes from a DOUBLE sum and
is equal too); the bin-plane geometry, drops and counts agree exactly."""
import numpy as np
import pytest

from conftest import small_obs

CASES = [dict(rmode="NORM", robust=0.0), dict(rmode="NORM", robust=-1.0, shift=(30.0, -45.0)),
         dict(rmode="ABS", robust=0.05, ds=0.01), dict(rmode="NONE"), dict(rmode="NORM", nbu=64, nbv=100)]


@pytest.fixture(scope="module")
def obs_geoms(orc):
    out = {}
    for shift in ((0.0, 0.0), (30.0, -45.0)):
        o = small_obs(imsize=128, cell=4.0, ntime=48, jitter=True, flag_frac=0.05, shift=shift)
        p = orc.params(o["imsize"], o["cell"], fov=1.0, rmode="NONE", vdec=o["vdec"], shift=shift)
        out[shift] = (o, orc.geom(p))
    return out


def test_oracle_weights_are_local_densities(orc, obs_geoms):
    o, g = obs_geoms[(0.0, 0.0)]
    nw, rc, st = orc.grduruwt(o["u"], o["v"], o["w"], o["wt"], 1.0 / g.uscale, 1.0 / g.vscale,
                              np.array(list(g.shift)), rmode="NONE")
    assert rc == 0 and st["ndrop"] == 0
    good = o["wt"] > 0
    assert st["nsel"] == good.sum()
    # NONE: newwt = WT / (local sum); a point's own weight is in its sum, so newwt <= 1
    assert np.all(nw[good] > 0) and np.all(nw[good] <= 1.0 + 1e-6)
    assert np.array_equal(nw[~good], o["wt"][~good])
    # the local sums agree with a direct count of neighbours (either conjugation) for almost all
    u, v, wt = o["u"][good], o["v"][good], o["wt"][good]
    r = st["uradius"]
    sums = o["wt"][good] / nw[good]
    rng = np.random.default_rng(0)
    idx = rng.choice(len(u), 200, replace=False)
    agree = 0
    for k in idx:
        d1 = (u - u[k]) ** 2 + (v - v[k]) ** 2
        d2 = (u + u[k]) ** 2 + (v + v[k]) ** 2
        direct = wt[(np.minimum(d1, d2) < r * r)].sum()
        agree += abs(direct - sums[k]) <= 1e-4 * direct
    assert agree >= 190


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[str(i) for i in range(len(CASES))])
def test_gpu_ungridded_weights_match_oracle(gpu_ctx, orc, obs_geoms, case):
    from sde_gb300.imaging import weights_ungridded
    kw = dict(case)
    shift = kw.pop("shift", (0.0, 0.0))
    o, g = obs_geoms[shift]
    got, st = weights_ungridded(gpu_ctx, _geom_py(g), o["u"], o["v"], o["w"], o["wt"], **kw)
    ref, rc, rst = orc.grduruwt(o["u"], o["v"], o["w"], o["wt"], 1.0 / g.uscale, 1.0 / g.vscale,
                                np.array(list(g.shift)), **kw)
    assert rc == 0
    assert (st["nbu"], st["nbv"], st["ndrop"], st["nsel"]) == (rst["nbu"], rst["nbv"], rst["ndrop"], rst["nsel"])
    assert st["f2"] == np.float32(rst["f2"])
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


class _geom_py:
    """The oracle geometry in the form imaging.weights_ungridded reads (uscale, vscale, shift)."""

    def __init__(self, g):
        self.uscale, self.vscale = g.uscale, g.vscale
        self.shift = np.array(list(g.shift), np.float64)
