"""GPU parity tests: each CUDA kernel against the oracle on the same seeded inputs.

Bars: weight-density counts and reweighted WT bit-exact; grids within 1e-5 of the grid's
peak; images within 1e-5 of the image peak inside CRDNHALF's window (the CLEAN region; see
test_oracle.test_fp32_gridder_close_to_fp64 for why the corners are looser); degridded
visibilities within 1e-5 of the largest model visibility with identical WT flags; Hogbom
component positions and residuals identical on identical inputs."""
import numpy as np
import pytest

from conftest import rel_err, small_obs

pytestmark = pytest.mark.gpu


def _dev(ctx, a, dt=None):
    return ctx.tensor(a, dt)


def _geom(o, fov=1.0):
    from sde_gb300.imaging import Geom
    return Geom(o["imsize"], o["cell"], vra=o["vra"], vdec=o["vdec"], shift=o["shift"], fov=fov)


def _window(n):
    lo = n // 4
    return slice(lo, lo + n // 2 - 1)


@pytest.mark.parametrize("case", ["small", "shift"])
@pytest.mark.parametrize("rmode", ["UNIFORM", "NORM", "ABS", "NONE"])
def test_weights_bit_exact(gpu_ctx, orc, obs_small, obs_shift, case, rmode):
    o = obs_small if case == "small" else obs_shift
    ctx = gpu_ctx
    g = _geom(o)
    u, v, w, wt = (_dev(ctx, o[k]) for k in ("u", "v", "w", "wt"))
    gwt = ctx.zeros((g.nv, g.nu), ctx.torch.float32)
    newwt = wt.clone()
    rob = (0.5, 0.0, 0.0) if rmode != "ABS" else (0.3, 0.0, 0.0)
    st = ctx.weights(g, u, v, w, wt, rmode=rmode, robust=rob, ds=0.7, gwt=gwt, newwt=newwt)
    ctx.sync()
    if rmode == "UNIFORM":
        ref_new, ref_g, nd = orc.grduwt2d(o["wt"], o["u"], o["v"], o["w"], g.wuscale, g.wvscale,
                                          g.uorigin, g.vorigin, g.nu, g.nv, g.shift)
    else:
        rc, ref_new, ref_g, nd, sw, slw, f2 = orc.grdruw2d(
            o["wt"], o["u"], o["v"], o["w"], g.wuscale, g.wvscale, g.uorigin, g.vorigin, g.nu,
            g.nv, g.shift, rmode, rob, ds=0.7)
        assert rc == 0
        assert np.float32(st.f2) == np.float32(f2)
    got_g = gwt.cpu().numpy()
    got_new = newwt.cpu().numpy()
    assert np.array_equal(got_g.view(np.uint32), ref_g.view(np.uint32))
    touched = o["wt"] > 0
    assert np.array_equal(got_new[touched].view(np.uint32), ref_new[touched].view(np.uint32))
    assert np.array_equal(got_new[~touched], o["wt"][~touched])
    assert st.ndrop == nd


@pytest.mark.parametrize("case", ["small", "shift"])
@pytest.mark.parametrize("psf", [False, True])
def test_grid_matches_grdh2d(gpu_ctx, orc, obs_small, obs_shift, case, psf):
    from sde_gb300.imaging import Plan
    o = obs_small if case == "small" else obs_shift
    ctx = gpu_ctx
    g = _geom(o)
    t = {k: _dev(ctx, o[k]) for k in ("u", "v", "w", "wt")}
    t["vis"] = _dev(ctx, o["vis"])
    plan = Plan(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"])
    grid = ctx.grid_buffer(g)
    sw = plan.grid(grid, psf=psf)
    got = grid.cpu().numpy()[:, :g.nu]
    rc, ref, rsw, lsw = orc.grdh2d(o["vis"], o["wt"], o["u"], o["v"], o["w"], g.uscale,
                                   g.vscale, g.uorigin, g.vorigin, g.nu, g.nv, g.shift, psf=psf)
    assert rc == 0
    assert rel_err(got, ref) < 1e-5
    assert abs(sw - rsw) <= 1e-5 * abs(rsw)
    plan.close()


# 2048 and up: the column pass fed by TMA (two columns per CTA); 1800 in 2048: the forward
# pass's rows outside the image; FFTs of 4096 and 8192: the row passes on row pairs fed by
# bulk copies (3600 wide: an image narrower than the FFT; 4095 rows: a pair with one row)
@pytest.mark.parametrize("n,fnu,ny", [(256, 256, 256), (200, 256, 200), (128, 128, 128),
                                      (2048, 2048, 2048), (1800, 2048, 1800), (4096, 4096, 4096),
                                      (3600, 4096, 4095), (8192, 8192, 8192)])
def test_fft_both_directions(gpu_ctx, orc, n, fnu, ny):
    ctx = gpu_ctx
    from sde_gb300.imaging import fftpwr2
    rng = np.random.default_rng(n + ny)
    nx = n
    nv, nu = fnu, fnu // 2 + 1
    pitch = (nu + 3) & ~3
    X = (rng.standard_normal((nv, nu)) + 1j * rng.standard_normal((nv, nu))).astype(np.complex64)
    ref_img, _ = orc.fftr2d(nx, ny, fnu, nv, -1, xarray=X)
    Xp = np.zeros((nv, pitch), np.complex64)
    Xp[:, :nu] = X
    grid = _dev(ctx, Xp)
    img = ctx.empty((ny, nx), ctx.torch.float32)

    class G:
        pass
    gg = G()
    gg.pitch, gg.nx, gg.ny, gg.fnu, gg.nv = pitch, nx, ny, fnu, nv
    ctx.image_from_grid(gg, grid, img, correct=False)
    assert rel_err(img.cpu().numpy(), ref_img) < 2e-6
    # forward
    im = rng.standard_normal((ny, nx)).astype(np.float32)
    _, refX = orc.fftr2d(nx, ny, fnu, nv, +1, rarray=im)
    grid2 = ctx.zeros((nv, pitch), ctx.torch.complex64)
    ctx.grid_from_image(gg, _dev(ctx, im), grid2, correct=False)
    assert rel_err(grid2.cpu().numpy()[:, :nu], refX) < 2e-6
    # with the grid correction fused
    ccflen = 1 + fftpwr2(max(nx, ny)) // 2
    ccf = orc.grdccf(ccflen)
    cenx, ceny = float((nx + 1) // 2), float((ny + 1) // 2)
    ctx.image_from_grid(gg, _dev(ctx, Xp), img, correct=True)
    ref_c = orc.pixcor2d(ref_img, ccf, cenx, ceny)
    wx, wy = _window(nx), _window(ny)
    assert rel_err(img.cpu().numpy()[wy, wx], ref_c[wy, wx]) < 2e-6
    corrected = orc.pixcor2d(im, ccf, cenx, ceny)
    _, refX2 = orc.fftr2d(nx, ny, fnu, nv, +1, rarray=corrected)
    ctx.grid_from_image(gg, _dev(ctx, im), grid2, correct=True)
    assert rel_err(grid2.cpu().numpy()[:, :nu], refX2) < 2e-6


@pytest.mark.parametrize("case,rmode", [("small", "UNIFORM"), ("shift", "NORM")])
def test_uvmap_matches_reference(gpu_ctx, orc, obs_small, obs_shift, case, rmode):
    from sde_gb300.imaging import uvmap
    o = obs_small if case == "small" else obs_shift
    ctx = gpu_ctx
    g = _geom(o)
    t = {k: _dev(ctx, o[k]) for k in ("u", "v", "w", "wt", "vis")}
    res = uvmap(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"], rmode=rmode,
                robust=(0.0, 0.0, 0.0))
    ctx.sync()
    p = orc.params(o["imsize"], o["cell"], fov=1.0, rmode="NONE" if rmode == "UNIFORM" else rmode,
                   vdec=o["vdec"], shift=o["shift"])
    rd, rp, rwt, rmax, rsw, rc = orc.uvmap(p, o["u"], o["v"], o["w"], o["vis"], o["wt"])
    assert rc == 0
    assert np.array_equal(t["wt"].cpu().numpy().view(np.uint32), rwt.view(np.uint32))
    d = res["dirty"].cpu().numpy()
    ps = res["psf"].cpu().numpy()
    w = _window(o["imsize"])
    assert np.abs(d - rd)[w, w].max() / np.abs(rd).max() < 1e-5
    assert np.abs(ps - rp)[w, w].max() < 1e-5
    assert np.abs(d - rd).max() / np.abs(rd).max() < 5e-3
    res["plan"].close()


@pytest.mark.parametrize("imsize,cell", [(256, 2.0), (2048, 0.25)])
def test_plan_image_equals_grid_then_fft(gpu_ctx, obs_small, imsize, cell):
    """sde_plan_image (GRDH2D's finalize inside the column pass where that pass is TMA-fed,
    2048 rows and up) gives the image and column-transformed grid of sde_plan_grid +
    sde_image_from_grid, for the PSF and the PSF-normalised dirty image.  Two gridding passes
    differ at FP32 rounding (work items meet in the raw grid through atomic adds in no fixed
    order), so the bars are the image bars: 1e-5 of the peak inside the CLEAN window, 5e-3
    over the image (grid correction amplifies rounding at the corners), 1e-5 of the grid peak."""
    from sde_gb300.imaging import Geom, Plan
    o = obs_small
    ctx = gpu_ctx
    g = Geom(imsize, cell, vdec=o["vdec"])
    t = {k: _dev(ctx, o[k]) for k in ("u", "v", "w", "wt", "vis")}
    plan = Plan(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"])
    torch = ctx.torch
    for psf in (True, False):
        peak = ctx.zeros(1, torch.float32) + 0.5
        ga, gb = ctx.grid_buffer(g), ctx.grid_buffer(g)
        ia, ib = ctx.image_buffer(g), ctx.image_buffer(g)
        sw_a = plan.grid(ga, psf=psf)
        ctx.image_from_grid(g, ga, ia, scale_dev=None if psf else peak)
        sw_b = plan.image(ib, gb, psf=psf, scale_dev=None if psf else peak, sumwt=True)
        ctx.sync()
        assert sw_a == sw_b
        a, b = ia.cpu().numpy(), ib.cpu().numpy()
        w = _window(imsize)
        pk = np.abs(a).max()
        assert np.abs(a - b)[w, w].max() / pk < 1e-5
        assert np.abs(a - b).max() / pk < 5e-3
        assert float((ga - gb).abs().max()) / float(ga.abs().max()) < 1e-5
    plan.close()


@pytest.mark.parametrize("case", ["small", "shift"])
def test_degrid_matches_grddeh2d(gpu_ctx, orc, obs_small, obs_shift, case):
    from sde_gb300.imaging import Plan
    o = obs_small if case == "small" else obs_shift
    ctx = gpu_ctx
    g = _geom(o)
    rng = np.random.default_rng(5)
    model = np.zeros((g.ny, g.nx), np.float32)
    w = _window(g.nx)
    for _ in range(12):
        iy, ix = rng.integers(w.start, w.stop, 2)
        model[iy, ix] += rng.uniform(0.05, 1.0)
    # model grid exactly as vismodel builds it
    ccf = orc.grdccf(1 + g.fnu // 2)
    corr = orc.pixcor2d(model, ccf, g.cenx, g.ceny)
    _, mgrid = orc.fftr2d(g.nx, g.ny, g.fnu, g.nv, +1, rarray=corr)
    ref_vis, ref_wt, ref_nbad = orc.grddeh2d(o["vis"], o["wt"], o["u"], o["v"], o["w"],
                                             g.uscale, g.vscale, g.uorigin, g.vorigin, mgrid,
                                             g.shift)
    t = {k: _dev(ctx, o[k]) for k in ("u", "v", "w", "wt", "vis")}
    plan = Plan(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"])
    gp = np.zeros((g.nv, g.pitch), np.complex64)
    gp[:, :g.nu] = mgrid
    vis_out = t["vis"].clone()
    wt_out = t["wt"].clone()
    nbad = plan.degrid(_dev(ctx, gp), vis_out, wt_out)
    got_v = vis_out.cpu().numpy()
    got_w = wt_out.cpu().numpy()
    assert nbad == ref_nbad
    assert np.array_equal(np.sign(got_w), np.sign(ref_wt))
    assert np.array_equal(got_w, ref_wt)
    scale = np.abs(ref_vis[ref_wt > 0]).max()
    assert np.abs(got_v - ref_vis).max() / scale < 1e-5
    # the same model through the GPU FFT (vismodel path)
    from sde_gb300.imaging import vismodel
    vis2 = t["vis"].clone()
    wt2 = t["wt"].clone()
    vismodel(ctx, g, plan, _dev(ctx, model), vis2, wt2)
    assert np.abs(vis2.cpu().numpy() - ref_vis).max() / scale < 1e-5
    plan.close()


def _reflection_rows_outside(g, u, v):
    """GRDDEH2D's FP32 cells (grd/grddeh2d.f:103-114): True where a visibility inside the
    reference's bounds has a mirrored row 2*VORIGIN - (NVC + offv) outside 1..NV."""
    ul = np.float64(g.uscale) * u.astype(np.float64)
    vl = (np.float64(g.vscale) * v.astype(np.float64)).astype(np.float32)
    pos = ul > 0
    uc = np.where(pos, ul.astype(np.float32) + np.float32(g.uorigin),
                  -ul.astype(np.float32) + np.float32(g.uorigin))
    vc = np.where(pos, vl + np.float32(g.vorigin), -vl + np.float32(g.vorigin))
    nuc = np.floor(uc + 0.5).astype(int)
    nvc = np.floor(vc + 0.5).astype(int)
    inside = (nuc + 3 <= g.nu) & (nvc + 3 <= g.nv) & (nvc - 3 >= 1)
    mirror_out = (2 * g.vorigin - (nvc + 3) < 1) | (2 * g.vorigin - (nvc - 3) > g.nv)
    return inside & (nuc <= 3) & mirror_out, uc, vc, nuc, nvc, pos


def _degrid_skip_outside(orc, g, gvis, uc, vc, nuc, nvc, pos):
    """The reflection branch in FP64 with taps whose row lies outside the grid left out of
    the sum and of SUMWT (the GPU's reading of an access the reference leaves undefined)."""
    cf, supp, osamp = orc.grdcf()
    cf = np.asarray(cf, np.float64)
    cfo = (supp + 1) * osamp + 1
    out = []
    for a, b, nu_, nv_, p in zip(uc, vc, nuc, nvc, pos):
        dui = int(np.floor(np.float32(osamp) * (np.float32(nu_) - a) + np.float32(0.5)))
        dvi = int(np.floor(np.float32(osamp) * (np.float32(nv_) - b) + np.float32(0.5)))
        ucen, vcen = nu_ - g.uorigin, nv_ - g.vorigin
        acc, sw = 0j, 0.0
        for offu in range(-supp, supp + 1):
            us = 1 if ucen + offu >= 0 else -1
            ui = g.uorigin + us * (ucen + offu)
            for offv in range(-supp, supp + 1):
                vi = g.vorigin + us * (vcen + offv)
                if vi < 1 or vi > g.nv:
                    continue
                wgt = cf[dui + osamp * offu + cfo - 1] * cf[dvi + osamp * offv + cfo - 1]
                f = complex(gvis[vi - 1, ui - 1])
                acc += (f if us > 0 else f.conjugate()) * wgt
                sw += wgt
        val = acc / sw
        out.append(val.conjugate() if p else val)
    return np.array(out)


def test_degrid_reflection_branch(gpu_ctx, orc):
    """GRDDEH2D's axis-reflection branch (grd/grddeh2d.f:123-158): visibilities within SUPP
    cells of the v axis, over the whole v range.  Those whose mirrored rows 2*VORIGIN - v
    stay inside the grid are degridded by the tiled kernel (from the u = 0 tile's mirrored
    halo) and must match the oracle.  Where a mirrored row leaves the grid the reference
    reads outside GVIS (no bounds check in that loop): those take the exception path, which
    leaves the outside taps out, and are checked against that rule in FP64."""
    import ctypes as C
    from sde_gb300 import _abi
    from sde_gb300.imaging import Geom, Plan
    ctx = gpu_ctx
    g = Geom(64, 8.0, vdec=40.0)
    rng = np.random.default_rng(21)
    n = 3000
    ucell = rng.uniform(-3.45, 3.45, n)
    vcell = rng.uniform(-27.0, 27.0, n)
    # rows at the v edges: NVC = 61 / 60 (a mirrored row off the grid / inside) and
    # NVC = 4 / 3 (tiled / outside GRDDEH2D's bounds)
    vcell[:40] = np.repeat([29.0, 28.0, -28.0, -29.0], 10) + rng.uniform(-0.3, 0.3, 40)
    u = (ucell / g.uscale).astype(np.float32)
    v = (vcell / g.vscale).astype(np.float32)
    w = rng.uniform(-50, 50, n).astype(np.float32)
    vis = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
    wt = np.ones(n, np.float32)
    gvis = (rng.normal(size=(g.nv, g.nu)) + 1j * rng.normal(size=(g.nv, g.nu))).astype(np.complex64)
    edge, uc, vc, nuc, nvc, pos = _reflection_rows_outside(g, u, v)
    assert 0 < edge.sum() < 40
    d = ~edge  # where the reference is defined
    ref_vis, ref_wt, ref_nbad = orc.grddeh2d(vis[d], wt[d], u[d], v[d], w[d], g.uscale, g.vscale,
                                             g.uorigin, g.vorigin, gvis, g.shift)
    t = {k: _dev(ctx, x) for k, x in (("u", u), ("v", v), ("w", w), ("wt", wt), ("vis", vis))}
    plan = Plan(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"])
    a, b, nexc = C.c_int64(), C.c_int64(), C.c_int64()
    _abi.lib().sde_plan_stats(plan.h, C.byref(a), C.byref(b), C.byref(nexc))
    assert 0 < nexc.value < 40  # only edge rows; the near-axis bulk is tiled
    gp = np.zeros((g.nv, g.pitch), np.complex64)
    gp[:, :g.nu] = gvis
    gd = _dev(ctx, gp)
    vis_out = t["vis"].clone()
    wt_out = t["wt"].clone()
    nbad = plan.degrid(gd, vis_out, wt_out)
    got_v = vis_out.cpu().numpy()
    got_w = wt_out.cpu().numpy()
    assert nbad == ref_nbad
    assert np.array_equal(got_w[d], ref_wt)
    scale = np.abs(ref_vis[ref_wt > 0]).max()
    assert np.abs(got_v[d] - ref_vis).max() / scale < 1e-5
    e64 = _degrid_skip_outside(orc, g, gvis, uc[edge], vc[edge], nuc[edge], nvc[edge], pos[edge])
    assert np.all(got_w[edge] > 0)
    assert np.abs(got_v[edge] - e64).max() / scale < 1e-5
    # residual form: observed - model, read back in the caller's order
    plan.degrid_residual(gd)
    res = t["vis"].clone()
    plan.residual(res)
    r = res.cpu().numpy()
    ok = ref_wt > 0
    assert np.abs(r[d][ok] - (vis[d] - ref_vis)[ok]).max() / scale < 1e-5
    assert np.abs(r[edge] - (vis[edge] - e64)).max() / scale < 1e-5
    plan.close()


def test_residual_cycle_consistent(gpu_ctx, orc, obs_small):
    """Residual = observed - model in the gridding frame equals gridding (obs - degrid)."""
    from sde_gb300.imaging import Plan
    o = obs_small
    ctx = gpu_ctx
    g = _geom(o)
    t = {k: _dev(ctx, o[k]) for k in ("u", "v", "w", "wt", "vis")}
    plan = Plan(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"])
    model = np.zeros((g.ny, g.nx), np.float32)
    model[g.ny // 2 - 1, g.nx // 2 - 1] = 1.0
    mgrid = ctx.grid_buffer(g)
    ctx.grid_from_image(g, _dev(ctx, model), mgrid)
    plan.degrid_residual(mgrid)
    res_user = t["vis"].clone()
    plan.residual(res_user)
    vis_m = t["vis"].clone()
    wt_m = t["wt"].clone()
    plan.degrid(mgrid, vis_m, wt_m)
    r = res_user.cpu().numpy()
    expect = o["vis"] - vis_m.cpu().numpy()
    ok = o["wt"] > 0
    assert np.abs(r[ok] - expect[ok]).max() < 1e-5
    plan.close()


def test_hogbom_positions_identical(gpu_ctx, orc, obs_small):
    o = obs_small
    p = orc.params(o["imsize"], o["cell"], fov=1.0, vdec=o["vdec"])
    rd, rp, *_ = orc.uvmap(p, o["u"], o["v"], o["w"], o["vis"], o["wt"])
    n = o["imsize"]
    w = _window(n)
    drt = np.ascontiguousarray(rd[w, w])
    ref = orc.pix2drcl(drt, rp, np.ones_like(drt), 0.1, 300)
    ctx = gpu_ctx
    got = ctx.hogbom(_dev(ctx, drt), _dev(ctx, rp), 300, 0.1)
    assert got["ansub"] == ref["ansub"]
    na = ref["ansub"]
    assert np.array_equal(got["cx"].cpu().numpy()[:na], ref["cx"][:na])
    assert np.array_equal(got["cy"].cpu().numpy()[:na], ref["cy"][:na])
    assert np.array_equal(got["cflux"].cpu().numpy()[:na], ref["cflux"][:na])
    assert np.array_equal(got["res"].cpu().numpy(), ref["res"])
    assert np.array_equal(got["cln"].cpu().numpy(), ref["cln"])
    assert np.float32(got["tflux"]) == np.float32(ref["tflux"])
    assert np.float32(got["maxres"]) == np.float32(ref["maxres"])


def test_hogbom_flux_and_negative_stops(gpu_ctx, orc):
    rng = np.random.default_rng(1)
    n = 64
    yy, xx = np.mgrid[0:2 * n, 0:2 * n]
    psf = np.exp(-((xx - n + 1) ** 2 + (yy - n + 1) ** 2) / 6.0).astype(np.float32)
    drt = (0.01 * rng.standard_normal((n - 1, n - 1))).astype(np.float32)
    drt[20, 30] += 1.0
    drt[40, 10] -= 0.6
    ctx = gpu_ctx
    for nsub, flux in [(200, 0.5), (-200, 0.0)]:
        ref = orc.pix2drcl(drt, psf, np.ones_like(drt), 0.2, nsub, flux=flux)
        got = ctx.hogbom(_dev(ctx, drt), _dev(ctx, psf), nsub, 0.2, flux=flux)
        assert got["ansub"] == ref["ansub"] and got["ansub"] < 200
        na = ref["ansub"]
        assert np.array_equal(got["cx"].cpu().numpy()[:na], ref["cx"][:na])
        assert np.float32(got["maxres"]) == np.float32(ref["maxres"])
        assert np.array_equal(got["res"].cpu().numpy(), ref["res"])
