"""GPU parity on the benchmark's own configurations, against the oracle.

* The plain single field at its full size (84,240 visibilities, uniform weighting onto a
  512^2 grid at 1", Hogbom 1000 iterations at gain 0.1 on CRDNHALF's 255^2 window), end to
  end: weights bit-exact, the points dropped off the grid counted as the reference counts
  them, dirty image and PSF within 1e-5 of the peak, and CLEAN components identical.
* The large single field's uv coverage at 4096^2 on a 1/16 subsample (4,043,520
  visibilities on the full 2049 x 4096 grid, robust NORM R=0): enough points per 64x64 tile
  that the densest tiles take the compensated cross-item path, and a grid large enough for
  the TMA column pass with the finalize inside it.  Weights bit-exact, dirty image and PSF
  within 1e-5 of the peak of the oracle's FP32 and of the FP64 oracle, degridding within
  1e-5 of the largest model visibility.
* GRDRUW2D's azimuthal mode (AZ-NORM), which evaluates ATAN2 and 10**x per visibility.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DENSE_TILE_VIS = 65536  # a 64x64 tile with this many visibilities is gridded compensated


def _t(ctx, a):
    return ctx.tensor(a)


def _first_mismatch(a, b):
    d = np.nonzero(a != b)[0]
    return int(d[0]) if len(d) else None


def test_config1_uvmap_and_hogbom_end_to_end(gpu_ctx, orc):
    from sde_gb300 import synth
    from sde_gb300.imaging import Geom, hogbom, uvmap
    ctx = gpu_ctx
    c = synth.config1()
    n = c["imsize"]
    assert len(c["u"]) == 84240
    g = Geom(n, c["cellsize"], vdec=c["vdec"])
    t = {k: _t(ctx, c[k]) for k in ("u", "v", "w", "vis", "wt")}
    res = uvmap(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"], rmode="UNIFORM")
    ctx.sync()
    p = orc.params(n, c["cellsize"], fov=1.0, rmode="NONE", vdec=c["vdec"])  # 'NONE' = GRDUWT2D
    rd, rp, rwt, rmax, rsw, rc = orc.uvmap(p, c["u"], c["v"], c["w"], c["vis"], c["wt"])
    assert rc == 0
    # uniform weights bit-exact; points off the weighting grid flagged and counted
    # (grd/grduwt2d.f:138-145), then GRDH2D's own bounds (grd/grdh2d.f:151-153)
    assert np.array_equal(t["wt"].cpu().numpy().view(np.uint32), rwt.view(np.uint32))
    og = orc.geom(p)
    _, _, ndrop = orc.grduwt2d(c["wt"], c["u"], c["v"], c["w"], og.uscale, og.vscale, og.uorigin,
                               og.vorigin, og.nu, og.nv, np.array(list(og.shift)))
    assert res["wstats"].ndrop == ndrop == int((rwt <= 0).sum())
    # the points GRDH2D grids: its SUMWT with unit weights on the reweighted points
    ones = (rwt > 0).astype(np.float32)
    _, _, ngrid, _ = orc.grdh2d(c["vis"], ones, c["u"], c["v"], c["w"], og.uscale, og.vscale,
                                og.uorigin, og.vorigin, og.nu, og.nv, np.array(list(og.shift)),
                                psf=True)
    assert res["plan"].nvis == int(ngrid)
    print("config 1: %d visibilities, %d dropped off the weighting grid, %d more outside "
          "GRDH2D's bounds, %d gridded" % (len(rwt), ndrop, int(ones.sum() - ngrid), int(ngrid)))
    d, ps = res["dirty"].cpu().numpy(), res["psf"].cpu().numpy()
    lo, hi = g.window()
    W = slice(lo, hi)
    assert hi - lo == 255
    assert np.abs(d - rd)[W, W].max() / np.abs(rd).max() < 1e-5
    assert np.abs(ps - rp)[W, W].max() < 1e-5
    # Hogbom on identical inputs (the oracle's dirty window and PSF): identical components
    drt = np.ascontiguousarray(rd[W, W])
    ref = orc.pix2drcl(drt, rp, np.ones_like(drt), c["gain"], c["niter"])
    got = ctx.hogbom(_t(ctx, drt), _t(ctx, rp), c["niter"], c["gain"])
    assert got["ansub"] == ref["ansub"] == c["niter"]
    for k in ("cx", "cy", "cflux"):
        assert np.array_equal(got[k].cpu().numpy(), ref[k]), k
    assert np.array_equal(got["res"].cpu().numpy(), ref["res"])
    assert np.array_equal(got["cln"].cpu().numpy(), ref["cln"])
    # the whole chain: GPU dirty -> GPU Hogbom against oracle dirty -> oracle Hogbom.  The
    # dirty images differ at FP32 rounding, so the component lists agree until two pixels'
    # |residual| tie within the two residuals' difference.  Where the lists part (iteration
    # k), both chains are rerun for k iterations: their residuals must agree within 1e-5 of
    # the peak, and the two pixels chosen must tie within twice that difference.
    gch = hogbom(ctx, g, res["dirty"], res["psf"], c["niter"], c["gain"])
    gx, gy = gch["cx"].cpu().numpy(), gch["cy"].cpu().numpy()
    k = _first_mismatch(gx * 100000 + gy, ref["cx"] * 100000 + ref["cy"])
    if k is not None:
        rk = orc.pix2drcl(drt, rp, np.ones_like(drt), c["gain"], k)["res"]
        gk = hogbom(ctx, g, res["dirty"], res["psf"], k, c["gain"])["res"].cpu().numpy()
        ek = float(np.abs(gk - rk).max())
        assert ek <= 1e-5 * np.abs(rd).max(), ek
        a = abs(float(rk[gy[k] - 1, gx[k] - 1]))
        b = abs(float(rk[ref["cy"][k] - 1, ref["cx"][k] - 1]))
        assert 0.0 <= b - a <= 2.0 * ek + 1e-9, (k, a, b, ek)
    kk = c["niter"] if k is None else k
    assert np.allclose(gch["cflux"].cpu().numpy()[:kk], ref["cflux"][:kk], rtol=1e-4, atol=1e-6)
    assert abs(gch["tflux"] - ref["tflux"]) <= 1e-3 * abs(ref["tflux"])
    print("config 1 chain: components identical for %s of %d iterations; TFLUX %.6f vs %.6f"
          % ("all" if k is None else k, c["niter"], gch["tflux"], ref["tflux"]))
    res["plan"].close()


def _config2_subsample(orc, stride=16, nsrc=20):
    from sde_gb300 import synth
    (u, v, w), seed = synth.config2_uvw()
    u, v, w = u[::stride].copy(), v[::stride].copy(), w[::stride].copy()
    flux, l, m = synth.point_sky(200, 4096 * 0.5, seed)
    vis = orc.point_vis(u, v, flux[:nsrc], l[:nsrc], m[:nsrc])
    rng = np.random.default_rng(seed + 2)
    vis += (rng.normal(0, 1e-3, len(u)) + 1j * rng.normal(0, 1e-3, len(u))).astype(np.complex64)
    return u, v, w, vis, np.ones(len(u), np.float32)


def _dense_tiles(g, u, v):
    """Tiles of 64x64 raw-grid cells (GRDH2D's cell + SUPP) holding >= DENSE_TILE_VIS points."""
    uc = np.float64(g.uscale) * u.astype(np.float64)
    vc = np.float64(g.vscale) * v.astype(np.float64)
    pos = uc > 0
    uc = np.where(pos, uc, -uc) + g.uorigin
    vc = np.where(pos, vc, -vc) + g.vorigin
    tile = ((np.rint(uc).astype(np.int64) + 3) // 64) * 4096 + np.rint(vc).astype(np.int64) // 64
    _, cnt = np.unique(tile, return_counts=True)
    return int((cnt >= DENSE_TILE_VIS).sum())


def test_config2_subsample_4096_against_oracle_and_fp64(gpu_ctx, orc):
    from sde_gb300.imaging import Geom, uvmap, vismodel
    ctx = gpu_ctx
    u, v, w, vis, wt = _config2_subsample(orc)
    g = Geom(4096, 0.5, vdec=40.0)
    assert (g.nu, g.nv) == (2049, 4096)
    ndense = _dense_tiles(g, u, v)
    assert ndense >= 1  # the compensated cross-item path is exercised
    t = {k: _t(ctx, x) for k, x in (("u", u), ("v", v), ("w", w), ("vis", vis), ("wt", wt))}
    res = uvmap(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"], rmode="NORM",
                robust=(0.0, 0.0, 0.0))
    ctx.sync()
    p = orc.params(4096, 0.5, fov=1.0, rmode="NORM", vdec=40.0)
    rd, rp, rwt, rmax, rsw, rc = orc.uvmap(p, u, v, w, vis, wt)
    assert rc == 0
    gw = t["wt"].cpu().numpy()
    assert np.array_equal(gw.view(np.uint32), rwt.view(np.uint32))
    d, ps = res["dirty"].cpu().numpy(), res["psf"].cpu().numpy()
    lo, hi = g.window()
    W = slice(lo, hi)
    pk = np.abs(rd).max()
    e_ref = np.abs(d - rd)[W, W].max() / pk
    assert e_ref < 1e-5
    assert np.abs(ps - rp)[W, W].max() < 1e-5
    # against the FP64 oracle (the same algorithm in double) with the same weights
    og = orc.geom(p)
    p64 = orc.uvmap_image64_mt(og, u, v, w, vis, rwt, True)
    d64 = orc.uvmap_image64_mt(og, u, v, w, vis, rwt, False) / p64.max()
    e64 = np.abs(d - d64)[W, W].max() / np.abs(d64).max()
    e64_ref = np.abs(rd - d64)[W, W].max() / np.abs(d64).max()
    assert e64 < 1e-5
    print("4096^2 subsample: %d vis, %d dense tiles; dirty vs oracle FP32 %.2e, vs FP64 %.2e "
          "(oracle FP32 vs FP64 %.2e)" % (len(u), ndense, e_ref, e64, e64_ref))
    # degridding a CLEAN-like model (vismodel's path: IMGGRIDC, r2c FFT, GRDDEH2D)
    rng = np.random.default_rng(3)
    model = np.zeros((g.ny, g.nx), np.float32)
    for _ in range(50):
        iy, ix = rng.integers(lo, hi, 2)
        model[iy, ix] += rng.uniform(0.01, 1.0)
    ccf = orc.grdccf(1 + g.fnu // 2)
    _, mgrid = orc.fftr2d(g.nx, g.ny, g.fnu, g.nv, +1, rarray=orc.pixcor2d(model, ccf, g.cenx, g.ceny))
    ref_vis, ref_wt, ref_nbad = orc.grddeh2d(vis, rwt, u, v, w, og.uscale, og.vscale, og.uorigin,
                                             og.vorigin, mgrid, np.array(list(og.shift)))
    plan = res["plan"]
    gp = np.zeros((g.nv, g.pitch), np.complex64)
    gp[:, :g.nu] = mgrid
    vis_out, wt_out = t["vis"].clone(), t["wt"].clone()
    nbad = plan.degrid(_t(ctx, gp), vis_out, wt_out)
    assert nbad == ref_nbad
    assert np.array_equal(wt_out.cpu().numpy(), ref_wt)
    scale = np.abs(ref_vis[ref_wt > 0]).max()
    assert np.abs(vis_out.cpu().numpy() - ref_vis).max() / scale < 1e-5
    vis2, wt2 = t["vis"].clone(), t["wt"].clone()
    vismodel(ctx, g, plan, _t(ctx, model), vis2, wt2)
    assert np.abs(vis2.cpu().numpy() - ref_vis).max() / scale < 1e-5
    plan.close()


@pytest.mark.parametrize("case", ["small", "shift"])
def test_weights_az_norm(gpu_ctx, orc, obs_small, obs_shift, case):
    """GRDRUW2D's AZ-NORM mode (grd/grdruw2d.f:106-126, 225-230): the density grid GWT is
    bit-exact.  NEWWT evaluates, per visibility in REAL, T = ATAN2(V, U), then
    MOD(T - RPA + 2.5*PI, PI) - PI/2 and F2 = (5*10**(-ROB))**2 / ratio with
    ROB = ROBUST(1) - |T|*RBSCALE.  CUDA's atan2f/powf and the host's libm may round
    differently in the last place (as two platforms' Fortran libraries may), and the sum with
    2.5*PI (about 7.85) can then round to neighbouring REALs: |T| moves by up to two ulp(8),
    ROB by RBSCALE times that, and F2 (hence NEWWT) by 2*ln(10) times the ROB change.  The
    bound below is that amount plus a few ulp for the power and the divisions."""
    from sde_gb300.imaging import Geom
    o = obs_small if case == "small" else obs_shift
    ctx = gpu_ctx
    g = Geom(o["imsize"], o["cell"], vra=o["vra"], vdec=o["vdec"], shift=o["shift"])
    u, v, w, wt = (_t(ctx, o[k]) for k in ("u", "v", "w", "wt"))
    gwt = ctx.zeros((g.nv, g.nu), ctx.torch.float32)
    newwt = wt.clone()
    rob = (1.0, -1.0, 30.0)
    st = ctx.weights(g, u, v, w, wt, rmode="AZ-NORM", robust=rob, gwt=gwt, newwt=newwt)
    ctx.sync()
    rc, ref_new, ref_g, nd, sw, slw, f2 = orc.grdruw2d(
        o["wt"], o["u"], o["v"], o["w"], g.wuscale, g.wvscale, g.uorigin, g.vorigin, g.nu, g.nv,
        g.shift, "AZ-NORM", rob)
    assert rc == 0
    assert np.array_equal(gwt.cpu().numpy().view(np.uint32), ref_g.view(np.uint32))
    assert st.ndrop == nd
    got = newwt.cpu().numpy()
    touched = o["wt"] > 0
    a, b = got[touched], ref_new[touched]
    assert np.array_equal(np.sign(a), np.sign(b))
    ok = b > 0
    rbscale = (rob[0] - rob[1]) / (np.pi / 2.0)
    # up to two REAL steps of the sum near 8 (its rounding, and the subtraction of PI/2)
    tol = 2.0 * np.log(10.0) * rbscale * 2.0 * float(np.spacing(np.float32(8.0))) + 16.0 * float(np.finfo(np.float32).eps)
    rel = float(np.max(np.abs(a[ok] - b[ok]) / b[ok]))
    assert rel <= tol, (rel, tol)
    same = float(np.mean(a.view(np.uint32) == b.view(np.uint32)))
    assert same >= 0.25, same
    assert np.array_equal(got[~touched], o["wt"][~touched])
    print("AZ-NORM %s: %.1f%% of NEWWT bit-identical, max relative difference %.2e (bound %.2e)"
          % (case, 100 * same, rel, tol))


def test_imgtovis_padded_degrid_matches_oracle(gpu_ctx, orc, obs_small, obs_shift):
    """IMGTOVIS (img/imgtovis.f:55-84), the degrid of mosclean's major cycle
    (task/mosclean.f:361): IMGDOUBL pads the model to FFTPWR2(2N) with the reference pixel
    moved to the centre (bit-exact against the oracle's PIXRPAD), then the padded image's
    grid -- uv cells half as large -- is corrected, transformed and degridded; visibilities
    within 1e-5 of the largest, WT flags identical.  Both observations: with and without a
    phase-centre shift."""
    from sde_gb300.imaging import Geom, Plan, image_double, imgtovis, padded_geom
    ctx = gpu_ctx
    for o in (obs_small, obs_shift):
        g = Geom(o["imsize"], o["cell"], vra=o["vra"], vdec=o["vdec"], shift=o["shift"])
        rng = np.random.default_rng(17)
        model = np.zeros((g.ny, g.nx), np.float32)
        lo, hi = g.window()
        for _ in range(15):
            iy, ix = rng.integers(lo, hi, 2)
            model[iy, ix] += rng.uniform(0.05, 1.0)
        # the padding alone, bit for bit
        pad_ref, rx, ry = orc.imgdoubl(model, g.cenx, g.ceny)
        pad, gx, gy = image_double(ctx, _t(ctx, model), g.cenx, g.ceny)
        assert np.array_equal(pad.cpu().numpy(), pad_ref) and (gx, gy) == (rx, ry)
        pg = padded_geom(g)
        assert (pg.nx, pg.nu, pg.nv) == (2 * g.nx, g.nx + 1, 2 * g.nx) and (pg.cenx, pg.ceny) == (rx, ry)
        p = orc.params(o["imsize"], o["cell"], fov=1.0, vdec=o["vdec"], shift=o["shift"])
        ref_vis, ref_wt = orc.imgtovis(p, o["u"], o["v"], o["w"], o["vis"], o["wt"], model)
        t = {k: _t(ctx, o[k]) for k in ("u", "v", "w", "wt", "vis")}
        plan = Plan(ctx, pg, t["u"], t["v"], t["w"], t["vis"], t["wt"])
        vis_out, wt_out = t["vis"].clone(), t["wt"].clone()
        imgtovis(ctx, g, plan, _t(ctx, model), vis_out, wt_out)
        got_w = wt_out.cpu().numpy()
        assert np.array_equal(got_w, ref_wt)
        ok = ref_wt > 0
        scale = np.abs(ref_vis[ok]).max()
        assert np.abs(vis_out.cpu().numpy()[ok] - ref_vis[ok]).max() / scale < 1e-5
        plan.close()
