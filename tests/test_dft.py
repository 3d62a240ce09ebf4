"""Direct Fourier transforms: uvmap's DFT option (VISDFT -> VISDFT3D, vis/visdft3d.f) and
vismodel's (IMGDFT -> IMGDFT2D, img/imgdft2d.f).

The oracle holds both as the reference computes them (FP32 rotation recurrences) and with
exact phases in FP64.  The reference's own FP32 result is the recurrence's: its error grows
along each row.  The GPU computes exact phases (split-head reduction) with compensated sums;
the bar is 1e-5 of the peak against FP64 (the spec precision target), and the GPU must
be at least as close to FP64 as the reference's own arithmetic."""
import numpy as np
import pytest

from conftest import small_obs


@pytest.fixture(scope="module")
def obs():
    o = small_obs(imsize=128, cell=4.0, ntime=24, jitter=True, flag_frac=0.05)
    return o


CASES = [  # nx, ny, refx, refy, cell (arcsec)
    (64, 64, 32.0, 32.0, 4.0),
    (100, 72, 50.5, 36.0, 3.0),
]


def test_oracle_reference_dft_error_is_bounded(orc, obs):
    """Documents the reference's FP32 recurrence error against exact phases."""
    o = obs
    n = 64
    d32, p32, rc = orc.visdft2d(o["vis"], o["wt"], o["u"], o["v"], n, n, 32, -4 / 3600, 32, 4 / 3600)
    d64, p64, rc2 = orc.visdft2d(o["vis"], o["wt"], o["u"], o["v"], n, n, 32, -4 / 3600, 32, 4 / 3600, fp64=True)
    assert rc == rc2 == 0
    assert abs(p64.max() - 1.0) < 1e-12 and np.unravel_index(np.argmax(p64), p64.shape) == (31, 31)
    assert np.abs(d32 - d64).max() / np.abs(d64).max() < 1e-4
    assert np.abs(p32 - p64).max() < 1e-3


def test_oracle_no_valid_data(orc, obs):
    wt = -np.ones_like(obs["wt"])
    assert orc.visdft2d(obs["vis"], wt, obs["u"], obs["v"], 8, 8, 4, -1e-3, 4, 1e-3)[2] == -1


@pytest.mark.gpu
@pytest.mark.parametrize("nx,ny,rx,ry,cell", CASES)
def test_gpu_dft_image_matches_fp64(gpu_ctx, orc, obs, nx, ny, rx, ry, cell):
    from sde_gb300.imaging import dft_image
    ctx, o = gpu_ctx, obs
    dx, dy = -cell / 3600.0, cell / 3600.0
    t = {k: ctx.tensor(o[k]) for k in ("u", "v", "wt", "vis")}
    r = dft_image(ctx, t["u"], t["v"], t["vis"], t["wt"], nx, ny, rx, dx, ry, dy)
    ctx.sync()
    gd, gp = r["dirty"].cpu().numpy(), r["psf"].cpu().numpy()
    d64, p64, rc = orc.visdft2d(o["vis"], o["wt"], o["u"], o["v"], nx, ny, rx, dx, ry, dy, fp64=True)
    d32, p32, _ = orc.visdft2d(o["vis"], o["wt"], o["u"], o["v"], nx, ny, rx, dx, ry, dy)
    pk = np.abs(d64).max()
    e_gpu, e_ref = np.abs(gd - d64).max() / pk, np.abs(d32 - d64).max() / pk
    print("dirty error vs FP64: GPU %.2e, reference FP32 %.2e" % (e_gpu, e_ref))
    assert e_gpu < 1e-5 and e_gpu <= e_ref
    assert np.abs(gp - p64).max() < 1e-5 and np.abs(gp - p64).max() <= np.abs(p32 - p64).max()


@pytest.mark.gpu
@pytest.mark.parametrize("nx,ny,rx,ry,cell", CASES)
def test_gpu_dft_vis_matches_fp64(gpu_ctx, orc, obs, nx, ny, rx, ry, cell):
    from sde_gb300.imaging import dft_vis
    ctx, o = gpu_ctx, obs
    dx, dy = -cell / 3600.0, cell / 3600.0
    rng = np.random.default_rng(5)
    img = np.zeros((ny, nx), np.float32)
    img[rng.integers(0, ny, 40), rng.integers(0, nx, 40)] = rng.uniform(-0.5, 2.0, 40).astype(np.float32)
    img[ny // 2, nx // 3] = 3.0
    m = 3000  # a sample of the visibilities keeps the FP64 oracle fast
    u, v, wt = o["u"][:m], o["v"][:m], o["wt"][:m]
    vis0 = (np.arange(m) + 1j).astype(np.complex64)
    vt = ctx.tensor(vis0)
    dft_vis(ctx, ctx.tensor(img), rx, dx, ry, dy, ctx.tensor(u), ctx.tensor(v), ctx.tensor(wt), vt)
    ctx.sync()
    got = vt.cpu().numpy()
    v64 = orc.imgdft2d(img, rx, dx, ry, dy, wt, u, v, vis_in=vis0, fp64=True)
    v32 = orc.imgdft2d(img, rx, dx, ry, dy, wt, u, v, vis_in=vis0)
    good = wt > 0
    assert np.array_equal(got[~good], vis0[~good])  # flagged points keep their VIS
    pk = np.abs(v64[good]).max()
    e_gpu = np.abs(got[good] - v64[good]).max() / pk
    e_ref = np.abs(v32[good] - v64[good]).max() / pk
    print("vis error vs FP64: GPU %.2e, reference FP32 %.2e" % (e_gpu, e_ref))
    assert e_gpu < 1e-5 and e_gpu <= e_ref


@pytest.mark.gpu
def test_gpu_dft_no_valid_data(gpu_ctx, obs):
    from sde_gb300 import _abi
    from sde_gb300.imaging import dft_image
    ctx = gpu_ctx
    t = {k: ctx.tensor(obs[k]) for k in ("u", "v", "vis")}
    wt = ctx.tensor(-np.ones_like(obs["wt"]))
    with pytest.raises(RuntimeError):
        dft_image(ctx, t["u"], t["v"], t["vis"], wt, 16, 16, 8, -1e-3, 8, 1e-3)
    assert "No valid data" in _abi.last_error()


# ---------------------------------------------------------------------------------------
# MODIMG2D: component models into an image
COMPS = [("POIN", 1.0, 3.0, -2.0, 0.0, 0.0, 0.0), ("GAUS", 2.0, 10.0, 5.0, 8.0, 4.0, 30.0),
         ("DISK", 1.5, -20.0, 10.0, 12.0, 6.0, -45.0), ("RECT", 0.5, 15.0, -15.0, 10.0, 5.0, 10.0),
         ("SPHE", 1.0, -10.0, -20.0, 10.0, 10.0, 0.0), ("SHEL", 1.0, 20.0, 20.0, 12.0, 8.0, 60.0),
         ("PLOR", 1.0, 0.0, 0.0, 6.0, 3.0, 20.0), ("POIN", -0.25, 3.0, -2.0, 0.0, 0.0, 0.0),
         ("GAUS", 0.7, -3.0, 4.0, 2.5, 1.5, -10.0)]


def test_oracle_model_components(orc):
    img, rc = orc.modimg2d(COMPS, 64, 64, 32, -1.0, 32, 1.0)
    assert rc == 0
    # the two points land on NINT(32 + 3/-1), NINT(32 - 2/1) = (29, 30), 1-based
    one, _ = orc.modimg2d([COMPS[0]], 64, 64, 32, -1.0, 32, 1.0)
    assert one[29, 28] == 1.0 and one.sum() == 1.0
    # a shell is normalised to its flux by a direct pixel sum
    sh, _ = orc.modimg2d([COMPS[5]], 64, 64, 32, -1.0, 32, 1.0)
    assert abs(float(sh.astype(np.float64).sum()) - 1.0) < 1e-5
    assert orc.modimg2d([("GAUS", 1.0, 0, 0, 0.0, 1.0, 0)], 8, 8, 4, -1.0, 4, 1.0)[1] == -2
    assert orc.modimg2d(COMPS, 8, 8, 4, 0.0, 4, 1.0)[1] == -1


@pytest.mark.gpu
@pytest.mark.parametrize("nx,ny,refx,deltx,refy,delty", [(64, 64, 32, -1.0, 32, 1.0), (90, 70, 45.5, -0.75, 30, 0.6)])
def test_gpu_model_image_matches_reference(gpu_ctx, orc, nx, ny, refx, deltx, refy, delty):
    """Same per-pixel REAL arithmetic in component order: equal to the reference's up to the
    last-place rounding of exp/pow (1e-6 of the peak), points and edges identical."""
    from sde_gb300.imaging import model_image
    ctx = gpu_ctx
    base = np.linspace(-1, 1, nx * ny, dtype=np.float32).reshape(ny, nx)  # added into
    got = model_image(ctx, COMPS, nx, ny, refx, deltx, refy, delty, image=ctx.tensor(base))
    ctx.sync()
    g = got.cpu().numpy()
    ref, rc = orc.modimg2d(COMPS, nx, ny, refx, deltx, refy, delty, image=base)
    assert rc == 0
    pk = np.abs(ref).max()
    assert np.abs(g - ref).max() / pk < 1e-6
    # components without transcendental terms are bit-exact
    exact = [c for c in COMPS if c[0] in ("POIN", "DISK", "RECT", "SPHE")]
    g2 = model_image(ctx, exact, nx, ny, refx, deltx, refy, delty).cpu().numpy()
    r2, _ = orc.modimg2d(exact, nx, ny, refx, deltx, refy, delty)
    assert np.array_equal(g2, r2)


@pytest.mark.gpu
def test_gpu_model_image_errors(gpu_ctx):
    from sde_gb300 import _abi
    from sde_gb300.imaging import model_image
    for comps, msg in (([("GAUS", 1.0, 0, 0, 0.0, 1.0, 0)], "Major axis zero"),
                       ([("BLOB", 1.0, 0, 0, 1.0, 1.0, 0)], "Unknown model type BLOB for component    1")):
        with pytest.raises(RuntimeError):
            model_image(gpu_ctx, comps, 8, 8, 4, -1.0, 4, 1.0)
        assert msg in _abi.last_error()
