"""Clark CLEAN (the default algorithm of SDE's clean task: task/clean.f CLARK branch,
img/imgcclea.f, pix/pix2drcc.f, pix/pix2drli.f, pix/pixrabsh.f, pix/pixflim.f,
pix/pix2drma.f, img/imgresid.f, img/imgsubps.f).

The oracle (oracle/sde_oracle.c orc_clark) is pinned on the reference's own logged run of
test/timer (test/timings.sun3:232-240: clean of reqdata/3C10MAP.FTS with 3C10BEAM.FTS,
Niter 20000, Flux 3e-3, Gain 0.1, Numcl 16384, Bpatch 64): the first two major cycles'
messages agree to every printed digit.  The GPU (sde_clark) is checked against the oracle:
the first major cycle (list from the dirty image itself) bit for bit, the first three
cycles' messages as printed, and the converged result of the whole run."""
import numpy as np
import pytest

GOLD_LOG = [(974, 5, 5.7758e-01, 3.1695e-01), (1253, 47, 4.5179e-01, 2.4370e00)]
TIMER = dict(niter=20000, gain=0.1, flux=3e-3, numcl=16384, bpatch=64)


@pytest.fixture(scope="module")
def gold():
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "3c10.npz"))


def _same_printed(a, b):
    """Equal as IMGCCLEA prints them: I6, I7, 1PE12.4, 1PE12.4 (img/imgcclea.f:277)."""
    return a[0] == b[0] and a[1] == b[1] and "%.4E" % a[2] == "%.4E" % b[2] and "%.4E" % a[3] == "%.4E" % b[3]


def test_oracle_reproduces_reference_log(orc, gold):
    r = orc.clark(gold["map"], gold["beam"], **TIMER)
    assert r["rc"] == 0
    for got, want in zip(r["trace"][:2], GOLD_LOG):
        assert _same_printed(got, want), (got, want)
    # later cycles: the 1991 log drifts from FP32 (its residual comes from a long FFT
    # convolution on a different machine) but stays within 2 % while it converges
    assert abs(r["trace"][2][2] - 0.27713) / 0.27713 < 0.02


def test_oracle_cleans_a_point(orc, gold):
    """dirty = PSF: the components sum to the unit flux at the window centre."""
    psf = gold["beam"]
    r = orc.clark(psf, psf, niter=50, gain=0.5, bpatch=64)
    assert r["rc"] == 0
    assert abs(float(r["comp"].sum()) - 1.0) < 1e-6
    assert abs(float(r["comp"][31, 31]) - 1.0) < 1e-6  # 1-based (32, 32) of the 64-pixel window
    assert np.abs(r["resid"]).max() < 1e-6


def test_oracle_zero_image_is_an_error(orc, gold):
    z = np.zeros((128, 128), np.float32)
    assert orc.clark(z, gold["beam"], niter=10)["rc"] == -1  # 'Zero range in values'


# ---------------------------------------------------------------------------------------
def _gpu(ctx, dirty, psf, **kw):
    from sde_gb300.imaging import clark
    box = kw.pop("box", None)
    r = clark(ctx, ctx.tensor(dirty), ctx.tensor(psf), box=None if box is None else ctx.tensor(box), **kw)
    ctx.sync()
    for k in ("comp", "resid", "cl", "cx", "cy"):
        r[k] = r[k].cpu().numpy()
    return r


@pytest.mark.gpu
def test_gpu_first_major_cycle_bit_exact(gpu_ctx, orc, gold):
    """Niter small enough for one major cycle: the list comes from the dirty image itself,
    so the minor cycle, component list and component image equal the oracle's bit for bit."""
    for niter, numcl, bp in ((5, 16384, 64), (40, 32768, 128), (300, 2000, 32)):
        kw = dict(niter=niter, gain=0.1, flux=0.0, numcl=numcl, bpatch=bp)
        o = orc.clark(gold["map"], gold["beam"], **kw)
        g = _gpu(gpu_ctx, gold["map"], gold["beam"], **kw)
        assert g["ncycles"] >= 1 and o["ncycles"] >= 1
        a = o["trace"][0][1]
        assert g["trace"][0][:2] == o["trace"][0][:2]
        assert np.array_equal(g["cl"][:a], o["cl"][:a])
        assert np.array_equal(g["cx"][:a], o["cx"][:a]) and np.array_equal(g["cy"][:a], o["cy"][:a])
        assert g["extside"] == o["extside"]
        if g["ncycles"] == 1:
            assert np.array_equal(g["comp"], o["comp"])
            assert g["maxres"] == o["maxres"] and g["tflux"] == o["tflux"]


@pytest.mark.gpu
def test_gpu_reproduces_reference_log_and_oracle(gpu_ctx, orc, gold):
    o = orc.clark(gold["map"], gold["beam"], **TIMER)
    g = _gpu(gpu_ctx, gold["map"], gold["beam"], **TIMER)
    for got, want in zip(g["trace"][:2], GOLD_LOG):
        assert _same_printed(got, want), (got, want)
    # the whole run against the oracle: from the second major cycle on, the residual comes
    # from FP32 FFTs of a different summation order; both are deterministic, and CLEAN turns
    # a last-bit difference near a threshold into one component more or less, after which
    # the runs take different (equally valid) paths to the same flux limit.  So: the first
    # three cycles agree as printed, and the converged results agree.
    print("gpu", g["trace"], "\noracle", o["trace"])
    for gt, ot in zip(g["trace"][:3], o["trace"][:3]):
        assert _same_printed(gt, ot), (gt, ot)
    assert abs(g["maxres"]) <= TIMER["flux"] and abs(o["maxres"]) <= TIMER["flux"]
    assert abs(g["tflux"] - o["tflux"]) / o["tflux"] < 1e-2
    # different components, residuals at the same level: rms within 5 %, and no pixel apart by
    # more than the residual level itself (~1 % of the peak)
    pk = float(np.abs(gold["map"]).max())
    rg, ro = (float(np.sqrt((x.astype(np.float64) ** 2).mean())) for x in (g["resid"], o["resid"]))
    assert abs(rg - ro) / ro < 0.05
    assert np.abs(g["resid"] - o["resid"]).max() / pk < 3e-2
    assert abs(float(g["comp"].sum()) - float(o["comp"].sum())) / float(o["comp"].sum()) < 1e-2


@pytest.mark.gpu
def test_gpu_box_and_point(gpu_ctx, orc, gold):
    psf = gold["beam"]
    g = _gpu(gpu_ctx, psf, psf, niter=50, gain=0.5, bpatch=64)
    assert abs(float(g["comp"].sum()) - 1.0) < 1e-6 and np.abs(g["resid"]).max() < 1e-6
    # a box that excludes the left half: no component there, oracle equal on the first cycle
    box = np.ones((64, 64), np.float32)
    box[:, :32] = 0.0
    kw = dict(niter=30, gain=0.1, numcl=16384, bpatch=64, box=box)
    o = orc.clark(gold["map"], gold["beam"], **kw)
    g = _gpu(gpu_ctx, gold["map"], gold["beam"], **kw)
    assert np.all(g["comp"][:, :32] == 0)
    a = o["trace"][0][1]
    assert np.array_equal(g["cl"][:a], o["cl"][:a])


@pytest.mark.gpu
def test_gpu_zero_image_reports_reference_error(gpu_ctx, gold):
    from sde_gb300 import _abi
    with pytest.raises(RuntimeError):
        _gpu(gpu_ctx, np.zeros((128, 128), np.float32), gold["beam"], niter=10)
    assert "Zero range in values" in _abi.last_error()
