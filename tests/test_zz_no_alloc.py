"""The allocation-free Hogbom entry point (sde_hogbom_noalloc).

Callers whose device memory all comes from their own allocator or a fixed arena, and loops
that must not allocate once running, cannot let the library call cudaMalloc.  For them
sde_hogbom_noalloc runs the CLEAN minor cycle on arrays they already own, with its scratch
in a static device array.  This test calls it through the C ABI twice in a row (the second
call sees the first call's leftovers in that shared array) and checks both results against
the allocating entry point sde_hogbom on the same inputs: component list, residual, clean
image and scalars must be identical, the bar every Hogbom test here holds.

It sits in its own file, named to be collected last, and builds its own inputs, so it passes
both alone in a fresh process and after the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(n=96, seed=3):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:2 * n, 0:2 * n]
    psf = np.exp(-((xx - n + 1) ** 2 + 0.7 * (yy - n + 1) ** 2) / 9.0).astype(np.float32)
    psf += (0.02 * np.cos(0.4 * (xx - n + 1)) * np.exp(-((yy - n + 1) ** 2) / 200.0)).astype(np.float32)
    drt = (0.01 * rng.standard_normal((n - 1, n - 1))).astype(np.float32)
    for _ in range(6):
        iy, ix = rng.integers(10, n - 11, 2)
        a = rng.uniform(-0.5, 1.0)
        drt += a * psf[n - 1 - iy:2 * n - 2 - iy, n - 1 - ix:2 * n - 2 - ix]
    box = np.ones_like(drt)
    return drt, psf, box


def test_noalloc_hogbom_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sde_gb300 import _abi
    L = _abi.lib()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    drt, psf, box = _inputs()
    ny, nx = drt.shape
    pny, pnx = psf.shape
    niter, gain = 400, 0.15
    d_drt = torch.from_numpy(drt).to(dev)
    d_psf = torch.from_numpy(psf).to(dev)
    d_box = torch.from_numpy(box).to(dev)
    p = lambda t: C.c_void_p(t.data_ptr())

    def outputs():
        return (torch.zeros((ny, nx), dtype=torch.float32, device=dev),
                torch.zeros((ny, nx), dtype=torch.float32, device=dev),
                torch.zeros(niter, dtype=torch.float32, device=dev),
                torch.zeros(niter, dtype=torch.int32, device=dev),
                torch.zeros(niter, dtype=torch.int32, device=dev))

    # reference: the allocating entry point
    h = C.c_void_p()
    assert L.sde_ctx_create(C.byref(h), 0) == 0
    stream = torch.cuda.current_stream(dev)
    assert L.sde_ctx_set_stream(h, C.c_void_p(stream.cuda_stream)) == 0
    cln0, res0, cf0, cx0, cy0 = outputs()
    r0 = _abi.CleanResult()
    rc = L.sde_hogbom(h, p(d_drt), p(d_psf), p(d_box), nx, ny, pnx, pny, gain, niter, 1, 0.0, 0.0,
                      p(cln0), p(res0), p(cf0), p(cx0), p(cy0), None, C.byref(r0))
    assert rc == 0, _abi.last_error()
    torch.cuda.synchronize()
    L.sde_ctx_destroy(h)

    for call in range(2):
        cln, res, cf, cx, cy = outputs()
        r = _abi.CleanResult()
        rc = L.sde_hogbom_noalloc(C.c_void_p(stream.cuda_stream), p(d_drt), p(d_psf), p(d_box),
                                  nx, ny, pnx, pny, gain, niter, 1, 0.0, 0.0, p(cln), p(res),
                                  p(cf), p(cx), p(cy), None, C.byref(r))
        assert rc == 0, _abi.last_error()
        torch.cuda.synchronize()
        assert r.ansub == r0.ansub
        na = r0.ansub if r0.ansub > 0 else niter
        assert torch.equal(cx[:na], cx0[:na]) and torch.equal(cy[:na], cy0[:na]), call
        assert torch.equal(cf[:na], cf0[:na]), call
        assert torch.equal(res, res0) and torch.equal(cln, cln0), call
        assert np.float32(r.maxres) == np.float32(r0.maxres)
        assert np.float32(r.tflux) == np.float32(r0.tflux)


def test_noalloc_rejects_oversized_window():
    """The size check runs before any device work.  It is exercised in a child process that
    sees no GPU, so that if the check ever moved below the launches the call would fail with a
    device error instead of launching kernels on the placeholder addresses."""
    import os
    import subprocess
    import sys
    code = (
        "import ctypes as C, sys\n"
        "sys.path.insert(0, %r)\n"
        "from sde_gb300 import _abi\n"
        "L = _abi.lib()\n"
        "r = _abi.CleanResult()\n"
        "one = C.c_void_p(16)\n"
        "rc = L.sde_hogbom_noalloc(None, one, one, None, 65536, 65536, 3, 3, 0.1, 10, 1, 0.0, 0.0,\n"
        "                          one, one, one, one, one, None, C.byref(r))\n"
        "assert rc == _abi.SDE_EINVAL, rc\n"
        "assert '2^31-1' in _abi.last_error(), _abi.last_error()\n"
        "print('ok')\n" % os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
