import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as O
    O.lib()
    return O


def small_obs(imsize=256, cell=2.0, ntime=48, nchan=1, seed=7, dec=40.0, jitter=False,
              shift=(0.0, 0.0), flag_frac=0.0, arm_m=3000.0):
    """Seeded Y-array observation small enough for the oracle to finish in seconds."""
    from sde_gb300 import synth
    pos = synth.y_array(27, arm_m, seed)
    freqs = 1.4e9 * (1.0 + 0.05 * np.arange(nchan))
    u, v, w = synth.uvw_tracks(pos, dec, 8.0, 8.0 * 3600.0 / ntime, freqs)
    as2r = math.radians(1.0 / 3600.0)
    fov = imsize * cell
    flux = np.array([1.0, 0.3, 0.1, 0.05])
    l = np.array([0.0, 0.12, -0.2, 0.3]) * fov * as2r
    m = np.array([0.0, -0.08, 0.15, -0.25]) * fov * as2r
    vis = synth.visibilities(u, v, flux, l, m, 1e-3, seed,
                             gauss=[(0.2, -0.1 * fov * as2r, -0.2 * fov * as2r, 8 * cell * as2r)])
    rng = np.random.default_rng(seed + 11)
    if jitter:
        wt = rng.uniform(0.2, 3.0, len(u)).astype(np.float32)
    else:
        wt = np.ones(len(u), np.float32)
    if flag_frac > 0:
        wt[rng.uniform(size=len(u)) < flag_frac] = np.float32(-1.0)
    return dict(u=u, v=v, w=w, vis=vis, wt=wt, imsize=imsize, cell=cell, vra=0.0, vdec=dec,
                shift=shift)


@pytest.fixture(scope="session")
def obs_small():
    return small_obs()


@pytest.fixture(scope="session")
def obs_shift():
    # phase-centre shift: exercises the FP64 rotation, degrid exceptions, jittered weights
    return small_obs(imsize=128, cell=4.0, ntime=40, seed=9, dec=55.0, jitter=True,
                     shift=(30.0, -20.0), flag_frac=0.05)


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.fixture(scope="session")
def gpu_ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sde_gb300.imaging import Context
    ctx = Context(0)
    yield ctx
    ctx.close()
