"""Served imaging: each job's image is the same alone and in a concurrent mix, admission
keeps the device footprint under the budget, and latency records are consistent.

The bar for "the same" is the dirty-image bar of every test here: 1e-5 of the image peak
inside the CRDNHALF window (float atomics make summation order, and so the last bits,
depend on scheduling; the grid correction amplifies that towards the image corners)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _window(n):
    lo = n // 4 + 1
    length = min(3 * n // 4 - 1 - lo + 1, n // 2 - 1)
    return slice(lo - 1, lo - 1 + length)


@pytest.fixture(scope="module")
def jobs():
    from sde_gb300 import serve
    return [serve.make_job(i, sizes=(256, 512), ants=(27, 32), ints=(1, 12), chans=(1, 6))
            for i in range(10)]


@pytest.fixture(scope="module")
def server():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sde_gb300.serve import Server
    s = Server(nslots=4, hbm_budget=8 << 30)
    yield s
    s.close()


def test_each_job_same_alone_and_in_the_mix(server, jobs):
    import torch
    from sde_gb300.serve import run_job
    rec, mixed = server.run(jobs, keep_images=True)  # all arrive at once: concurrent mix
    assert server.max_running > 1
    alone = [run_job(server.slots[0].ctx, j, torch) for j in jobs]  # one at a time
    for a, b, j in zip(alone, mixed, jobs):
        w = _window(j["imsize"])
        pk = np.abs(a).max()
        assert np.abs(a - b)[w, w].max() / pk < 1e-5, j["id"]
        assert np.abs(a - b).max() / pk < 5e-3, j["id"]


def test_admission_holds_the_budget(jobs):
    from sde_gb300.serve import Server, footprint_bytes
    sizes = [footprint_bytes(j["nvis"], j["imsize"]) for j in jobs]
    budget = 2 * max(sizes)
    s = Server(nslots=4, hbm_budget=budget)
    try:
        rec = s.run(jobs)
        assert all(r is not None for r in rec)
        assert s.max_reserved <= budget
        assert s.max_running <= 4
    finally:
        s.close()


def test_stream_records_and_latency(server, jobs):
    from sde_gb300.serve import poisson_arrivals, summarize
    arr = poisson_arrivals(len(jobs), 100.0)
    rec = server.run(jobs, arrivals=arr)
    for r, a in zip(rec, arr):
        assert r["finish"] >= r["start"] >= r["admitted"] >= a - 1e-3
        assert r["latency_ms"] > 0
    s = summarize(rec)
    assert s["p50_ms"] <= s["p99_ms"] <= s["max_ms"]
    assert s["jobs"] == len(jobs)


def test_native_job_equals_uvmap_composition(server, jobs, orc):
    """sde_uvmap (one native call) gives the image of the host-side uvmap composition and
    of the oracle's uvmap, for a natural and a robust job."""
    import torch
    from sde_gb300.imaging import Geom, uvmap
    from sde_gb300.serve import run_job
    ctx = server.slots[0].ctx
    for j in [x for x in jobs if x["natural"]][:1] + [x for x in jobs if not x["natural"]][:1]:
        native = run_job(ctx, j, torch)
        g = Geom(j["imsize"], j["cell"], vdec=j["dec"])
        t = {k: ctx.tensor(j[k], torch.float32) for k in ("u", "v", "w", "wt")}
        t["vis"] = ctx.tensor(np.asarray(j["vis"], np.complex64).view(np.float32), torch.float32)
        with torch.cuda.stream(ctx.stream):
            if j["natural"]:
                r = uvmap(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"], weighting=False)
            else:
                r = uvmap(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"], rmode="NORM",
                          robust=(j["robust"], 0.0, 0.0))
            ctx.stream.synchronize()
        comp = r["dirty"].cpu().numpy()
        r["plan"].close()
        w = _window(j["imsize"])
        pk = np.abs(comp).max()
        assert np.abs(native - comp)[w, w].max() / pk < 1e-5
        if not j["natural"]:
            p = orc.params(j["imsize"], j["cell"], fov=1.0, rmode="NORM",
                           robust=(j["robust"], 0.0, 0.0), vdec=j["dec"])
            rd, *_ = orc.uvmap(p, j["u"], j["v"], j["w"], j["vis"], j["wt"])
            assert np.abs(native - rd)[w, w].max() / np.abs(rd).max() < 1e-5
