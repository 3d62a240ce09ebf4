"""Served imaging: a stream of uvmap jobs of different sizes, imaged as they arrive.

Each job is what task/uvmap.f does for one snapshot or channel set: weighting (natural or
robust), PSF, dirty image divided by the PSF peak (task/uvmap.f:212-491).  The server keeps
a fixed set of execution slots; each slot is a host thread with its own CUDA stream and
library context (plans, scratch, grids stay resident on the device while the job runs).
Jobs are admitted in arrival order when a slot is free and their estimated device footprint
fits the HBM budget that the jobs already running leave free; a job larger than the whole
budget runs alone.  Jobs admitted while others are on the GPU run concurrently (their
kernels overlap across the slots' streams): continuous batching at job granularity, with
no job waiting for a batch to fill.  Latency is arrival -> dirty image on the host.

The reference has no server: SDE runs one task per process (its PVM farm, pvm/vistoimgh.f,
hands whole images to worker processes).  Nothing here changes the imaging arithmetic: a
job's image is the single-job uvmap image whether it runs alone or in a mix.
"""
import ctypes as C
import math
import queue
import threading
import time

import numpy as np

from . import _abi, synth
from ._abi import check, lib
from .imaging import Context, Geom

CONFIG5 = dict(rate_hz=200.0, ants=(27, 64), ints=(1, 60), chans=(1, 64), sizes=(256, 4096),
               robust=(-2.0, 2.0), p_natural=0.5, dt_s=10.0, dec=40.0, arm_m=5000.0,
               f_lo=1.2e9, f_hi=1.6e9, cell_arcsec=1.5, n_src=8)


def make_job(idx, seed=synth.SEED_BASE + 5, cfg=None, vis_fn=None, sizes=None, ants=None,
             ints=None, chans=None):
    """Job idx of the seeded config-5 population (host arrays + imaging parameters)."""
    c = dict(CONFIG5, **(cfg or {}))
    rng = np.random.default_rng(seed * 1000003 + idx)
    a = ants or c["ants"]
    n_ant = int(rng.integers(a[0], a[1] + 1))
    it = ints or c["ints"]
    nint = int(rng.integers(it[0], it[1] + 1))
    ch = chans or c["chans"]
    nch = int(rng.integers(ch[0], ch[1] + 1))
    sz = sizes or c["sizes"]
    e_lo, e_hi = int(round(math.log2(sz[0]))), int(round(math.log2(sz[1])))
    imsize = 2 ** int(rng.integers(e_lo, e_hi + 1))
    natural = bool(rng.uniform() < c["p_natural"])
    robust = float(rng.uniform(*c["robust"]))
    pos = synth.y_array(n_ant, c["arm_m"], seed + idx)
    freqs = c["f_lo"] + (np.arange(nch) + 0.5) * ((c["f_hi"] - c["f_lo"]) / nch)
    hours = nint * c["dt_s"] / 3600.0
    u, v, w = synth.uvw_tracks(pos, c["dec"], hours, c["dt_s"], freqs)
    a2r = math.radians(1.0 / 3600.0)
    half = 0.35 * imsize * c["cell_arcsec"] * a2r
    srng = np.random.default_rng(seed + 7 * idx)
    flux = srng.uniform(0.05, 1.0, c["n_src"])
    l = srng.uniform(-half, half, c["n_src"])
    m = srng.uniform(-half, half, c["n_src"])
    fn = vis_fn or synth.visibilities
    vis = np.asarray(fn(u, v, flux, l, m, 1e-3, seed + idx), np.complex64)
    return dict(id=idx, u=u, v=v, w=w, vis=vis, wt=np.ones(len(u), np.float32), imsize=imsize,
                cell=c["cell_arcsec"], dec=c["dec"], natural=natural, robust=robust,
                nvis=len(u))


def footprint_bytes(nvis, imsize):
    """Device bytes a running job holds: inputs (24 B/vis), plan (~45 B/vis) and build
    scratch (~70 B/vis), grid and its raw accumulation (2 x 8 B x NU x NV), PSF and dirty
    image (2 x 4 B x N^2), 4 MB of fixed tables."""
    nu_nv = (imsize // 2 + 1) * imsize
    return int(140 * nvis + 16 * nu_nv + 8 * imsize * imsize + (4 << 20))


class _Slot:
    def __init__(self, device, torch):
        self.stream = torch.cuda.Stream(device=device)
        with torch.cuda.stream(self.stream):
            self.ctx = Context(device.index if device.index is not None else 0, stream=self.stream)


def run_job(ctx, job, torch, pinned=None, out=None):
    """uvmap of one job on ctx's stream through the one-call native job (sde_uvmap): host
    arrays in, dirty image (host) out.  pinned: page-locked tensors of the job's arrays;
    out: a page-locked float32 tensor of the image's shape to write into."""
    g = Geom(job["imsize"], job["cell"], vdec=job["dec"])
    a = _abi.UvmapArgs()
    a.spec = g.spec()
    a.nx, a.ny = g.nx, g.ny
    a.rmode = -1 if job["natural"] else 1  # natural: keep WT; else GRDRUW2D 'NORM'
    a.robust = (C.c_float * 3)(float(job["robust"]), 0.0, 0.0)
    a.ds = 0.0
    a.wuscale, a.wvscale = float(g.wuscale), float(g.wvscale)
    a.out_where = _abi.SDE_HOST
    if pinned is not None:
        ptr = {k: C.c_void_p(t.data_ptr()) for k, t in pinned.items()}
    else:
        arrs = {k: np.ascontiguousarray(job[k], np.float32) for k in ("u", "v", "w", "wt")}
        arrs["vis"] = np.asarray(job["vis"], np.complex64)
        ptr = {k: x.ctypes.data_as(C.c_void_p) for k, x in arrs.items()}
    if out is None:
        out = torch.empty((g.ny, g.nx), dtype=torch.float32, pin_memory=True)
    res = _abi.UvmapResult()
    check(lib().sde_uvmap(ctx.h, C.byref(a), int(job["nvis"]), ptr["u"], ptr["v"], ptr["w"],
                          ptr["vis"], ptr["wt"], _abi.SDE_HOST, C.c_void_p(out.data_ptr()), None,
                          C.byref(res)), "sde_uvmap")
    return out.numpy()


class Server:
    """Slots x streams executing jobs concurrently under an HBM admission budget."""

    def __init__(self, nslots=4, hbm_budget=48 << 30, device=0):
        import torch
        self.torch = torch
        self.device = torch.device("cuda", device)
        torch.cuda.set_device(self.device)
        self.slots = [_Slot(self.device, torch) for _ in range(nslots)]
        self.budget = int(hbm_budget)
        self._lock = threading.Condition()
        self._reserved = 0
        self._running = 0
        self.max_reserved = 0
        self.max_running = 0

    def close(self):
        for s in self.slots:
            s.ctx.close()
        self.slots = []

    # admission: in arrival order, when a slot is free and the footprint fits what the
    # running jobs leave free (a job larger than the budget waits until nothing runs)
    def _admit(self, nbytes):
        with self._lock:
            while not (self._running < len(self.slots) and
                       (self._running == 0 or self._reserved + nbytes <= self.budget)):
                self._lock.wait()
            self._reserved += nbytes
            self._running += 1
            self.max_reserved = max(self.max_reserved, self._reserved)
            self.max_running = max(self.max_running, self._running)

    def _release(self, nbytes):
        with self._lock:
            self._reserved -= nbytes
            self._running -= 1
            self._lock.notify_all()

    def run(self, jobs, arrivals=None, pinned=None, keep_images=False):
        """Serve jobs (dicts from make_job) arriving at arrivals[i] seconds after start
        (None: all at once).  Returns per-job records (arrival, start, finish, ...)."""
        torch = self.torch
        n = len(jobs)
        arrivals = [0.0] * n if arrivals is None else list(arrivals)
        order = sorted(range(n), key=lambda i: arrivals[i])
        admit_q = queue.Queue()
        rec = [None] * n
        images = [None] * n if keep_images else None
        t0 = time.perf_counter()
        errors = []

        def dispatcher():
            # admits strictly in arrival order; a slot worker takes each admitted job
            for i in order:
                delay = t0 + arrivals[i] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                nb = footprint_bytes(jobs[i]["nvis"], jobs[i]["imsize"])
                self._admit(nb)
                admit_q.put((i, nb, time.perf_counter()))
            for _ in self.slots:
                admit_q.put(None)

        def worker(slot):
            torch.cuda.set_device(self.device)
            outbuf = {}
            while True:
                item = admit_q.get()
                if item is None:
                    return
                i, nb, t_adm = item
                try:
                    t_start = time.perf_counter()
                    n_im = jobs[i]["imsize"]
                    if n_im not in outbuf:
                        outbuf[n_im] = torch.empty((n_im, n_im), dtype=torch.float32, pin_memory=True)
                    img = run_job(slot.ctx, jobs[i], torch, None if pinned is None else pinned[i],
                                  outbuf[n_im])
                    t_fin = time.perf_counter()
                    rec[i] = dict(id=jobs[i]["id"], nvis=jobs[i]["nvis"], imsize=jobs[i]["imsize"],
                                  arrival=arrivals[i], admitted=t_adm - t0, start=t_start - t0,
                                  finish=t_fin - t0, latency_ms=(t_fin - t0 - arrivals[i]) * 1e3,
                                  bytes=nb)
                    if keep_images:
                        images[i] = img.copy()
                except Exception as e:  # surfaced after the run
                    errors.append((i, repr(e)))
                finally:
                    self._release(nb)

        th = [threading.Thread(target=worker, args=(s,), daemon=True) for s in self.slots]
        for t in th:
            t.start()
        d = threading.Thread(target=dispatcher, daemon=True)
        d.start()
        d.join()
        for t in th:
            t.join()
        if errors:
            raise RuntimeError("served jobs failed: %s" % errors[:3])
        return (rec, images) if keep_images else rec


def poisson_arrivals(n, rate_hz, seed=synth.SEED_BASE + 55):
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_hz, n))


def summarize(rec):
    lat = np.array([r["latency_ms"] for r in rec])
    nvis = sum(r["nvis"] for r in rec)
    span = max(r["finish"] for r in rec) - min(r["arrival"] for r in rec)
    return dict(jobs=len(rec), p50_ms=float(np.percentile(lat, 50)),
                p99_ms=float(np.percentile(lat, 99)), max_ms=float(lat.max()),
                mvis_s=nvis / span / 1e6, images_s=len(rec) / span, span_s=span)
