#!/usr/bin/env python
"""Benchmark of the imaging hot path on the large single-field workload.

Workload (one "step" = one CLEAN major cycle's grid + degrid):
  27 antennas on a Y of 21 km arms (seeded), 8 h at 10 s integrations x 64 channels over
  1.2-1.6 GHz = 64,696,320 complex64 visibilities; sky of 200 seeded power-law point sources
  (0.1 mJy - 1 Jy, index -1.5) + 1 mJy noise; robust weighting RMODE=NORM, R=0; 4096^2 image
  at 0.5" cells (grid 2049 x 4096).  Per step: grid the residual visibilities (GRDH2D),
  inverse FFT + grid correction + PSF-peak scaling (dirty image), grid-correct + forward FFT
  of the CLEAN model image (IMGGRIDC + IMGFFT), degrid it and form residual = observed -
  model (GRDDEH2D + ARRSUBTR).  Weighting, plan build (sort into uv tiles), PSF and the
  CLEAN model are made once before the timed region.

  value : Mvis/s with everything resident in HBM (visibility arrays 1.55 GB >> 129 MB L2,
          so no L2 flush is needed between steps).
  e2e   : the same step through the Fortran drop-in C ABI (grdh2d_, fftr2d_, pixcor2d_,
          grddeh2d_) on pinned HOST arrays, transfers and plan builds inside the timing.
  --impl reference : the reference's CPU path (the C restatement in oracle/, compiled with
          the host compiler) on this machine's cores, on a bounded sample of the same
          workload, extrapolated to the full step.
"""
import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

def max_over_ranks(x, tdist=None, device=None):
    """x on a single process; with a process group up, the largest x over all ranks (the
    slowest replica sets the whole job's time)."""
    if tdist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def whole_job_mvis(nvis_per_rank, world, seconds_per_step):
    """Whole-job Mvis/s of `world` replicas that each process nvis_per_rank visibilities per
    step, timed by the slowest replica (weak scaling)."""
    return nvis_per_rank * world / seconds_per_step / 1e6


METRIC = "Mvis/s grid+degrid @4096^2 (one CLEAN major cycle per step)"
IMSIZE, CELL, VDEC = 4096, 0.5, 40.0
NCHAN = 64
NSRC = 200


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="single",
                    choices=["single", "mosaic", "serve", "precision", "clark"],
                    help="single: the large single field (headline); mosaic: config 4 "
                         "(49 uneven pointings, batched vs per-pointing); serve: config 5 "
                         "(Poisson stream of jobs, continuous batching); precision: config 3 "
                         "(557 M vis at 8192^2: dirty image error vs the FP64 oracle); clark: "
                         "Clark CLEAN of a 4096^2 dirty image (clean task's default algorithm)")
    ap.add_argument("--no-extras", action="store_true",
                    help="single workload: skip the compact mosaic/serve summaries")
    ap.add_argument("--nchan", type=int, default=NCHAN, help="channels (64 = full workload)")
    ap.add_argument("--e2e-steps", type=int, default=6)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-precision", action="store_true",
                    help="single workload: skip the dirty image's error against the FP64 oracle")
    ap.add_argument("--clean-iters", type=int, default=200)
    ap.add_argument("--plan-opts", default=None,
                    help="item_max,chunk_max of the plan's work items and chunks (library defaults if unset)")
    return ap.parse_args()


def workload_config(nchan, nvis, world=1):
    """The workload's config, identical in both arms (a replica per rank when world > 1)."""
    return {"workload": "large single field: 27-antenna Y (21 km arms), 8 h x 10 s x %d ch "
                        "1.2-1.6 GHz, %d vis, 200 power-law sources + noise, robust NORM R=0, "
                        "4096^2 @ 0.5\" (grid 2049x4096)" % (nchan, nvis),
            "nvis": nvis, "imsize": IMSIZE, "cellsize_arcsec": CELL, "grid": [2049, 4096],
            "kernel": "SF prolate spheroidal 7x7, 128x oversampled",
            "l2": "inputs 1.55 GB > 129 MB L2 (no flush needed)",
            "parallelism": "replicas x%d" % world if world > 1 else "single job"}


# ------------------------------------------------------------------------------------------
def make_uvw(nchan):
    from sde_gb300 import synth
    (u, v, w), seed = synth.config2_uvw(n_chan=nchan)
    return u, v, w, seed


def make_vis_torch(torch, u_d, v_d, seed, device):
    """Visibilities of the seeded sky, computed on the device in chunks (FP32 phases)."""
    from sde_gb300 import synth
    flux, l, m = synth.point_sky(NSRC, IMSIZE * CELL, seed)
    n = u_d.numel()
    re = torch.zeros(n, dtype=torch.float32, device=device)
    im = torch.zeros(n, dtype=torch.float32, device=device)
    two_pi = 2.0 * math.pi
    for S, ll, mm in zip(flux, l, m):
        ph = (u_d * float(two_pi * ll)).add_(v_d * float(two_pi * mm))  # SDE's sign
        re.add_(torch.cos(ph), alpha=float(S))
        im.add_(torch.sin(ph), alpha=float(S))
        del ph
    g = torch.Generator(device=device)
    g.manual_seed(seed + 2)
    re.add_(torch.randn(n, generator=g, device=device), alpha=1e-3)
    im.add_(torch.randn(n, generator=g, device=device), alpha=1e-3)
    return torch.complex(re, im)


def make_vis_numpy_sample(u, v, seed, idx):
    from sde_gb300 import synth
    flux, l, m = synth.point_sky(NSRC, IMSIZE * CELL, seed)
    return synth.visibilities(u[idx], v[idx], flux, l, m, 1e-3, seed)


# ------------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 100 ms during the timed region.

    start() returns once the first sample has been written, so the timed steps that follow
    are covered by samples."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.path = None
        self.gpu = gpu_index

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.fh,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        t0 = time.time()
        while time.time() - t0 < 5.0 and self.proc.poll() is None:
            self.fh.flush()
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "power_w_max": max(power), "samples": len(sm), "reasons": sorted(reasons)}


# ------------------------------------------------------------------------------------------
def reference_times(u, v, w, vis, wt, shift_geom, sample_frac, oracle_mod, fft_full=True):
    """One reference step on a sample: grid+degrid of the sampled visibilities on the full
    4096^2 grid plus the full-size FFTs/corrections; returns component times (s)."""
    O = oracle_mod
    g = shift_geom
    s = np.array(list(g.shift))
    t0 = time.perf_counter()
    rc, grid, sw, lsw = O.grdh2d(vis, wt, u, v, w, g.uscale, g.vscale, g.uorigin, g.vorigin,
                                 g.nu, g.nv, s)
    t1 = time.perf_counter()
    img, _ = O.fftr2d(IMSIZE, IMSIZE, g.fnu, g.nv, -1, xarray=grid)
    ccf = O.grdccf(1 + g.fnu // 2)
    img = O.pixcor2d(img, ccf, g.cenx, g.ceny)
    model = np.zeros_like(img)
    model[IMSIZE // 2 - 1, IMSIZE // 2 - 1] = 1.0
    mc = O.pixcor2d(model, ccf, g.cenx, g.ceny)
    _, mgrid = O.fftr2d(IMSIZE, IMSIZE, g.fnu, g.nv, +1, rarray=mc)
    t2 = time.perf_counter()
    O.grddeh2d(vis, wt, u, v, w, g.uscale, g.vscale, g.uorigin, g.vorigin, mgrid, s)
    t3 = time.perf_counter()
    return {"grid": t1 - t0, "fft": t2 - t1, "degrid": t3 - t2}


def run_reference(args):
    """--impl reference: the reference's CPU path (the oracle's C restatement, 1 thread like
    SDE) on this host, over ONE FULL major cycle of the workload -- every one of the
    visibilities gridded (GRDH2D) and degridded (GRDDEH2D) once, the inverse FFT with grid
    correction of the gridded residual, and the correction and forward FFT of the model.
    GRDH2D's visibility loop is split into K consecutive ranges, one per timed step (the
    accumulation is the oracle's orc_grdh2d_acc, so the grid is that of one pass over all of
    them), and each step degrids the same range; step 0 also transforms the model and the
    last step finalizes the grid and transforms it.  The K steps together are exactly one
    unsampled major cycle, so ms_per_step = cycle time / K is measured, not extrapolated.
    Warm-up steps grid and degrid the first range into a scratch grid."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    from sde_gb300 import synth
    O.lib()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    t_setup = time.perf_counter()
    u, v, w, seed = make_uvw(args.nchan)
    nvis = len(u)
    flux, l, m = synth.point_sky(NSRC, IMSIZE * CELL, seed)
    vis = O.point_vis(u, v, flux, l, m)  # the same sky in double on the host's threads
    rng = np.random.default_rng(seed + 2)
    vis += (rng.normal(0, 1e-3, nvis) + 1j * rng.normal(0, 1e-3, nvis)).astype(np.complex64)
    p = O.params(IMSIZE, CELL, fov=1.0, rmode="NORM", vdec=VDEC)
    g = O.geom(p)
    shift = np.array(list(g.shift))
    # once per job, outside the timing (as the GPU arm's weighting)
    rc, wt, *_ = O.grdruw2d(np.ones(nvis, np.float32), u, v, w, g.uscale, g.vscale, g.uorigin,
                            g.vorigin, g.nu, g.nv, shift, "NORM", [0.0, 0.0, 0.0])
    cf, _, _ = O.grdcf()
    ccf = O.grdccf(1 + g.fnu // 2)
    model = np.zeros((IMSIZE, IMSIZE), np.float32)
    model[IMSIZE // 2 - 1, IMSIZE // 2 - 1] = 1.0
    setup_s = time.perf_counter() - t_setup
    K = max(1, args.steps)
    cuts = [nvis * k // K for k in range(K + 1)]

    def degrid(mgrid, a, b):
        out, _, _ = O.grddeh2d(vis[a:b], wt[a:b], u[a:b], v[a:b], w[a:b], g.uscale, g.vscale,
                               g.uorigin, g.vorigin, mgrid, shift, cf=cf)
        return vis[a:b] - out  # residual = observed - model (ARRSUBTR)

    # warm-up: the first range into a scratch grid, degridded from an empty model grid
    zero_grid = np.zeros((g.nv, g.nu), np.complex64)
    for _ in range(args.warmup):
        W = O.Grdh2dParts(g, cf)
        W.add(vis, wt, u, v, w, cuts[0], cuts[1])
        degrid(zero_grid, cuts[0], cuts[1])
    P = O.Grdh2dParts(g, cf)
    comp = {"grid": 0.0, "degrid": 0.0, "fft": 0.0}
    step_s = []
    mgrid = None
    for k in range(K):
        t0 = time.perf_counter()
        if k == 0:
            mc = O.pixcor2d(model, ccf, g.cenx, g.ceny)  # IMGGRIDC, then IMGFFT (r2c)
            _, mgrid = O.fftr2d(IMSIZE, IMSIZE, g.fnu, g.nv, +1, rarray=mc)
        t1 = time.perf_counter()
        P.add(vis, wt, u, v, w, cuts[k], cuts[k + 1])
        t2 = time.perf_counter()
        degrid(mgrid, cuts[k], cuts[k + 1])
        t3 = time.perf_counter()
        if k == K - 1:
            rc = P.end()
            img, _ = O.fftr2d(IMSIZE, IMSIZE, g.fnu, g.nv, -1, xarray=P.grid)
            img = O.pixcor2d(img, ccf, g.cenx, g.ceny)
        t4 = time.perf_counter()
        comp["fft"] += (t1 - t0) + (t4 - t3)
        comp["grid"] += t2 - t1
        comp["degrid"] += t3 - t2
        step_s.append(t4 - t0)
    total = sum(step_s)
    value = nvis / total / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mvis/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / K * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded uv tracks, power-law sky, noise)",
        "config": workload_config(args.nchan, nvis, world),
        "cpu_baseline": {"value": value, "unit": "Mvis/s", "cores": 1, "kind": "port",
                         "sample": "none: one full major cycle over all %d visibilities (GRDH2D's "
                                   "loop split into %d consecutive ranges, one per step) on the "
                                   "full 4096^2 grid, with the full-size FFTs and corrections; "
                                   "C restatement of the reference (oracle/), gcc -O2, "
                                   "single-threaded like SDE" % (nvis, K),
                         "components_s": comp, "cycle_s": total, "cpu": _cpu_model()},
        "e2e": {"value": value, "unit": "Mvis/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "setup_s": setup_s,
    }
    print(json.dumps(line))


def precision_vs_fp64(geom, u, v, w, vis, wt, dirty, psf):
    """The GPU's PSF-normalised dirty image and PSF of the workload against the FP64 oracle
    (oracle/: the same gridder, inverse FFT and correction in double, on the host's threads,
    with the GPU's reweighted WT): max |GPU - FP64| over CRDNHALF's window and over the whole
    image, as a fraction of the FP64 image's peak."""
    from oracle import oracle as O
    O.lib()
    p = O.params(IMSIZE, CELL, fov=1.0, rmode="NORM", vdec=VDEC)
    og = O.geom(p)
    t0 = time.perf_counter()
    p64 = O.uvmap_image64_mt(og, u, v, w, vis, wt, True)
    d64 = O.uvmap_image64_mt(og, u, v, w, vis, wt, False)
    secs = time.perf_counter() - t0
    pk = p64.max()
    d64 /= pk
    p64 /= pk
    lo, hi = geom.window()
    W = slice(lo, hi)
    dpk = np.abs(d64).max()
    out = {"dirty_window": float(np.abs(dirty - d64)[W, W].max() / dpk),
           "dirty_image": float(np.abs(dirty - d64).max() / dpk),
           "psf_window": float(np.abs(psf - p64)[W, W].max()),
           "psf_image": float(np.abs(psf - p64).max()),
           "bar": 1e-5, "unit": "fraction of the FP64 image peak",
           "oracle": "FP64 restatement of GRDH2D + FFTR2D(-1) + PIXCOR2D (oracle/), %d host threads, %.1f s"
                     % (max(1, min(os.cpu_count() or 1, 64)), secs),
           "window": [lo, hi]}
    out["within_bar"] = out["dirty_window"] <= 1e-5 and out["psf_window"] <= 1e-5
    return out


def _cpu_model():
    try:
        for l in open("/proc/cpuinfo"):
            if l.lower().startswith(("model name", "cpu part")):
                return l.split(":", 1)[1].strip() + " x%d" % os.cpu_count()
    except Exception:
        pass
    return "x%d" % (os.cpu_count() or 0)


# ------------------------------------------------------------------------------------------
def run_gpu(args):
    import torch
    from sde_gb300 import _abi
    from sde_gb300._abi import lib
    from sde_gb300.imaging import Context, Geom, MajorCycle, Plan, components_image

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    # ---- CPU baseline sample first (no GPU state yet), rank 0 only -------------------
    u, v, w, seed = make_uvw(args.nchan)
    nvis = len(u)
    cpu_base = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle as O
        O.lib()
        nsamp = min(nvis, 505440)
        idx = np.linspace(0, nvis - 1, nsamp).astype(np.int64)
        vs_ = make_vis_numpy_sample(u, v, seed, idx)
        p = O.params(IMSIZE, CELL, fov=1.0, rmode="NORM", vdec=VDEC)
        og = O.geom(p)
        wts = np.ones(nsamp, np.float32)
        t = reference_times(u[idx], v[idx], w[idx], vs_, wts, og, nsamp / nvis, O)
        t2 = reference_times(u[idx], v[idx], w[idx], vs_, wts, og, nsamp / nvis, O)
        per = {k: min(t[k], t2[k]) for k in t}
        step_s = (per["grid"] + per["degrid"]) * nvis / nsamp + per["fft"]
        cpu_base = {"value": nvis / step_s / 1e6, "unit": "Mvis/s", "cores": 1, "kind": "port",
                    "sample": "2 steps: grid+degrid of %d of %d visibilities on the full "
                              "4096^2 grid scaled x%.0f, plus full-size FFTs; oracle/ C "
                              "restatement, 1 thread" % (nsamp, nvis, nvis / nsamp),
                    "cpu": _cpu_model()}

    # ---- device data --------------------------------------------------------------------
    ctx = Context(local)
    geom = Geom(IMSIZE, CELL, vdec=VDEC)
    ud = torch.from_numpy(u).to(dev)
    vd = torch.from_numpy(v).to(dev)
    wd = torch.from_numpy(w).to(dev)
    vis = make_vis_torch(torch, ud, vd, seed + rank, dev)
    wt0 = torch.ones(nvis, dtype=torch.float32, device=dev)
    popts = tuple(int(x) for x in args.plan_opts.split(",")) if args.plan_opts else None

    def timed_setup():
        """weighting (in place, on a fresh copy of the input weights) and the plan build:
        device time of the weighting, wall time of the plan build"""
        w_ = wt0.clone()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        st_ = ctx.weights(geom, ud, vd, wd, w_, rmode="NORM", robust=(0.0, 0.0, 0.0))
        ev1.record()
        torch.cuda.synchronize()
        t0_ = time.perf_counter()
        pl_ = Plan(ctx, geom, ud, vd, wd, vis, w_, opts=popts)
        torch.cuda.synchronize()
        return w_, st_, pl_, ev0.elapsed_time(ev1), (time.perf_counter() - t0_) * 1e3

    # the first call also allocates the context's scratch buffers and loads the kernels; a
    # process that images more than one field, or a server, pays the repeat call's time
    _, _, plan, weights_first_ms, plan_first_ms = timed_setup()
    plan.close()
    wt, wst, plan, weights_ms, plan_ms = timed_setup()
    nplan = plan.nvis
    t0 = time.perf_counter()
    # PSF, normalisation, first dirty image and a CLEAN model (outside the timing)
    grid = ctx.grid_buffer(geom)
    psf = ctx.image_buffer(geom)
    maxpsf = ctx.zeros(1, torch.float32)
    plan.grid(grid, psf=True)
    ctx.image_from_grid(geom, grid, psf)
    ctx.image_max(psf, maxpsf)
    ctx.scale_by_inverse(psf, maxpsf)
    torch.cuda.synchronize()
    psf_ms = (time.perf_counter() - t0) * 1e3
    mc = MajorCycle(ctx, geom, plan, maxpsf, psf)
    mc.grid_step()
    dirty0 = mc.dirty.clone()  # the observed field's dirty image (checked against FP64 below)
    torch.cuda.synchronize()
    L = lib()

    # CRDNHALF's window of the dirty image, cut out before the timing: the first strided copy
    # of a process makes torch load that kernel (hundreds of ms), which is not CLEAN's time
    wlo, whi = geom.window()
    drt = mc.dirty[wlo:whi, wlo:whi].contiguous()
    torch.cuda.synchronize()

    def timed_hogbom():
        """wall time of one Hogbom call through the library, and k_hogbom's device time"""
        L.sde_ctx_reset_stats(ctx.h)
        L.sde_ctx_profile(ctx.h, 1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = ctx.hogbom(drt, psf, args.clean_iters, 0.1)
        torch.cuda.synchronize()
        wall = (time.perf_counter() - t0) * 1e3
        tot, cnt = C.c_double(), C.c_int64()
        L.sde_ctx_kernel_stats(ctx.h, b"hogbom", C.byref(tot), C.byref(cnt))
        L.sde_ctx_profile(ctx.h, 0)
        return r, wall, tot.value

    cl, hogbom_first_ms, hogbom_first_kernel_ms = timed_hogbom()
    cl, hogbom_ms, hogbom_kernel_ms = timed_hogbom()
    model = components_image(ctx, geom, cl["cln"])
    torch.cuda.synchronize()

    def step():
        mc.grid_step()
        mc.degrid_step(model)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        tdist.barrier()
    L.sde_ctx_reset_stats(ctx.h)
    L.sde_ctx_profile(ctx.h, 1)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    if dist:
        tdist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    if dist:
        tdist.barrier()
    elapsed_ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    launches = L.sde_ctx_launches(ctx.h)
    kern = {}
    for name in ("grid", "fold_lo", "finalize", "col_fft_fin", "col_fft", "row_c2r", "row_r2c", "degrid",
                 "degrid_exc"):
        tot, cnt = C.c_double(), C.c_int64()
        L.sde_ctx_kernel_stats(ctx.h, name.encode(), C.byref(tot), C.byref(cnt))
        if cnt.value:
            kern[name] = {"ms_avg": tot.value / cnt.value, "launches": cnt.value}
    L.sde_ctx_profile(ctx.h, 0)
    elapsed_ms = max_over_ranks(elapsed_ms, tdist if dist else None, dev)
    ms_per_step = elapsed_ms / args.steps
    value = whole_job_mvis(nvis, world, ms_per_step / 1e3)

    # ---- roofline for the dominant kernel --------------------------------------------
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    grid_bytes = geom.nu * geom.nv * 8
    dom = max(("grid", "degrid"), key=lambda k: kern.get(k, {}).get("ms_avg", 0.0))
    alg_bytes = 24 * nvis + grid_bytes
    dom_ms = kern.get(dom, {}).get("ms_avg", float("nan"))
    achieved = alg_bytes / (dom_ms / 1e3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        try:
            traffic = json.load(open(tp)).get(dom)
        except Exception:
            traffic = None
    pair_ms = kern.get("grid", {}).get("ms_avg", 0) + kern.get("degrid", {}).get("ms_avg", 0)
    roofline = {"bound": "hbm", "kernel": "k_" + dom, "achieved": achieved, "peak": hbm_peak,
                "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
                "peak_source": "measured" if peaks else "fallback",
                "alg_bytes_per_launch": alg_bytes,
                "alg_bytes_formula": "24 B/vis (u,v,w,vis,wt) + NU*NV*8 grid",
                "grid_plus_degrid": {"ms": pair_ms,
                                     "achieved_gbs": (48 * nvis + 2 * grid_bytes) / (pair_ms / 1e3) / 1e9,
                                     "frac": (48 * nvis + 2 * grid_bytes) / (pair_ms / 1e3) / 1e9 / hbm_peak}}

    # ---- one whole imaging job: weighting, plan, PSF, then 5 major cycles, each a step
    # (grid + dirty image + model FFT + degrid) and a Hogbom minor cycle -------------------
    ncyc = 5
    job_ms = weights_ms + plan_ms + psf_ms + ncyc * (ms_per_step + hogbom_ms)
    job = {"cycles": ncyc, "clean_iters_per_cycle": args.clean_iters, "ms": job_ms,
           "setup": "weighting and plan build as a repeat call (first call in once_per_job_ms)",
           "mvis_s": whole_job_mvis(nvis * ncyc, world, job_ms / 1e3),
           "parts_ms": {"weights": weights_ms, "plan_build": plan_ms, "psf": psf_ms,
                        "major_cycle_steps": ncyc * ms_per_step, "hogbom": ncyc * hogbom_ms}}

    # ---- the dirty image's error against the FP64 oracle at full size (rank 0) -----------
    prec = None
    if rank == 0 and not dist and not args.no_precision:
        prec = precision_vs_fp64(geom, u, v, w, vis.cpu().numpy(), wt.cpu().numpy(),
                                 dirty0.cpu().numpy(), psf.cpu().numpy())

    # ---- e2e through the Fortran drop-in ABI on pinned host arrays ---------------------
    e2e = None
    if args.e2e_steps > 0:  # every replica, timed by the slowest
        e2e = run_e2e(args, torch, L, geom, plan, ud, vd, wd, vis, wt, model, nvis,
                      tdist if dist else None, dev, world)
        # the same through ordinary (pageable) host memory, beside it
        e2e["pageable"] = run_e2e(args, torch, L, geom, plan, ud, vd, wd, vis, wt, model, nvis,
                                  tdist if dist else None, dev, world, pinned_host=False)

    line = {
        "metric": METRIC, "value": value, "unit": "Mvis/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded uv tracks, power-law sky, noise)",
        "config": workload_config(args.nchan, nvis, world),
        "gpu_launches": int(launches),
        "roofline": roofline,
        "kernels_ms": kern,
        "clocks": clk,
        "e2e": e2e,
        "cpu_baseline": cpu_base,
        "once_per_job_ms": {"weights": weights_ms, "plan_build": plan_ms, "psf": psf_ms,
                            "weights_first_call": weights_first_ms, "plan_build_first_call": plan_first_ms,
                            "hogbom_%d_iter" % args.clean_iters: hogbom_ms,
                            "hogbom_kernel_%d_iter" % args.clean_iters: hogbom_kernel_ms,
                            "hogbom_first_call": hogbom_first_ms,
                            "hogbom_first_call_kernel": hogbom_first_kernel_ms},
        "job": job,
        "precision": prec,
        "plan": dict(gridding_vis=int(nplan), bytes=int(plan.nbytes), ndrop_weighting=int(wst.ndrop),
                     **_plan_stats(L, plan)),
    }
    plan.close()
    ctx.close()
    if rank == 0 and not dist and not args.no_extras:
        # compact batched / served results beside the headline (outside its timed region)
        try:
            line["mosaic"] = run_mosaic(args, compact=True)
        except Exception as e:  # reported, never silently dropped
            line["mosaic"] = {"error": repr(e)}
        try:
            line["serve"] = run_serve(args, compact=True)
        except Exception as e:
            line["serve"] = {"error": repr(e)}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        tdist.destroy_process_group()


MOSAIC_METRIC = "Mvis/s mosaic dirty imaging (49 uneven pointings, batched + CUDA graph)"


def _device_vis_fn(torch, dev):
    """synth.visibilities on the device (FP64 phases), same sign and noise model."""
    def fn(u, v, flux, l, m, noise, seed):
        ud = torch.as_tensor(u, device=dev, dtype=torch.float64)
        vd = torch.as_tensor(v, device=dev, dtype=torch.float64)
        acc = torch.zeros(len(u), dtype=torch.complex128, device=dev)
        for S, ll, mm in zip(flux, l, m):
            acc += float(S) * torch.exp(2j * math.pi * (ud * float(ll) + vd * float(mm)))
        rng = np.random.default_rng(seed + 2)
        out = acc.to(torch.complex64).cpu().numpy()
        if noise > 0:
            out += (rng.normal(0, noise, len(u)) + 1j * rng.normal(0, noise, len(u))).astype(np.complex64)
        return out
    return fn


def run_mosaic(args, compact=False):
    """Config 4: dirty mosaic of 49 uneven pointings.  A step is the dirty imaging pass of
    the whole mosaic (every pointing gridded, transformed, PSF-normalised, combined)."""
    import torch
    from sde_gb300 import mosaic, synth
    from sde_gb300.imaging import Context
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ctx = Context(local)
    pts, c = synth.config4(vis_fn=_device_vis_fn(torch, ctx.device))
    nvis_in = sum(len(p["u"]) for p in pts)
    tune = mosaic.autotune(ctx, pts, c["cell_arcsec"], reps=3)
    m = mosaic.Mosaic(ctx, pts, c["cell_arcsec"], opts=tune["best"])
    nvis = m.nvis
    steps = max(args.steps if not compact else 20, 1)
    warm = max(args.warmup, 3)

    def timed(fn):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ctx.stream)
        for _ in range(steps):
            fn()
        e1.record(ctx.stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    clocks = ClockSampler(local)
    clocks.start()
    graph_ms = timed(lambda: m.dirty(graph=True))
    clk = clocks.stop()
    eager_ms = timed(lambda: m.dirty(graph=False))
    loop_ms = timed(lambda: m.dirty_loop())
    nodes = m.graph_nodes
    m.close()
    # e2e: host arrays -> device, weighting, plans, batch, PSF, dirty mosaic, mosaic to host
    e2e_ms = []
    for _ in range(1 if compact else 2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        me = mosaic.Mosaic(ctx, pts, c["cell_arcsec"], opts=tune["best"])
        me.dirty(graph=False)
        mos = me.read(-1)
        torch.cuda.synchronize()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        me.close()
    h2d = sum(p["u"].nbytes * 3 + p["vis"].nbytes + p["wt"].nbytes for p in pts)
    res = {
        "batched_graph": {"ms": graph_ms, "mvis_s": nvis / graph_ms / 1e3,
                          "dirty_images_s": m.n / graph_ms * 1e3, "graph_nodes": nodes},
        "batched_eager": {"ms": eager_ms, "mvis_s": nvis / eager_ms / 1e3,
                          "dirty_images_s": m.n / eager_ms * 1e3},
        "per_pointing_loop": {"ms": loop_ms, "mvis_s": nvis / loop_ms / 1e3,
                              "dirty_images_s": m.n / loop_ms * 1e3},
        "speedup_vs_loop": loop_ms / graph_ms,
        "autotune": {"chosen": list(tune["best"]),
                     "table_ms": [[list(k), round(v, 4)] for k, v in tune["table"]]},
        "nvis": int(nvis), "pointings": m.n,
        "image_sizes": sorted(int(p["imsize"]) for p in pts),
        "mosaic_px": [m.layout["mnx"], m.layout["mny"]],
    }
    if compact:
        ctx.close()
        return res
    line = {
        "metric": MOSAIC_METRIC, "value": res["batched_graph"]["mvis_s"], "unit": "Mvis/s",
        "n_gpus": 1, "steps": steps, "warmup": warm, "ms_per_step": graph_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded config 4: hex mosaic, Gaussian PB 30', log-uniform Nvis, pow2 sizes)",
        "config": {"workload": "config 4 mosaic: %d pointings, %d vis, images %s, 2\" cells, "
                               "uniform weighting, linear mosaic %dx%d" % (m.n, nvis_in,
                                                                         "256-2048", m.layout["mnx"],
                                                                         m.layout["mny"]),
                   "l2": "per-pointing visibility records 16 B x %d vis" % nvis},
        "gpu_launches": int(nodes),
        "clocks": clk,
        "e2e": {"value": nvis_in / statistics.mean(e2e_ms) / 1e3, "unit": "Mvis/s",
                "ms_per_step": statistics.mean(e2e_ms), "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(mos.nbytes),
                "path": "Mosaic(host pointings): upload, weighting, plans, batch, PSF; dirty; "
                        "mosaic to host"},
        "cpu_baseline": _mosaic_cpu_baseline(pts, c) if rank == 0 and not args.no_cpu_baseline else None,
        "mosaic": res,
    }
    ctx.close()
    return line


def _mosaic_cpu_baseline(pts, c, budget_s=12.0):
    """The reference's per-pointing uvmap (oracle/ C restatement, 1 thread) on a sample of
    the pointings (smallest images first, until the time budget), Mvis/s over the sample."""
    from oracle import oracle as O
    O.lib()
    order = sorted(range(len(pts)), key=lambda i: (pts[i]["imsize"], len(pts[i]["u"])))
    done, nv, t_all = [], 0, 0.0
    for i in order:
        p = pts[i]
        par = O.params(p["imsize"], c["cell_arcsec"], fov=1.0, rmode="NONE", vdec=c["dec"])
        t0 = time.perf_counter()
        O.uvmap(par, p["u"], p["v"], p["w"], p["vis"], p["wt"])
        t_all += time.perf_counter() - t0
        nv += len(p["u"])
        done.append(i)
        if t_all > budget_s:
            break
    return {"value": nv / t_all / 1e6, "unit": "Mvis/s", "cores": 1, "kind": "port",
            "sample": "uvmap (uniform weights, PSF, dirty) of %d of %d pointings (%d vis, "
                      "images %s), oracle/ C restatement, 1 thread"
                      % (len(done), len(pts), nv, sorted({pts[i]["imsize"] for i in done})),
            "dirty_images_s": len(done) / t_all}


SERVE_METRIC = ("Mvis/s served uvmap jobs (config 5 population, all queued), "
                "with p50/p99 ms latency at 200 jobs/s Poisson")


def run_serve(args, compact=False):
    """Config 5: uvmap jobs of the seeded config-5 population (27-64 antennas, 1-60
    integrations, 1-64 channels, 256^2-4096^2, natural or robust R in [-2, 2]) served by
    slot-parallel continuous batching.  (1) A Poisson stream at 200 jobs/s: p50/p99
    latency, arrival to dirty image on the host.  (2) Saturation: the same jobs all queued
    at once, served (several slots) vs serial (one slot, one job at a time): Mvis/s."""
    import torch
    from sde_gb300 import serve
    from sde_gb300._abi import lib
    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ntpl = 24 if compact else 48
    tpl = [serve.make_job(i, vis_fn=_device_vis_fn(torch, dev)) for i in range(ntpl)]

    def pin(j):
        d = {}
        for k in ("u", "v", "w", "wt"):
            d[k] = torch.from_numpy(np.ascontiguousarray(j[k])).pin_memory()
        d["vis"] = torch.from_numpy(np.asarray(j["vis"], np.complex64).view(np.float32)).pin_memory()
        return d

    pins = [pin(j) for j in tpl]
    duration = 2.0 if compact else 5.0
    rate = serve.CONFIG5["rate_hz"]
    n_stream = int(rate * duration)
    rng = np.random.default_rng(serve.synth.SEED_BASE + 56)
    pick = rng.integers(ntpl, size=n_stream)
    jobs = [tpl[k] for k in pick]
    pinned = [pins[k] for k in pick]
    arrivals = serve.poisson_arrivals(n_stream, rate)
    nslots = 6
    srv = serve.Server(nslots=nslots, hbm_budget=64 << 30, device=local)
    srv.run(jobs[:2 * nslots], None, pinned[:2 * nslots])  # warm-up: tables, allocator
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    rec = srv.run(jobs, arrivals, pinned)
    clk = clocks.stop()
    st = serve.summarize(rec)
    st.update(offered_jobs_s=rate, max_running=srv.max_running,
              max_reserved_gb=srv.max_reserved / 2 ** 30)
    nsat = 48 if compact else 96
    t0 = time.perf_counter()
    srv.run(jobs[:nsat], None, pinned[:nsat])
    t_served = time.perf_counter() - t0
    launches = sum(lib().sde_ctx_launches(sl.ctx.h) for sl in srv.slots)
    srv.close()
    one = serve.Server(nslots=1, hbm_budget=64 << 30, device=local)
    one.run(jobs[:2], None, pinned[:2])
    t0 = time.perf_counter()
    one.run(jobs[:nsat], None, pinned[:nsat])
    t_serial = time.perf_counter() - t0
    one.close()
    nv_sat = sum(j["nvis"] for j in jobs[:nsat])
    res = {
        "stream": st,
        "saturated": {"jobs": nsat, "nvis": int(nv_sat), "slots": nslots,
                      "served_mvis_s": nv_sat / t_served / 1e6, "served_images_s": nsat / t_served,
                      "serial_mvis_s": nv_sat / t_serial / 1e6, "serial_images_s": nsat / t_serial,
                      "speedup": t_serial / t_served},
        "templates": ntpl,
        "job_nvis_mean": float(np.mean([j["nvis"] for j in jobs])),
    }
    if compact:
        return res
    h2d = float(np.mean([j["nvis"] * 24 for j in jobs]))
    d2h = float(np.mean([j["imsize"] ** 2 * 4 for j in jobs]))
    line = {
        "metric": SERVE_METRIC, "value": res["saturated"]["served_mvis_s"], "unit": "Mvis/s",
        "n_gpus": 1, "steps": nsat, "warmup": 2 * nslots,
        "ms_per_step": t_served / nsat * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded config-5 job population, %d templates)" % ntpl,
        "config": {"workload": "config 5 served uvmap: Poisson %g jobs/s for %g s (%d jobs), "
                               "27-64 ants, 1-60 ints, 1-64 ch, 256-4096 px, natural or robust"
                               % (rate, duration, n_stream), "slots": nslots,
                   "hbm_budget_gb": 64},
        "gpu_launches": int(launches),
        "clocks": clk,
        "latency_ms": {"p50": st["p50_ms"], "p99": st["p99_ms"], "max": st["max_ms"]},
        "e2e": {"value": res["saturated"]["served_mvis_s"], "unit": "Mvis/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "path": "host (pinned) job arrays -> weighting, plan, PSF, dirty -> image to host"},
        "cpu_baseline": _serve_cpu_baseline(tpl) if rank == 0 and not args.no_cpu_baseline else None,
        "serve": res,
    }
    return line


def _serve_cpu_baseline(tpl, budget_s=12.0):
    """uvmap of a sample of the job population with the oracle/ C restatement (1 thread)."""
    from oracle import oracle as O
    O.lib()
    order = sorted(range(len(tpl)), key=lambda i: tpl[i]["nvis"] * max(tpl[i]["imsize"], 1024))
    nv, t_all, done = 0, 0.0, 0
    for i in order:
        j = tpl[i]
        par = O.params(j["imsize"], j["cell"], fov=1.0,
                       rmode="NONE" if j["natural"] else "NORM", vdec=j["dec"])
        t0 = time.perf_counter()
        O.uvmap(par, j["u"], j["v"], j["w"], j["vis"], j["wt"])
        t_all += time.perf_counter() - t0
        nv += j["nvis"]
        done += 1
        if t_all > budget_s:
            break
    return {"value": nv / t_all / 1e6, "unit": "Mvis/s", "cores": 1, "kind": "port",
            "sample": "uvmap of the %d cheapest of %d job templates (%d vis), oracle/ C "
                      "restatement, 1 thread" % (done, len(tpl), nv),
            "images_s": done / t_all}


def _plan_stats(L, plan):
    a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
    L.sde_plan_stats(plan.h, C.byref(a), C.byref(b), C.byref(c))
    return {"work_items": a.value, "chunks": b.value, "degrid_exceptions": c.value}


def _shim_stats(L):
    h, m = C.c_int64(), C.c_int64()
    L.sde_shim_cache_stats(C.byref(h), C.byref(m))
    return {"hits": h.value, "misses": m.value}


def run_precision(args):
    """Config 3: dirty image of 557 M visibilities at 8192^2 (natural weights) from the GPU
    path, with and without compensated cross-item sums, against the FP64 oracle (the same
    algorithm in double on the host); max |error| over the CRDNHALF window and the image as
    a fraction of the FP64 peak."""
    import torch
    from oracle import precision
    from sde_gb300 import synth
    from sde_gb300.imaging import Context
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ctx = Context(local)
    t0 = time.perf_counter()
    (u, v, w), seed = synth.config3_uvw()
    c = synth.CONFIG3
    flux, l, m = synth.point_sky(200, c["imsize"] * c["cellsize"], seed)
    vis = _device_vis_fn(torch, ctx.device)(u, v, flux[:c["n_src"]], l[:c["n_src"]],
                                            m[:c["n_src"]], c["noise"], seed)
    wt = np.ones(len(u), np.float32)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    r = precision.study(ctx, (u, v, w, vis, wt), imsize=c["imsize"], cell=c["cellsize"],
                        vdec=c["vdec"], reference=False)
    study_s = time.perf_counter() - t0
    ctx.close()
    return {
        "metric": "dirty-image error vs FP64 oracle, config 3 (557 M vis, 8192^2), CRDNHALF window",
        "value": r["compensated"]["window"], "unit": "fraction of image peak",
        "higher_is_better": False, "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": None,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded config 3: 64 ants, 12 h x 5 s x 32 ch, 20 sources)",
        "config": {"workload": "config 3 precision: %d vis, %d^2 at %g\"" % (len(u), c["imsize"],
                                                                           c["cellsize"])},
        "precision": r, "seconds": {"generate": gen_s, "study": study_s},
    }


CLARK_KW = dict(niter=5000, gain=0.1, flux=0.0, numcl=32768, bpatch=128)


def run_clark(args):
    """Clark CLEAN (task/clean.f CLARK branch with IMGCCLEA) of the dirty image of a seeded
    27-antenna Y-array observation (8 h, 4 channels, four point sources and a Gaussian) at
    4096^2 and 0.25"; a step is one whole CLEAN of 5000 iterations from the same dirty image
    and PSF (minor cycles on the device, image-plane residual by FFT each major cycle)."""
    import torch
    from sde_gb300 import synth
    from sde_gb300._abi import lib
    from sde_gb300.imaging import Context, Geom, clark, uvmap
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if rank != 0:
        return None
    torch.cuda.set_device(local)
    n, cell, ntime, nchan, dec, seed = 4096, 0.25, 192, 4, 40.0, 7
    pos = synth.y_array(27, 3000.0, seed)
    u, v, w = synth.uvw_tracks(pos, dec, 8.0, 8.0 * 3600.0 / ntime, 1.4e9 * (1.0 + 0.05 * np.arange(nchan)))
    as2r = math.radians(1.0 / 3600.0)
    fov = n * cell * as2r
    vis = synth.visibilities(u, v, np.array([1.0, 0.3, 0.1, 0.05]), np.array([0.0, 0.12, -0.2, 0.3]) * fov,
                             np.array([0.0, -0.08, 0.15, -0.25]) * fov, 1e-3, seed,
                             gauss=[(0.2, -0.1 * fov, -0.2 * fov, 8 * cell * as2r)])
    ctx = Context(local)
    g = Geom(n, cell, vdec=dec)
    t = {k: ctx.tensor(a) for k, a in (("u", u), ("v", v), ("w", w), ("vis", vis),
                                       ("wt", np.ones(len(u), np.float32)))}
    r = uvmap(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"], rmode="UNIFORM")
    dirty, psf = r["dirty"], r["psf"]
    for _ in range(max(1, args.warmup)):
        res = clark(ctx, dirty, psf, **CLARK_KW)
    ctx.sync()
    L = lib()
    L.sde_ctx_reset_stats(ctx.h)
    L.sde_ctx_profile(ctx.h, 1)
    steps = max(1, min(args.steps, 10))
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        res = clark(ctx, dirty, psf, **CLARK_KW)
        ctx.sync()
        times.append(time.perf_counter() - t0)
    kern = {}
    for k in ("clark_select", "clark_minor", "clark_cmul", "clark_sub", "col_fft", "row_c2r", "row_r2c"):
        tot, cnt = C.c_double(), C.c_int64()
        L.sde_ctx_kernel_stats(ctx.h, k.encode(), C.byref(tot), C.byref(cnt))
        if cnt.value:
            kern[k] = {"ms_per_clean": tot.value / steps, "launches_per_clean": cnt.value // steps}
    L.sde_ctx_profile(ctx.h, 0)
    ms = statistics.median(times) * 1e3
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        dn, pn = dirty.cpu().numpy(), psf.cpu().numpy()
        t0 = time.perf_counter()
        ro = O.clark(dn, pn, **CLARK_KW)
        cpu = {"value": (time.perf_counter() - t0) * 1e3, "unit": "ms per CLEAN", "cores": 1, "kind": "port",
               "sample": "the same CLEAN (same dirty image and PSF) by the oracle C restatement, 1 thread",
               "aniter": int(ro["aniter"]), "ncycles": int(ro["ncycles"])}
    return {"metric": "ms per Clark CLEAN (4096^2, 5000 iterations)", "value": ms, "unit": "ms",
            "higher_is_better": False, "n_gpus": 1, "steps": steps, "warmup": max(1, args.warmup),
            "dtype": "f32", "data": "synthetic (seeded 27-antenna Y array, 8 h x 4 ch, 4 points + Gaussian)",
            "config": {"workload": "Clark CLEAN of a 4096^2 dirty image, %d vis, uniform weighting" % len(u),
                       **CLARK_KW},
            "aniter": int(res["aniter"]), "ncycles": int(res["ncycles"]), "kernels": kern,
            "ms_each": [round(x * 1e3, 3) for x in times], "cpu_baseline": cpu}


def run_e2e(args, torch, L, geom, plan, ud, vd, wd, vis, wt, model, nvis, tdist=None, dev=None, world=1,
            pinned_host=True):
    """Same step through grdh2d_/fftr2d_/pixcor2d_/grddeh2d_ with host buffers -- page-locked
    (pinned_host) or ordinary pageable memory, as a Fortran program's MEMR arrays are; with a
    process group, every replica runs it and the slowest one's time counts."""
    from sde_gb300 import _abi
    P = C.c_void_p

    def pinned(t):
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=pinned_host)
        h.copy_(t)
        return h

    hu, hv, hw = pinned(ud), pinned(vd), pinned(wd)
    hvis, hwt = pinned(vis), pinned(wt)
    hwt2 = pinned(wt)
    nu, nv, n = geom.nu, geom.nv, geom.nx
    hgrid = torch.zeros((nv, nu), dtype=torch.complex64, pin_memory=pinned_host)
    himg = torch.zeros((n, n), dtype=torch.float32, pin_memory=pinned_host)
    hmodel = pinned(model)
    hmc = torch.zeros((n, n), dtype=torch.float32, pin_memory=pinned_host)
    hmgrid = torch.zeros((nv, nu), dtype=torch.complex64, pin_memory=pinned_host)
    hout = pinned(vis)
    from sde_gb300.imaging import fftpwr2
    # the caller-side tables, built by the library's GRDCF/GRDCCF entry points
    cf = np.zeros(1 + 8 * 129, np.float32)
    L.grdcf_(b"SF", cf.ctypes.data_as(P), C.byref(C.c_int()), C.byref(C.c_int()), 2)
    ccflen = 1 + fftpwr2(n) // 2
    ccf = np.zeros(ccflen, np.float32)
    L.grdccf_(b"SF", ccf.ctypes.data_as(P), C.byref(C.c_int(ccflen)), 2)
    I = lambda x: C.byref(C.c_int(int(x)))
    Fv = lambda x: C.byref(C.c_float(float(x)))
    ptr = lambda t: P(t.data_ptr())
    shift = geom.shift.copy()
    sumwt = C.c_float()
    psf0 = C.c_int(0)

    def step():
        L.grdh2d_(ptr(hvis), ptr(hwt), ptr(hu), ptr(hv), ptr(hw), I(nvis), Fv(geom.uscale), Fv(0),
                  Fv(geom.vscale), Fv(0), I(geom.uorigin), I(geom.vorigin), ptr(hgrid),
                  C.byref(psf0), I(nu), I(nv), cf.ctypes.data_as(P), I(3), I(128),
                  cf.ctypes.data_as(P), I(3), I(128), shift.ctypes.data_as(P), C.byref(sumwt))
        L.fftr2d_(ptr(himg), ptr(hgrid), None, None, None, I(n), I(n), I(geom.fnu), I(nv), I(-1))
        L.pixcor2d_(ptr(himg), I(n), I(n), ccf.ctypes.data_as(P), I(ccflen), b"CORRECT",
                    ptr(himg), Fv(geom.cenx), Fv(geom.ceny), 7)
        L.pixcor2d_(ptr(hmodel), I(n), I(n), ccf.ctypes.data_as(P), I(ccflen), b"CORRECT",
                    ptr(hmc), Fv(geom.cenx), Fv(geom.ceny), 7)
        L.fftr2d_(ptr(hmc), ptr(hmgrid), None, None, None, I(n), I(n), I(geom.fnu), I(nv), I(1))
        L.grddeh2d_(ptr(hout), ptr(hwt2), ptr(hu), ptr(hv), ptr(hw), I(nvis), Fv(geom.uscale),
                    Fv(0), Fv(geom.vscale), Fv(0), I(geom.uorigin), I(geom.vorigin), ptr(hmgrid),
                    I(nu), I(nv), cf.ctypes.data_as(P), I(3), I(128), cf.ctypes.data_as(P), I(3),
                    I(128), shift.ctypes.data_as(P))
        if _abi.sysi().error:
            raise RuntimeError("drop-in call reported an error")

    step()  # warm-up (allocates the shim's device buffers)
    torch.cuda.synchronize()
    if tdist is not None:
        tdist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        step()
    torch.cuda.synchronize()
    dt = max_over_ranks((time.perf_counter() - t0) / args.e2e_steps, tdist, dev)
    gb = nu * nv * 8
    img = n * n * 4
    # grdh2d_: VIS, WT, U, V, W up, grid down; fftr2d_(-1): grid up, image and the
    # column-transformed grid down; pixcor2d_ x2: image up and down; fftr2d_(+1): image up,
    # grid down; grddeh2d_: U, V, W, WT and the model grid up, VIS down -- plus VIS and WT up
    # when some WT <= 0 (the points GRDDEH2D leaves as they are), and WT down when a point
    # was not degridded (WT negated)
    flagged = bool((hwt <= 0).any().item())
    negated = bool(((hwt2 < 0) & (hwt > 0)).any().item())
    h2d = 24 * nvis + gb + img + img + img + 16 * nvis + gb + (12 * nvis if flagged else 0)
    d2h = gb + img + gb + img + img + gb + 8 * nvis + (4 * nvis if negated else 0)
    return {"value": whole_job_mvis(nvis, world, dt), "unit": "Mvis/s", "ms_per_step": dt * 1e3,
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "path": "grdh2d_ -> fftr2d_(-1) -> pixcor2d_ x2 -> fftr2d_(+1) -> grddeh2d_, %s "
                    "host arrays; every call uploads its inputs and downloads its outputs; "
                    "GRDH2D/GRDDEH2D reuse their tile plan when U, V, W, WT are bitwise "
                    "unchanged (compared on the device)" % ("pinned" if pinned_host else "pageable"),
            "flagged_wt": flagged, "negated_wt": negated,
            "plan_cache": _shim_stats(L)}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "mosaic":
        line = run_mosaic(args)
        if line:
            print(json.dumps(line))
    elif args.workload == "serve":
        line = run_serve(args)
        if line:
            print(json.dumps(line))
    elif args.workload == "precision":
        line = run_precision(args)
        if line:
            print(json.dumps(line))
    elif args.workload == "clark":
        line = run_clark(args)
        if line:
            print(json.dumps(line))
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
