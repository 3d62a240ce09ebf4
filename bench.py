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
    ap.add_argument("--nchan", type=int, default=NCHAN, help="channels (64 = full workload)")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--clean-iters", type=int, default=200)
    return ap.parse_args()


def workload_config(nchan, nvis):
    return {"workload": "large single field: 27-antenna Y (21 km arms), 8 h x 10 s x %d ch "
                        "1.2-1.6 GHz, %d vis, 200 power-law sources + noise, robust NORM R=0, "
                        "4096^2 @ 0.5\" (grid 2049x4096)" % (nchan, nvis),
            "nvis": nvis, "imsize": IMSIZE, "cellsize_arcsec": CELL, "grid": [2049, 4096],
            "kernel": "SF prolate spheroidal 7x7, 128x oversampled",
            "l2": "inputs 1.55 GB > 129 MB L2 (no flush needed)"}


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
        ph = (u_d * float(-two_pi * ll)).add_(v_d * float(-two_pi * mm))
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
    """--impl reference: the reference's CPU path timed on this host's cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    O.lib()
    u, v, w, seed = make_uvw(args.nchan)
    nvis = len(u)
    # bounded sample: one channel's worth of visibilities, spread over all channels
    nsamp = min(nvis, 1010880)
    idx = np.linspace(0, nvis - 1, nsamp).astype(np.int64)
    us, vs, ws = u[idx], v[idx], w[idx]
    vis = make_vis_numpy_sample(u, v, seed, idx)
    wt = np.ones(nsamp, np.float32)
    p = O.params(IMSIZE, CELL, fov=1.0, rmode="NORM", vdec=VDEC)
    g = O.geom(p)
    rc, wt, *_ = O.grdruw2d(wt, us, vs, ws, g.uscale, g.vscale, g.uorigin, g.vorigin, g.nu, g.nv,
                            np.array(list(g.shift)), "NORM", [0.0, 0.0, 0.0])
    scale = nvis / nsamp
    times = []
    for k in range(args.warmup + args.steps):
        t = reference_times(us, vs, ws, vis, wt, g, nsamp / nvis, O)
        if k >= args.warmup:
            times.append(t)
    per = {k: statistics.mean(t[k] for t in times) for k in times[0]}
    step_s = (per["grid"] + per["degrid"]) * scale + per["fft"]
    value = nvis / step_s / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mvis/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": workload_config(args.nchan, nvis),
        "cpu_baseline": {"value": value, "unit": "Mvis/s", "cores": 1, "kind": "port",
                         "sample": "grid+degrid of %d of %d visibilities (every %.0fth) on the "
                                   "full 4096^2 grid, scaled x%.1f, plus the full-size FFTs "
                                   "and grid corrections; C restatement of the reference "
                                   "(oracle/), gcc -O2, single-threaded like SDE"
                                   % (nsamp, nvis, scale, scale),
                         "components_s": per, "cpu": _cpu_model()},
        "e2e": {"value": value, "unit": "Mvis/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


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
    from sde_gb300.imaging import Context, Geom, MajorCycle, Plan, components_image, hogbom

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
    wt = torch.ones(nvis, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    wst = ctx.weights(geom, ud, vd, wd, wt, rmode="NORM", robust=(0.0, 0.0, 0.0))
    ev1.record()
    torch.cuda.synchronize()
    weights_ms = ev0.elapsed_time(ev1)
    t0 = time.perf_counter()
    plan = Plan(ctx, geom, ud, vd, wd, vis, wt)
    torch.cuda.synchronize()
    plan_ms = (time.perf_counter() - t0) * 1e3
    nplan = plan.nvis
    # PSF, normalisation, first dirty image and a CLEAN model (outside the timing)
    grid = ctx.grid_buffer(geom)
    psf = ctx.image_buffer(geom)
    maxpsf = ctx.zeros(1, torch.float32)
    plan.grid(grid, psf=True)
    ctx.image_from_grid(geom, grid, psf)
    ctx.image_max(psf, maxpsf)
    ctx.scale_by_inverse(psf, maxpsf)
    mc = MajorCycle(ctx, geom, plan, maxpsf, psf)
    mc.grid_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cl = hogbom(ctx, geom, mc.dirty, psf, args.clean_iters, 0.1)
    torch.cuda.synchronize()
    hogbom_ms = (time.perf_counter() - t0) * 1e3
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
    L = lib()
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
    for name in ("grid", "finalize", "col_fft", "row_c2r", "row_r2c", "degrid", "degrid_exc"):
        tot, cnt = C.c_double(), C.c_int64()
        L.sde_ctx_kernel_stats(ctx.h, name.encode(), C.byref(tot), C.byref(cnt))
        if cnt.value:
            kern[name] = {"ms_avg": tot.value / cnt.value, "launches": cnt.value}
    L.sde_ctx_profile(ctx.h, 0)
    if dist:
        t = torch.tensor([elapsed_ms], device=dev)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    ms_per_step = elapsed_ms / args.steps
    value = nvis * world / (ms_per_step / 1e3) / 1e6

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

    # ---- e2e through the Fortran drop-in ABI on pinned host arrays ---------------------
    e2e = None
    if rank == 0 and args.e2e_steps > 0:
        e2e = run_e2e(args, torch, L, geom, plan, ud, vd, wd, vis, wt, model, nvis)

    line = {
        "metric": METRIC, "value": value, "unit": "Mvis/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded uv tracks, power-law sky, noise)",
        "config": dict(workload_config(args.nchan, nvis), parallelism="replicas" if world > 1 else "1 GPU"),
        "gpu_launches": int(launches),
        "roofline": roofline,
        "kernels_ms": kern,
        "clocks": clk,
        "e2e": e2e,
        "cpu_baseline": cpu_base,
        "once_per_job_ms": {"weights": weights_ms, "plan_build": plan_ms,
                            "hogbom_%d_iter" % args.clean_iters: hogbom_ms},
        "plan": {"gridding_vis": int(nplan), "bytes": int(plan.nbytes), "ndrop_weighting": int(wst.ndrop)},
    }
    if rank == 0:
        print(json.dumps(line))
    plan.close()
    ctx.close()
    if dist:
        tdist.destroy_process_group()


def run_e2e(args, torch, L, geom, plan, ud, vd, wd, vis, wt, model, nvis):
    """Same step through grdh2d_/fftr2d_/pixcor2d_/grddeh2d_ with pinned host buffers."""
    from sde_gb300 import _abi
    P = C.c_void_p

    def pinned(t):
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t)
        return h

    hu, hv, hw = pinned(ud), pinned(vd), pinned(wd)
    hvis, hwt = pinned(vis), pinned(wt)
    hwt2 = pinned(wt)
    nu, nv, n = geom.nu, geom.nv, geom.nx
    hgrid = torch.zeros((nv, nu), dtype=torch.complex64, pin_memory=True)
    himg = torch.zeros((n, n), dtype=torch.float32, pin_memory=True)
    hmodel = pinned(model)
    hmc = torch.zeros((n, n), dtype=torch.float32, pin_memory=True)
    hmgrid = torch.zeros((nv, nu), dtype=torch.complex64, pin_memory=True)
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
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        step()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / args.e2e_steps
    gb = nu * nv * 8
    img = n * n * 4
    h2d = 24 * nvis + gb + img + img + img + (24 + 12) * nvis + gb
    d2h = gb + img + gb + img + img + gb + 12 * nvis
    return {"value": nvis / dt / 1e6, "unit": "Mvis/s", "ms_per_step": dt * 1e3,
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "path": "grdh2d_ -> fftr2d_(-1) -> pixcor2d_ x2 -> fftr2d_(+1) -> grddeh2d_, pinned "
                    "host arrays, each call uploads, builds its tile plan and downloads"}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
