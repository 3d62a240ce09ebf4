// api.cu -- context management, the resident plan API, and the Fortran-77 drop-in entry
// points (grdh2d_, grddeh2d_, grduwt2d_, grdruw2d_, fftr2d_, pixcor2d_, pix2drcl_,
// pixisama_) with the reference's ERROR/ERRREPOR/MSGPUT conventions.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>

#include "common.cuh"

// ---------------------------------------------------------------------------------------
// error text
static thread_local char g_err[512] = "";

void sde_set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

extern "C" const char *sde_last_error(void) { return g_err; }
extern "C" int sde_version(void) { return 1; }

// ---------------------------------------------------------------------------------------
// 'SF' tables on the host: the prolate spheroidal function m=6, alpha=1 by F. Schwab's
// rational approximation (as in grd/grdsf.f), the gridding function (1-nu^2) psi(nu)
// sampled 128x over support 3 and normalised to unit sum (grd/grdcf.f:53-64, 84-90), and the
// grid-correction table psi((i-1)/(CCFLEN-1)) (grd/grdccf.f:48-52).
double sf_grdsf(double nu) {
    static const double P[2][5] = {
        {8.203343e-2, -3.644705e-1, 6.278660e-1, -5.335581e-1, 2.312756e-1},
        {4.028559e-3, -3.697768e-2, 1.021332e-1, -1.201436e-1, 6.412774e-2}};
    static const double Q[2][3] = {{1.0, 8.212018e-1, 2.078043e-1}, {1.0, 9.599102e-1, 2.918724e-1}};
    int part;
    double nuend;
    if (nu >= 0.0 && nu < 0.75) {
        part = 0;
        nuend = 0.75;
    } else if (nu >= 0.75 && nu <= 1.0) {
        part = 1;
        nuend = 1.0;
    } else {
        return 0.0;
    }
    double x = nu * nu - nuend * nuend;
    double top = P[part][0], bot = Q[part][0];
    for (int k = 1; k <= 4; k++) top = top + P[part][k] * pow(x, (double)k);
    for (int k = 1; k <= 2; k++) bot = bot + Q[part][k] * pow(x, (double)k);
    return bot != 0.0 ? top / bot : 0.0;
}

void sf_cf_table(float *cf) {
    const int off = (SUPP + 1) * OSAMP;  // 0-based centre
    for (int i = 0; i < CFLEN; i++) cf[i] = 0.0f;
    for (int i = 0; i <= SUPP * OSAMP; i++) {
        double nu = (double)i / (double)(SUPP * OSAMP);
        cf[off + i] = (float)((1 - pow(nu, 2.0)) * sf_grdsf(nu));
        cf[off - i] = cf[off + i];
    }
    float sum = 0.0f;
    for (int i = -(SUPP + 1) * OSAMP; i <= (SUPP + 1) * OSAMP; i++) sum = sum + cf[off + i];
    for (int i = -(SUPP + 1) * OSAMP; i <= (SUPP + 1) * OSAMP; i++) cf[off + i] = cf[off + i] / sum;
}

void sf_ccf_table(float *ccf, int ccflen) {
    for (int i = 1; i <= ccflen; i++) ccf[i - 1] = (float)sf_grdsf((double)(i - 1) / (double)(ccflen - 1));
}

int fftpwr2(int i) {
    if (i < 1) return 1;
    int lg = (int)lroundf(logf((float)i) / logf(2.0f));
    int p = 1;
    for (int k = 0; k < lg; k++) p *= 2;
    while (p < i) p *= 2;
    return p;
}

// ---------------------------------------------------------------------------------------
// context
static void drain_events(sde_ctx *c);

// Device memory is stream-ordered (cudaMallocAsync / cudaFreeAsync on the context's stream,
// from the device's pool, which keeps freed memory for reuse): allocating and freeing never
// synchronises the device, so contexts working on different streams (concurrent jobs) do not
// stall one another.  Memory used on another stream is synchronised with the context's
// stream first (the context, batch and table set-up paths do).
int ctx_alloc(sde_ctx *ctx, void **p, size_t bytes) {
    cudaError_t e = cudaMallocAsync(p, bytes ? bytes : 16, ctx->stream);
    if (e != cudaSuccess) {
        *p = nullptr;
        sde_set_error("cudaMallocAsync(%zu): %s", bytes, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? SDE_ENOMEM : SDE_ECUDA;
    }
    return SDE_OK;
}

void ctx_free(sde_ctx *ctx, void *p, size_t bytes) {
    if (p) cudaFreeAsync(p, ctx->stream);
}

int ctx_read_small(sde_ctx *ctx, cudaStream_t st, void *dst, const void *src, size_t bytes) {
    if (bytes > H_SMALL_BYTES) {
        sde_set_error("ctx_read_small: %zu bytes", bytes);
        return SDE_EINVAL;
    }
    SDE_CUDA_TRY(cudaMemcpyAsync(ctx->h_small, src, bytes, cudaMemcpyDeviceToHost, st));
    SDE_CUDA_TRY(cudaStreamSynchronize(st));
    memcpy(dst, ctx->h_small, bytes);
    return SDE_OK;
}

int ctx_scratch(sde_ctx *ctx, const char *name, size_t bytes, void **out) {
    DevBuf &b = ctx->scratch[name];
    if (b.bytes < bytes) {
        if (b.p) {
            ctx_free(ctx, b.p, b.bytes);  // stream-ordered: after the work that used it
            ctx->bytes -= (int64_t)b.bytes;
            b.p = nullptr;
            b.bytes = 0;
        }
        size_t want = bytes + bytes / 8 + 256;
        SDE_TRY(ctx_alloc(ctx, &b.p, want));
        b.bytes = want;
        ctx->bytes += (int64_t)want;
    }
    *out = b.p;
    return SDE_OK;
}

int ctx_twiddles(sde_ctx *ctx, int n, const float2 **out) {
    auto it = ctx->twiddles.find(n);
    if (it != ctx->twiddles.end()) {
        *out = it->second;
        return SDE_OK;
    }
    int h = n > 0 ? n : 1;  // full period: exp(+2 pi i k/n), k < n
    std::vector<float2> t((size_t)h);
    for (int k = 0; k < h; k++) {
        double a = 2.0 * M_PI * (double)k / (double)n;
        t[(size_t)k] = make_float2((float)cos(a), (float)sin(a));
    }
    float2 *d;
    SDE_TRY(ctx_alloc(ctx, (void **)&d, sizeof(float2) * (size_t)h));
    // pageable source: returns once the host data has been staged, so t may go away
    SDE_CUDA_TRY(cudaMemcpyAsync(d, t.data(), sizeof(float2) * (size_t)h, cudaMemcpyHostToDevice,
                                 ctx->stream));
    ctx->bytes += (int64_t)(sizeof(float2) * h);
    ctx->twiddles[n] = d;
    *out = d;
    return SDE_OK;
}

extern "C" int sde_ctx_create(sde_ctx **out, int device) {
    if (!out) return SDE_EINVAL;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        sde_set_error("no CUDA device: %s", e != cudaSuccess ? cudaGetErrorString(e) : "count 0");
        return SDE_ENODEV;
    }
    if (device < 0 || device >= ndev) {
        sde_set_error("device %d out of range", device);
        return SDE_EINVAL;
    }
    SDE_CUDA_TRY(cudaSetDevice(device));
    sde_ctx *c = new sde_ctx();
    c->device = device;
    int rc = SDE_OK;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        sde_set_error("device setup failed");
        delete c;
        return SDE_ECUDA;
    }
    c->own_stream = true;
    c->num_sms = prop.multiProcessorCount;
    {
        // the default pool keeps memory freed by cudaFreeAsync for reuse instead of
        // returning it at every synchronisation
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    if ((rc = ctx_alloc(c, (void **)&c->d_status, sizeof(int) * STATUS_COUNT)) ||
        (rc = ctx_alloc(c, (void **)&c->d_cf, sizeof(float) * CFLEN)) ||
        (rc = ctx_alloc(c, (void **)&c->d_cft, sizeof(float) * 129 * 8))) {
        sde_ctx_destroy(c);
        return rc;
    }
    if (cudaMallocHost((void **)&c->h_status, sizeof(int) * STATUS_COUNT) != cudaSuccess ||
        cudaMallocHost((void **)&c->h_small, H_SMALL_BYTES) != cudaSuccess) {
        sde_ctx_destroy(c);
        return SDE_ENOMEM;
    }
    if ((rc = clean_preload(c)) != SDE_OK) {
        sde_ctx_destroy(c);
        return rc;
    }
    float cf[CFLEN];
    sf_cf_table(cf);
    cudaMemcpyAsync(c->d_cf, cf, sizeof cf, cudaMemcpyHostToDevice, c->stream);
    cudaMemsetAsync(c->d_status, 0, sizeof(int) * STATUS_COUNT, c->stream);
    if ((rc = ctx_build_cft(c)) != SDE_OK || cudaStreamSynchronize(c->stream) != cudaSuccess) {
        sde_ctx_destroy(c);
        return rc ? rc : SDE_ECUDA;
    }
    *out = c;
    return SDE_OK;
}

extern "C" int sde_ctx_destroy(sde_ctx *c) {
    if (!c) return SDE_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    drain_events(c);
    for (auto &kv : c->scratch) ctx_free(c, kv.second.p, kv.second.bytes);
    for (auto &kv : c->twiddles) ctx_free(c, kv.second, 0);
    ctx_free(c, c->d_status, 0);
    ctx_free(c, c->d_cf, 0);
    ctx_free(c, c->d_cft, 0);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->h_small) cudaFreeHost(c->h_small);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return SDE_OK;
}

extern "C" int sde_ctx_sync(sde_ctx *c) {
    if (!c) return SDE_EINVAL;
    SDE_CUDA_TRY(cudaMemcpyAsync(c->h_status, c->d_status, sizeof(int) * STATUS_COUNT,
                                 cudaMemcpyDeviceToHost, c->stream));
    SDE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (c->h_status[STATUS_TIMEOUT]) {
        cudaMemsetAsync(c->d_status, 0, sizeof(int) * STATUS_COUNT, c->stream);
        sde_set_error("a bounded device wait timed out");
        return SDE_ETIMEDOUT;
    }
    return SDE_OK;
}

extern "C" void *sde_ctx_stream(sde_ctx *c) { return c ? (void *)c->stream : nullptr; }

extern "C" int sde_ctx_set_stream(sde_ctx *c, void *stream) {
    if (!c) return SDE_EINVAL;
    SDE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    c->stream = (cudaStream_t)stream;
    c->own_stream = false;
    return SDE_OK;
}

extern "C" int64_t sde_ctx_bytes_in_use(sde_ctx *c) { return c ? c->bytes : 0; }

static void drain_events(sde_ctx *c) {
    for (auto &e : c->evq) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, e.a, e.b) == cudaSuccess) {
            auto &k = c->kstats[e.name];
            k.first += ms;
            k.second += 1;
        }
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    c->evq.clear();
}

extern "C" int sde_ctx_profile(sde_ctx *c, int enable) {
    if (!c) return SDE_EINVAL;
    c->profile = enable != 0;
    return SDE_OK;
}

extern "C" int sde_ctx_kernel_stats(sde_ctx *c, const char *kernel, double *total_ms, int64_t *count) {
    if (!c || !kernel) return SDE_EINVAL;
    SDE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    drain_events(c);
    auto it = c->kstats.find(kernel);
    if (total_ms) *total_ms = it == c->kstats.end() ? 0.0 : it->second.first;
    if (count) *count = it == c->kstats.end() ? 0 : it->second.second;
    return SDE_OK;
}

extern "C" int sde_ctx_reset_stats(sde_ctx *c) {
    if (!c) return SDE_EINVAL;
    SDE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    drain_events(c);
    c->kstats.clear();
    c->nlaunch = 0;
    return SDE_OK;
}

extern "C" int64_t sde_ctx_launches(sde_ctx *c) { return c ? c->nlaunch : 0; }

extern "C" int sde_ctx_set_compensated(sde_ctx *c, int on) {
    if (!c) return SDE_EINVAL;
    c->compensated = on != 0;
    return SDE_OK;
}

// ---------------------------------------------------------------------------------------
// plan-level operations
static int ensure_sums(sde_plan *pl) {
    if (!pl->sums_ready) {
        SDE_TRY(plan_sums(pl, &pl->h_lsumwt, &pl->h_sumwt));
        pl->sums_ready = true;
    }
    return SDE_OK;
}

// Raw accumulation of one gridding pass of pl in the context's scratch; the compensation
// plane, when on, is folded in (*raw_lo = nullptr after) or left for finalize.
static int plan_raw_pass(sde_plan *pl, int what, float2 **raw, float2 **raw_lo) {
    sde_ctx *ctx = pl->ctx;
    const size_t cells = (size_t)pl->spec.nv * pl->pitch;
    SDE_TRY(ctx_scratch(ctx, "raw_grid", sizeof(float2) * cells * (ctx->compensated ? 2 : 1), (void **)raw));
    *raw_lo = ctx->compensated ? *raw + cells : nullptr;
    // the compensation plane stays zero between passes (the fold re-zeroes what a pass
    // wrote); it is cleared only when the scratch is new
    const bool lo_clean = *raw_lo && ctx->lo_clean == *raw_lo;
    ctx->lo_clean = nullptr;
    SDE_TRY(plan_grid_raw(pl, what, *raw, *raw_lo, lo_clean));
    SDE_TRY(plan_fold_lo(pl, *raw, *raw_lo));
    if (*raw_lo && pl->core_lo) {
        ctx->lo_clean = *raw_lo;
        *raw_lo = nullptr;  // folded into raw
    }
    return SDE_OK;
}

extern "C" int sde_plan_grid(sde_plan *pl, int what, float *grid, int pitch, float *sumwt) {
    if (!pl || !grid || pitch < pl->spec.nu || (what != SDE_GRID_VIS && what != SDE_GRID_PSF)) {
        sde_set_error("sde_plan_grid: bad arguments");
        return SDE_EINVAL;
    }
    sde_ctx *ctx = pl->ctx;
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    SDE_TRY(ensure_sums(pl));
    const int nu = pl->spec.nu, nv = pl->spec.nv;
    if (pl->h_lsumwt == 0.0) {
        SDE_CUDA_TRY(cudaMemset2DAsync(grid, (size_t)pitch * 8, 0, (size_t)nu * 8, nv, ctx->stream));
        if (sumwt) *sumwt = (float)pl->h_sumwt;
        sde_set_error("No weight!");
        return SDE_ENOWEIGHT;
    }
    float2 *raw, *raw_lo;
    SDE_TRY(plan_raw_pass(pl, what, &raw, &raw_lo));
    // LSUMWT = FLOAT(NU-1)*FLOAT(NV)/LSUMWT (grd/grdh2d.f:218), applied in FP32
    const float scale = (float)((double)((float)(nu - 1) * (float)nv) / pl->h_lsumwt);
    if (pitch == pl->pitch) {
        SDE_TRY(grid_finalize_scale(ctx, raw, raw_lo, (float2 *)grid, nu, nv, pitch, pl->spec.uorigin,
                                    pl->spec.vorigin, pl->spec.supp, scale));
    } else {
        float2 *tmp;
        SDE_TRY(ctx_scratch(ctx, "fin_grid", sizeof(float2) * (size_t)nv * pl->pitch, (void **)&tmp));
        SDE_TRY(grid_finalize_scale(ctx, raw, raw_lo, tmp, nu, nv, pl->pitch, pl->spec.uorigin,
                                    pl->spec.vorigin, pl->spec.supp, scale));
        SDE_CUDA_TRY(cudaMemcpy2DAsync(grid, (size_t)pitch * 8, tmp, (size_t)pl->pitch * 8,
                                       (size_t)nu * 8, nv, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    if (sumwt) *sumwt = (float)pl->h_sumwt;
    return SDE_OK;
}

extern "C" int sde_plan_image(sde_plan *pl, int what, int nx, int ny, int correct,
                              const float *scale_dev, float *image, float *grid, int pitch,
                              float *sumwt) {
    if (!pl || !image || nx < 1 || ny < 1 || (grid && pitch < pl->spec.nu) ||
        (what != SDE_GRID_VIS && what != SDE_GRID_PSF)) {
        sde_set_error("sde_plan_image: bad arguments");
        return SDE_EINVAL;
    }
    sde_ctx *ctx = pl->ctx;
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    const int nu = pl->spec.nu, nv = pl->spec.nv, fnu = 2 * (nu - 1);
    SDE_TRY(check_fft_shape(nx, ny, fnu, nv));
    SDE_TRY(ensure_sums(pl));
    float2 *g = (float2 *)grid;
    if (!g || pitch != pl->pitch)
        SDE_TRY(ctx_scratch(ctx, "img_grid", sizeof(float2) * (size_t)nv * pl->pitch, (void **)&g));
    if (pl->h_lsumwt == 0.0) {
        SDE_CUDA_TRY(cudaMemsetAsync(image, 0, sizeof(float) * (size_t)nx * ny, ctx->stream));
        if (grid) SDE_CUDA_TRY(cudaMemset2DAsync(grid, (size_t)pitch * 8, 0, (size_t)nu * 8, nv, ctx->stream));
        if (sumwt) *sumwt = (float)pl->h_sumwt;
        sde_set_error("No weight!");
        return SDE_ENOWEIGHT;
    }
    float2 *raw, *raw_lo;
    SDE_TRY(plan_raw_pass(pl, what, &raw, &raw_lo));
    // LSUMWT = FLOAT(NU-1)*FLOAT(NV)/LSUMWT (grd/grdh2d.f:218), applied in FP32
    const float scale = (float)((double)((float)(nu - 1) * (float)nv) / pl->h_lsumwt);
    SDE_TRY(image_from_raw(ctx, raw, raw_lo, nu, nv, pl->spec.uorigin, pl->spec.vorigin, pl->spec.supp,
                           scale, (float *)g, pl->pitch, nx, ny, fnu, correct, scale_dev, image));
    if (grid && (float2 *)grid != g)
        SDE_CUDA_TRY(cudaMemcpy2DAsync(grid, (size_t)pitch * 8, g, (size_t)pl->pitch * 8, (size_t)nu * 8, nv,
                                       cudaMemcpyDeviceToDevice, ctx->stream));
    if (sumwt) *sumwt = (float)pl->h_sumwt;
    return SDE_OK;
}

extern "C" int sde_plan_degrid_residual(sde_plan *pl, const float *grid, int pitch) {
    if (!pl || !grid || pitch < pl->spec.nu) return SDE_EINVAL;
    SDE_CUDA_TRY(cudaSetDevice(pl->ctx->device));
    return plan_degrid(pl, grid, pitch, 0, nullptr, nullptr, nullptr);
}

extern "C" int sde_plan_reset_residual(sde_plan *pl) {
    if (!pl) return SDE_EINVAL;
    if (pl->nvis > 0)
        SDE_CUDA_TRY(cudaMemcpy2DAsync(reinterpret_cast<char *>(pl->rec) + sizeof(float2),
                                       sizeof(float4), pl->fobs, sizeof(float2), sizeof(float2),
                                       (size_t)pl->nvis, cudaMemcpyDeviceToDevice,
                                       pl->ctx->stream));
    return SDE_OK;
}

extern "C" int sde_plan_degrid(sde_plan *pl, const float *grid, int pitch, float *vis_out,
                               float *wt_out, int where, int64_t *nbad) {
    if (!pl || !grid || !vis_out || !wt_out || pitch < pl->spec.nu) return SDE_EINVAL;
    sde_ctx *ctx = pl->ctx;
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    const size_t n = (size_t)(pl->nvis_in > 0 ? pl->nvis_in : 1);
    float2 *dv = (float2 *)vis_out;
    float *dw = wt_out;
    const size_t nin = (size_t)pl->nvis_in;
    if (where == SDE_HOST) {
        SDE_TRY(ctx_scratch(ctx, "dg_vis", 8 * n, (void **)&dv));
        SDE_TRY(ctx_scratch(ctx, "dg_wt", 4 * n, (void **)&dw));
        // Every visibility with WT > 0 is written (degridded value, or 0 and WT negated);
        // only the others keep the caller's values, so VIS and WT go up only if there are
        // such visibilities.
        if (pl->nuntouched > 0) {
            SDE_CUDA_TRY(cudaMemcpyAsync(dv, vis_out, 8 * nin, cudaMemcpyHostToDevice, ctx->stream));
            SDE_CUDA_TRY(cudaMemcpyAsync(dw, wt_out, 4 * nin, cudaMemcpyHostToDevice, ctx->stream));
        }
    }
    unsigned long long *nb;  // [0] points not degridded (SUMWT <= 0), [1] WT negated
    SDE_TRY(ctx_scratch(ctx, "dg_nbad", 16, (void **)&nb));
    SDE_CUDA_TRY(cudaMemsetAsync(nb, 0, 16, ctx->stream));
    SDE_TRY(plan_degrid(pl, grid, pitch, 1, dv, dw, nb));
    if (where == SDE_HOST)
        SDE_CUDA_TRY(cudaMemcpyAsync(vis_out, dv, 8 * nin, cudaMemcpyDeviceToHost, ctx->stream));
    if (nbad || where == SDE_HOST) {
        unsigned long long h[2] = {0, 0};
        SDE_CUDA_TRY(cudaMemcpyAsync(h, nb, 16, cudaMemcpyDeviceToHost, ctx->stream));
        SDE_TRY(sde_ctx_sync(ctx));
        if (nbad) *nbad = (int64_t)h[0];
        // WT keeps the caller's values (the plan's WT) unless a point was not degridded
        if (where == SDE_HOST && h[1] > 0) {
            SDE_CUDA_TRY(cudaMemcpyAsync(wt_out, dw, 4 * nin, cudaMemcpyDeviceToHost, ctx->stream));
            SDE_TRY(sde_ctx_sync(ctx));
        }
    }
    return SDE_OK;
}

extern "C" int sde_plan_get_residual(sde_plan *pl, float *vis_out, int where) {
    if (!pl || !vis_out) return SDE_EINVAL;
    sde_ctx *ctx = pl->ctx;
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    if (where == SDE_DEVICE) return plan_scatter_residual(pl, (float2 *)vis_out);
    float2 *d;
    const size_t n = (size_t)(pl->nvis_in > 0 ? pl->nvis_in : 1);
    SDE_TRY(ctx_scratch(ctx, "gr_vis", 8 * n, (void **)&d));
    SDE_CUDA_TRY(cudaMemcpyAsync(d, vis_out, 8 * (size_t)pl->nvis_in, cudaMemcpyHostToDevice, ctx->stream));
    SDE_TRY(plan_scatter_residual(pl, d));
    SDE_CUDA_TRY(cudaMemcpyAsync(vis_out, d, 8 * (size_t)pl->nvis_in, cudaMemcpyDeviceToHost, ctx->stream));
    SDE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SDE_OK;
}

extern "C" int sde_plan_set_vis(sde_plan *pl, const float *vis, int where) {
    if (!pl || !vis) return SDE_EINVAL;
    sde_ctx *ctx = pl->ctx;
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    const float2 *d = (const float2 *)vis;
    if (where == SDE_HOST) {
        float2 *t;
        const size_t n = (size_t)(pl->nvis_in > 0 ? pl->nvis_in : 1);
        SDE_TRY(ctx_scratch(ctx, "sv_vis", 8 * n, (void **)&t));
        SDE_CUDA_TRY(cudaMemcpyAsync(t, vis, 8 * (size_t)pl->nvis_in, cudaMemcpyHostToDevice, ctx->stream));
        d = t;
    }
    return plan_set_vis_dev(pl, d);
}

// ---------------------------------------------------------------------------------------
// Fortran-77 drop-in layer.
extern "C" {
sde_sysi_common sysi_ = {0, 80, 0, 0, 0, 1, 0};

__attribute__((weak)) void errrepor_(const char *reason, const char *routine, const char *text,
                                     size_t lreason, size_t lroutine, size_t ltext) {
    fprintf(stderr, "E%.*s in routine %.*s, %.*s\n", (int)lreason, reason, (int)lroutine, routine,
            (int)ltext, text);
    sysi_.error = 1;
}

__attribute__((weak)) void msgput_(const char *msg, const char *type, size_t lmsg, size_t ltype) {
    if (sysi_.sysmsg) fprintf(stderr, "%.*s: %.*s\n", (int)ltype, type, (int)lmsg, msg);
}
}

static std::mutex g_shim_mu;
static sde_ctx *g_shim_ctx = nullptr;

// Copies between the drop-ins' caller arrays and the device.  SDE's arrays are ordinary
// pageable memory, which cudaMemcpyAsync stages through the driver's buffers (14 GB/s on
// first touch, ~190 GB/s at best, measured on GB300).  Where the device reads and writes
// pageable host memory directly (cudaDevAttrPageableMemoryAccess), a copy kernel moves large
// pageable arrays at the link's rate (~200 GB/s) on a few SMs; pinned and device memory, small
// copies and unaligned ones go to the CUDA copy as before.  Either way the copy is ordered on
// the given stream, and every drop-in waits for its stream before it returns, so the caller's
// array is only touched during the call.
static constexpr size_t SHIM_KCOPY_MIN = 256 * 1024;
static constexpr int SHIM_KCOPY_CTAS = 32;

__global__ void __launch_bounds__(512) k_copy16(uint4 *__restrict__ dst, const uint4 *__restrict__ src, int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n; i += 4 * stride) {
        const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n; i += stride) dst[i] = src[i];
}

__global__ void __launch_bounds__(512) k_copy4_2d(char *__restrict__ dst, size_t dpitch,
                                                  const char *__restrict__ src, size_t spitch,
                                                  int64_t words, int64_t rows) {
    for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
        uint32_t *d = reinterpret_cast<uint32_t *>(dst + r * dpitch);
        const uint32_t *sr = reinterpret_cast<const uint32_t *>(src + r * spitch);
        for (int64_t w = threadIdx.x; w < words; w += blockDim.x) d[w] = sr[w];
    }
}

static bool shim_pageable_direct(const void *host) {
    static int access[64];
    static bool known[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    if (!known[dev]) {
        int a = 0;
        if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) a = 0;
        access[dev] = a;
        known[dev] = true;
    }
    if (!access[dev]) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeUnregistered;
}

static cudaError_t shim_memcpy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st) {
    const bool h2d = kind == cudaMemcpyHostToDevice, d2h = kind == cudaMemcpyDeviceToHost;
    if (bytes >= SHIM_KCOPY_MIN && (h2d || d2h) && bytes % 16 == 0 &&
        (reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) % 16 == 0 &&
        shim_pageable_direct(h2d ? src : dst)) {
        k_copy16<<<SHIM_KCOPY_CTAS, 512, 0, st>>>(static_cast<uint4 *>(dst), static_cast<const uint4 *>(src),
                                                  (int64_t)(bytes / 16));
        return cudaGetLastError();
    }
    return cudaMemcpyAsync(dst, src, bytes, kind, st);
}

static cudaError_t shim_memcpy2d(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width,
                                 size_t rows, cudaMemcpyKind kind, cudaStream_t st) {
    const bool h2d = kind == cudaMemcpyHostToDevice, d2h = kind == cudaMemcpyDeviceToHost;
    if (width * rows >= SHIM_KCOPY_MIN && (h2d || d2h) && width % 4 == 0 && dpitch % 4 == 0 &&
        spitch % 4 == 0 && (reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) % 4 == 0 &&
        shim_pageable_direct(h2d ? src : dst)) {
        k_copy4_2d<<<SHIM_KCOPY_CTAS * 4, 512, 0, st>>>(static_cast<char *>(dst), dpitch,
                                                        static_cast<const char *>(src), spitch,
                                                        (int64_t)(width / 4), (int64_t)rows);
        return cudaGetLastError();
    }
    return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, rows, kind, st);
}

// The drop-ins' context: on device SDE_DEVICE if set, else on the calling thread's current
// device (0 unless the caller chose another), created by the first drop-in call.
static sde_ctx *shim_ctx() {
    if (!g_shim_ctx) {
        const char *d = getenv("SDE_DEVICE");
        int dev = 0;
        if (d)
            dev = atoi(d);
        else if (cudaGetDevice(&dev) != cudaSuccess)
            dev = 0;
        if (sde_ctx_create(&g_shim_ctx, dev) != SDE_OK) g_shim_ctx = nullptr;
    }
    return g_shim_ctx;
}

static void report(const char *reason, const char *routine, const char *text) {
    errrepor_(reason, routine, text, strlen(reason), strlen(routine), strlen(text));
}

static void report_rc(int rc, const char *routine) {
    char buf[600];
    snprintf(buf, sizeof buf, "%s", sde_last_error());
    const char *reason = rc == SDE_EINVAL ? "Bad argument" : rc == SDE_ENOMEM ? "No memory" : "GPU failure";
    report(reason, routine, buf);
}

static int fstr_eq(const char *s, size_t len, const char *lit) {
    size_t n = len;
    while (n > 0 && s[n - 1] == ' ') n--;
    return strlen(lit) == n && strncmp(s, lit, n) == 0;
}

// upload the caller's 'SF'-style table into the plan (1+2*(SUPP+1)*OSAMP values)
static int plan_use_table(sde_plan *pl, const float *cf) {
    SDE_CUDA_TRY(shim_memcpy(pl->cf, cf, sizeof(float) * (2 * (SUPP + 1) * OSAMP + 1),
                                 cudaMemcpyHostToDevice, pl->ctx->stream));
    return plan_build_cft(pl);
}

static int check_table_args(const float *fnu, const float *fnv, int suppu, int osampu, int suppv,
                            int osampv, const char *routine) {
    if (suppu != SUPP || suppv != SUPP || osampu != OSAMP || osampv != OSAMP) {
        char t[128];
        snprintf(t, sizeof t, "support %d/%d, oversampling %d/%d: only the SF kernel (3, 128) is "
                 "implemented", suppu, suppv, osampu, osampv);
        report("Bad argument", routine, t);
        return 0;
    }
    if (memcmp(fnu, fnv, sizeof(float) * (2 * (SUPP + 1) * OSAMP + 1)) != 0) {
        report("Bad argument", routine, "different u and v functions are not implemented");
        return 0;
    }
    return 1;
}

static void fill_spec(sde_gridspec *s, int nu, int nv, float us, float uo, float vs, float vo,
                      int uor, int vor, const double *shift) {
    s->nu = nu;
    s->nv = nv;
    s->uscale = us;
    s->uoffset = uo;
    s->vscale = vs;
    s->voffset = vo;
    s->uorigin = uor;
    s->vorigin = vor;
    s->supp = SUPP;
    s->osamp = OSAMP;
    memcpy(s->shift, shift, sizeof s->shift);
}

// GRDSF / GRDCF / GRDCCF (grd/grdsf.f, grd/grdcf.f, grd/grdccf.f): host-side table
// builders the callers of the gridder use; 'SF' and 'BOX' codes.
extern "C" double grdsf_(double *nu) { return sf_grdsf(*nu); }

extern "C" void grdcf_(char *cfcode, float *cf, int *cfsupp, int *cfosamp, size_t len) {
    if (sysi_.error) return;
    if (len >= 2 && strncmp(cfcode, "SF", 2) == 0) {
        sf_cf_table(cf);
        *cfsupp = SUPP;
        *cfosamp = OSAMP;
    } else if (len >= 3 && strncmp(cfcode, "BOX", 3) == 0) {
        const int osamp = 128, supp = 1, off = (supp + 1) * osamp;
        for (int i = 0; i <= osamp / 2; i++) cf[off + i] = cf[off - i] = 1.0f;
        for (int i = osamp / 2 + 1; i <= 2 * osamp; i++) cf[off + i] = cf[off - i] = 0.0f;
        float sum = 0.0f;
        for (int i = -(supp + 1) * osamp; i <= (supp + 1) * osamp; i++) sum = sum + cf[off + i];
        for (int i = -(supp + 1) * osamp; i <= (supp + 1) * osamp; i++) cf[off + i] = cf[off + i] / sum;
        *cfsupp = supp;
        *cfosamp = osamp;
    } else {
        report("Bad argument", "GRDCF", "Cannot make convolution function");
    }
}

extern "C" void grdccf_(char *ccfcode, float *ccf, int *ccflen, size_t len) {
    if (sysi_.error) return;
    if (len >= 2 && strncmp(ccfcode, "SF", 2) == 0) {
        sf_ccf_table(ccf, *ccflen);
    } else if (len >= 3 && strncmp(ccfcode, "BOX", 3) == 0) {
        const float PI = 3.141592554f;
        ccf[0] = 1.0f;
        for (int i = 2; i <= *ccflen; i++) {
            double nu = (double)(i - 1) / (double)(*ccflen - 1);
            float x = 0.5f * PI * (float)nu;
            ccf[i - 1] = sinf(x) / x;
        }
    } else {
        report("Bad argument", "GRDCCF", "Cannot make convolution correction function");
    }
}

// ---- plan cache of the drop-ins ---------------------------------------------------------
// VISGRID and VISDEGRI call GRDH2D / GRDDEH2D every major cycle with the same U, V, W, WT and
// new VIS.  The shim keeps the plan of its last call with a device copy of the U, V, W, WT it
// was built from.  Every call still uploads its arrays; when they are bitwise identical to
// the cached ones (compared on the device) and the grid geometry and the caller's gridding
// function are the same, only the visibilities are replaced (the frame transform of
// sde_plan_set_vis) instead of sorting again.  Any difference rebuilds the plan.
struct ShimCache {
    sde_plan *pl = nullptr;
    sde_gridspec spec{};
    int64_t nvis = -1;
    uint64_t cf_hash = 0;
    float *inputs = nullptr;  // u | v | w | wt of the cached plan (device)
    size_t cap = 0;           // bytes of inputs
    int64_t hits = 0, misses = 0;
};
static ShimCache g_pc;

// flag = 1 if the n words differ anywhere.  a and b have the same alignment modulo 16
// bytes: the head words up to the first 16-byte boundary go one by one, the body as 16-byte
// loads (four in flight per thread), the tail word by word.
__global__ void k_words_differ(const uint32_t *__restrict__ a, const uint32_t *__restrict__ b,
                               int64_t n, int *flag) {
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t head = (int64_t)((4 - (((uintptr_t)a >> 2) & 3)) & 3);
    if (head > n) head = n;
    uint32_t diff = 0;
    if (tid < head) diff |= a[tid] ^ b[tid];
    const int64_t n4 = (n - head) >> 2;
    const uint4 *a4 = reinterpret_cast<const uint4 *>(a + head);
    const uint4 *b4 = reinterpret_cast<const uint4 *>(b + head);
    int64_t i = tid;
    for (; i + 3 * stride < n4; i += 4 * stride) {
        uint4 x[4], y[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            x[k] = a4[i + k * stride];
            y[k] = b4[i + k * stride];
        }
#pragma unroll
        for (int k = 0; k < 4; k++)
            diff |= (x[k].x ^ y[k].x) | (x[k].y ^ y[k].y) | (x[k].z ^ y[k].z) | (x[k].w ^ y[k].w);
    }
    for (; i < n4; i += stride) {
        const uint4 x = a4[i], y = b4[i];
        diff |= (x.x ^ y.x) | (x.y ^ y.y) | (x.z ^ y.z) | (x.w ^ y.w);
    }
    for (int64_t j = head + 4 * n4 + tid; j < n; j += stride) diff |= a[j] ^ b[j];
    if (diff) *flag = 1;
}

static uint64_t hash_floats(const float *x, size_t n) {
    uint64_t h = 1469598103934665603ull;  // FNV-1a over the bit patterns
    const unsigned char *b = reinterpret_cast<const unsigned char *>(x);
    for (size_t i = 0; i < n * sizeof(float); i++) h = (h ^ b[i]) * 1099511628211ull;
    return h;
}

static void shim_cache_drop() {
    if (g_pc.pl) sde_plan_destroy(g_pc.pl);
    g_pc.pl = nullptr;
    g_pc.nvis = -1;
}

// The plan for this call (owned by the cache: callers do not destroy it).  vis may be NULL
// (GRDDEH2D: VIS is output only).
// Copies of the drop-ins' inputs run on a second stream so that work on the context's stream
// overlaps them: the cached plan takes the new visibilities (set_vis) while U, V, W, WT are
// still arriving, each array is compared as soon as it has arrived, and a caller's extra
// upload (GRDDEH2D's model grid) follows the inputs while the comparison runs.
struct ShimStreams {
    cudaStream_t copy = nullptr;
    cudaEvent_t ev[7] = {};
};
static ShimStreams g_ss;

static int shim_streams() {
    if (g_ss.copy) return SDE_OK;
    SDE_CUDA_TRY(cudaStreamCreateWithFlags(&g_ss.copy, cudaStreamNonBlocking));
    for (auto &e : g_ss.ev) SDE_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return SDE_OK;
}

struct Upload2D {  // an extra host -> device 2-D copy issued behind the inputs
    void *dst;
    size_t dpitch;
    const void *src;
    size_t spitch, width, rows;
};

static int shim_plan_build(sde_ctx *ctx, const sde_gridspec &sp, int64_t n, const float *in, const float *dvis,
                           const float *cf, uint64_t h, sde_plan **out);

static int shim_plan(sde_ctx *ctx, const sde_gridspec &sp, int64_t n, const float *u,
                     const float *v, const float *w, const float *vis, const float *wt,
                     const float *cf, sde_plan **out, const Upload2D *extra = nullptr) {
    cudaStream_t st = ctx->stream;
    SDE_TRY(shim_streams());
    cudaStream_t cs = g_ss.copy;
    float *in = nullptr, *dvis = nullptr;
    const size_t nb = sizeof(float) * (size_t)(n > 0 ? n : 1);
    SDE_TRY(ctx_scratch(ctx, "shim_in", 4 * nb, (void **)&in));
    SDE_TRY(ctx_scratch(ctx, "shim_vis", 2 * nb, (void **)&dvis));
    int *flag = nullptr;
    SDE_TRY(ctx_scratch(ctx, "shim_flag", sizeof(int), (void **)&flag));
    const uint64_t h = hash_floats(cf, 2 * (SUPP + 1) * OSAMP + 1);
    const bool cached = g_pc.pl && g_pc.nvis == n && g_pc.cf_hash == h &&
                        memcmp(&g_pc.spec, &sp, sizeof sp) == 0;
    SDE_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), st));
    if (n > 0 && vis) SDE_CUDA_TRY(shim_memcpy(dvis, vis, 2 * nb, cudaMemcpyHostToDevice, st));
    // the copy stream follows everything queued so far (scratch allocations, earlier users
    // of the buffers, the visibilities' copy)
    SDE_CUDA_TRY(cudaEventRecord(g_ss.ev[0], st));
    SDE_CUDA_TRY(cudaStreamWaitEvent(cs, g_ss.ev[0], 0));
    if (n > 0 && vis && cached) SDE_TRY(sde_plan_set_vis(g_pc.pl, dvis, SDE_DEVICE));  // speculative
    const float *src[4] = {u, v, w, wt};
    for (int k = 0; k < 4 && n > 0; k++) {
        SDE_CUDA_TRY(shim_memcpy(in + k * n, src[k], nb, cudaMemcpyHostToDevice, cs));
        SDE_CUDA_TRY(cudaEventRecord(g_ss.ev[1 + k], cs));
    }
    if (extra)
        SDE_CUDA_TRY(shim_memcpy2d(extra->dst, extra->dpitch, extra->src, extra->spitch,
                                       extra->width, extra->rows, cudaMemcpyHostToDevice, cs));
    SDE_CUDA_TRY(cudaEventRecord(g_ss.ev[5], cs));
    if (cached) {
        for (int k = 0; k < 4 && n > 0; k++) {
            SDE_CUDA_TRY(cudaStreamWaitEvent(st, g_ss.ev[1 + k], 0));
            k_words_differ<<<ctx->num_sms * 4, 256, 0, st>>>(
                reinterpret_cast<const uint32_t *>(in + k * n),
                reinterpret_cast<const uint32_t *>(g_pc.inputs + k * n), n, flag);
            SDE_CHECK_LAUNCH();
        }
    }
    SDE_CUDA_TRY(cudaStreamWaitEvent(st, g_ss.ev[5], 0));
    if (cached) {
        int hf = 1;
        SDE_CUDA_TRY(shim_memcpy(&hf, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
        SDE_CUDA_TRY(cudaStreamSynchronize(st));
        if (!hf) {
            g_pc.hits++;
            *out = g_pc.pl;
            return SDE_OK;
        }
    }
    if (!vis && n > 0) SDE_CUDA_TRY(cudaMemsetAsync(dvis, 0, 2 * nb, st));
    return shim_plan_build(ctx, sp, n, in, dvis, cf, h, out);
}

// A new plan from the device copies of U, V, W, WT (in, 4n floats) and VIS, kept in the cache
// with its inputs.
static int shim_plan_build(sde_ctx *ctx, const sde_gridspec &sp, int64_t n, const float *in, const float *dvis,
                           const float *cf, uint64_t h, sde_plan **out) {
    cudaStream_t st = ctx->stream;
    const size_t nb = sizeof(float) * (size_t)(n > 0 ? n : 1);
    shim_cache_drop();
    sde_plan *pl = nullptr;
    SDE_TRY(sde_plan_create(ctx, &sp, n, in, in + n, in + 2 * n, dvis, in + 3 * n, SDE_DEVICE, &pl));
    int rc = plan_use_table(pl, cf);
    if (rc == SDE_OK && 4 * nb > g_pc.cap) {
        if (g_pc.inputs) ctx_free(ctx, g_pc.inputs, g_pc.cap);
        g_pc.inputs = nullptr;
        g_pc.cap = 0;
        rc = ctx_alloc(ctx, (void **)&g_pc.inputs, 4 * nb);
        if (rc == SDE_OK) g_pc.cap = 4 * nb;
    }
    if (rc == SDE_OK && n > 0) {
        cudaError_t e = shim_memcpy(g_pc.inputs, in, 4 * nb, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) {
            sde_set_error("%s", cudaGetErrorString(e));
            rc = SDE_ECUDA;
        }
    }
    if (rc != SDE_OK) {
        sde_plan_destroy(pl);
        return rc;
    }
    g_pc.pl = pl;
    g_pc.spec = sp;
    g_pc.nvis = n;
    g_pc.cf_hash = h;
    g_pc.misses++;
    *out = pl;
    return SDE_OK;
}

extern "C" int sde_shim_cache_stats(int64_t *hits, int64_t *misses) {
    if (hits) *hits = g_pc.hits;
    if (misses) *misses = g_pc.misses;
    return SDE_OK;
}

extern "C" int sde_shim_cache_clear(void) {
    std::lock_guard<std::mutex> lk(g_shim_mu);
    shim_cache_drop();
    if (g_pc.inputs && g_shim_ctx) ctx_free(g_shim_ctx, g_pc.inputs, g_pc.cap);
    g_pc.inputs = nullptr;
    g_pc.cap = 0;
    return SDE_OK;
}

// GRDH2D against the cached plan while its inputs are still arriving: VIS goes up first and
// the cached plan grids it, and the grid comes down, while U, V, W, WT are uploaded and
// compared on the copy stream.  If one of them changed, the plan is rebuilt and the grid
// made and returned again (GVIS and SUMWT are outputs only).  *done = 0: no cached plan.
static int shim_grid_speculative(sde_ctx *ctx, const sde_gridspec &sp, int64_t n, const float *vis, const float *wt,
                                 const float *u, const float *v, const float *w, const float *cf, int psf,
                                 float *gvis, int nu, int nv, float *sumwt, int *done) {
    *done = 0;
    const uint64_t h = hash_floats(cf, 2 * (SUPP + 1) * OSAMP + 1);
    if (!(g_pc.pl && n > 0 && g_pc.nvis == n && g_pc.cf_hash == h && memcmp(&g_pc.spec, &sp, sizeof sp) == 0))
        return SDE_OK;
    cudaStream_t st = ctx->stream;
    SDE_TRY(shim_streams());
    cudaStream_t cs = g_ss.copy;
    const size_t nb = sizeof(float) * (size_t)n;
    float *in = nullptr, *dvis = nullptr;
    float2 *dg = nullptr;
    int *flag = nullptr;
    const int pitch = sde_grid_pitch(nu);
    SDE_TRY(ctx_scratch(ctx, "shim_in", 4 * nb, (void **)&in));
    SDE_TRY(ctx_scratch(ctx, "shim_vis", 2 * nb, (void **)&dvis));
    SDE_TRY(ctx_scratch(ctx, "shim_flag", sizeof(int), (void **)&flag));
    SDE_TRY(ctx_scratch(ctx, "shim_grid", sizeof(float2) * (size_t)pitch * nv, (void **)&dg));
    SDE_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), st));
    SDE_CUDA_TRY(shim_memcpy(dvis, vis, 2 * nb, cudaMemcpyHostToDevice, st));
    SDE_CUDA_TRY(cudaEventRecord(g_ss.ev[0], st));
    SDE_CUDA_TRY(cudaStreamWaitEvent(cs, g_ss.ev[0], 0));
    // the grid of the cached plan and its way back on the main stream ...
    sde_plan *pl = g_pc.pl;
    if (!psf) SDE_TRY(sde_plan_set_vis(pl, dvis, SDE_DEVICE));
    float sw = 0.0f;
    int rc = sde_plan_grid(pl, psf ? SDE_GRID_PSF : SDE_GRID_VIS, (float *)dg, pitch, &sw);
    if (rc != SDE_OK && rc != SDE_ENOWEIGHT) return rc;
    SDE_CUDA_TRY(shim_memcpy2d(gvis, (size_t)nu * 8, dg, (size_t)pitch * 8, (size_t)nu * 8, (size_t)nv,
                                   cudaMemcpyDeviceToHost, st));
    // ... while U, V, W, WT go up and are compared on the copy stream
    const float *src[4] = {u, v, w, wt};
    for (int k = 0; k < 4; k++) {
        SDE_CUDA_TRY(shim_memcpy(in + k * n, src[k], nb, cudaMemcpyHostToDevice, cs));
        k_words_differ<<<ctx->num_sms * 4, 256, 0, cs>>>(reinterpret_cast<const uint32_t *>(in + k * n),
                                                        reinterpret_cast<const uint32_t *>(g_pc.inputs + k * n), n,
                                                        flag);
        SDE_CHECK_LAUNCH();
    }
    int hf = 1;
    SDE_CUDA_TRY(shim_memcpy(&hf, flag, sizeof(int), cudaMemcpyDeviceToHost, cs));
    SDE_CUDA_TRY(cudaStreamSynchronize(cs));
    SDE_CUDA_TRY(cudaStreamSynchronize(st));
    *done = 1;
    if (!hf) {
        g_pc.hits++;
        *sumwt = sw;
        return rc;
    }
    // an input changed: a new plan from the arrived inputs, the grid again
    SDE_TRY(shim_plan_build(ctx, sp, n, in, dvis, cf, h, &pl));
    rc = sde_plan_grid(pl, psf ? SDE_GRID_PSF : SDE_GRID_VIS, (float *)dg, pitch, &sw);
    if (rc != SDE_OK && rc != SDE_ENOWEIGHT) return rc;
    SDE_CUDA_TRY(shim_memcpy2d(gvis, (size_t)nu * 8, dg, (size_t)pitch * 8, (size_t)nu * 8, (size_t)nv,
                                   cudaMemcpyDeviceToHost, st));
    SDE_CUDA_TRY(cudaStreamSynchronize(st));
    *sumwt = sw;
    return rc;
}

extern "C" void grdh2d_(float *vis, float *wt, float *u, float *v, float *w, int *nvis,
                        float *uscale, float *uoffset, float *vscale, float *voffset, int *uorigin,
                        int *vorigin, float *gvis, int *psf, int *nu, int *nv, float *gridfnu,
                        int *suppu, int *osampu, float *gridfnv, int *suppv, int *osampv,
                        double *shift, float *sumwt) {
    if (sysi_.error) return;
    std::lock_guard<std::mutex> lk(g_shim_mu);
    const char *R = "GRDH2D";
    if (!check_table_args(gridfnu, gridfnv, *suppu, *osampu, *suppv, *osampv, R)) return;
    sde_ctx *ctx = shim_ctx();
    if (!ctx) {
        report("No GPU", R, sde_last_error());
        return;
    }
    sde_gridspec sp;
    fill_spec(&sp, *nu, *nv, *uscale, *uoffset, *vscale, *voffset, *uorigin, *vorigin, shift);
    int done = 0;
    float ssw = 0.0f;
    int rs = shim_grid_speculative(ctx, sp, *nvis, vis, wt, u, v, w, gridfnu, *psf, gvis, *nu, *nv, &ssw, &done);
    if (done || rs != SDE_OK) {
        if (rs == SDE_OK || rs == SDE_ENOWEIGHT) *sumwt = ssw;
        if (rs == SDE_ENOWEIGHT)
            report("Bad argument", R, "No weight!");
        else if (rs != SDE_OK)
            report_rc(rs, R);
        return;
    }
    sde_plan *pl = nullptr;
    int rc = shim_plan(ctx, sp, *nvis, u, v, w, vis, wt, gridfnu, &pl);
    float2 *dg = nullptr;
    const int pitch = sde_grid_pitch(*nu);
    if (rc == SDE_OK) rc = ctx_scratch(ctx, "shim_grid", sizeof(float2) * (size_t)pitch * *nv, (void **)&dg);
    float sw = 0.0f;
    if (rc == SDE_OK) rc = sde_plan_grid(pl, *psf ? SDE_GRID_PSF : SDE_GRID_VIS, (float *)dg, pitch, &sw);
    if (rc == SDE_OK || rc == SDE_ENOWEIGHT) {
        cudaError_t e = shim_memcpy2d(gvis, (size_t)*nu * 8, dg, (size_t)pitch * 8, (size_t)*nu * 8,
                                          *nv, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess && rc == SDE_OK) {
            sde_set_error("%s", cudaGetErrorString(e));
            rc = SDE_ECUDA;
        }
        *sumwt = sw;
    }
    if (rc == SDE_ENOWEIGHT)
        report("Bad argument", R, "No weight!");
    else if (rc != SDE_OK)
        report_rc(rc, R);
}

// Host arrays of a slow-Z call on the device: vis, wt, u, v, w, both tables (uploads in order)
static int h23_upload(sde_ctx *ctx, int64_t n, const float *vis, const float *wt, const float *u,
                      const float *v, const float *w, const float *fnu, int lu, const float *fnv, int lv,
                      float **d) {
    const size_t nb = (size_t)(n > 0 ? n : 1);
    SDE_TRY(ctx_scratch(ctx, "h23_in", sizeof(float) * (nb * 6 + (size_t)lu + (size_t)lv), (void **)d));
    float *p = *d;
    const float *src[7] = {vis, wt, u, v, w, fnu, fnv};
    const size_t len[7] = {2 * (size_t)n, (size_t)n, (size_t)n, (size_t)n, (size_t)n, (size_t)lu, (size_t)lv};
    const size_t off[7] = {0, 2 * nb, 3 * nb, 4 * nb, 5 * nb, 6 * nb, 6 * nb + (size_t)lu};
    for (int i = 0; i < 7; i++)
        if (len[i]) SDE_CUDA_TRY(shim_memcpy(p + off[i], src[i], sizeof(float) * len[i], cudaMemcpyHostToDevice,
                                                 ctx->stream));
    return SDE_OK;
}

// GRDH23D (grd/grdh23d.f), VISGRID's slow-Z gridder (vis/visgrid.f:219-226)
extern "C" void grdh23d_(float *vis, float *wt, float *u, float *v, float *w, int *nvis, float *uscale,
                         float *uoffset, float *vscale, float *voffset, int *uorigin, int *vorigin, float *gvis,
                         int *psf, int *nu, int *nv, float *gridfnu, int *suppu, int *osampu, float *gridfnv,
                         int *suppv, int *osampv, int *nz, float *cellz, float *refz, double *shift, float *sumwt) {
    if (sysi_.error) return;
    std::lock_guard<std::mutex> lk(g_shim_mu);
    const char *R = "GRDH23D";
    sde_ctx *ctx = shim_ctx();
    if (!ctx) {
        report("No GPU", R, sde_last_error());
        return;
    }
    const int64_t n = *nvis > 0 ? *nvis : 0;
    const size_t nb = (size_t)(n > 0 ? n : 1);
    const int lu = 2 * (*suppu + 1) * *osampu + 1, lv = 2 * (*suppv + 1) * *osampv + 1;
    const size_t cells = (size_t)*nu * *nv * (*nz > 0 ? *nz : 0);
    float *d = nullptr, *dg = nullptr;
    int rc = (*nu < 2 || *nv < 2 || *nz < 1 || *suppu < 0 || *suppv < 0 || *osampu < 1 || *osampv < 1) ? SDE_EINVAL
                                                                                                    : SDE_OK;
    if (rc == SDE_EINVAL) sde_set_error("bad grid or table sizes");
    if (rc == SDE_OK) rc = h23_upload(ctx, n, vis, wt, u, v, w, gridfnu, lu, gridfnv, lv, &d);
    if (rc == SDE_OK) rc = ctx_scratch(ctx, "h23_grid", sizeof(float2) * cells, (void **)&dg);
    float sw = 0.0f;
    if (rc == SDE_OK)
        rc = grid_h23d(ctx, n, d, d + 2 * nb, d + 3 * nb, d + 4 * nb, d + 5 * nb, *uscale, *uoffset, *vscale, *voffset,
                       *uorigin, *vorigin, *psf, *nu, *nv, d + 6 * nb, *suppu, *osampu, d + 6 * nb + lu, *suppv,
                       *osampv, *nz, *cellz, *refz, shift, dg, &sw);
    if (rc == SDE_OK || rc == SDE_ENOWEIGHT) {
        cudaError_t e = shim_memcpy(gvis, dg, sizeof(float2) * cells, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess && rc == SDE_OK) {
            sde_set_error("%s", cudaGetErrorString(e));
            rc = SDE_ECUDA;
        }
        *sumwt = sw;
    }
    if (rc == SDE_ENOWEIGHT)
        report("Bad argument", R, "No weight!");
    else if (rc != SDE_OK)
        report_rc(rc, R);
}

// GRDDEH23 (grd/grddeh23.f), VISDEGRI's slow-Z degridder (vis/visdegri.f:154-160)
extern "C" void grddeh23_(float *vis, float *wt, float *u, float *v, float *w, int *nvis, float *uscale,
                          float *uoffset, float *vscale, float *voffset, int *uorigin, int *vorigin, float *gvis,
                          int *nu, int *nv, float *intfnu, int *suppu, int *osampu, float *intfnv, int *suppv,
                          int *osampv, int *nz, float *cellz, float *refz, double *shift) {
    if (sysi_.error) return;
    std::lock_guard<std::mutex> lk(g_shim_mu);
    const char *R = "GRDDEH23";
    sde_ctx *ctx = shim_ctx();
    if (!ctx) {
        report("No GPU", R, sde_last_error());
        return;
    }
    const int64_t n = *nvis > 0 ? *nvis : 0;
    const size_t nb = (size_t)(n > 0 ? n : 1);
    const int lu = 2 * (*suppu + 1) * *osampu + 1, lv = 2 * (*suppv + 1) * *osampv + 1;
    const size_t cells = (size_t)*nu * *nv * (*nz > 0 ? *nz : 0);
    float *d = nullptr, *dg = nullptr;
    int rc = (*nu < 2 || *nv < 2 || *nz < 1 || *suppu < 0 || *suppv < 0 || *osampu < 1 || *osampv < 1) ? SDE_EINVAL
                                                                                                    : SDE_OK;
    if (rc == SDE_EINVAL) sde_set_error("bad grid or table sizes");
    if (rc == SDE_OK) rc = h23_upload(ctx, n, vis, wt, u, v, w, intfnu, lu, intfnv, lv, &d);
    if (rc == SDE_OK) rc = ctx_scratch(ctx, "h23_mgrid", sizeof(float2) * cells, (void **)&dg);
    if (rc == SDE_OK) {
        cudaError_t e = shim_memcpy(dg, gvis, sizeof(float2) * cells, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) {
            sde_set_error("%s", cudaGetErrorString(e));
            rc = SDE_ECUDA;
        }
    }
    int64_t nbad = 0;
    if (rc == SDE_OK)
        rc = degrid_h23(ctx, n, d, d + 2 * nb, d + 3 * nb, d + 4 * nb, d + 5 * nb, *uscale, *uoffset, *vscale, *voffset,
                        *uorigin, *vorigin, dg, *nu, *nv, d + 6 * nb, *suppu, *osampu, d + 6 * nb + lu, *suppv,
                        *osampv, *nz, *cellz, *refz, shift, &nbad);
    if (rc == SDE_OK && n > 0) {
        cudaError_t e = shim_memcpy(vis, d, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = shim_memcpy(wt, d + 2 * nb, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) {
            sde_set_error("%s", cudaGetErrorString(e));
            rc = SDE_ECUDA;
        }
    }
    if (rc != SDE_OK) {
        report_rc(rc, R);
        return;
    }
    if (nbad > 0) {  // grd/grddeh23.f:185-189
        char m[96];
        snprintf(m, sizeof m, "%7lld points were not successfully degridded", (long long)nbad);
        msgput_(m, "W", strlen(m), 1);
    }
}

// GRDQH2D (grd/grdqh2d.f), VISGRID's gridder for the 'BOX' function (vis/visgrid.f:154-158)
extern "C" void grdqh2d_(float *vis, float *wt, float *u, float *v, float *w, int *nvis, float *uscale,
                         float *uoffset, float *vscale, float *voffset, int *uorigin, int *vorigin, float *gvis,
                         int *psf, int *nu, int *nv, double *shift, float *sumwt) {
    if (sysi_.error) return;
    std::lock_guard<std::mutex> lk(g_shim_mu);
    const char *R = "GRDQH2D";
    sde_ctx *ctx = shim_ctx();
    if (!ctx) {
        report("No GPU", R, sde_last_error());
        return;
    }
    const int64_t n = *nvis > 0 ? *nvis : 0;
    const size_t nb = (size_t)(n > 0 ? n : 1);
    float *din = nullptr, *dg = nullptr;
    int rc = ctx_scratch(ctx, "box_in", sizeof(float) * nb * 6, (void **)&din);
    if (rc == SDE_OK) rc = ctx_scratch(ctx, "box_grid", sizeof(float2) * (size_t)*nu * *nv, (void **)&dg);
    float *dvis = din, *dwt = din + 2 * nb, *du = dwt + nb, *dv = du + nb, *dw = dv + nb;
    cudaStream_t st = ctx->stream;
    cudaError_t e = cudaSuccess;
    if (rc == SDE_OK && n > 0) {
        e = shim_memcpy(dvis, vis, sizeof(float) * 2 * n, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = shim_memcpy(dwt, wt, sizeof(float) * n, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = shim_memcpy(du, u, sizeof(float) * n, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = shim_memcpy(dv, v, sizeof(float) * n, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = shim_memcpy(dw, w, sizeof(float) * n, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) {
            sde_set_error("%s", cudaGetErrorString(e));
            rc = SDE_ECUDA;
        }
    }
    float sw = 0.0f;
    if (rc == SDE_OK)
        rc = grid_box(ctx, n, dvis, dwt, du, dv, dw, *uscale, *uoffset, *vscale, *voffset, *uorigin, *vorigin, *psf,
                      *nu, *nv, shift, dg, *nu, &sw, nullptr);
    if (rc == SDE_OK || rc == SDE_ENOWEIGHT) {
        e = shim_memcpy(gvis, dg, sizeof(float2) * (size_t)*nu * *nv, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess && rc == SDE_OK) {
            sde_set_error("%s", cudaGetErrorString(e));
            rc = SDE_ECUDA;
        }
        *sumwt = sw;
    }
    if (rc == SDE_ENOWEIGHT)
        report("Bad argument", R, "No weight!");
    else if (rc != SDE_OK)
        report_rc(rc, R);
}

// GRDDEH2D against the cached plan while its inputs are still arriving.  WT goes up first and
// is compared with the cached plan's: when it matches and that plan has no points with
// WT <= 0 (whose VIS the caller keeps), every VIS is written whatever U, V, W turn out to be,
// so the model grid goes up next, the degrid runs and VIS comes down while U, V, W are
// uploaded and compared on the copy stream (the two directions of the link at once).  If U,
// V or W changed, the plan is rebuilt and VIS written again.  *done = 0: not attempted
// (no cached plan, WT changed, or flagged points): the caller takes the ordinary path.
static int shim_degrid_speculative(sde_ctx *ctx, const sde_gridspec &sp, int64_t n, const float *u, const float *v,
                                   const float *w, float *wt, const float *cf, const float *gvis, int nu, int nv,
                                   float *vis, int64_t *nbad, int *done) {
    *done = 0;
    const uint64_t h = hash_floats(cf, 2 * (SUPP + 1) * OSAMP + 1);
    if (!(g_pc.pl && n > 0 && g_pc.nvis == n && g_pc.cf_hash == h && memcmp(&g_pc.spec, &sp, sizeof sp) == 0 &&
          g_pc.pl->nuntouched == 0))
        return SDE_OK;
    cudaStream_t st = ctx->stream;
    SDE_TRY(shim_streams());
    cudaStream_t cs = g_ss.copy;
    const size_t nb = sizeof(float) * (size_t)n;
    float *in = nullptr, *dvis = nullptr, *dw = nullptr;
    float2 *dv = nullptr, *dg = nullptr;
    int *flag = nullptr;
    unsigned long long *cnt = nullptr;
    const int pitch = sde_grid_pitch(nu);
    SDE_TRY(ctx_scratch(ctx, "shim_in", 4 * nb, (void **)&in));
    SDE_TRY(ctx_scratch(ctx, "shim_flag2", 2 * sizeof(int), (void **)&flag));
    SDE_TRY(ctx_scratch(ctx, "shim_grid", sizeof(float2) * (size_t)pitch * nv, (void **)&dg));
    SDE_TRY(ctx_scratch(ctx, "dg_vis", 2 * nb, (void **)&dv));
    SDE_TRY(ctx_scratch(ctx, "dg_wt", nb, (void **)&dw));
    SDE_TRY(ctx_scratch(ctx, "dg_nbad", 16, (void **)&cnt));
    SDE_CUDA_TRY(cudaMemsetAsync(flag, 0, 2 * sizeof(int), st));
    SDE_CUDA_TRY(cudaMemsetAsync(cnt, 0, 16, st));
    SDE_CUDA_TRY(cudaEventRecord(g_ss.ev[0], st));
    SDE_CUDA_TRY(cudaStreamWaitEvent(cs, g_ss.ev[0], 0));
    // WT first, compared on the copy stream
    SDE_CUDA_TRY(shim_memcpy(in + 3 * n, wt, nb, cudaMemcpyHostToDevice, cs));
    k_words_differ<<<ctx->num_sms * 4, 256, 0, cs>>>(reinterpret_cast<const uint32_t *>(in + 3 * n),
                                                    reinterpret_cast<const uint32_t *>(g_pc.inputs + 3 * n), n,
                                                    flag);
    SDE_CHECK_LAUNCH();
    int fw = 1;
    SDE_CUDA_TRY(shim_memcpy(&fw, flag, sizeof(int), cudaMemcpyDeviceToHost, cs));
    SDE_CUDA_TRY(cudaStreamSynchronize(cs));
    if (fw) return SDE_OK;  // WT changed: the ordinary path
    // the model grid, the degrid with the cached plan and VIS down on the main stream ...
    SDE_CUDA_TRY(shim_memcpy2d(dg, (size_t)pitch * 8, gvis, (size_t)nu * 8, (size_t)nu * 8, (size_t)nv,
                                   cudaMemcpyHostToDevice, st));
    SDE_TRY(plan_degrid(g_pc.pl, (const float *)dg, pitch, 1, dv, dw, cnt));
    SDE_CUDA_TRY(shim_memcpy(vis, dv, 2 * nb, cudaMemcpyDeviceToHost, st));
    // ... while U, V, W go up and are compared on the copy stream
    const float *src[3] = {u, v, w};
    for (int k = 0; k < 3; k++) {
        SDE_CUDA_TRY(shim_memcpy(in + k * n, src[k], nb, cudaMemcpyHostToDevice, cs));
        k_words_differ<<<ctx->num_sms * 4, 256, 0, cs>>>(reinterpret_cast<const uint32_t *>(in + k * n),
                                                        reinterpret_cast<const uint32_t *>(g_pc.inputs + k * n), n,
                                                        flag + 1);
        SDE_CHECK_LAUNCH();
    }
    int fuvw = 1;
    SDE_CUDA_TRY(shim_memcpy(&fuvw, flag + 1, sizeof(int), cudaMemcpyDeviceToHost, cs));
    unsigned long long hc[2] = {0, 0};
    SDE_CUDA_TRY(shim_memcpy(hc, cnt, 16, cudaMemcpyDeviceToHost, st));
    SDE_CUDA_TRY(cudaStreamSynchronize(cs));
    SDE_CUDA_TRY(cudaStreamSynchronize(st));
    *done = 1;
    if (!fuvw) {
        g_pc.hits++;
        *nbad = (int64_t)hc[0];
        if (hc[1] > 0) {  // points not degridded: WT negated
            SDE_CUDA_TRY(shim_memcpy(wt, dw, nb, cudaMemcpyDeviceToHost, st));
            SDE_CUDA_TRY(cudaStreamSynchronize(st));
        }
        return SDE_OK;
    }
    // U, V or W changed: a new plan from the arrived inputs, then the ordinary degrid
    SDE_TRY(ctx_scratch(ctx, "shim_vis", 2 * nb, (void **)&dvis));
    SDE_CUDA_TRY(cudaMemsetAsync(dvis, 0, 2 * nb, st));
    sde_plan *pl = nullptr;
    SDE_TRY(shim_plan_build(ctx, sp, n, in, dvis, cf, h, &pl));
    return sde_plan_degrid(pl, (const float *)dg, pitch, vis, wt, SDE_HOST, nbad);
}

extern "C" void grddeh2d_(float *vis, float *wt, float *u, float *v, float *w, int *nvis,
                          float *uscale, float *uoffset, float *vscale, float *voffset,
                          int *uorigin, int *vorigin, float *gvis, int *nu, int *nv, float *intfnu,
                          int *suppu, int *osampu, float *intfnv, int *suppv, int *osampv,
                          double *shift) {
    if (sysi_.error) return;
    std::lock_guard<std::mutex> lk(g_shim_mu);
    const char *R = "GRDDEH2D";
    if (!check_table_args(intfnu, intfnv, *suppu, *osampu, *suppv, *osampv, R)) return;
    sde_ctx *ctx = shim_ctx();
    if (!ctx) {
        report("No GPU", R, sde_last_error());
        return;
    }
    sde_gridspec sp;
    fill_spec(&sp, *nu, *nv, *uscale, *uoffset, *vscale, *voffset, *uorigin, *vorigin, shift);
    sde_plan *pl = nullptr;
    float2 *dg = nullptr;
    const int pitch = sde_grid_pitch(*nu);
    int64_t nbad = 0;
    int done = 0;
    int rc = shim_degrid_speculative(ctx, sp, *nvis, u, v, w, wt, intfnu, gvis, *nu, *nv, vis, &nbad, &done);
    if (rc == SDE_OK && !done) {
        rc = ctx_scratch(ctx, "shim_grid", sizeof(float2) * (size_t)pitch * *nv, (void **)&dg);
        // the model grid goes up behind U, V, W, WT, while they are compared with the cached plan's
        const Upload2D gup{dg, (size_t)pitch * 8, gvis, (size_t)*nu * 8, (size_t)*nu * 8, (size_t)*nv};
        if (rc == SDE_OK) rc = shim_plan(ctx, sp, *nvis, u, v, w, nullptr, wt, intfnu, &pl, &gup);
        if (rc == SDE_OK) rc = sde_plan_degrid(pl, (const float *)dg, pitch, vis, wt, SDE_HOST, &nbad);
    }
    if (rc != SDE_OK) {
        report_rc(rc, R);
        return;
    }
    if (nbad > 0) {
        char m[64];
        snprintf(m, sizeof m, "%7lld points were not successfully degridded", (long long)nbad);
        msgput_(m, "W", strlen(m), 1);
    }
}

static void weights_shim(float *wt, float *u, float *v, float *w, int *nvis, float *uscale,
                         float *uoffset, float *vscale, float *voffset, int *uorigin, int *vorigin,
                         float *newwt, float *gwt, int *nu, int *nv, double *shift, int rmode,
                         float *robust, float ds, const char *R) {
    sde_ctx *ctx = shim_ctx();
    if (!ctx) {
        report("No GPU", R, sde_last_error());
        return;
    }
    const size_t n = (size_t)(*nvis > 0 ? *nvis : 1), ncell = (size_t)*nu * *nv;
    float *du, *dv, *dw, *dwt, *dnew, *dg;
    int rc = SDE_OK;
    if ((rc = ctx_scratch(ctx, "sh_u", 4 * n, (void **)&du)) ||
        (rc = ctx_scratch(ctx, "sh_v", 4 * n, (void **)&dv)) ||
        (rc = ctx_scratch(ctx, "sh_w", 4 * n, (void **)&dw)) ||
        (rc = ctx_scratch(ctx, "sh_wt", 4 * n, (void **)&dwt)) ||
        (rc = ctx_scratch(ctx, "sh_new", 4 * n, (void **)&dnew)) ||
        (rc = ctx_scratch(ctx, "sh_gwt", 4 * ncell, (void **)&dg))) {
        report_rc(rc, R);
        return;
    }
    const bool alias = newwt == wt;
    cudaStream_t st = ctx->stream;
    size_t nb = 4 * (size_t)*nvis;
    shim_memcpy(du, u, nb, cudaMemcpyHostToDevice, st);
    shim_memcpy(dv, v, nb, cudaMemcpyHostToDevice, st);
    shim_memcpy(dw, w, nb, cudaMemcpyHostToDevice, st);
    shim_memcpy(dwt, wt, nb, cudaMemcpyHostToDevice, st);
    if (!alias) shim_memcpy(dnew, newwt, nb, cudaMemcpyHostToDevice, st);
    sde_wstats stats;
    rc = sde_weights(ctx, rmode, robust, ds, dwt, du, dv, dw, *nvis, *uscale, *uoffset, *vscale,
                     *voffset, *uorigin, *vorigin, *nu, *nv, shift, alias ? dwt : dnew, dg, &stats);
    if (rc == SDE_OK) {
        shim_memcpy(newwt, alias ? dwt : dnew, nb, cudaMemcpyDeviceToHost, st);
        shim_memcpy(gwt, dg, 4 * ncell, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) rc = SDE_ECUDA;
    }
    if (rc == SDE_EBADMODE) {
        report("Logic error", R, "Unrecognized RMODE");
        return;
    }
    if (rc != SDE_OK) {
        report_rc(rc, R);
        return;
    }
    if (stats.ndrop > 0) {
        char m[64];
        snprintf(m, sizeof m, "%7lld points dropped off reweighting grid!", (long long)stats.ndrop);
        msgput_(m, "W", strlen(m), 1);
        const char *m2 = "These points are now flagged bad";
        msgput_(m2, "W", strlen(m2), 1);
    }
}

extern "C" void grduwt2d_(float *wt, float *u, float *v, float *w, int *nvis, float *uscale,
                          float *uoffset, float *vscale, float *voffset, int *uorigin, int *vorigin,
                          float *newwt, float *gwt, int *nu, int *nv, double *shift) {
    if (sysi_.error) return;
    std::lock_guard<std::mutex> lk(g_shim_mu);
    float rob[3] = {0.f, 0.f, 0.f};
    weights_shim(wt, u, v, w, nvis, uscale, uoffset, vscale, voffset, uorigin, vorigin, newwt, gwt,
                 nu, nv, shift, 0, rob, 0.0f, "GRDUWT2D");
}

extern "C" void grdruw2d_(float *wt, float *u, float *v, float *w, int *nvis, float *uscale,
                          float *uoffset, float *vscale, float *voffset, int *uorigin, int *vorigin,
                          float *newwt, float *gwt, int *nu, int *nv, double *shift, char *rmode,
                          float *robust, float *ds, size_t rmode_len) {
    if (sysi_.error) return;
    std::lock_guard<std::mutex> lk(g_shim_mu);
    int m;
    if (fstr_eq(rmode, rmode_len, "NORM"))
        m = 1;
    else if (fstr_eq(rmode, rmode_len, "ABS"))
        m = 2;
    else if (fstr_eq(rmode, rmode_len, "AZ-NORM"))
        m = 3;
    else if (fstr_eq(rmode, rmode_len, "NONE"))
        m = 4;
    else {
        // the reference grids first, then rejects the mode (grd/grdruw2d.f:190-192)
        report("Logic error", "GRDRUW2D", "Unrecognized RMODE");
        return;
    }
    float rob[3] = {robust[0], m == 3 ? robust[1] : 0.f, m == 3 ? robust[2] : 0.f};
    weights_shim(wt, u, v, w, nvis, uscale, uoffset, vscale, voffset, uorigin, vorigin, newwt, gwt,
                 nu, nv, shift, m, rob, *ds, "GRDRUW2D");
}

extern "C" void fftr2d_(float *rarray, float *xarray, float *work, float *work2, float *rwork,
                        int *nx, int *ny, int *fnu, int *nv, int *dir) {
    if (sysi_.error) return;
    std::lock_guard<std::mutex> lk(g_shim_mu);
    const char *R = "FFTR2D";
    sde_ctx *ctx = shim_ctx();
    if (!ctx) {
        report("No GPU", R, sde_last_error());
        return;
    }
    const int nu = *fnu / 2 + 1, pitch = sde_grid_pitch(nu);
    float2 *dg;
    float *di;
    int rc = ctx_scratch(ctx, "fft_grid", sizeof(float2) * (size_t)pitch * *nv, (void **)&dg);
    if (rc == SDE_OK) rc = ctx_scratch(ctx, "fft_img", sizeof(float) * (size_t)*nx * *ny, (void **)&di);
    if (rc != SDE_OK) {
        report_rc(rc, R);
        return;
    }
    cudaStream_t st = ctx->stream;
    if (*dir < 0) {
        shim_memcpy2d(dg, (size_t)pitch * 8, xarray, (size_t)nu * 8, (size_t)nu * 8, *nv,
                          cudaMemcpyHostToDevice, st);
        rc = sde_image_from_grid(ctx, (float *)dg, pitch, *nx, *ny, *fnu, *nv, 0, nullptr, di);
        if (rc == SDE_OK) {
            shim_memcpy(rarray, di, sizeof(float) * (size_t)*nx * *ny, cudaMemcpyDeviceToHost, st);
            // FFTR2D leaves the column-transformed grid in XARRAY (fft/fftr2d.f:82-90)
            shim_memcpy2d(xarray, (size_t)nu * 8, dg, (size_t)pitch * 8, (size_t)nu * 8, *nv,
                              cudaMemcpyDeviceToHost, st);
        }
    } else {
        shim_memcpy(di, rarray, sizeof(float) * (size_t)*nx * *ny, cudaMemcpyHostToDevice, st);
        rc = sde_grid_from_image(ctx, di, *nx, *ny, *fnu, *nv, 0, (float *)dg, pitch);
        if (rc == SDE_OK)
            shim_memcpy2d(xarray, (size_t)nu * 8, dg, (size_t)pitch * 8, (size_t)nu * 8, *nv,
                              cudaMemcpyDeviceToHost, st);
    }
    if (rc == SDE_OK && cudaStreamSynchronize(st) != cudaSuccess) rc = SDE_ECUDA;
    if (rc != SDE_OK) report_rc(rc, R);
}

namespace {
__global__ void k_pixcor2d(const float *in, int nx, int ny, const float *cf, int correct,
                           float *out, float scalex, float scaley, float cenx, float ceny) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (int64_t)nx * ny) return;
    const int iy = (int)(k / nx) + 1, ix = (int)(k - (int64_t)(iy - 1) * nx) + 1;
    const int icy = 1 + abs(nint_f(__fmul_rn(scaley, __fsub_rn((float)iy, ceny))));
    const int icx = 1 + abs(nint_f(__fmul_rn(scalex, __fsub_rn((float)ix, cenx))));
    const float f = __fmul_rn(cf[icx - 1], cf[icy - 1]);
    out[k] = correct ? __fdiv_rn(in[k], f) : __fmul_rn(f, in[k]);
}
}  // namespace

extern "C" void pixcor2d_(float *in, int *nx, int *ny, float *cf, int *cflen, char *mode,
                          float *out, float *cenx, float *ceny, size_t mode_len) {
    if (sysi_.error) return;
    std::lock_guard<std::mutex> lk(g_shim_mu);
    const char *R = "PIXCOR2D";
    int correct;
    if (mode_len >= 5 && strncmp(mode, "APPLY", 5) == 0)
        correct = 0;
    else if (mode_len >= 7 && strncmp(mode, "CORRECT", 7) == 0)
        correct = 1;
    else {
        report("Bad argument", R, "Unknown mode");
        return;
    }
    sde_ctx *ctx = shim_ctx();
    if (!ctx) {
        report("No GPU", R, sde_last_error());
        return;
    }
    const int fnx = fftpwr2(*nx), fny = fftpwr2(*ny);
    const float sx = (float)(*cflen - 1) * 2.0f / (float)fnx, sy = (float)(*cflen - 1) * 2.0f / (float)fny;
    const size_t npix = (size_t)*nx * *ny;
    float *di, *dc;
    if (ctx_scratch(ctx, "pc_img", 4 * npix, (void **)&di) || ctx_scratch(ctx, "pc_cf", 4 * (size_t)*cflen, (void **)&dc)) {
        report_rc(SDE_ENOMEM, R);
        return;
    }
    cudaStream_t st = ctx->stream;
    shim_memcpy(di, in, 4 * npix, cudaMemcpyHostToDevice, st);
    shim_memcpy(dc, cf, 4 * (size_t)*cflen, cudaMemcpyHostToDevice, st);
    KTimer kt(ctx, "pixcor2d");
    k_pixcor2d<<<ceil_div((int64_t)npix, 256), 256, 0, st>>>(di, *nx, *ny, dc, correct, di, sx, sy, *cenx, *ceny);
    shim_memcpy(out, di, 4 * npix, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        sde_set_error("%s", cudaGetErrorString(cudaGetLastError()));
        report_rc(SDE_ECUDA, R);
    }
}

extern "C" void pix2drcl_(float *drt, float *psf, float *box, int *nx, int *ny, int *pnx, int *pny,
                          float *gain, int *nsub, int *bsub, float *flux, float *cln, float *res,
                          int *ansub, float *maxres, float *tflux, float *cflux, int *cx, int *cy) {
    if (sysi_.error) return;
    std::lock_guard<std::mutex> lk(g_shim_mu);
    const char *R = "PIX2DRCL";
    sde_ctx *ctx = shim_ctx();
    if (!ctx) {
        report("No GPU", R, sde_last_error());
        return;
    }
    const size_t npix = (size_t)*nx * *ny, pnpix = (size_t)*pnx * *pny;
    const int nabs = *nsub < 0 ? -*nsub : *nsub;
    const size_t nc = (size_t)(nabs > 0 ? nabs : 1);
    float *dd, *dp, *db, *dcl, *dr, *dcf;
    int *dcx, *dcy;
    if (ctx_scratch(ctx, "hb_drt", 4 * npix, (void **)&dd) || ctx_scratch(ctx, "hb_psf", 4 * pnpix, (void **)&dp) ||
        ctx_scratch(ctx, "hb_box", 4 * npix, (void **)&db) || ctx_scratch(ctx, "hb_cln", 4 * npix, (void **)&dcl) ||
        ctx_scratch(ctx, "hb_res", 4 * npix, (void **)&dr) || ctx_scratch(ctx, "hb_cf", 4 * nc, (void **)&dcf) ||
        ctx_scratch(ctx, "hb_cx", 4 * nc, (void **)&dcx) || ctx_scratch(ctx, "hb_cy", 4 * nc, (void **)&dcy)) {
        report_rc(SDE_ENOMEM, R);
        return;
    }
    cudaStream_t st = ctx->stream;
    shim_memcpy(dd, drt, 4 * npix, cudaMemcpyHostToDevice, st);
    shim_memcpy(dp, psf, 4 * pnpix, cudaMemcpyHostToDevice, st);
    shim_memcpy(db, box, 4 * npix, cudaMemcpyHostToDevice, st);
    shim_memcpy(dcl, cln, 4 * npix, cudaMemcpyHostToDevice, st);
    if (nabs > 0) {
        shim_memcpy(dcf, cflux, 4 * (size_t)nabs, cudaMemcpyHostToDevice, st);
        shim_memcpy(dcx, cx, 4 * (size_t)nabs, cudaMemcpyHostToDevice, st);
        shim_memcpy(dcy, cy, 4 * (size_t)nabs, cudaMemcpyHostToDevice, st);
    }
    sde_clean_result out;
    int rc = sde_hogbom(ctx, dd, dp, db, *nx, *ny, *pnx, *pny, *gain, *nsub, *bsub, *flux, *tflux, dcl,
                        dr, dcf, dcx, dcy, nullptr, &out);
    if (rc != SDE_OK) {
        report_rc(rc, R);
        return;
    }
    shim_memcpy(cln, dcl, 4 * npix, cudaMemcpyDeviceToHost, st);
    shim_memcpy(res, dr, 4 * npix, cudaMemcpyDeviceToHost, st);
    if (nabs > 0) {
        shim_memcpy(cflux, dcf, 4 * (size_t)nabs, cudaMemcpyDeviceToHost, st);
        shim_memcpy(cx, dcx, 4 * (size_t)nabs, cudaMemcpyDeviceToHost, st);
        shim_memcpy(cy, dcy, 4 * (size_t)nabs, cudaMemcpyDeviceToHost, st);
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        report_rc(SDE_ECUDA, R);
        return;
    }
    *ansub = out.ansub;
    *maxres = out.maxres;
    *tflux = out.tflux;
}

extern "C" int pixisama_(int *n, float *a, int *i) {
    if (sysi_.error) return *i;
    std::lock_guard<std::mutex> lk(g_shim_mu);
    if (*n <= 0) return *i;
    sde_ctx *ctx = shim_ctx();
    if (!ctx) {
        report("No GPU", "PIXISAMA", sde_last_error());
        return *i;
    }
    float *d;
    if (ctx_scratch(ctx, "isa_in", 4 * (size_t)*n, (void **)&d)) {
        report_rc(SDE_ENOMEM, "PIXISAMA");
        return *i;
    }
    shim_memcpy(d, a, 4 * (size_t)*n, cudaMemcpyHostToDevice, ctx->stream);
    int64_t idx = 0;
    if (sde_isamax0(ctx, d, *n, &idx) != SDE_OK) {
        report_rc(SDE_ECUDA, "PIXISAMA");
        return *i;
    }
    return idx == 0 ? *i : (int)idx;
}
