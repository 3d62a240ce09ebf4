// jobs.cu -- a whole uvmap job in one call: the device work of task/uvmap.f (weighting,
// PSF, dirty image, both divided by the PSF peak, task/uvmap.f:212-491) from host or device
// arrays to host or device images, with no return to the caller in between.  A server runs
// many of these concurrently, one per stream (sde_gb300/serve.py); doing the sequence here
// keeps the host side of a job to one call.
#include <string.h>

#include "common.cuh"

extern "C" int sde_uvmap(sde_ctx *ctx, const sde_uvmap_args *a, int64_t nvis, const float *u,
                         const float *v, const float *w, const float *vis, const float *wt,
                         int where, float *dirty, float *psf, sde_uvmap_result *res) {
    if (!ctx || !a || nvis < 0 || !dirty || (nvis > 0 && (!u || !v || !w || !vis || !wt)) ||
        a->nx < 1 || a->ny < 1 || a->rmode < -1 || a->rmode > 4) {
        sde_set_error("sde_uvmap: bad arguments");
        return SDE_EINVAL;
    }
    const sde_gridspec &sp = a->spec;
    const int fnu = 2 * (sp.nu - 1), nv = sp.nv;
    SDE_TRY(check_fft_shape(a->nx, a->ny, fnu, nv));
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const size_t n = (size_t)(nvis > 0 ? nvis : 1);
    // inputs on the device; WT always into scratch (weighting rewrites it)
    float *du = const_cast<float *>(u), *dv = const_cast<float *>(v), *dw = const_cast<float *>(w);
    float *dvis = const_cast<float *>(vis), *dwt = nullptr;
    SDE_TRY(ctx_scratch(ctx, "job_wt", sizeof(float) * n, (void **)&dwt));
    const cudaMemcpyKind kin = where == SDE_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    if (where == SDE_HOST) {
        SDE_TRY(ctx_scratch(ctx, "job_u", sizeof(float) * n, (void **)&du));
        SDE_TRY(ctx_scratch(ctx, "job_v", sizeof(float) * n, (void **)&dv));
        SDE_TRY(ctx_scratch(ctx, "job_w", sizeof(float) * n, (void **)&dw));
        SDE_TRY(ctx_scratch(ctx, "job_vis", sizeof(float) * 2 * n, (void **)&dvis));
        if (nvis > 0) {
            SDE_CUDA_TRY(cudaMemcpyAsync(du, u, sizeof(float) * nvis, kin, st));
            SDE_CUDA_TRY(cudaMemcpyAsync(dv, v, sizeof(float) * nvis, kin, st));
            SDE_CUDA_TRY(cudaMemcpyAsync(dw, w, sizeof(float) * nvis, kin, st));
            SDE_CUDA_TRY(cudaMemcpyAsync(dvis, vis, sizeof(float) * 2 * nvis, kin, st));
        }
    }
    if (nvis > 0) SDE_CUDA_TRY(cudaMemcpyAsync(dwt, wt, sizeof(float) * nvis, kin, st));
    sde_uvmap_result r{};
    if (a->rmode >= 0) {
        sde_wstats ws{};
        SDE_TRY(sde_weights(ctx, a->rmode, a->robust, a->ds, dwt, du, dv, dw, nvis, a->wuscale, 0.0f,
                            a->wvscale, 0.0f, sp.uorigin, sp.vorigin, sp.nu, sp.nv, sp.shift, dwt,
                            nullptr, &ws));
        r.ndrop = ws.ndrop;
    }
    sde_plan *pl = nullptr;
    SDE_TRY(sde_plan_create(ctx, &sp, nvis, du, dv, dw, dvis, dwt, SDE_DEVICE, &pl));
    r.ngrid = pl->nvis;
    const int pitch = sde_grid_pitch(sp.nu);
    const int64_t npix = (int64_t)a->nx * a->ny;
    float *grid = nullptr, *dpsf = nullptr, *ddirty = dirty, *peak = nullptr;
    int rc = ctx_scratch(ctx, "job_grid", sizeof(float2) * (size_t)pitch * nv, (void **)&grid);
    if (rc == SDE_OK) rc = ctx_scratch(ctx, "job_psf", sizeof(float) * (size_t)npix, (void **)&dpsf);
    if (rc == SDE_OK) rc = ctx_scratch(ctx, "job_peak", sizeof(float), (void **)&peak);
    if (rc == SDE_OK && a->out_where == SDE_HOST)
        rc = ctx_scratch(ctx, "job_dirty", sizeof(float) * (size_t)npix, (void **)&ddirty);
    float sw = 0.0f;
    if (rc == SDE_OK) rc = sde_plan_image(pl, SDE_GRID_PSF, a->nx, a->ny, 1, nullptr, dpsf, grid, pitch, &sw);
    if (rc == SDE_OK) rc = sde_image_max(ctx, dpsf, npix, peak);
    if (rc == SDE_OK) rc = sde_plan_image(pl, SDE_GRID_VIS, a->nx, a->ny, 1, peak, ddirty, grid, pitch, nullptr);
    if (rc == SDE_OK && psf) rc = sde_image_scale_by_inverse(ctx, dpsf, npix, peak);
    if (rc == SDE_OK) {
        cudaError_t e = cudaSuccess;
        if (a->out_where == SDE_HOST)
            e = cudaMemcpyAsync(dirty, ddirty, sizeof(float) * (size_t)npix, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && psf)
            e = cudaMemcpyAsync(psf, dpsf, sizeof(float) * (size_t)npix,
                                a->out_where == SDE_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st);
        // the peak through the context's pinned bytes (a pageable read would go through the
        // driver's staging, shared with the other slots' streams)
        if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_small, peak, sizeof(float), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) memcpy(&r.psf_peak, ctx->h_small, sizeof(float));
        if (e != cudaSuccess) {
            sde_set_error("sde_uvmap: %s", cudaGetErrorString(e));
            rc = SDE_ECUDA;
        }
    }
    r.sumwt = sw;
    sde_plan_destroy(pl);
    if (res) *res = r;
    return rc;
}
