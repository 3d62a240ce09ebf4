// box.cu -- GRDQH2D (grd/grdqh2d.f), the gridder VISGRID calls for the 'BOX' gridding
// function (vis/visgrid.f:154-158): each visibility, phase-rotated by the shift matrix, is
// added to its nearest cell; the u = 0 column is made Hermitian, then the grid is shifted one
// column left and scaled by (NU-1)*NV/LSUMWT.  One thread per visibility adds into a raw
// grid (atomics: FP32 sums in no fixed order); the column fold and the shift run on the raw
// grid into the caller's grid.
#include <math.h>

#include "common.cuh"

namespace {

struct BoxSums {
    double sumwt, lsumwt;
    unsigned long long ngrid;
};

__global__ void k_box_grid(const float2 *__restrict__ vis, const float *__restrict__ wt, const float *__restrict__ u,
                           const float *__restrict__ v, const float *__restrict__ w, int64_t nvis, float uscale,
                           float uoffset, float vscale, float voffset, int uorigin, int vorigin, int psf, int nu,
                           int nv, double s11, double s21, double s31, double s12, double s22, double s32,
                           double s13, double s23, double s33, float twopi, float2 *raw, BoxSums *sums) {
    double sw = 0.0, lw = 0.0;
    unsigned long long ng = 0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nvis; k += (int64_t)gridDim.x * blockDim.x) {
        const float wk = wt[k];
        if (!(wk > 0.f)) continue;
        const double uu = u[k], vv = v[k], ww = w[k];
        // grd/grdqh2d.f:77-83: DOUBLE products summed left to right, stored REAL
        const float ul = (float)__dadd_rn(__dadd_rn(__dmul_rn(s11, uu), __dmul_rn(s21, vv)), __dmul_rn(s31, ww));
        const float vl = (float)__dadd_rn(__dadd_rn(__dmul_rn(s12, uu), __dmul_rn(s22, vv)), __dmul_rn(s32, ww));
        const float wl = (float)__dadd_rn(__dadd_rn(__dmul_rn(s13, uu), __dmul_rn(s23, vv)), __dmul_rn(s33, ww));
        const float phase = __fmul_rn(twopi, __fsub_rn(wl, w[k]));
        const float c = cosf(phase), s = -sinf(phase);
        const float2 a = vis ? vis[k] : make_float2(0.f, 0.f);
        float2 f = make_float2(__fsub_rn(__fmul_rn(a.x, c), __fmul_rn(a.y, s)),
                               __fadd_rn(__fmul_rn(a.x, s), __fmul_rn(a.y, c)));
        float uc = __fadd_rn(__fmul_rn(uscale, ul), uoffset);
        float vc = __fadd_rn(__fmul_rn(vscale, vl), voffset);
        sw += wk;
        if (uc > 0.f) {
            f.y = -f.y;
            uc = __fadd_rn(uc, (float)uorigin);
            vc = __fadd_rn(vc, (float)vorigin);
        } else {
            uc = __fadd_rn(-uc, (float)uorigin);
            vc = __fadd_rn(-vc, (float)vorigin);
        }
        if (psf) f = make_float2(1.f, 0.f);
        const int ug = (int)lroundf(uc) + 1, vg = (int)lroundf(vc);
        if (ug < 1 || ug > nu || vg < 1 || vg > nv) continue;
        float2 *cell = raw + (size_t)(vg - 1) * nu + (ug - 1);
        atomicAdd(&cell->x, __fmul_rn(wk, f.x));
        atomicAdd(&cell->y, __fmul_rn(wk, f.y));
        lw += wk;
        ng++;
    }
    for (int d = 16; d > 0; d >>= 1) {
        sw += __shfl_xor_sync(0xffffffffu, sw, d);
        lw += __shfl_xor_sync(0xffffffffu, lw, d);
        ng += __shfl_xor_sync(0xffffffffu, ng, d);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&sums->sumwt, sw);
        atomicAdd(&sums->lsumwt, lw);
        atomicAdd(&sums->ngrid, ng);
    }
}

// grd/grdqh2d.f:115-121: GVIS(UZ, VZ+OFF) += CONJG(GVIS(UZ, VZ-OFF)); GVIS(UZ, VZ-OFF) =
// CONJG(GVIS(UZ, VZ+OFF)) for OFF = 0 .. NV/2-1 (each OFF touches its own pair of cells)
__global__ void k_box_fold(float2 *raw, int nu, int nv, int uz, int vz) {
    const int off = blockIdx.x * blockDim.x + threadIdx.x;
    if (off >= nv / 2) return;
    const int vp = vz + off, vm = vz - off;
    if (uz < 1 || uz > nu || vp < 1 || vp > nv || vm < 1 || vm > nv) return;
    float2 *p = raw + (size_t)(vp - 1) * nu + (uz - 1), *m = raw + (size_t)(vm - 1) * nu + (uz - 1);
    float2 a = *p;
    const float2 b = *m;
    a = make_float2(__fadd_rn(a.x, b.x), __fsub_rn(a.y, b.y));
    *p = a;
    *m = make_float2(a.x, -a.y);
}

// grd/grdqh2d.f:126-131: GVIS(U, V) = LSUMWT * GVIS(U+1, V), GVIS(NU, V) = 0, LSUMWT =
// FLOAT(NU-1)*FLOAT(NV)/LSUMWT
__global__ void k_box_final(const float2 *__restrict__ raw, int nu, int nv, const BoxSums *sums, float2 *grid,
                            int pitch) {
    const float scale = __fdiv_rn(__fmul_rn((float)(nu - 1), (float)nv), (float)sums->lsumwt);
    const int64_t n = (int64_t)nu * nv;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = k / nu, c = k % nu;
        float2 g = make_float2(0.f, 0.f);
        if (c < nu - 1) {
            const float2 a = raw[r * nu + c + 1];
            g = make_float2(__fmul_rn(scale, a.x), __fmul_rn(scale, a.y));
        }
        grid[r * pitch + c] = g;
    }
}

}  // namespace

int grid_box(sde_ctx *ctx, int64_t nvis, const float *vis, const float *wt, const float *u, const float *v,
             const float *w, float uscale, float uoffset, float vscale, float voffset, int uorigin, int vorigin,
             int psf, int nu, int nv, const double *shift, float *grid, int pitch, float *sumwt, int64_t *ngrid) {
    if (!ctx || nvis < 0 || nu < 2 || nv < 2 || pitch < nu || !grid || !shift ||
        (nvis > 0 && (!wt || !u || !v || !w || (!psf && !vis)))) {
        sde_set_error("sde_grid_box: bad arguments");
        return SDE_EINVAL;
    }
    cudaStream_t st = ctx->stream;
    float2 *raw;
    BoxSums *sums;
    SDE_TRY(ctx_scratch(ctx, "box_raw", sizeof(float2) * (size_t)nu * nv, (void **)&raw));
    SDE_TRY(ctx_scratch(ctx, "box_sums", sizeof(BoxSums), (void **)&sums));
    SDE_CUDA_TRY(cudaMemsetAsync(raw, 0, sizeof(float2) * (size_t)nu * nv, st));
    SDE_CUDA_TRY(cudaMemsetAsync(sums, 0, sizeof(BoxSums), st));
    const float twopi = 8.0f * atanf(1.0f);
    {
        KTimer kt(ctx, "box_grid");
        const unsigned nb = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(nvis, (int64_t)256),
                                                                              (int64_t)ctx->num_sms * 8));
        k_box_grid<<<nb, 256, 0, st>>>(reinterpret_cast<const float2 *>(vis), wt, u, v, w, nvis, uscale, uoffset,
                                       vscale, voffset, uorigin, vorigin, psf, nu, nv, shift[0], shift[1], shift[2],
                                       shift[3], shift[4], shift[5], shift[6], shift[7], shift[8], twopi, raw, sums);
        SDE_CHECK_LAUNCH();
    }
    k_box_fold<<<(unsigned)ceil_div(nv / 2, 256), 256, 0, st>>>(raw, nu, nv, uorigin + 1, vorigin);
    SDE_CHECK_LAUNCH();
    BoxSums h{};
    SDE_CUDA_TRY(cudaMemcpyAsync(&h, sums, sizeof h, cudaMemcpyDeviceToHost, st));
    SDE_CUDA_TRY(cudaStreamSynchronize(st));
    if (sumwt) *sumwt = (float)h.sumwt;
    if (ngrid) *ngrid = (int64_t)h.ngrid;
    if (h.lsumwt == 0.0) {
        sde_set_error("No weight!");  // grd/grdqh2d.f:122-124: the grid stays as gridded
        SDE_CUDA_TRY(cudaMemcpy2DAsync(grid, sizeof(float2) * pitch, raw, sizeof(float2) * nu, sizeof(float2) * nu,
                                       nv, cudaMemcpyDeviceToDevice, st));
        return SDE_ENOWEIGHT;
    }
    k_box_final<<<ctx->num_sms * 4, 256, 0, st>>>(raw, nu, nv, sums, reinterpret_cast<float2 *>(grid), pitch);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

extern "C" int sde_grid_box(sde_ctx *ctx, int64_t nvis, const float *vis, const float *wt, const float *u,
                            const float *v, const float *w, float uscale, float uoffset, float vscale, float voffset,
                            int uorigin, int vorigin, int psf, int nu, int nv, const double *shift, float *grid,
                            int pitch, float *sumwt) {
    if (!ctx) return SDE_EINVAL;
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    return grid_box(ctx, nvis, vis, wt, u, v, w, uscale, uoffset, vscale, voffset, uorigin, vorigin, psf, nu, nv,
                    shift, grid, pitch, sumwt, nullptr);
}
