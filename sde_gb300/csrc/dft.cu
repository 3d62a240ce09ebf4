// dft.cu -- the direct Fourier transforms of uvmap's and vismodel's DFT options:
//   VISDFT3D (vis/visdft3d.f, 2-D): dirty(ix,iy) = RNORM sum_k WT_k Re(V_k E_k(ix,iy)),
//            psf(ix,iy) = RNORM sum_k WT_k Re(E_k(ix,iy)), E = exp(-i CF (u DX (ix-RX) + v DY (iy-RY)))
//   IMGDFT2D (img/imgdft2d.f): V_k = sum_{ix,iy} I(ix,iy) conj(E_k(ix,iy)) for WT_k > 0
// with CF = 2 pi^2/180 (DX, DY in degrees), RNORM = 1/sum WT over WT > 0.
// Both are dense contractions over visibilities x pixels.  E separates into a row factor and
// a column factor, so a CTA tile stages, per chunk of visibilities, the factors of its 64
// columns and 64 rows in shared memory and accumulates the tile in registers (2 FMA per
// visibility and pixel).  Phases are exact to FP32 rounding: the turns per pixel, g, are
// split into two 8-bit heads and a tail (a head times a pixel offset of at most 16 bits is
// exact in FP32, so is its fractional part; the tail's product is 2^-15 of the phase); the
// reference's rotation recurrence, whose error grows along each row, is not used.  Sums over
// chunks are compensated (TwoSum).
#include "common.cuh"

namespace {

constexpr int DT = 64;       // tile: 64 x 64 pixels (image) or 64 visibilities x 64 rows (vis)
constexpr int DK = 32;       // visibilities (or columns) per staged chunk
constexpr int DTHR = 256;

// per visibility: turns per pixel along x and y, each as two 8-bit heads and a tail, and
// the weights
struct DftVis {
    float4 gx;  // h1, h2, tail, 0
    float4 gy;
    float4 w;   // (RNORM WT V) re, im; RNORM WT; 0     (zero for WT <= 0)
};

__device__ __forceinline__ double head8(double x) {
    if (x == 0.0) return 0.0;
    int e;
    frexp(x, &e);
    const double q = ldexp(1.0, e - 8);
    return rint(x / q) * q;  // at most 8 significant bits
}

__device__ __forceinline__ float4 split3(double g) {
    const double h1 = head8(g), r = g - h1, h2 = head8(r);
    return make_float4((float)h1, (float)h2, (float)(r - h2), 0.f);
}

// exp(2 pi i s t), t = (h1 + h2 + l) n for a pixel offset n (|n| < 2^15, a multiple of 1/2):
// h n is exact for both heads, so are their fractional parts
__device__ __forceinline__ float2 cis_turns(float4 g, float n, float s) {
    const float p1 = __fmul_rn(g.x, n), p2 = __fmul_rn(g.y, n);
    const float f = __fadd_rn(__fsub_rn(p1, rintf(p1)), __fsub_rn(p2, rintf(p2)));
    const float t = __fmaf_rn(g.z, n, f);
    float sn, cs;
    sincospif(2.f * t, &sn, &cs);
    return make_float2(cs, s * sn);
}

__device__ __forceinline__ void two_sum(float &hi, float &lo, float x) {
    const float s = __fadd_rn(hi, x);
    const float bp = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    hi = s;
    lo = __fadd_rn(lo, err);
}

__global__ void k_dft_sumwt(const float *__restrict__ wt, int64_t n, double *sum) {
    double s = 0.0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        if (wt[k] > 0.f) s += wt[k];
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, s);
}

// CF u DX / (2 pi) = u DX pi/180 turns per pixel
__global__ void k_dft_prep(const float *__restrict__ u, const float *__restrict__ v, const float2 *__restrict__ vis,
                           const float *__restrict__ wt, int64_t n, double dx, double dy, const double *sumwt,
                           DftVis *out) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double d2r = 3.14159265358979323846 / 180.0;
    DftVis r;
    r.gx = split3((double)u[k] * dx * d2r);
    r.gy = split3((double)v[k] * dy * d2r);
    const float w = wt ? wt[k] : 1.f;
    if (w > 0.f) {
        const float c = sumwt ? (float)((double)w / *sumwt) : 1.f;
        const float2 vv = vis ? vis[k] : make_float2(0.f, 0.f);
        r.w = make_float4(c * vv.x, c * vv.y, c, 0.f);
    } else {
        r.w = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    out[k] = r;
}

// VISDFT3D tile: thread (tx, ty) owns pixels (x0 + tx + 16a, y0 + ty + 16b), a, b < 4; the
// visibilities are split over blockIdx.z (kper each, a multiple of DK) into partial images
// (hi, lo) that k_dft_reduce adds in split order
template <bool PSF>
__global__ void __launch_bounds__(DTHR) k_dft_image(const DftVis *__restrict__ pv, int64_t nvis, int nx, int ny,
                                                    float rx, float ry, int64_t kper, float2 *part) {
    __shared__ float2 ex[DK][DT];
    __shared__ float2 by[DK][DT];
    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const int x0 = blockIdx.x * DT, y0 = blockIdx.y * DT;
    float hi[4][4], lo[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) hi[a][b] = lo[a][b] = 0.f;
    const int64_t kb = (int64_t)blockIdx.z * kper, ke = min(nvis, kb + kper);
    for (int64_t k0 = kb; k0 < ke; k0 += DK) {
        __syncthreads();
        // factors of the chunk: ex[k][i] = exp(-2 pi i gx (x0+i+1-RX)), by[k][j] = w exp(-2 pi i gy (y0+j+1-RY))
        for (int e = t; e < DK * DT; e += DTHR) {
            const int k = e / DT, i = e % DT;
            const int64_t kk = k0 + k;
            float2 fx = make_float2(0.f, 0.f), fy = make_float2(0.f, 0.f);
            if (kk < ke) {
                const DftVis r = pv[kk];
                fx = cis_turns(r.gx, (float)(x0 + i + 1) - rx, -1.f);
                const float2 c = cis_turns(r.gy, (float)(y0 + i + 1) - ry, -1.f);
                if (PSF) {
                    fy = make_float2(r.w.z * c.x, r.w.z * c.y);
                } else {
                    fy = make_float2(__fsub_rn(__fmul_rn(r.w.x, c.x), __fmul_rn(r.w.y, c.y)),
                                     __fadd_rn(__fmul_rn(r.w.x, c.y), __fmul_rn(r.w.y, c.x)));
                }
            }
            ex[k][i] = fx;
            by[k][i] = fy;
        }
        __syncthreads();
        float acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) acc[a][b] = 0.f;
#pragma unroll 4
        for (int k = 0; k < DK; k++) {
            float2 xa[4], yb[4];
#pragma unroll
            for (int a = 0; a < 4; a++) xa[a] = ex[k][tx + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; b++) yb[b] = by[k][ty + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++)
                    acc[a][b] = fmaf(xa[a].x, yb[b].x, fmaf(-xa[a].y, yb[b].y, acc[a][b]));
        }
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) two_sum(hi[a][b], lo[a][b], acc[a][b]);
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int ix = x0 + tx + 16 * a, iy = y0 + ty + 16 * b;
            if (ix < nx && iy < ny)
                part[((size_t)blockIdx.z * ny + iy) * nx + ix] = make_float2(hi[a][b], lo[a][b]);
        }
}

// the partial images of the visibility splits, added in split order (compensated)
__global__ void k_dft_reduce(const float2 *__restrict__ part, int nsplit, int64_t npix, float *out) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (int64_t)gridDim.x * blockDim.x) {
        float hi = 0.f, lo = 0.f;
        for (int s = 0; s < nsplit; s++) {
            const float2 q = part[(size_t)s * npix + p];
            two_sum(hi, lo, q.x);
            lo = __fadd_rn(lo, q.y);
        }
        out[p] = __fadd_rn(hi, lo);
    }
}

// IMGDFT2D: CTA = 64 visibilities; for each band of 64 rows, T(k, row) = sum_x I(x, row)
// exp(2 pi i gx (x+1-RX)) over chunks of 32 columns (thread (tk, tr) owns visibilities
// tk + 16a and rows tr + 16b), then V_k += sum_rows exp(2 pi i gy (row+1-RY)) T(k, row).
__global__ void __launch_bounds__(DTHR) k_dft_vis(const float *__restrict__ image, int nx, int ny, float rx,
                                                  float ry, const DftVis *__restrict__ pv, int64_t nvis,
                                                  float2 *vis) {
    __shared__ float2 ex[DK][DT];      // [column][visibility]
    __shared__ float img[DK][DT + 1];  // [column][row], padded: the row-wise fill is conflict-free
    __shared__ float2 part[16][DT];    // per row group, per visibility
    const int t = threadIdx.x, tk = t & 15, tr = t >> 4;
    const int64_t v0 = (int64_t)blockIdx.x * DT;
    float hr = 0.f, hi_ = 0.f, lr = 0.f, li = 0.f;  // compensated sum of visibility v0 + t
    for (int y0 = 0; y0 < ny; y0 += DT) {
        float2 tacc[4][4];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) tacc[a][b] = make_float2(0.f, 0.f);
        for (int c0 = 0; c0 < nx; c0 += DK) {
            __syncthreads();
            for (int e = t; e < DK * DT; e += DTHR) {
                const int c = e / DT, i = e % DT;
                const int64_t kk = v0 + i;
                float2 fx = make_float2(0.f, 0.f);
                if (kk < nvis && c0 + c < nx) fx = cis_turns(pv[kk].gx, (float)(c0 + c + 1) - rx, 1.f);
                ex[c][i] = fx;
                // image rows along the warp's columns: coalesced reads
                const int ic = e % DK, ir = e / DK;
                img[ic][ir] = (c0 + ic < nx && y0 + ir < ny) ? image[(size_t)(y0 + ir) * nx + c0 + ic] : 0.f;
            }
            __syncthreads();
#pragma unroll 4
            for (int c = 0; c < DK; c++) {
                float2 xa[4];
                float ib[4];
#pragma unroll
                for (int a = 0; a < 4; a++) xa[a] = ex[c][tk + 16 * a];
#pragma unroll
                for (int b = 0; b < 4; b++) ib[b] = img[c][tr + 16 * b];
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        tacc[a][b].x = fmaf(ib[b], xa[a].x, tacc[a][b].x);
                        tacc[a][b].y = fmaf(ib[b], xa[a].y, tacc[a][b].y);
                    }
            }
        }
        // rows of this band: multiply by the row factor and sum over the thread's rows
        float2 s[4];
#pragma unroll
        for (int a = 0; a < 4; a++) {
            s[a] = make_float2(0.f, 0.f);
            const int64_t kk = v0 + tk + 16 * a;
            if (kk >= nvis) continue;
            const float4 gy = pv[kk].gy;
#pragma unroll
            for (int b = 0; b < 4; b++) {
                const int row = y0 + tr + 16 * b;
                if (row >= ny) continue;
                const float2 f = cis_turns(gy, (float)(row + 1) - ry, 1.f);
                s[a].x = fmaf(f.x, tacc[a][b].x, fmaf(-f.y, tacc[a][b].y, s[a].x));
                s[a].y = fmaf(f.x, tacc[a][b].y, fmaf(f.y, tacc[a][b].x, s[a].y));
            }
        }
        __syncthreads();
#pragma unroll
        for (int a = 0; a < 4; a++) part[tr][tk + 16 * a] = s[a];
        __syncthreads();
        if (t < DT) {
            float2 band = make_float2(0.f, 0.f);
            for (int g = 0; g < 16; g++) {
                band.x += part[g][t].x;
                band.y += part[g][t].y;
            }
            two_sum(hr, lr, band.x);
            two_sum(hi_, li, band.y);
        }
    }
    if (t < DT) {
        const int64_t kk = v0 + t;
        if (kk < nvis && pv[kk].w.z > 0.f) vis[kk] = make_float2(__fadd_rn(hr, lr), __fadd_rn(hi_, li));
    }
}

int fail(const char *m) {
    sde_set_error("%s", m);
    return SDE_EINVAL;
}

}  // namespace

extern "C" int sde_dft_image(sde_ctx *ctx, int64_t nvis, const float *u, const float *v, const float *vis,
                             const float *wt, int nx, int ny, double refx, double deltx, double refy,
                             double delty, float *dirty, float *psf) {
    if (!ctx || nvis < 1 || !u || !v || !wt || nx < 1 || ny < 1 || (!dirty && !psf) || (dirty && !vis))
        return fail("sde_dft_image: bad arguments");
    // pixel offsets |ix - REF| < 2^14 keep the split phases exact
    if (nx > 8192 || ny > 8192 || fabs(refx) > 8192 || fabs(refy) > 8192)
        return fail("sde_dft_image: image over 8192 pixels or reference pixel outside +-8192");
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    double *sw;
    DftVis *pv;
    SDE_TRY(ctx_scratch(ctx, "dft_sumwt", sizeof(double), (void **)&sw));
    SDE_TRY(ctx_scratch(ctx, "dft_vis", sizeof(DftVis) * (size_t)nvis, (void **)&pv));
    SDE_CUDA_TRY(cudaMemsetAsync(sw, 0, sizeof(double), st));
    k_dft_sumwt<<<ctx->num_sms * 4, 256, 0, st>>>(wt, nvis, sw);
    k_dft_prep<<<(unsigned)ceil_div(nvis, (int64_t)256), 256, 0, st>>>(
        u, v, reinterpret_cast<const float2 *>(vis), wt, nvis, deltx, delty, sw, pv);
    SDE_CHECK_LAUNCH();
    double h = 0.0;
    SDE_CUDA_TRY(cudaMemcpyAsync(&h, sw, sizeof h, cudaMemcpyDeviceToHost, st));
    SDE_CUDA_TRY(cudaStreamSynchronize(st));
    if (!(h > 0.0)) {
        sde_set_error("No valid data");  // vis/visdft3d.f:44
        return SDE_EINVAL;
    }
    // enough CTAs for every SM: the visibilities split over blockIdx.z
    const int tiles = (int)(ceil_div(nx, DT) * ceil_div(ny, DT));
    const int64_t chunks = ceil_div(nvis, (int64_t)DK);
    const int nsplit = (int)std::max<int64_t>(1, std::min<int64_t>(chunks, ceil_div((int64_t)ctx->num_sms * 4, (int64_t)tiles)));
    const int64_t kper = ceil_div(chunks, (int64_t)nsplit) * DK;
    const int64_t npix = (int64_t)nx * ny;
    float2 *part;
    SDE_TRY(ctx_scratch(ctx, "dft_part", sizeof(float2) * (size_t)nsplit * npix, (void **)&part));
    const dim3 grid((unsigned)ceil_div(nx, DT), (unsigned)ceil_div(ny, DT), (unsigned)nsplit);
    KTimer kt(ctx, "dft_image");
    for (int which = 0; which < 2; which++) {
        float *out = which ? psf : dirty;
        if (!out) continue;
        if (which) k_dft_image<true><<<grid, DTHR, 0, st>>>(pv, nvis, nx, ny, (float)refx, (float)refy, kper, part);
        else k_dft_image<false><<<grid, DTHR, 0, st>>>(pv, nvis, nx, ny, (float)refx, (float)refy, kper, part);
        k_dft_reduce<<<ctx->num_sms * 4, 256, 0, st>>>(part, nsplit, npix, out);
        SDE_CHECK_LAUNCH();
    }
    return SDE_OK;
}

extern "C" int sde_dft_vis(sde_ctx *ctx, const float *image, int nx, int ny, double refx, double deltx,
                           double refy, double delty, int64_t nvis, const float *u, const float *v,
                           const float *wt, float *vis) {
    if (!ctx || !image || nx < 1 || ny < 1 || nvis < 1 || !u || !v || !wt || !vis)
        return fail("sde_dft_vis: bad arguments");
    if (nx > 8192 || ny > 8192 || fabs(refx) > 8192 || fabs(refy) > 8192)
        return fail("sde_dft_vis: image over 8192 pixels or reference pixel outside +-8192");
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    DftVis *pv;
    SDE_TRY(ctx_scratch(ctx, "dft_vis", sizeof(DftVis) * (size_t)nvis, (void **)&pv));
    k_dft_prep<<<(unsigned)ceil_div(nvis, (int64_t)256), 256, 0, st>>>(u, v, nullptr, wt, nvis, deltx, delty,
                                                                      nullptr, pv);
    SDE_CHECK_LAUNCH();
    KTimer kt(ctx, "dft_vis");
    k_dft_vis<<<(unsigned)ceil_div(nvis, (int64_t)DT), DTHR, 0, st>>>(image, nx, ny, (float)refx, (float)refy, pv,
                                                                    nvis, reinterpret_cast<float2 *>(vis));
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}
