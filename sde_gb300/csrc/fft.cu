// fft.cu -- the half-plane 2-D FFT of FFTR2D with the grid correction fused.
//
// Conventions (fft/fftr2d.f, fft/fftx1d.f, fft/fftr1d.f, fft/fftr1d2.f, fft/fftr.f,
// fft/fftx.f): along v, FFTX1D cyclically shifts the column by c = (NV+1)/2-1 on the way in
// and out; FFTX with ISIG=-1 is sum x exp(+2 pi i jk/M)/M, with ISIG=+1 sum x exp(-2 pi i
// jk/M).  Along u, FFTR1D2 centres the NX image pixels in FNU, FFTR1D shifts by
// (FNU+1)/2-1, and FFTR is the real<->half-complex transform (inverse: (1/N) sum over the
// Hermitian extension, reading only the real parts of the DC and Nyquist terms; forward:
// the plain DFT).  Grid correction (pix/pixcor2d.f:58-64) divides by CCF(ICFX)*CCF(ICFY)
// with the table of grd/grdccf.f.
//
// Kernels: a column pass keeps C whole columns of the grid in shared memory (C*NV*8 bytes,
// reading C*8 contiguous bytes per row), and a row pass keeps one half-length complex
// transform per row in shared memory; both use radix-2 butterflies over a twiddle table
// computed in double precision on the host.
#include <math.h>

#include "common.cuh"

namespace {

constexpr int FFT_THREADS = 512;

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ unsigned brev(unsigned k, int logn) {
    return logn == 0 ? 0u : (__brev(k) >> (32 - logn));
}

// In-place radix-2 DIT over `ncol` independent transforms of length n stored back to back
// in s (each already in bit-reversed order).  tw[k*tws] = exp(+2 pi i k/n) for k < n/2.
__device__ void block_fft(float2 *s, int n, int logn, int ncol, const float2 *__restrict__ tw,
                          int tws, bool inverse) {
    const int half = n >> 1;
    const int total = half * ncol;
    for (int st = 0; st < logn; st++) {
        const int h = 1 << st;
        const int step = half >> st;  // W_{2h}^j = W_n^{j n/(2h)}
        for (int b = threadIdx.x; b < total; b += blockDim.x) {
            const int col = b / half, bb = b - col * half;
            const int j = bb & (h - 1);
            const int i = ((bb >> st) << (st + 1)) + j;
            float2 w = __ldg(&tw[(size_t)j * step * tws]);
            if (!inverse) w.y = -w.y;
            float2 *base = s + (size_t)col * n;
            const float2 x = base[i], y = base[i + h];
            const float2 t = cmul(y, w);
            base[i] = make_float2(x.x + t.x, x.y + t.y);
            base[i + h] = make_float2(x.x - t.x, x.y - t.y);
        }
        __syncthreads();
    }
}

// Column pass along v, in place on grid [nv][pitch].  inverse: FFTX ISIG=-1 (1/nv);
// forward: ISIG=+1.  Forward mode treats rows outside [r0, r1) as zero (FFTR2D's padding,
// fft/fftr2d.f:57-70).
__global__ void __launch_bounds__(FFT_THREADS) k_col_fft(float2 *grid, int pitch, int nu, int nv,
                                                          int lognv, int ccols,
                                                          const float2 *__restrict__ tw,
                                                          int inverse, int r0, int r1) {
    extern __shared__ float2 s[];
    const int u0 = blockIdx.x * ccols;
    const int c = (nv + 1) / 2 - 1;
    const int total = nv * ccols;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int v = idx / ccols, j = idx - v * ccols;
        const int u = u0 + j;
        float2 x = make_float2(0.f, 0.f);
        if (u < nu && (inverse || (v >= r0 && v < r1))) x = grid[(int64_t)v * pitch + u];
        int k = v - c;
        if (k < 0) k += nv;
        s[(size_t)j * nv + brev((unsigned)k, lognv)] = x;
    }
    __syncthreads();
    block_fft(s, nv, lognv, ccols, tw, 1, inverse != 0);
    const float sc = inverse ? 1.0f / (float)nv : 1.0f;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int v = idx / ccols, j = idx - v * ccols;
        const int u = u0 + j;
        if (u >= nu) continue;
        int k = v - c;
        if (k < 0) k += nv;
        float2 z = s[(size_t)j * nv + k];
        if (inverse) {
            z.x = z.x * sc;
            z.y = z.y * sc;
        }
        grid[(int64_t)v * pitch + u] = z;
    }
}

struct CorrParams {
    const float *ccf;  // nullptr: no grid correction
    float scalex, scaley, cenx, ceny;
};

__device__ __forceinline__ float corr_factor(const CorrParams &cp, int ix1, int iy1) {
    const int icx = 1 + abs(nint_f(__fmul_rn(cp.scalex, __fsub_rn((float)ix1, cp.cenx))));
    const int icy = 1 + abs(nint_f(__fmul_rn(cp.scaley, __fsub_rn((float)iy1, cp.ceny))));
    return __fmul_rn(cp.ccf[icx - 1], cp.ccf[icy - 1]);
}

// Row pass grid -> image (c2r), one CTA per image row, with grid correction and an
// optional final scale OUT = s*IN (ARRSCALE by 1/max, pix/pixrscal.f).
__global__ void __launch_bounds__(FFT_THREADS) k_row_c2r(const float2 *__restrict__ grid,
                                                          int pitch, int fnu, int logh,
                                                          int nx, int ny, int ibegy,
                                                          const float2 *__restrict__ tw,
                                                          CorrParams cp,
                                                          const float *__restrict__ scale_dev,
                                                          float *image) {
    extern __shared__ float2 s[];
    const int iy = blockIdx.x;
    const int H = fnu >> 1;
    const float2 *X = grid + (int64_t)(iy + ibegy) * pitch;
    for (int k = threadIdx.x; k < H; k += blockDim.x) {
        float2 a = X[k], b = X[H - k];
        if (k == 0) {
            a.y = 0.f;
            b.y = 0.f;
        }
        // A = (X[k] + conj X[H-k]) / 2 ; B = (X[k] - conj X[H-k]) e^{+2 pi i k/N} / 2
        const float2 A = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
        const float2 d = make_float2(0.5f * (a.x - b.x), 0.5f * (a.y + b.y));
        const float2 B = cmul(d, __ldg(&tw[k]));
        // Z = A + i B
        s[brev((unsigned)k, logh)] = make_float2(A.x - B.y, A.y + B.x);
    }
    __syncthreads();
    block_fft(s, H, logh, 1, tw, 2, true);
    const float inv = 1.0f / (float)H;
    const int cu = (fnu + 1) / 2 - 1, ioff = (fnu - nx) / 2;
    const float sc = scale_dev ? 1.0f / *scale_dev : 1.0f;
    float *out = image + (int64_t)iy * nx;
    for (int ix = threadIdx.x; ix < nx; ix += blockDim.x) {
        int n = ix + ioff - cu;
        if (n < 0) n += fnu;
        const float2 z = s[n >> 1];
        float val = ((n & 1) ? z.y : z.x) * inv;
        if (cp.ccf) val = __fdiv_rn(val, corr_factor(cp, ix + 1, iy + 1));
        if (scale_dev) val = __fadd_rn(__fmul_rn(sc, val), 0.0f);
        out[ix] = val;
    }
}

// Row pass image -> grid (r2c), one CTA per image row; grid correction on the way in.
__global__ void __launch_bounds__(FFT_THREADS) k_row_r2c(const float *__restrict__ image, int nx,
                                                          int ny, int fnu, int logh, int ibegy,
                                                          const float2 *__restrict__ tw,
                                                          CorrParams cp, float2 *grid, int pitch,
                                                          int nu) {
    extern __shared__ float2 s[];
    const int iy = blockIdx.x;
    const int H = fnu >> 1;
    const int cu = (fnu + 1) / 2 - 1, ioff = (fnu - nx) / 2;
    const float *row = image + (int64_t)iy * nx;
    for (int m = threadIdx.x; m < H; m += blockDim.x) {
        float xv[2];
#pragma unroll
        for (int e = 0; e < 2; e++) {
            int k = 2 * m + e;                // x'[k] = R[(k + cu) mod fnu]
            int n = k + cu;
            if (n >= fnu) n -= fnu;
            const int ix = n - ioff;          // R[ioff + ix] = image[ix]
            float val = 0.f;
            if (ix >= 0 && ix < nx) {
                val = row[ix];
                if (cp.ccf) val = __fdiv_rn(val, corr_factor(cp, ix + 1, iy + 1));
            }
            xv[e] = val;
        }
        s[brev((unsigned)m, logh)] = make_float2(xv[0], xv[1]);
    }
    __syncthreads();
    block_fft(s, H, logh, 1, tw, 2, false);
    float2 *X = grid + (int64_t)(iy + ibegy) * pitch;
    for (int k = threadIdx.x; k <= H; k += blockDim.x) {
        const float2 zk = s[k == H ? 0 : k];
        const float2 zc = s[k == 0 || k == H ? 0 : H - k];
        // A = (Z[k] + conj Z[H-k])/2, B = (Z[k] - conj Z[H-k])/(2i), X = A + e^{-2 pi i k/N} B
        const float2 A = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y - zc.y));
        const float2 B = make_float2(0.5f * (zk.y + zc.y), -0.5f * (zk.x - zc.x));
        float2 w = k < H ? __ldg(&tw[k]) : make_float2(-1.f, 0.f);
        w.y = -w.y;
        const float2 t = cmul(B, w);
        float2 x = make_float2(A.x + t.x, A.y + t.y);
        if (k == 0 || k == H) x.y = 0.f;
        X[k] = x;
    }
}

int col_cols(int nv) {
    int c = 16384 / nv;
    if (c < 1) c = 1;
    if (c > 16) c = 16;
    return c;
}

int ilog2(int n) {
    int l = 0;
    while ((1 << l) < n) l++;
    return l;
}

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

int corr_params(sde_ctx *ctx, int nx, int ny, CorrParams *cp) {
    int fnx = fftpwr2(nx), fny = fftpwr2(ny);
    int ccflen = 1 + fftpwr2(nx > ny ? nx : ny) / 2;
    char name[48];
    snprintf(name, sizeof name, "ccf_%d", ccflen);
    auto it = ctx->scratch.find(name);
    float *d = nullptr;
    if (it == ctx->scratch.end() || it->second.bytes < sizeof(float) * (size_t)ccflen) {
        SDE_TRY(ctx_scratch(ctx, name, sizeof(float) * (size_t)ccflen, (void **)&d));
        std::vector<float> h((size_t)ccflen);
        sf_ccf_table(h.data(), ccflen);
        SDE_CUDA_TRY(cudaMemcpy(d, h.data(), sizeof(float) * (size_t)ccflen, cudaMemcpyHostToDevice));
    } else {
        d = (float *)it->second.p;
    }
    cp->ccf = d;
    cp->scalex = (float)(ccflen - 1) * 2.0f / (float)fnx;
    cp->scaley = (float)(ccflen - 1) * 2.0f / (float)fny;
    cp->cenx = (float)((nx + 1) / 2);
    cp->ceny = (float)((ny + 1) / 2);
    return SDE_OK;
}

int check_fft_args(int nx, int ny, int fnu, int nv, int pitch) {
    if (!is_pow2(fnu) || !is_pow2(nv) || fnu < 4 || nv < 2 || fnu > 16384 || nv > 16384 || nx < 1 ||
        ny < 1 || nx > fnu || ny > nv || pitch < fnu / 2 + 1) {
        sde_set_error("FFT: unsupported sizes nx=%d ny=%d fnu=%d nv=%d pitch=%d (power-of-two "
                      "FNU/NV up to 16384 required)", nx, ny, fnu, nv, pitch);
        return SDE_EINVAL;
    }
    return SDE_OK;
}

}  // namespace

int sde_image_from_grid(sde_ctx *ctx, float *grid, int pitch, int nx, int ny, int fnu, int nv,
                        int correct, const float *scale_dev, float *image) {
    if (!ctx || !grid || !image) return SDE_EINVAL;
    SDE_TRY(check_fft_args(nx, ny, fnu, nv, pitch));
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    const int nu = fnu / 2 + 1;
    const float2 *twv, *twu;
    SDE_TRY(ctx_twiddles(ctx, nv, &twv));
    SDE_TRY(ctx_twiddles(ctx, fnu, &twu));
    const int cc = col_cols(nv);
    const size_t smc = sizeof(float2) * (size_t)cc * nv;
    SDE_CUDA_TRY(cudaFuncSetAttribute(k_col_fft, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc));
    {
        KTimer kt(ctx, "col_fft");
        k_col_fft<<<ceil_div(nu, cc), FFT_THREADS, smc, ctx->stream>>>((float2 *)grid, pitch, nu, nv,
                                                                       ilog2(nv), cc, twv, 1, 0, nv);
    }
    SDE_CHECK_LAUNCH();
    CorrParams cp = {nullptr, 0.f, 0.f, 0.f, 0.f};
    if (correct) SDE_TRY(corr_params(ctx, nx, ny, &cp));
    const int ibegy = (nv + 1) / 2 - (ny + 1) / 2;  // 0-based first grid row
    const size_t smr = sizeof(float2) * (size_t)(fnu / 2);
    SDE_CUDA_TRY(cudaFuncSetAttribute(k_row_c2r, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr));
    KTimer kt(ctx, "row_c2r");
    k_row_c2r<<<ny, FFT_THREADS, smr, ctx->stream>>>((const float2 *)grid, pitch, fnu,
                                                     ilog2(fnu / 2), nx, ny, ibegy, twu, cp,
                                                     scale_dev, image);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

int sde_grid_from_image(sde_ctx *ctx, const float *image, int nx, int ny, int fnu, int nv,
                        int correct, float *grid, int pitch) {
    if (!ctx || !grid || !image) return SDE_EINVAL;
    SDE_TRY(check_fft_args(nx, ny, fnu, nv, pitch));
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    const int nu = fnu / 2 + 1;
    const float2 *twv, *twu;
    SDE_TRY(ctx_twiddles(ctx, nv, &twv));
    SDE_TRY(ctx_twiddles(ctx, fnu, &twu));
    CorrParams cp = {nullptr, 0.f, 0.f, 0.f, 0.f};
    if (correct) SDE_TRY(corr_params(ctx, nx, ny, &cp));
    const int ibegy = (nv + 1) / 2 - (ny + 1) / 2;
    const size_t smr = sizeof(float2) * (size_t)(fnu / 2);
    SDE_CUDA_TRY(cudaFuncSetAttribute(k_row_r2c, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr));
    {
        KTimer kt(ctx, "row_r2c");
        k_row_r2c<<<ny, FFT_THREADS, smr, ctx->stream>>>(image, nx, ny, fnu, ilog2(fnu / 2), ibegy,
                                                         twu, cp, (float2 *)grid, pitch, nu);
    }
    SDE_CHECK_LAUNCH();
    const int cc = col_cols(nv);
    const size_t smc = sizeof(float2) * (size_t)cc * nv;
    SDE_CUDA_TRY(cudaFuncSetAttribute(k_col_fft, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc));
    KTimer kt(ctx, "col_fft");
    k_col_fft<<<ceil_div(nu, cc), FFT_THREADS, smc, ctx->stream>>>((float2 *)grid, pitch, nu, nv,
                                                                   ilog2(nv), cc, twv, 0, ibegy,
                                                                   ibegy + ny);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}
