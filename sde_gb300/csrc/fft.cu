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

// ---- register-resident radix-2/4/8/16 DFTs --------------------------------------------
// dft<R, INV>(v): v[k] <- sum_r v[r] w^(rk), w = exp(-2 pi i/R) (forward) or exp(+2 pi i/R).
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {  // a * (-i) forward, a * (+i) inverse
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
template <bool INV>
__device__ __forceinline__ void dft2(float2 &a, float2 &b) {
    const float2 t = a;
    a = make_float2(t.x + b.x, t.y + b.y);
    b = make_float2(t.x - b.x, t.y - b.y);
}
template <bool INV>
__device__ __forceinline__ void dft4(float2 &v0, float2 &v1, float2 &v2, float2 &v3) {
    float2 a0 = make_float2(v0.x + v2.x, v0.y + v2.y), a1 = make_float2(v0.x - v2.x, v0.y - v2.y);
    float2 a2 = make_float2(v1.x + v3.x, v1.y + v3.y), a3 = mul_mi<INV>(make_float2(v1.x - v3.x, v1.y - v3.y));
    v0 = make_float2(a0.x + a2.x, a0.y + a2.y);
    v2 = make_float2(a0.x - a2.x, a0.y - a2.y);
    v1 = make_float2(a1.x + a3.x, a1.y + a3.y);
    v3 = make_float2(a1.x - a3.x, a1.y - a3.y);
}
// constant twiddles exp(-+2 pi i m/16), m = 0..15, used inside dft8/dft16
__device__ __forceinline__ float2 w16(int m, bool inv) {
    const float c[4] = {1.0f, 0.92387953251128674f, 0.70710678118654752f, 0.38268343236508977f};
    m &= 15;
    float re, im;  // exp(-2 pi i m/16)
    const int q = m >> 2, r = m & 3;
    float cr = c[r], sr = r ? c[4 - r] : 0.0f;  // cos, sin of 2 pi r/16
    // rotate by -q*pi/2
    switch (q) {
        case 0: re = cr; im = -sr; break;
        case 1: re = -sr; im = -cr; break;
        case 2: re = -cr; im = sr; break;
        default: re = sr; im = cr; break;
    }
    return make_float2(re, inv ? -im : im);
}
template <bool INV>
__device__ __forceinline__ void dft8(float2 *v) {
    // r = r1 + 4 r2 (r1 < 4, r2 < 2); k = 2 k1 + k2
#pragma unroll
    for (int r1 = 0; r1 < 4; r1++) dft2<INV>(v[r1], v[r1 + 4]);  // -> Y[r1][k2] at v[r1 + 4 k2]
#pragma unroll
    for (int r1 = 1; r1 < 4; r1++) v[r1 + 4] = cmul(v[r1 + 4], w16(2 * r1, INV));  // w8^(r1 k2)
    dft4<INV>(v[0], v[1], v[2], v[3]);
    dft4<INV>(v[4], v[5], v[6], v[7]);
    // X[2 k1 + k2] = v[k1 + 4 k2]
    float2 t[8];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++)
#pragma unroll
        for (int k2 = 0; k2 < 2; k2++) t[2 * k1 + k2] = v[k1 + 4 * k2];
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = t[k];
}
template <bool INV>
__device__ __forceinline__ void dft16(float2 *v) {
    // r = r1 + 4 r2; k = 4 k1 + k2
#pragma unroll
    for (int r1 = 0; r1 < 4; r1++) dft4<INV>(v[r1], v[r1 + 4], v[r1 + 8], v[r1 + 12]);
#pragma unroll
    for (int r1 = 1; r1 < 4; r1++)
#pragma unroll
        for (int k2 = 1; k2 < 4; k2++) v[r1 + 4 * k2] = cmul(v[r1 + 4 * k2], w16(r1 * k2, INV));
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) dft4<INV>(v[4 * k2], v[4 * k2 + 1], v[4 * k2 + 2], v[4 * k2 + 3]);
    float2 t[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++)
#pragma unroll
        for (int k2 = 0; k2 < 4; k2++) t[4 * k1 + k2] = v[k1 + 4 * k2];
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = t[k];
}
template <int R, bool INV>
__device__ __forceinline__ void dftR(float2 *v) {
    if (R == 16) dft16<INV>(v);
    else if (R == 8) dft8<INV>(v);
    else if (R == 4) dft4<INV>(v[0], v[1], v[2], v[3]);
    else dft2<INV>(v[0], v[1]);
}

// bulk copy of nbytes (multiple of 16, both addresses 16-byte aligned) into shared memory
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t nbytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(reinterpret_cast<uint64_t>(src)), "r"(nbytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ bool bar_wait_bounded(uint32_t bar) {
    uint32_t done = 0;
    for (int spin = 0; spin < (1 << 24) && !done; spin++) {
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;"
            " selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(bar)
            : "memory");
    }
    return done != 0;
}

__device__ __forceinline__ void bar_init_one(uint32_t bar) {
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
        asm volatile("fence.mbarrier_init.release.cluster;");
        asm volatile("fence.proxy.async.shared::cta;");
    }
    __syncthreads();
}

// Shared-memory index of element i of a transform: an XOR swizzle of the low four bits by
// bits 4..7 spreads the stride-16 stores of the first radix-16 pass over all banks.
__device__ __forceinline__ int swz(int i) { return i ^ ((i >> 4) & 15); }

// One Stockham pass of radix R over `ncol` transforms of length n = 2^logn stored back to
// back in s (in place: every thread loads its R inputs, barrier, stores its R outputs,
// barrier).  tw[t*tws] = exp(+2 pi i t/n), t < n (double-precision table rounded to float).
template <int R, int LOGR, bool INV>
__device__ __forceinline__ void stockham_pass(float2 *s, int logn, int logns, int ncol,
                                              const float2 *__restrict__ tw, int tws) {
    const int lognb = logn - LOGR, nb = 1 << lognb, ns = 1 << logns;
    const int total = nb * ncol;
    const int tshift = logn - logns - LOGR;  // t = jm * r * n/(ns R)
    for (int base = 0; base < total; base += blockDim.x) {
        const int b = base + threadIdx.x;
        float2 v[R];
        int col = 0, j = 0;
        if (b < total) {
            col = b >> lognb;
            j = b & (nb - 1);
            const float2 *src = s + ((size_t)col << logn);
#pragma unroll
            for (int r = 0; r < R; r++) v[r] = src[swz(j + r * nb)];
        }
        __syncthreads();
        if (b < total) {
            const int jm = j & (ns - 1);
            if (jm) {
#pragma unroll
                for (int r = 1; r < R; r++) {
                    float2 w = __ldg(&tw[(size_t)((jm * r) << tshift) * tws]);
                    if (!INV) w.y = -w.y;
                    v[r] = cmul(v[r], w);
                }
            }
            dftR<R, INV>(v);
            float2 *dst = s + ((size_t)col << logn);
            const int od = ((j >> logns) << (logns + LOGR)) + jm;
#pragma unroll
            for (int r = 0; r < R; r++) dst[swz(od + r * ns)] = v[r];
        }
        __syncthreads();
    }
}

// Full in-place FFT of ncol transforms of length n = 2^logn (2..16384) in smem (swizzled
// index swz), natural order in and out.  inverse: exp(+), unscaled.
__device__ void block_fft(float2 *s, int logn, int ncol, const float2 *__restrict__ tw, int tws,
                          bool inverse) {
    int logns = 0;
    while (logns < logn) {
        const int rem = logn - logns;
        if (rem >= 4) {
            if (inverse) stockham_pass<16, 4, true>(s, logn, logns, ncol, tw, tws);
            else stockham_pass<16, 4, false>(s, logn, logns, ncol, tw, tws);
            logns += 4;
        } else if (rem == 3) {
            if (inverse) stockham_pass<8, 3, true>(s, logn, logns, ncol, tw, tws);
            else stockham_pass<8, 3, false>(s, logn, logns, ncol, tw, tws);
            logns += 3;
        } else if (rem == 2) {
            if (inverse) stockham_pass<4, 2, true>(s, logn, logns, ncol, tw, tws);
            else stockham_pass<4, 2, false>(s, logn, logns, ncol, tw, tws);
            logns += 2;
        } else {
            if (inverse) stockham_pass<2, 1, true>(s, logn, logns, ncol, tw, tws);
            else stockham_pass<2, 1, false>(s, logn, logns, ncol, tw, tws);
            logns += 1;
        }
    }
}

// Column pass along v, in place on grid [nv][pitch].  inverse: FFTX ISIG=-1 (1/nv);
// forward: ISIG=+1.  Forward mode treats rows outside [r0, r1) as zero (FFTR2D's padding,
// fft/fftr2d.f:57-70).  A CTA keeps ccols (even, power of two) whole columns in shared
// memory; rows are read as 16-byte pairs of columns, LB rows in flight per thread.
constexpr int COL_THREADS = 256;
constexpr int LB = 16;
__global__ void __launch_bounds__(COL_THREADS) k_col_fft(float2 *grid, int pitch, int nu, int nv,
                                                          int lognv, int logcc,
                                                          const float2 *__restrict__ tw,
                                                          int inverse, int r0, int r1) {
    extern __shared__ float2 s[];
    const int ccols = 1 << logcc;
    const int u0 = blockIdx.x * ccols;
    const int c = (nv + 1) / 2 - 1;
    const int lp = logcc - 1;               // pairs per row = ccols/2
    const int total = nv << lp;             // (row, pair) items
    for (int base = 0; base < total; base += COL_THREADS * LB) {
        float4 x[LB];
#pragma unroll
        for (int i = 0; i < LB; i++) {
            const int idx = base + i * COL_THREADS + threadIdx.x;
            const int v = idx >> lp, jp = idx & ((1 << lp) - 1);
            const int u = u0 + 2 * jp;
            x[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (idx < total && u < nu && (inverse || (v >= r0 && v < r1)))
                x[i] = *reinterpret_cast<const float4 *>(&grid[(int64_t)v * pitch + u]);
        }
#pragma unroll
        for (int i = 0; i < LB; i++) {
            const int idx = base + i * COL_THREADS + threadIdx.x;
            if (idx >= total) continue;
            const int v = idx >> lp, jp = idx & ((1 << lp) - 1);
            int k = v - c;
            if (k < 0) k += nv;
            s[((size_t)(2 * jp) << lognv) + swz(k)] = make_float2(x[i].x, x[i].y);
            s[((size_t)(2 * jp + 1) << lognv) + swz(k)] = make_float2(x[i].z, x[i].w);
        }
    }
    __syncthreads();
    block_fft(s, lognv, ccols, tw, 1, inverse != 0);
    const float sc = inverse ? 1.0f / (float)nv : 1.0f;
    for (int idx = threadIdx.x; idx < total; idx += COL_THREADS) {
        const int v = idx >> lp, jp = idx & ((1 << lp) - 1);
        const int u = u0 + 2 * jp;
        if (u >= nu) continue;
        int k = v - c;
        if (k < 0) k += nv;
        float2 z0 = s[((size_t)(2 * jp) << lognv) + swz(k)];
        float2 z1 = s[((size_t)(2 * jp + 1) << lognv) + swz(k)];
        if (inverse) {
            z0.x *= sc; z0.y *= sc; z1.x *= sc; z1.y *= sc;
        }
        // grid rows are 16-byte aligned (pitch % 4 == 0), u is even
        *reinterpret_cast<float4 *>(&grid[(int64_t)v * pitch + u]) = make_float4(z0.x, z0.y, z1.x, z1.y);
    }
}

struct CorrParams {
    const float *ccf;    // nullptr: no grid correction
    const float *corrx;  // CCF(ICFX) for each image column (pix/pixcor2d.f:62)
    const float *corry;  // CCF(ICFY) for each image row (pix/pixcor2d.f:60)
};

// PIXCOR2D's correction VAL / (CCF(ICFX)*CCF(ICFY)) (pix/pixcor2d.f:58-64) of an image
// pixel going into a forward transform.  For a zero pixel and a positive divisor the
// quotient is the pixel itself (sign included), so the division is skipped there: the model
// images a CLEAN major cycle transforms are mostly zero.
__device__ __forceinline__ float pixcor_in(float val, float cx, float cy) {
    const float d = __fmul_rn(cx, cy);
    return (val == 0.0f && d > 0.0f) ? val : __fdiv_rn(val, d);
}


// Row pass grid -> image (c2r), one CTA per image row, with grid correction and an
// optional final scale OUT = s*IN (ARRSCALE by 1/max, pix/pixrscal.f).
__global__ void __launch_bounds__(FFT_THREADS) k_row_c2r(const float2 *__restrict__ grid,
                                                          int pitch, int fnu, int rows,
                                                          int nx, int ny, int ibegy,
                                                          const float2 *__restrict__ tw,
                                                          CorrParams cp,
                                                          const float *__restrict__ scale_dev,
                                                          float *image) {
    extern __shared__ float2 s[];
    const int H = fnu >> 1;
    const int logh = __ffs(H) - 1;
    const int iy0 = blockIdx.x * rows;
    for (int t = threadIdx.x; t < H * rows; t += blockDim.x) {
        const int rr = t >> logh, k = t & (H - 1);
        const int iy = iy0 + rr;
        if (iy >= ny) {
            s[(rr << logh) + swz(k)] = make_float2(0.f, 0.f);
            continue;
        }
        const float2 *X = grid + (int64_t)(iy + ibegy) * pitch;
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
        s[(rr << logh) + swz(k)] = make_float2(A.x - B.y, A.y + B.x);
    }
    __syncthreads();
    block_fft(s, logh, rows, tw, 2, true);
    const float inv = 1.0f / (float)H;
    const int cu = (fnu + 1) / 2 - 1, ioff = (fnu - nx) / 2;
    const float sc = scale_dev ? 1.0f / *scale_dev : 1.0f;
    for (int rr = 0; rr < rows; rr++) {
        const int iy = iy0 + rr;
        if (iy >= ny) break;
        float *out = image + (int64_t)iy * nx;
        const float cfy = cp.ccf ? cp.corry[iy] : 1.0f;
        for (int ix = threadIdx.x; ix < nx; ix += blockDim.x) {
        int n = ix + ioff - cu;
        if (n < 0) n += fnu;
        const float2 z = s[(rr << logh) + swz(n >> 1)];
        float val = ((n & 1) ? z.y : z.x) * inv;
        if (cp.ccf) val = __fdiv_rn(val, __fmul_rn(cp.corrx[ix], cfy));
        if (scale_dev) val = __fadd_rn(__fmul_rn(sc, val), 0.0f);
        out[ix] = val;
        }
    }
}

// Row pass image -> grid (r2c), one CTA per image row; grid correction on the way in.
__global__ void __launch_bounds__(FFT_THREADS) k_row_r2c(const float *__restrict__ image, int nx,
                                                          int ny, int fnu, int rows, int ibegy,
                                                          const float2 *__restrict__ tw,
                                                          CorrParams cp, float2 *grid, int pitch,
                                                          int nu) {
    extern __shared__ float2 s[];
    const int H = fnu >> 1;
    const int logh = __ffs(H) - 1;
    const int cu = (fnu + 1) / 2 - 1, ioff = (fnu - nx) / 2;
    const int iy0 = blockIdx.x * rows;
    for (int t = threadIdx.x; t < H * rows; t += blockDim.x) {
        const int rr = t >> logh, m = t & (H - 1);
        const int iy = iy0 + rr;
        if (iy >= ny) {
            s[(rr << logh) + swz(m)] = make_float2(0.f, 0.f);
            continue;
        }
        const float cfy = cp.ccf ? cp.corry[iy] : 1.0f;
        const float *row = image + (int64_t)iy * nx;
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
                if (cp.ccf) val = pixcor_in(val, cp.corrx[ix], cfy);
            }
            xv[e] = val;
        }
        s[(rr << logh) + swz(m)] = make_float2(xv[0], xv[1]);
    }
    __syncthreads();
    block_fft(s, logh, rows, tw, 2, false);
    for (int rr = 0; rr < rows; rr++) {
        const int iy = iy0 + rr;
        if (iy >= ny) break;
        float2 *X = grid + (int64_t)(iy + ibegy) * pitch;
        const float2 *sr = s + (rr << logh);
        for (int k = threadIdx.x; k <= H; k += blockDim.x) {
        const float2 zk = sr[swz(k == H ? 0 : k)];
        const float2 zc = sr[swz(k == 0 || k == H ? 0 : H - k)];
        // A = (Z[k] + conj Z[H-k])/2, B = (Z[k] - conj Z[H-k])/(2i), X = A + e^{-2 pi i k/N} B
        const float2 A = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y - zc.y));
        const float2 B = make_float2(0.5f * (zk.y + zc.y), -0.5f * (zk.x - zc.x));
        float2 w = k < H ? __ldg(&tw[k]) : make_float2(-1.f, 0.f);
        w.y = -w.y;
        const float2 bw = cmul(B, w);
        float2 x = make_float2(A.x + bw.x, A.y + bw.y);
        if (k == 0 || k == H) x.y = 0.f;
        X[k] = x;
        }
    }
}

// rows per CTA and threads for the row passes: one radix-16 butterfly per thread per pass,
// at least 128 threads and 16 KB of shared memory per CTA
void row_shape(int fnu, int *rows, int *thr) {
    const int H = fnu / 2;
    int per = H / 16 < 32 ? 32 : H / 16;
    int r = 1;
    while (r * per < 128 || (size_t)r * H * 8 < 16384) r *= 2;
    if (r * per > FFT_THREADS) r = FFT_THREADS / per > 0 ? FFT_THREADS / per : 1;
    *rows = r;
    *thr = r * per > FFT_THREADS ? FFT_THREADS : r * per;
}

// log2 of the columns per CTA: 128 KB of columns, between 2 and 16 columns
int col_logcc(int nv) {
    int c = 16384 / nv;
    if (c < 2) c = 2;
    if (c > 16) c = 16;
    int l = 0;
    while ((1 << l) < c) l++;
    return l;
}

int ilog2(int n) {
    int l = 0;
    while ((1 << l) < n) l++;
    return l;
}

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// Per-axis grid-correction factors CCF(1 + |NINT(SCALE*(I - CEN))|) with PIXCOR2D's REAL
// arithmetic (pix/pixcor2d.f:44-63), computed on the host once per image shape.
int corr_params(sde_ctx *ctx, int nx, int ny, CorrParams *cp) {
    int fnx = fftpwr2(nx), fny = fftpwr2(ny);
    int ccflen = 1 + fftpwr2(nx > ny ? nx : ny) / 2;
    char name[64];
    snprintf(name, sizeof name, "ccf_%d_%d", nx, ny);
    auto it = ctx->scratch.find(name);
    float *d = nullptr;
    const size_t need = sizeof(float) * (size_t)(ccflen + nx + ny);
    if (it == ctx->scratch.end() || it->second.bytes < need) {
        SDE_TRY(ctx_scratch(ctx, name, need, (void **)&d));
        std::vector<float> h((size_t)(ccflen + nx + ny));
        sf_ccf_table(h.data(), ccflen);
        const float scalex = (float)(ccflen - 1) * 2.0f / (float)fnx;
        const float scaley = (float)(ccflen - 1) * 2.0f / (float)fny;
        const float cenx = (float)((nx + 1) / 2), ceny = (float)((ny + 1) / 2);
        for (int ix = 1; ix <= nx; ix++)
            h[(size_t)ccflen + ix - 1] = h[(size_t)abs((int)lroundf(scalex * ((float)ix - cenx)))];
        for (int iy = 1; iy <= ny; iy++)
            h[(size_t)ccflen + nx + iy - 1] = h[(size_t)abs((int)lroundf(scaley * ((float)iy - ceny)))];
        SDE_CUDA_TRY(cudaMemcpyAsync(d, h.data(), need, cudaMemcpyHostToDevice, ctx->stream));
    } else {
        d = (float *)it->second.p;
    }
    cp->ccf = d;
    cp->corrx = d + ccflen;
    cp->corry = d + ccflen + nx;
    return SDE_OK;
}

int check_fft_args(int nx, int ny, int fnu, int nv, int pitch) {
    if (!is_pow2(fnu) || !is_pow2(nv) || fnu < 4 || nv < 2 || fnu > 8192 || nv > 8192 || nx < 1 ||
        ny < 1 || nx > fnu || ny > nv || pitch < fnu / 2 + 1) {
        sde_set_error("FFT: unsupported sizes nx=%d ny=%d fnu=%d nv=%d pitch=%d (power-of-two "
                      "FNU/NV up to 8192 required, as ARRFFTR's MAXGAMMA=13)", nx, ny, fnu, nv, pitch);
        return SDE_EINVAL;
    }
    return SDE_OK;
}

// ---- compile-time-sized transforms ------------------------------------------------------
// The same Stockham decomposition as block_fft (radix-16 passes, then one radix-8/4/2 pass),
// with the transform length, the number of transforms in shared memory and the thread
// count fixed at compile time: every pass unrolls with constant strides, each thread keeps
// its butterflies' inputs in registers, and the kernels fit 64 registers (4+ resident CTAs
// of 256 threads per SM).

// v[r] *= w^r (r = 1..R-1) for w = tw[i1] (conjugated for the forward transform), with two
// table reads: w and w^4 = tw[i4]; the other powers are products (w^2 = w w, w^3 = w^2 w,
// w^(4a+b) = w^(4a) w^b), at most four roundings from the tabulated values.
template <int R, bool INV>
__device__ __forceinline__ void twiddle_powers(float2 *v, const float2 *__restrict__ tw, size_t i1,
                                               size_t i4) {
    float2 w1 = __ldg(&tw[i1]);
    if (!INV) w1.y = -w1.y;
    v[1] = cmul(v[1], w1);
    if (R == 2) return;
    const float2 w2 = cmul(w1, w1);
    v[2] = cmul(v[2], w2);
    const float2 w3 = cmul(w2, w1);
    v[3] = cmul(v[3], w3);
    if (R == 4) return;
    float2 w4 = __ldg(&tw[i4]);
    if (!INV) w4.y = -w4.y;
    float2 wa = w4;  // w^(4a)
#pragma unroll
    for (int a = 1; a < R / 4; a++) {
        if (a > 1) wa = cmul(wa, w4);
        v[4 * a] = cmul(v[4 * a], wa);
        v[4 * a + 1] = cmul(v[4 * a + 1], cmul(wa, w1));
        v[4 * a + 2] = cmul(v[4 * a + 2], cmul(wa, w2));
        v[4 * a + 3] = cmul(v[4 * a + 3], cmul(wa, w3));
    }
}

// One radix-2^LOGR pass over NT transforms of length 2^LOGN (T threads).
template <int LOGN, int LOGR, int LOGNS, bool INV, int NT, int T>
__device__ __forceinline__ void st_pass(float2 *s, const float2 *__restrict__ tw, int tws) {
    constexpr int R = 1 << LOGR, NB = 1 << (LOGN - LOGR), NS = 1 << LOGNS;
    constexpr int TOTAL = NB * NT;
    constexpr int PER = (TOTAL + T - 1) / T;
    constexpr int TSHIFT = LOGN - LOGNS - LOGR;
    float2 v[PER][R];
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int b = threadIdx.x + i * T;
        if (TOTAL % T == 0 || b < TOTAL) {
            const int col = b >> (LOGN - LOGR), j = b & (NB - 1);
            const float2 *src = s + (col << LOGN);
#pragma unroll
            for (int r = 0; r < R; r++) v[i][r] = src[swz(j + r * NB)];
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int b = threadIdx.x + i * T;
        if (TOTAL % T == 0 || b < TOTAL) {
            const int col = b >> (LOGN - LOGR), j = b & (NB - 1);
            const int jm = j & (NS - 1);
            if (LOGNS > 0 && jm)
                twiddle_powers<R, INV>(v[i], tw, (size_t)(jm << TSHIFT) * tws,
                                       (size_t)((4 * jm) << TSHIFT) * tws);
            dftR<R, INV>(v[i]);
            float2 *dst = s + (col << LOGN);
            const int od = ((j >> LOGNS) << (LOGNS + LOGR)) + jm;
#pragma unroll
            for (int r = 0; r < R; r++) dst[swz(od + r * NS)] = v[i][r];
        }
    }
    __syncthreads();
}

template <int LOGN, int LOGNS, bool INV, int NT, int T>
struct StPasses {
    static __device__ __forceinline__ void run(float2 *s, const float2 *__restrict__ tw, int tws) {
        constexpr int REM = LOGN - LOGNS;
        constexpr int LOGR = REM >= 4 ? 4 : REM;
        st_pass<LOGN, LOGR, LOGNS, INV, NT, T>(s, tw, tws);
        StPasses<LOGN, LOGNS + LOGR, INV, NT, T>::run(s, tw, tws);
    }
};
template <int LOGN, bool INV, int NT, int T>
struct StPasses<LOGN, LOGN, INV, NT, T> {
    static __device__ __forceinline__ void run(float2 *, const float2 *__restrict__, int) {}
};

// Shapes: columns per CTA and threads for a column transform of length 2^LOGN, rows per CTA
// and threads for a row transform of half-length 2^LOGH.
template <int LOGN>
struct ColShape {
    static constexpr int N = 1 << LOGN;
    static constexpr int CC = N >= 4096 ? 2 : (4096 / N > 64 ? 64 : 4096 / N);  // columns
    static constexpr int T0 = CC * N / 16;
    static constexpr int T = T0 < 128 ? 128 : (T0 > 1024 ? 1024 : T0);
    static constexpr size_t SMEM = sizeof(float2) * (size_t)CC * N;
    static constexpr int MINB = 1024 / T;  // resident CTAs the kernel is built for (64 regs)
};
template <int LOGH>
struct RowShape {
    static constexpr int H = 1 << LOGH;
    static constexpr int ROWS = H >= 2048 ? 2 : 4096 / H;
    static constexpr int T0 = ROWS * H / 16;
    static constexpr int T = T0 < 128 ? 128 : (T0 > 1024 ? 1024 : T0);
    static constexpr size_t SMEM = sizeof(float2) * (size_t)ROWS * H + 16;  // + an mbarrier
    static constexpr int MINB = 1024 / T;
};

// Column pass along v (as k_col_fft), CC columns per CTA read as 16-byte column pairs.
template <int LOGN, bool INV>
__global__ void __launch_bounds__(ColShape<LOGN>::T, ColShape<LOGN>::MINB)
    k_col_fft_t(const __grid_constant__ FftBatch bt, int pitch, int nu, const float2 *__restrict__ tw,
                int r0, int r1) {
    float2 *grid = bt.grid[blockIdx.y];
    using S = ColShape<LOGN>;
    constexpr int N = S::N, CC = S::CC, T = S::T;
    constexpr int LP = __builtin_ctz(CC) - 1;           // log2(column pairs per row)
    constexpr int TOTAL = N * CC / 2;                   // (row, pair) items
    constexpr int PER = (TOTAL + T - 1) / T;
    extern __shared__ float2 s[];
    const int u0 = blockIdx.x * CC;
    const int c = (N + 1) / 2 - 1;
    float4 x[PER];
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int idx = i * T + threadIdx.x;
        const int v = idx >> LP, jp = idx & ((1 << LP) - 1);
        const int u = u0 + 2 * jp;
        x[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if ((TOTAL % T == 0 || idx < TOTAL) && u < nu && (INV || (v >= r0 && v < r1)))
            x[i] = *reinterpret_cast<const float4 *>(&grid[(int64_t)v * pitch + u]);
    }
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int idx = i * T + threadIdx.x;
        if (TOTAL % T != 0 && idx >= TOTAL) continue;
        const int v = idx >> LP, jp = idx & ((1 << LP) - 1);
        int k = v - c;
        if (k < 0) k += N;
        s[((2 * jp) << LOGN) + swz(k)] = make_float2(x[i].x, x[i].y);
        s[((2 * jp + 1) << LOGN) + swz(k)] = make_float2(x[i].z, x[i].w);
    }
    __syncthreads();
    StPasses<LOGN, 0, INV, CC, T>::run(s, tw, 1);
    const float sc = INV ? 1.0f / (float)N : 1.0f;
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int idx = i * T + threadIdx.x;
        if (TOTAL % T != 0 && idx >= TOTAL) continue;
        const int v = idx >> LP, jp = idx & ((1 << LP) - 1);
        const int u = u0 + 2 * jp;
        if (u >= nu) continue;
        int k = v - c;
        if (k < 0) k += N;
        float2 z0 = s[((2 * jp) << LOGN) + swz(k)];
        float2 z1 = s[((2 * jp + 1) << LOGN) + swz(k)];
        if (INV) {
            z0.x *= sc; z0.y *= sc; z1.x *= sc; z1.y *= sc;
        }
        *reinterpret_cast<float4 *>(&grid[(int64_t)v * pitch + u]) = make_float4(z0.x, z0.y, z1.x, z1.y);
    }
}

// Row pass grid -> image (as k_row_c2r), ROWS rows per CTA, half-length 2^LOGH.
template <int LOGH>
__global__ void __launch_bounds__(RowShape<LOGH>::T, RowShape<LOGH>::MINB)
    k_row_c2r_t(const __grid_constant__ FftBatch bt, int pitch, int nx, int ny, int ibegy,
                const float2 *__restrict__ tw, CorrParams cp) {
    const float2 *__restrict__ grid = bt.grid[blockIdx.y];
    const float *__restrict__ scale_dev = bt.scale[blockIdx.y];
    float *image = bt.image[blockIdx.y];
    using S = RowShape<LOGH>;
    constexpr int H = S::H, ROWS = S::ROWS, T = S::T, FNU = 2 * H;
    constexpr int TOTAL = ROWS * H;
    constexpr int PER = (TOTAL + T - 1) / T;
    extern __shared__ float2 s[];
    const int iy0 = blockIdx.x * ROWS;
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int t = i * T + threadIdx.x;
        if (TOTAL % T != 0 && t >= TOTAL) continue;
        const int rr = t >> LOGH, k = t & (H - 1);
        const int iy = iy0 + rr;
        if (iy >= ny) {
            s[(rr << LOGH) + swz(k)] = make_float2(0.f, 0.f);
            continue;
        }
        const float2 *X = grid + (int64_t)(iy + ibegy) * pitch;
        float2 a = X[k], b = X[H - k];
        if (k == 0) {
            a.y = 0.f;
            b.y = 0.f;
        }
        const float2 A = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
        const float2 d = make_float2(0.5f * (a.x - b.x), 0.5f * (a.y + b.y));
        const float2 B = cmul(d, __ldg(&tw[k]));
        s[(rr << LOGH) + swz(k)] = make_float2(A.x - B.y, A.y + B.x);
    }
    __syncthreads();
    StPasses<LOGH, 0, true, ROWS, T>::run(s, tw, 2);
    const float inv = 1.0f / (float)H;
    const int cu = (FNU + 1) / 2 - 1, ioff = (FNU - nx) / 2;
    const float sc = scale_dev ? 1.0f / *scale_dev : 1.0f;
    for (int t = threadIdx.x; t < ROWS * nx; t += T) {
        const int rr = t / nx, ix = t - rr * nx;
        const int iy = iy0 + rr;
        if (iy >= ny) break;
        int n = ix + ioff - cu;
        if (n < 0) n += FNU;
        const float2 z = s[(rr << LOGH) + swz(n >> 1)];
        float val = ((n & 1) ? z.y : z.x) * inv;
        if (cp.ccf) val = __fdiv_rn(val, __fmul_rn(cp.corrx[ix], cp.corry[iy]));
        if (scale_dev) val = __fadd_rn(__fmul_rn(sc, val), 0.0f);
        image[(int64_t)iy * nx + ix] = val;
    }
}

// Row pass image -> grid (as k_row_r2c), ROWS rows per CTA, half-length 2^LOGH.
template <int LOGH>
__global__ void __launch_bounds__(RowShape<LOGH>::T, RowShape<LOGH>::MINB)
    k_row_r2c_t(const __grid_constant__ FftBatch bt, int nx, int ny, int ibegy,
                const float2 *__restrict__ tw, CorrParams cp, int pitch, int *status) {
    const float *__restrict__ image = bt.image[blockIdx.y];
    float2 *grid = bt.grid[blockIdx.y];
    using S = RowShape<LOGH>;
    constexpr int H = S::H, ROWS = S::ROWS, T = S::T, FNU = 2 * H;
    constexpr int TOTAL = ROWS * H;
    constexpr int PER = (TOTAL + T - 1) / T;
    extern __shared__ __align__(16) float2 s[];
    const int cu = (FNU + 1) / 2 - 1, ioff = (FNU - nx) / 2;
    const int iy0 = blockIdx.x * ROWS;
    if (ROWS == 2 && status) {
        // the CTA's image rows come in by bulk copy (row rr at floats [rr*FNU, rr*FNU+nx) of
        // s); every thread reads its inputs from there, then the FFT layout overwrites it
        // (measured: 0.099 -> 0.088 ms at 4096^2 against the L2-prefetch path below)
        const float *stg = reinterpret_cast<const float *>(s);
        const uint32_t sb = (uint32_t)__cvta_generic_to_shared(s);
        const uint32_t bb = (uint32_t)__cvta_generic_to_shared(s + ROWS * H);
        const bool two = iy0 + 1 < ny;
        bar_init_one(bb);
        if (threadIdx.x == 0) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bb),
                         "r"((uint32_t)((two ? 2 : 1) * nx * sizeof(float))));
            bulk_g2s(sb, image + (int64_t)iy0 * nx, nx * sizeof(float), bb);
            if (two) bulk_g2s(sb + FNU * sizeof(float), image + (int64_t)(iy0 + 1) * nx, nx * sizeof(float), bb);
        }
        if (!bar_wait_bounded(bb)) {
            atomicExch(&status[STATUS_TIMEOUT], 1);
            return;
        }
        float2 xin[PER];
#pragma unroll
        for (int i = 0; i < PER; i++) {
            const int t = i * T + threadIdx.x;
            const int rr = t >> LOGH, m = t & (H - 1);
            const int iy = iy0 + rr;
            xin[i] = make_float2(0.f, 0.f);
            if (iy >= ny) continue;
            const float cfy = cp.ccf ? cp.corry[iy] : 1.0f;
            float xv[2];
#pragma unroll
            for (int e = 0; e < 2; e++) {
                int n = 2 * m + e + cu;
                if (n >= FNU) n -= FNU;
                const int ix = n - ioff;
                float val = 0.f;
                if (ix >= 0 && ix < nx) {
                    val = stg[rr * FNU + ix];
                    if (cp.ccf) val = pixcor_in(val, cp.corrx[ix], cfy);
                }
                xv[e] = val;
            }
            xin[i] = make_float2(xv[0], xv[1]);
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < PER; i++) {
            const int t = i * T + threadIdx.x;
            s[((t >> LOGH) << LOGH) + swz(t & (H - 1))] = xin[i];
        }
    } else {
    // rows that do not start on 16-byte boundaries: the CTA's image rows start on their way
    // to L2 while the first loads are issued (0.107 -> 0.099 ms at 4096^2)
    if (threadIdx.x == 0)
        for (int rr = 0; rr < ROWS; rr++)
            if (iy0 + rr < ny) prefetch_l2_range(image + (int64_t)(iy0 + rr) * nx, 0, nx, 4);
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int t = i * T + threadIdx.x;
        if (TOTAL % T != 0 && t >= TOTAL) continue;
        const int rr = t >> LOGH, m = t & (H - 1);
        const int iy = iy0 + rr;
        if (iy >= ny) {
            s[(rr << LOGH) + swz(m)] = make_float2(0.f, 0.f);
            continue;
        }
        const float cfy = cp.ccf ? cp.corry[iy] : 1.0f;
        const float *row = image + (int64_t)iy * nx;
        float xv[2];
#pragma unroll
        for (int e = 0; e < 2; e++) {
            const int k = 2 * m + e;
            int n = k + cu;
            if (n >= FNU) n -= FNU;
            const int ix = n - ioff;
            float val = 0.f;
            if (ix >= 0 && ix < nx) {
                val = row[ix];
                if (cp.ccf) val = pixcor_in(val, cp.corrx[ix], cfy);
            }
            xv[e] = val;
        }
        s[(rr << LOGH) + swz(m)] = make_float2(xv[0], xv[1]);
    }
    }
    __syncthreads();
    StPasses<LOGH, 0, false, ROWS, T>::run(s, tw, 2);
    for (int t = threadIdx.x; t < ROWS * (H + 1); t += T) {
        const int rr = t / (H + 1), k = t - rr * (H + 1);
        const int iy = iy0 + rr;
        if (iy >= ny) break;
        float2 *X = grid + (int64_t)(iy + ibegy) * pitch;
        const float2 *sr = s + (rr << LOGH);
        const float2 zk = sr[swz(k == H ? 0 : k)];
        const float2 zc = sr[swz(k == 0 || k == H ? 0 : H - k)];
        const float2 A = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y - zc.y));
        const float2 B = make_float2(0.5f * (zk.y + zc.y), -0.5f * (zk.x - zc.x));
        float2 w = k < H ? __ldg(&tw[k]) : make_float2(-1.f, 0.f);
        w.y = -w.y;
        const float2 bw = cmul(B, w);
        float2 xo = make_float2(A.x + bw.x, A.y + bw.y);
        if (k == 0 || k == H) xo.y = 0.f;
        X[k] = xo;
    }
}

// ---- column pass fed by TMA -----------------------------------------------------------
// Two columns per CTA, held in shared memory as (col0, col1) complex pairs, one float4 per
// row: TMA box loads bring the 16 bytes of each row in (no load instructions, no L1
// wavefronts per row), every thread runs its radix-16 butterfly on both columns with one
// set of twiddles, and TMA box stores write the columns back.  The first pass reads in row
// order (FFTX1D's cyclic shift and, forward, the rows outside the image read as zero), the
// middle passes use an XOR swizzle for float4 elements, and the last pass writes in row
// order (inverse: times 1/N).  The tensor map's width (2*NU floats) keeps the loads of the
// padding column at zero and the stores out of it.
__device__ __forceinline__ int swz4(int i) { return i ^ ((i >> 4) & 7); }

template <int R, bool INV>
__device__ __forceinline__ void twiddle_powers2(float2 *a, float2 *b, const float2 *__restrict__ tw,
                                                size_t i1, size_t i4) {
    float2 w1 = __ldg(&tw[i1]);
    if (!INV) w1.y = -w1.y;
    a[1] = cmul(a[1], w1);
    b[1] = cmul(b[1], w1);
    if (R == 2) return;
    const float2 w2 = cmul(w1, w1);
    a[2] = cmul(a[2], w2);
    b[2] = cmul(b[2], w2);
    const float2 w3 = cmul(w2, w1);
    a[3] = cmul(a[3], w3);
    b[3] = cmul(b[3], w3);
    if (R == 4) return;
    float2 w4 = __ldg(&tw[i4]);
    if (!INV) w4.y = -w4.y;
    float2 wa = w4;
#pragma unroll
    for (int q = 1; q < R / 4; q++) {
        if (q > 1) wa = cmul(wa, w4);
        const float2 x1 = cmul(wa, w1), x2 = cmul(wa, w2), x3 = cmul(wa, w3);
        a[4 * q] = cmul(a[4 * q], wa);
        b[4 * q] = cmul(b[4 * q], wa);
        a[4 * q + 1] = cmul(a[4 * q + 1], x1);
        b[4 * q + 1] = cmul(b[4 * q + 1], x1);
        a[4 * q + 2] = cmul(a[4 * q + 2], x2);
        b[4 * q + 2] = cmul(b[4 * q + 2], x2);
        a[4 * q + 3] = cmul(a[4 * q + 3], x3);
        b[4 * q + 3] = cmul(b[4 * q + 3], x3);
    }
}

// GRDH2D's finalize (grd/grdh2d.f:202-226) applied while a column pass reads its input from
// the raw accumulation: out(u, v) = scale * (R(u+SUPP+1, v) + conj(R(UC-k, 2VC-v)) for the
// k = 0..SUPP columns next to the axis), 0 for u+1 > NU-SUPP; R is stored at raw index U
// (RAW_SHIFT) and already holds the folded compensation plane.  nullptr raw: no finalize.
struct FinParams {
    const float2 *raw;
    int raw_pitch, nu, nv, uorigin, vorigin, supp;
    float scale;
};
constexpr int FIN_MAXB = 8;  // grids per finalize-fused column launch (load + store maps)
struct FinBatch {
    FinParams f[FIN_MAXB];
};
__device__ __forceinline__ float2 fin_cell(const FinParams &f, float2 r, int u, int v) {
    const int u1 = u + 1, v1 = v + 1;
    if (u1 > f.nu - f.supp) return make_float2(0.f, 0.f);
    const int U = u1 + f.supp, UC = f.uorigin + f.supp, k = U - UC;
    if (k >= 0 && k <= f.supp) {
        const int dvv = v1 - f.vorigin, vm = 2 * f.vorigin - v1;
        if (dvv >= -(f.nv / 2) + 1 && dvv <= f.nv / 2 - 1 && vm >= 1 && vm <= f.nv) {
            const float2 m = f.raw[(int64_t)(vm - 1) * f.raw_pitch + (UC - k)];
            r.x = r.x + m.x;
            r.y = r.y - m.y;
        }
    }
    r.x *= f.scale;
    r.y *= f.scale;
    return r;
}

template <int LOGN, int LOGR, int LOGNS, bool INV, int T, bool FIRST, bool LAST, bool FIN = false>
__device__ __forceinline__ void st_pass2(float4 *s, const float2 *__restrict__ tw, int r0, int r1,
                                         const FinParams *fp = nullptr, int u0 = 0) {
    constexpr int N = 1 << LOGN, R = 1 << LOGR, NB = 1 << (LOGN - LOGR), NS = 1 << LOGNS;
    constexpr int PER = (NB + T - 1) / T;
    constexpr int TSHIFT = LOGN - LOGNS - LOGR;
    constexpr int C = N / 2 - 1;  // (N+1)/2 - 1 for even N
    float2 a[PER][R], b[PER][R];
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int j = threadIdx.x + i * T;
        if (NB % T == 0 || j < NB) {
#pragma unroll
            for (int r = 0; r < R; r++) {
                const int idx = j + r * NB;
                float4 x;
                if (FIRST) {
                    const int v = (idx + C) & (N - 1);
                    x = s[v];
                    if (!INV && (v < r0 || v >= r1)) x = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (FIN) {
                        const float2 c0 = fin_cell(*fp, make_float2(x.x, x.y), u0, v);
                        const float2 c1 = fin_cell(*fp, make_float2(x.z, x.w), u0 + 1, v);
                        x = make_float4(c0.x, c0.y, c1.x, c1.y);
                    }
                } else {
                    x = s[swz4(idx)];
                }
                a[i][r] = make_float2(x.x, x.y);
                b[i][r] = make_float2(x.z, x.w);
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int j = threadIdx.x + i * T;
        if (NB % T == 0 || j < NB) {
            const int jm = j & (NS - 1);
            if (LOGNS > 0 && jm)
                twiddle_powers2<R, INV>(a[i], b[i], tw, (size_t)(jm << TSHIFT), (size_t)((4 * jm) << TSHIFT));
            dftR<R, INV>(a[i]);
            dftR<R, INV>(b[i]);
            const int od = ((j >> LOGNS) << (LOGNS + LOGR)) + jm;
            const float sc = INV ? 1.0f / (float)N : 1.0f;
#pragma unroll
            for (int r = 0; r < R; r++) {
                const int p = od + r * NS;
                if (LAST) {
                    float4 y = make_float4(a[i][r].x, a[i][r].y, b[i][r].x, b[i][r].y);
                    if (INV) {
                        y.x *= sc; y.y *= sc; y.z *= sc; y.w *= sc;
                    }
                    s[(p + C) & (N - 1)] = y;
                } else {
                    s[swz4(p)] = make_float4(a[i][r].x, a[i][r].y, b[i][r].x, b[i][r].y);
                }
            }
        }
    }
    __syncthreads();
}

template <int LOGN, int LOGNS, bool INV, int T, bool FIN>
struct St2Passes {
    static __device__ __forceinline__ void run(float4 *s, const float2 *__restrict__ tw, int r0, int r1,
                                               const FinParams *fp, int u0) {
        constexpr int REM = LOGN - LOGNS;
        constexpr int LOGR = REM >= 4 ? 4 : REM;
        st_pass2<LOGN, LOGR, LOGNS, INV, T, LOGNS == 0, LOGNS + LOGR == LOGN, FIN && LOGNS == 0>(
            s, tw, r0, r1, fp, u0);
        St2Passes<LOGN, LOGNS + LOGR, INV, T, FIN>::run(s, tw, r0, r1, fp, u0);
    }
};
template <int LOGN, bool INV, int T, bool FIN>
struct St2Passes<LOGN, LOGN, INV, T, FIN> {
    static __device__ __forceinline__ void run(float4 *, const float2 *__restrict__, int, int,
                                               const FinParams *, int) {}
};

template <int LOGN>
struct ColTma {
    static constexpr int N = 1 << LOGN;
    static constexpr int T = N / 16 < 128 ? 128 : N / 16;  // one radix-16 butterfly per thread
    static constexpr int BOX = N < 256 ? N : 256;          // rows per TMA box
    static constexpr size_t SMEM = sizeof(float4) * (size_t)N + 16;
    static constexpr int MINB = 2 * SMEM <= 227 * 1024 ? 2 : 1;  // resident CTAs (shared memory)
};

// tensor maps of up to TMA_MAXB same-shape grids of one launch (blockIdx.y)
constexpr int TMA_MAXB = 16;
struct TmaBatch {
    CUtensorMap map[TMA_MAXB];
};

// FIN: the input is GRDH2D's raw accumulation (tensor map tb.map[blockIdx.y], boxes at raw
// index u + RAW_SHIFT) finalized on the way in (fp); the output goes to tb.map[blockIdx.y +
// store_off] (the final grid).
template <int LOGN, bool INV, bool FIN>
__global__ void __launch_bounds__(ColTma<LOGN>::T, ColTma<LOGN>::MINB)
    k_col_fft_tma(const __grid_constant__ TmaBatch tb, const float2 *__restrict__ tw, int r0,
                  int r1, int *status, int store_off, const __grid_constant__ FinBatch fb) {
    const FinParams &fp = fb.f[FIN ? blockIdx.y : 0];
    const CUtensorMap *tmap = &tb.map[blockIdx.y];
    const CUtensorMap *smap = &tb.map[blockIdx.y + store_off];
    const int xl = 4 * blockIdx.x + (FIN ? 2 * RAW_SHIFT : 0);  // load box: raw index u0+4
    using S = ColTma<LOGN>;
    constexpr int N = S::N, BOX = S::BOX;
    extern __shared__ __align__(128) unsigned char smem_ct[];
    float4 *s = reinterpret_cast<float4 *>(smem_ct);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_ct + sizeof(float4) * (size_t)N);
    const uint32_t sb = (uint32_t)__cvta_generic_to_shared(s);
    const uint32_t bb = (uint32_t)__cvta_generic_to_shared(bar);
    const int x = 4 * blockIdx.x;  // first float of this CTA's two complex columns
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bb));
        asm volatile("fence.mbarrier_init.release.cluster;");
        asm volatile("fence.proxy.async.shared::cta;");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bb),
                     "r"((uint32_t)(sizeof(float4) * N)));
        for (int b = 0; b < N / BOX; b++)
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                " [%0], [%1, {%2, %3}], [%4];" ::"r"(sb + (uint32_t)(b * BOX * sizeof(float4))),
                "l"(reinterpret_cast<uint64_t>(tmap)), "r"(xl), "r"(b * BOX), "r"(bb)
                : "memory");
    }
    {
        uint32_t done = 0;
        for (int spin = 0; spin < (1 << 24) && !done; spin++) {
            asm volatile(
                "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;"
                " selp.u32 %0, 1, 0, p; }"
                : "=r"(done)
                : "r"(bb)
                : "memory");
        }
        if (!done) {
            atomicExch(&status[STATUS_TIMEOUT], 1);
            return;
        }
    }
    St2Passes<LOGN, 0, INV, S::T, FIN>::run(s, tw, r0, r1, &fp, 2 * blockIdx.x);
    // the last pass's generic stores must be visible to the bulk copies that read them
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int b = 0; b < N / BOX; b++)
            asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                             reinterpret_cast<uint64_t>(smap)),
                         "r"(x), "r"(b * BOX), "r"(sb + (uint32_t)(b * BOX * sizeof(float4)))
                         : "memory");
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    }
}

template <int LOGN>
cudaError_t launch_col_tma(const TmaBatch &map, int nbatch, int nu, const float2 *tw, bool inverse,
                           int r0, int r1, int *status, cudaStream_t st, const FinBatch *fin = nullptr) {
    using S = ColTma<LOGN>;
    const dim3 nb((unsigned)((nu + 1) / 2), (unsigned)nbatch);
    cudaError_t e;
    if (fin) {
        e = cudaFuncSetAttribute(k_col_fft_tma<LOGN, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)S::SMEM);
        if (e != cudaSuccess) return e;
        k_col_fft_tma<LOGN, true, true><<<nb, S::T, S::SMEM, st>>>(map, tw, r0, r1, status, nbatch, *fin);
    } else if (inverse) {
        e = cudaFuncSetAttribute(k_col_fft_tma<LOGN, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)S::SMEM);
        if (e != cudaSuccess) return e;
        k_col_fft_tma<LOGN, true, false><<<nb, S::T, S::SMEM, st>>>(map, tw, r0, r1, status, 0, FinBatch{});
    } else {
        e = cudaFuncSetAttribute(k_col_fft_tma<LOGN, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)S::SMEM);
        if (e != cudaSuccess) return e;
        k_col_fft_tma<LOGN, false, false><<<nb, S::T, S::SMEM, st>>>(map, tw, r0, r1, status, 0, FinBatch{});
    }
    return cudaGetLastError();
}

// Column pass of n same-shape grids through the TMA kernel when 2^logn has an instance
// (2048..8192), TMA_MAXB grids per launch.
bool col_fft_tma(sde_ctx *ctx, int logn, float2 *const *grids, int n, int pitch, int nu, int nv,
                 const float2 *tw, bool inverse, int r0, int r1, cudaError_t *err, int *rc) {
    if (logn < 11 || logn > 13) return false;
    *rc = SDE_OK;
    *err = cudaSuccess;
    for (int b0 = 0; b0 < n && *rc == SDE_OK && *err == cudaSuccess; b0 += TMA_MAXB) {
        const int nb = n - b0 < TMA_MAXB ? n - b0 : TMA_MAXB;
        TmaBatch tb;
        for (int i = 0; i < nb && *rc == SDE_OK; i++)
            *rc = encode_tmap_f32_2d(&tb.map[i], grids[b0 + i], (uint64_t)nu * 2, (uint64_t)nv,
                                     (uint64_t)pitch * 8, 4, (uint32_t)(nv < 256 ? nv : 256));
        if (*rc != SDE_OK) break;
        switch (logn) {
            case 11: *err = launch_col_tma<11>(tb, nb, nu, tw, inverse, r0, r1, ctx->d_status, ctx->stream); break;
            case 12: *err = launch_col_tma<12>(tb, nb, nu, tw, inverse, r0, r1, ctx->d_status, ctx->stream); break;
            default: *err = launch_col_tma<13>(tb, nb, nu, tw, inverse, r0, r1, ctx->d_status, ctx->stream); break;
        }
    }
    return true;
}

// ---- c2r row pass on row pairs fed by bulk copies ---------------------------------------
// A CTA takes two grid rows (two image rows).  They come into shared memory with 1-D bulk
// copies (cp.async.bulk, mbarrier with a bounded wait); the first FFT pass reads that staging
// copy directly through FFTR's Hermitian pre-step, and its outputs overwrite it as (row0,
// row1) complex pairs, one float4 per element, so every thread runs its butterfly for both
// rows with one set of twiddles and one correction-table load.  The staging rows and the
// pair array are the same 16*H bytes.  (The same form for the r2c pass measured slower than
// the one-row-per-butterfly kernel: 0.103 vs 0.099 ms at 4096^2.)
struct SwzRead4 {
    const float4 *s;
    __device__ __forceinline__ float4 operator()(int i) const { return s[swz4(i)]; }
};
struct SwzWrite4 {
    float4 *s;
    __device__ __forceinline__ void operator()(int i, float4 y) const { s[swz4(i)] = y; }
};

template <int LOGN, int LOGR, int LOGNS, bool INV, int T, int TWS, class Rd, class Wr>
__device__ __forceinline__ void st_pass_fn(const float2 *__restrict__ tw, const Rd &rd, const Wr &wr) {
    constexpr int R = 1 << LOGR, NB = 1 << (LOGN - LOGR), NS = 1 << LOGNS;
    constexpr int PER = (NB + T - 1) / T;
    constexpr int TSHIFT = LOGN - LOGNS - LOGR;
    float2 a[PER][R], b[PER][R];
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int j = threadIdx.x + i * T;
        if (NB % T == 0 || j < NB) {
#pragma unroll
            for (int r = 0; r < R; r++) {
                const float4 x = rd(j + r * NB);
                a[i][r] = make_float2(x.x, x.y);
                b[i][r] = make_float2(x.z, x.w);
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int j = threadIdx.x + i * T;
        if (NB % T == 0 || j < NB) {
            const int jm = j & (NS - 1);
            if (LOGNS > 0 && jm)
                twiddle_powers2<R, INV>(a[i], b[i], tw, (size_t)(jm << TSHIFT) * TWS,
                                        (size_t)((4 * jm) << TSHIFT) * TWS);
            dftR<R, INV>(a[i]);
            dftR<R, INV>(b[i]);
            const int od = ((j >> LOGNS) << (LOGNS + LOGR)) + jm;
#pragma unroll
            for (int r = 0; r < R; r++)
                wr(od + r * NS, make_float4(a[i][r].x, a[i][r].y, b[i][r].x, b[i][r].y));
        }
    }
    __syncthreads();
}

// passes LOGNS.. of a length-2^LOGN transform over pairs in s (swizzled in and out)
template <int LOGN, int LOGNS, bool INV, int T, int TWS>
struct PairPasses {
    static __device__ __forceinline__ void run(float4 *s, const float2 *__restrict__ tw) {
        constexpr int REM = LOGN - LOGNS;
        constexpr int LOGR = REM >= 4 ? 4 : REM;
        st_pass_fn<LOGN, LOGR, LOGNS, INV, T, TWS>(tw, SwzRead4{s}, SwzWrite4{s});
        PairPasses<LOGN, LOGNS + LOGR, INV, T, TWS>::run(s, tw);
    }
};
template <int LOGN, bool INV, int T, int TWS>
struct PairPasses<LOGN, LOGN, INV, T, TWS> {
    static __device__ __forceinline__ void run(float4 *, const float2 *__restrict__) {}
};

template <int LOGH>
struct RowPair {
    static constexpr int H = 1 << LOGH;
    static constexpr int T = H / 16;
    static constexpr size_t SMEM = sizeof(float4) * (size_t)H + 16;
    static constexpr int MINB = T <= 128 ? 4 : 2;
};

// c2r first-pass input: FFTR's pre-step of element k for both staged grid rows
template <int H>
struct C2rRead {
    const float2 *stg;  // row 0 at [0, H), row 1 at [H, 2H)
    float2 xh0, xh1;    // X[H] of each row
    const float2 *__restrict__ tw;
    __device__ __forceinline__ float4 operator()(int k) const {
        const float2 w = __ldg(&tw[k]);
        float2 o[2];
#pragma unroll
        for (int rr = 0; rr < 2; rr++) {
            float2 a = stg[rr * H + k];
            float2 bb = k == 0 ? (rr ? xh1 : xh0) : stg[rr * H + H - k];
            if (k == 0) {
                a.y = 0.f;
                bb.y = 0.f;
            }
            const float2 A = make_float2(0.5f * (a.x + bb.x), 0.5f * (a.y - bb.y));
            const float2 d = make_float2(0.5f * (a.x - bb.x), 0.5f * (a.y + bb.y));
            const float2 B = cmul(d, w);
            o[rr] = make_float2(A.x - B.y, A.y + B.x);
        }
        return make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
    }
};

template <int LOGH>
__global__ void __launch_bounds__(RowPair<LOGH>::T, RowPair<LOGH>::MINB)
    k_row_c2r_pair(const __grid_constant__ FftBatch bt, int pitch, int nx, int ny, int ibegy,
                   const float2 *__restrict__ tw, CorrParams cp, int *status) {
    using S = RowPair<LOGH>;
    constexpr int H = S::H, T = S::T, FNU = 2 * H;
    const float2 *__restrict__ grid = bt.grid[blockIdx.y];
    const float *__restrict__ scale_dev = bt.scale[blockIdx.y];
    float *image = bt.image[blockIdx.y];
    extern __shared__ __align__(128) unsigned char smem_rp[];
    float4 *s = reinterpret_cast<float4 *>(smem_rp);
    const float2 *stg = reinterpret_cast<const float2 *>(smem_rp);
    const uint32_t sb = (uint32_t)__cvta_generic_to_shared(smem_rp);
    const uint32_t bb = (uint32_t)__cvta_generic_to_shared(smem_rp + sizeof(float4) * H);
    const int iy0 = 2 * blockIdx.x;
    const bool two = iy0 + 1 < ny;
    const float2 *X0 = grid + (int64_t)(iy0 + ibegy) * pitch;
    const float2 *X1 = two ? X0 + pitch : X0;
    bar_init_one(bb);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bb),
                     "r"((uint32_t)(2 * H * sizeof(float2))));
        bulk_g2s(sb, X0, H * sizeof(float2), bb);
        bulk_g2s(sb + H * sizeof(float2), X1, H * sizeof(float2), bb);
    }
    const float2 xh0 = X0[H], xh1 = X1[H];
    if (!bar_wait_bounded(bb)) {
        atomicExch(&status[STATUS_TIMEOUT], 1);
        return;
    }
    constexpr int LOGR0 = LOGH >= 4 ? 4 : LOGH;
    st_pass_fn<LOGH, LOGR0, 0, true, T, 2>(tw, C2rRead<H>{stg, xh0, xh1, tw}, SwzWrite4{s});
    PairPasses<LOGH, LOGR0, true, T, 2>::run(s, tw);
    const float inv = 1.0f / (float)H;
    const int cu = (FNU + 1) / 2 - 1, ioff = (FNU - nx) / 2;
    const float sc = scale_dev ? 1.0f / *scale_dev : 1.0f;
    const float cy0 = cp.ccf ? cp.corry[iy0] : 1.0f, cy1 = cp.ccf && two ? cp.corry[iy0 + 1] : 1.0f;
    float *im0 = image + (int64_t)iy0 * nx;
    for (int ix = threadIdx.x; ix < nx; ix += T) {
        int n = ix + ioff - cu;
        if (n < 0) n += FNU;
        const float4 z = s[swz4(n >> 1)];
        float v0 = ((n & 1) ? z.y : z.x) * inv, v1 = ((n & 1) ? z.w : z.z) * inv;
        if (cp.ccf) {
            const float cx = cp.corrx[ix];
            v0 = __fdiv_rn(v0, __fmul_rn(cx, cy0));
            v1 = __fdiv_rn(v1, __fmul_rn(cx, cy1));
        }
        if (scale_dev) {
            v0 = __fadd_rn(__fmul_rn(sc, v0), 0.0f);
            v1 = __fadd_rn(__fmul_rn(sc, v1), 0.0f);
        }
        im0[ix] = v0;
        if (two) im0[nx + ix] = v1;
    }
}

template <int LOGH>
cudaError_t launch_c2r_pair(const FftBatch &bt, int nbatch, int pitch, int nx, int ny, int ibegy,
                            const float2 *tw, CorrParams cp, int *status, cudaStream_t st) {
    using S = RowPair<LOGH>;
    cudaError_t e = cudaFuncSetAttribute(k_row_c2r_pair<LOGH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)S::SMEM);
    if (e != cudaSuccess) return e;
    k_row_c2r_pair<LOGH><<<dim3((unsigned)((ny + 1) / 2), (unsigned)nbatch), S::T, S::SMEM, st>>>(
        bt, pitch, nx, ny, ibegy, tw, cp, status);
    return cudaGetLastError();
}
// Whether the row-pair c2r kernel applies: half-lengths 1024..4096, grid rows that start
// on 16-byte boundaries (pitch even, 16-byte aligned grids), image rows of whole float4s.
static bool row_pair_ok(int logh, const FftBatch &bt, int nbatch, int pitch, int nx) {
    if (logh < 10 || logh > 12) return false;
    if ((pitch & 1) || (nx & 3)) return false;
    for (int b = 0; b < nbatch; b++)
        if (((uintptr_t)bt.grid[b] & 15u) || ((uintptr_t)bt.image[b] & 15u)) return false;
    return true;
}

// Launchers for the compile-time shapes: false if the size has no instance.
template <int LOGN>
cudaError_t launch_col_t(const FftBatch &bt, int nbatch, int pitch, int nu, const float2 *tw,
                         bool inverse, int r0, int r1, cudaStream_t st) {
    using S = ColShape<LOGN>;
    const dim3 nb((unsigned)((nu + S::CC - 1) / S::CC), (unsigned)nbatch);
    if (inverse) {
        cudaError_t e = cudaFuncSetAttribute(k_col_fft_t<LOGN, true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
        if (e != cudaSuccess) return e;
        k_col_fft_t<LOGN, true><<<nb, S::T, S::SMEM, st>>>(bt, pitch, nu, tw, r0, r1);
    } else {
        cudaError_t e = cudaFuncSetAttribute(k_col_fft_t<LOGN, false>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
        if (e != cudaSuccess) return e;
        k_col_fft_t<LOGN, false><<<nb, S::T, S::SMEM, st>>>(bt, pitch, nu, tw, r0, r1);
    }
    return cudaGetLastError();
}

template <int LOGH>
cudaError_t launch_c2r_t(const FftBatch &bt, int nbatch, int pitch, int nx, int ny, int ibegy,
                         const float2 *tw, CorrParams cp, cudaStream_t st) {
    using S = RowShape<LOGH>;
    cudaError_t e = cudaFuncSetAttribute(k_row_c2r_t<LOGH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)S::SMEM);
    if (e != cudaSuccess) return e;
    k_row_c2r_t<LOGH><<<dim3((unsigned)((ny + S::ROWS - 1) / S::ROWS), (unsigned)nbatch), S::T, S::SMEM,
                        st>>>(bt, pitch, nx, ny, ibegy, tw, cp);
    return cudaGetLastError();
}

template <int LOGH>
cudaError_t launch_r2c_t(const FftBatch &bt, int nbatch, int nx, int ny, int ibegy, const float2 *tw,
                         CorrParams cp, int pitch, int *status, cudaStream_t st) {
    using S = RowShape<LOGH>;
    cudaError_t e = cudaFuncSetAttribute(k_row_r2c_t<LOGH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)S::SMEM);
    if (e != cudaSuccess) return e;
    k_row_r2c_t<LOGH><<<dim3((unsigned)((ny + S::ROWS - 1) / S::ROWS), (unsigned)nbatch), S::T, S::SMEM,
                        st>>>(bt, nx, ny, ibegy, tw, cp, pitch, status);
    return cudaGetLastError();
}

#define SDE_LOG_CASES(X) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13)

// Column pass through the compile-time kernels when 2^logn has an instance.
bool col_fft_t(int logn, const FftBatch &bt, int nbatch, int pitch, int nu, const float2 *tw,
               bool inverse, int r0, int r1, cudaStream_t st, cudaError_t *err) {
    switch (logn) {
#define CASE(L) \
    case L: *err = launch_col_t<L>(bt, nbatch, pitch, nu, tw, inverse, r0, r1, st); return true;
        SDE_LOG_CASES(CASE)
#undef CASE
        default: return false;
    }
}
bool c2r_t(int logh, const FftBatch &bt, int nbatch, int pitch, int nx, int ny, int ibegy,
           const float2 *tw, CorrParams cp, cudaStream_t st, cudaError_t *err, int *status) {
    if (status && row_pair_ok(logh, bt, nbatch, pitch, nx)) {
        *err = logh == 10   ? launch_c2r_pair<10>(bt, nbatch, pitch, nx, ny, ibegy, tw, cp, status, st)
               : logh == 11 ? launch_c2r_pair<11>(bt, nbatch, pitch, nx, ny, ibegy, tw, cp, status, st)
                            : launch_c2r_pair<12>(bt, nbatch, pitch, nx, ny, ibegy, tw, cp, status, st);
        return true;
    }
    switch (logh) {
#define CASE(L) \
    case L: *err = launch_c2r_t<L>(bt, nbatch, pitch, nx, ny, ibegy, tw, cp, st); return true;
        SDE_LOG_CASES(CASE)
#undef CASE
        default: return false;
    }
}
bool r2c_t(int logh, const FftBatch &bt, int nbatch, int nx, int ny, int ibegy, const float2 *tw,
           CorrParams cp, int pitch, cudaStream_t st, cudaError_t *err, int *status) {
    // image rows staged by bulk copy when they start on 16-byte boundaries
    bool staged = status && (nx & 3) == 0;
    for (int b = 0; b < nbatch && staged; b++) staged = ((uintptr_t)bt.image[b] & 15u) == 0;
    int *st_status = staged ? status : nullptr;
    switch (logh) {
#define CASE(L) \
    case L: *err = launch_r2c_t<L>(bt, nbatch, nx, ny, ibegy, tw, cp, pitch, st_status, st); return true;
        SDE_LOG_CASES(CASE)
#undef CASE
        default: return false;
    }
}
#undef SDE_LOG_CASES

}  // namespace

int fft_images_from_grids(sde_ctx *ctx, int n, float2 *const *grids, float *const *images,
                          const float *const *scales, int pitch, int nx, int ny, int fnu, int nv,
                          int correct) {
    if (!ctx || n < 0) return SDE_EINVAL;
    if (n == 0) return SDE_OK;
    SDE_TRY(check_fft_args(nx, ny, fnu, nv, pitch));
    const int logn = ilog2(nv), logh = ilog2(fnu / 2);
    if (logn < 5 || logn > 13 || logh < 5 || logh > 13) {
        sde_set_error("batched FFT: no compiled shape for fnu=%d nv=%d", fnu, nv);
        return SDE_EINVAL;
    }
    const int nu = fnu / 2 + 1;
    const float2 *twv, *twu;
    SDE_TRY(ctx_twiddles(ctx, nv, &twv));
    SDE_TRY(ctx_twiddles(ctx, fnu, &twu));
    CorrParams cp = {nullptr, nullptr, nullptr};
    if (correct) SDE_TRY(corr_params(ctx, nx, ny, &cp));
    const int ibegy = (nv + 1) / 2 - (ny + 1) / 2;
    for (int b0 = 0; b0 < n; b0 += FFT_MAXB) {
        const int nb = n - b0 < FFT_MAXB ? n - b0 : FFT_MAXB;
        FftBatch bt{};
        for (int i = 0; i < nb; i++) {
            bt.grid[i] = grids[b0 + i];
            bt.image[i] = images[b0 + i];
            bt.scale[i] = scales ? scales[b0 + i] : nullptr;
        }
        cudaError_t e = cudaSuccess;
        {
            KTimer kt(ctx, "col_fft_batch");
            int trc = SDE_OK;
            if (col_fft_tma(ctx, logn, bt.grid, nb, pitch, nu, nv, twv, true, 0, nv, &e, &trc))
                SDE_TRY(trc);
            else
                col_fft_t(logn, bt, nb, pitch, nu, twv, true, 0, nv, ctx->stream, &e);
        }
        SDE_CUDA_TRY(e);
        {
            KTimer kt(ctx, "row_c2r_batch");
            c2r_t(logh, bt, nb, pitch, nx, ny, ibegy, twu, cp, ctx->stream, &e, ctx->d_status);
        }
        SDE_CUDA_TRY(e);
    }
    return SDE_OK;
}

bool fin_fused_shape(int nu, int nv) {
    const int logn = ilog2(nv);
    return logn >= 11 && logn <= 13 && (1 << logn) == nv && nu >= 2;
}

// Images of n same-shape gridding passes straight from their raw accumulations (compensation
// planes already folded: every fd[i].raw_lo is NULL): finalize-fused TMA column passes,
// FIN_MAXB grids per launch (fd[i].out receives the finalized, column-transformed grid), then
// the batched row c2r pass.  Shapes without a fused column pass: EINVAL.
int fft_images_from_raw(sde_ctx *ctx, int n, const FinalizeDesc *fd, float *const *images,
                        const float *const *scales, int nx, int ny, int correct) {
    if (!ctx || n < 0) return SDE_EINVAL;
    if (n == 0) return SDE_OK;
    const int nu = fd[0].nu, nv = fd[0].nv, pitch = fd[0].pitch, fnu = 2 * (nu - 1);
    for (int i = 0; i < n; i++)
        if (fd[i].raw_lo || fd[i].nu != nu || fd[i].nv != nv || fd[i].pitch != pitch) return SDE_EINVAL;
    SDE_TRY(check_fft_args(nx, ny, fnu, nv, pitch));
    if (!fin_fused_shape(nu, nv)) return SDE_EINVAL;
    const int logn = ilog2(nv), logh = ilog2(fnu / 2);
    const float2 *twv, *twu;
    SDE_TRY(ctx_twiddles(ctx, nv, &twv));
    SDE_TRY(ctx_twiddles(ctx, fnu, &twu));
    CorrParams cp = {nullptr, nullptr, nullptr};
    if (correct) SDE_TRY(corr_params(ctx, nx, ny, &cp));
    const int ibegy = (nv + 1) / 2 - (ny + 1) / 2;
    {
        KTimer kt(ctx, "col_fft_fin_batch");
        for (int b0 = 0; b0 < n; b0 += FIN_MAXB) {
            const int nb = n - b0 < FIN_MAXB ? n - b0 : FIN_MAXB;
            TmaBatch tb;
            FinBatch fb{};
            for (int i = 0; i < nb; i++) {
                const FinalizeDesc &f = fd[b0 + i];
                SDE_TRY(encode_tmap_f32_2d(&tb.map[i], f.raw, (uint64_t)pitch * 2, (uint64_t)nv,
                                           (uint64_t)pitch * 8, 4, 256));
                SDE_TRY(encode_tmap_f32_2d(&tb.map[nb + i], f.out, (uint64_t)nu * 2, (uint64_t)nv,
                                           (uint64_t)pitch * 8, 4, 256));
                fb.f[i] = FinParams{f.raw, pitch, nu, nv, f.uorigin, f.vorigin, f.supp, f.scale};
            }
            cudaError_t e;
            switch (logn) {
                case 11: e = launch_col_tma<11>(tb, nb, nu, twv, true, 0, nv, ctx->d_status, ctx->stream, &fb); break;
                case 12: e = launch_col_tma<12>(tb, nb, nu, twv, true, 0, nv, ctx->d_status, ctx->stream, &fb); break;
                default: e = launch_col_tma<13>(tb, nb, nu, twv, true, 0, nv, ctx->d_status, ctx->stream, &fb); break;
            }
            SDE_CUDA_TRY(e);
        }
    }
    for (int b0 = 0; b0 < n; b0 += FFT_MAXB) {
        const int nb = n - b0 < FFT_MAXB ? n - b0 : FFT_MAXB;
        FftBatch bt{};
        for (int i = 0; i < nb; i++) {
            bt.grid[i] = fd[b0 + i].out;
            bt.image[i] = images[b0 + i];
            bt.scale[i] = scales ? scales[b0 + i] : nullptr;
        }
        cudaError_t e = cudaSuccess;
        KTimer kt(ctx, "row_c2r_batch");
        c2r_t(logh, bt, nb, pitch, nx, ny, ibegy, twu, cp, ctx->stream, &e, ctx->d_status);
        SDE_CUDA_TRY(e);
    }
    return SDE_OK;
}

int check_fft_shape(int nx, int ny, int fnu, int nv) {
    return check_fft_args(nx, ny, fnu, nv, fnu / 2 + 1);
}

// The row c2r pass of a column-transformed grid into the image (FFTR2D's second half, with
// PIXCOR2D's correction and the PSF-peak scale when asked).
static int c2r_pass(sde_ctx *ctx, const float *grid, int pitch, int nx, int ny, int fnu, int nv,
                    int correct, const float *scale_dev, float *image, const float2 *twu) {
    CorrParams cp = {nullptr, nullptr, nullptr};
    if (correct) SDE_TRY(corr_params(ctx, nx, ny, &cp));
    const int ibegy = (nv + 1) / 2 - (ny + 1) / 2;  // 0-based first grid row
    KTimer kt(ctx, "row_c2r");
    cudaError_t e = cudaSuccess;
    FftBatch bt{};
    bt.grid[0] = (float2 *)grid;
    bt.image[0] = image;
    bt.scale[0] = scale_dev;
    if (!c2r_t(ilog2(fnu / 2), bt, 1, pitch, nx, ny, ibegy, twu, cp, ctx->stream, &e, ctx->d_status)) {
        int rows, thr;
        row_shape(fnu, &rows, &thr);
        const size_t smr = sizeof(float2) * (size_t)(fnu / 2) * rows;
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_row_c2r, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr));
        k_row_c2r<<<ceil_div(ny, rows), thr, smr, ctx->stream>>>((const float2 *)grid, pitch, fnu, rows,
                                                                nx, ny, ibegy, twu, cp, scale_dev, image);
        e = cudaGetLastError();
    }
    SDE_CUDA_TRY(e);
    return SDE_OK;
}

int sde_image_from_grid(sde_ctx *ctx, float *grid, int pitch, int nx, int ny, int fnu, int nv,
                        int correct, const float *scale_dev, float *image) {
    if (!ctx || !grid || !image) return SDE_EINVAL;
    SDE_TRY(check_fft_args(nx, ny, fnu, nv, pitch));
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    const int nu = fnu / 2 + 1;
    const float2 *twv, *twu;
    SDE_TRY(ctx_twiddles(ctx, nv, &twv));
    SDE_TRY(ctx_twiddles(ctx, fnu, &twu));
    {
        KTimer kt(ctx, "col_fft");
        cudaError_t e = cudaSuccess;
        FftBatch bt{};
        bt.grid[0] = (float2 *)grid;
        int trc = SDE_OK;
        float2 *g1 = (float2 *)grid;
        if (col_fft_tma(ctx, ilog2(nv), &g1, 1, pitch, nu, nv, twv, true, 0, nv, &e, &trc)) {
            SDE_TRY(trc);
        } else if (!col_fft_t(ilog2(nv), bt, 1, pitch, nu, twv, true, 0, nv, ctx->stream, &e)) {
            const int lcc = col_logcc(nv), cc = 1 << lcc;
            const size_t smc = sizeof(float2) * (size_t)cc * nv;
            SDE_CUDA_TRY(cudaFuncSetAttribute(k_col_fft, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc));
            k_col_fft<<<ceil_div(nu, cc), COL_THREADS, smc, ctx->stream>>>((float2 *)grid, pitch, nu, nv,
                                                                           ilog2(nv), lcc, twv, 1, 0, nv);
            e = cudaGetLastError();
        }
        SDE_CUDA_TRY(e);
    }
    return c2r_pass(ctx, grid, pitch, nx, ny, fnu, nv, correct, scale_dev, image, twu);
}

// The dirty image (or PSF) of a plan pass straight from the raw accumulation: where the
// column pass is TMA-fed (2048..8192 rows) it applies GRDH2D's finalize to its input and
// writes the column-transformed grid to grid; otherwise finalize into grid, then the column
// pass.  Then the row c2r pass.
int image_from_raw(sde_ctx *ctx, const float2 *raw, const float2 *raw_lo, int nu, int nv,
                   int uorigin, int vorigin, int supp, float scale, float *grid, int pitch, int nx,
                   int ny, int fnu, int correct, const float *scale_dev, float *image) {
    SDE_TRY(check_fft_args(nx, ny, fnu, nv, pitch));
    const int logn = ilog2(nv);
    if (raw_lo || logn < 11 || logn > 13 || nu != fnu / 2 + 1) {
        SDE_TRY(grid_finalize_scale(ctx, raw, raw_lo, (float2 *)grid, nu, nv, pitch, uorigin, vorigin,
                                    supp, scale));
        return sde_image_from_grid(ctx, grid, pitch, nx, ny, fnu, nv, correct, scale_dev, image);
    }
    const float2 *twv, *twu;
    SDE_TRY(ctx_twiddles(ctx, nv, &twv));
    SDE_TRY(ctx_twiddles(ctx, fnu, &twu));
    {
        KTimer kt(ctx, "col_fft_fin");
        TmaBatch tb;
        SDE_TRY(encode_tmap_f32_2d(&tb.map[0], raw, (uint64_t)pitch * 2, (uint64_t)nv, (uint64_t)pitch * 8, 4,
                                   256));
        SDE_TRY(encode_tmap_f32_2d(&tb.map[1], grid, (uint64_t)nu * 2, (uint64_t)nv, (uint64_t)pitch * 8, 4,
                                   256));
        FinBatch fb{};
        fb.f[0] = FinParams{raw, pitch, nu, nv, uorigin, vorigin, supp, scale};
        cudaError_t e;
        switch (logn) {
            case 11: e = launch_col_tma<11>(tb, 1, nu, twv, true, 0, nv, ctx->d_status, ctx->stream, &fb); break;
            case 12: e = launch_col_tma<12>(tb, 1, nu, twv, true, 0, nv, ctx->d_status, ctx->stream, &fb); break;
            default: e = launch_col_tma<13>(tb, 1, nu, twv, true, 0, nv, ctx->d_status, ctx->stream, &fb); break;
        }
        SDE_CUDA_TRY(e);
    }
    return c2r_pass(ctx, grid, pitch, nx, ny, fnu, nv, correct, scale_dev, image, twu);
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
    CorrParams cp = {nullptr, nullptr, nullptr};
    if (correct) SDE_TRY(corr_params(ctx, nx, ny, &cp));
    const int ibegy = (nv + 1) / 2 - (ny + 1) / 2;
    {
        KTimer kt(ctx, "row_r2c");
        cudaError_t e = cudaSuccess;
        FftBatch bt{};
        bt.grid[0] = (float2 *)grid;
        bt.image[0] = const_cast<float *>(image);
        if (!r2c_t(ilog2(fnu / 2), bt, 1, nx, ny, ibegy, twu, cp, pitch, ctx->stream, &e, ctx->d_status)) {
            int rows, thr;
            row_shape(fnu, &rows, &thr);
            const size_t smr = sizeof(float2) * (size_t)(fnu / 2) * rows;
            SDE_CUDA_TRY(cudaFuncSetAttribute(k_row_r2c, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr));
            k_row_r2c<<<ceil_div(ny, rows), thr, smr, ctx->stream>>>(image, nx, ny, fnu, rows, ibegy, twu,
                                                                    cp, (float2 *)grid, pitch, nu);
            e = cudaGetLastError();
        }
        SDE_CUDA_TRY(e);
    }
    KTimer kt(ctx, "col_fft");
    cudaError_t e = cudaSuccess;
    FftBatch bt{};
    bt.grid[0] = (float2 *)grid;
    int trc = SDE_OK;
    float2 *g1 = (float2 *)grid;
    if (col_fft_tma(ctx, ilog2(nv), &g1, 1, pitch, nu, nv, twv, false, ibegy, ibegy + ny, &e, &trc)) {
        SDE_TRY(trc);
    } else if (!col_fft_t(ilog2(nv), bt, 1, pitch, nu, twv, false, ibegy, ibegy + ny, ctx->stream, &e)) {
        const int lcc = col_logcc(nv), cc = 1 << lcc;
        const size_t smc = sizeof(float2) * (size_t)cc * nv;
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_col_fft, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc));
        k_col_fft<<<ceil_div(nu, cc), COL_THREADS, smc, ctx->stream>>>((float2 *)grid, pitch, nu, nv,
                                                                       ilog2(nv), lcc, twv, 0, ibegy,
                                                                       ibegy + ny);
        e = cudaGetLastError();
    }
    SDE_CUDA_TRY(e);
    return SDE_OK;
}
