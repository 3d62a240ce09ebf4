// clean.cu -- Hogbom CLEAN minor cycle (PIX2DRCL), PIXISAMA, and the uvmap PSF-peak
// normalisation (ARRSTAT max + ARRSCALE by 1/max).
//
// PIX2DRCL (pix/pix2drcl.f:67-130): RES = DRT*BOX; per iteration the first index of the
// strictly largest |RES| (PIXISAMA, pix/pixisama.f:45-53), stop tests, component record,
// then RES -= (PNTSUB*PSF(OFFX-IX,OFFY-IY))*BOX over the whole window in FP32.  Here one
// cooperative persistent launch runs every iteration: each CTA owns a contiguous slice of
// the window, applies the previous component's subtraction to it with the same FP32
// operations (no FMA), finds its slice's first maximum, and that maximum joins a global one
// (a packed key, one atomicMax per CTA) inside a grid barrier (bounded spin); every CTA then
// reads the same global (max, first index), so component positions are identical to the
// reference's.
#include <cooperative_groups.h>
#include <math.h>
#include <string.h>

#include <mutex>

#include "common.cuh"

namespace {

constexpr int CL_THREADS = 512;
constexpr size_t CL_SMEM_SLICE_MAX = 100 * 1024;  // largest RES slice kept in shared memory
constexpr int CL_BATCH = 4;                        // pixels per thread with PSF loads in flight
constexpr unsigned SPIN_LIMIT = 1u << 26;

struct Cand {
    float a;      // |value|
    int32_t idx;  // flat 0-based index, INT32_MAX if none
    float v;      // signed value
};

__device__ __forceinline__ Cand better(Cand x, Cand y) {
    // larger |a| wins; ties go to the smaller index (first occurrence)
    if (y.a > x.a || (y.a == x.a && y.idx < x.idx)) return y;
    return x;
}

__device__ Cand block_best(Cand c) {
    __shared__ Cand sh[32];
    for (int d = 16; d > 0; d >>= 1) {
        Cand o;
        o.a = __shfl_down_sync(0xffffffffu, c.a, d);
        o.idx = __shfl_down_sync(0xffffffffu, c.idx, d);
        o.v = __shfl_down_sync(0xffffffffu, c.v, d);
        c = better(c, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = c;
    __syncthreads();
    if (warp == 0) {
        c = lane < (int)(blockDim.x >> 5) ? sh[lane] : Cand{-1.0f, INT32_MAX, 0.0f};
        for (int d = 16; d > 0; d >>= 1) {
            Cand o;
            o.a = __shfl_down_sync(0xffffffffu, c.a, d);
            o.idx = __shfl_down_sync(0xffffffffu, c.idx, d);
            o.v = __shfl_down_sync(0xffffffffu, c.v, d);
            c = better(c, o);
        }
        if (lane == 0) sh[0] = c;
    }
    __syncthreads();
    Cand r = sh[0];
    __syncthreads();
    return r;
}

struct Barrier {
    unsigned count;  // arrivals since the launch (grid_sync)
    int stopreq[2];  // cancel requests published by CTA 0 before each barrier
    unsigned long long best[3];  // each iteration's maximum, as a packed key (cand_key)
};

// A candidate as a 64-bit key whose unsigned order is better()'s: |value| bits (|value| >= 0
// and not NaN here, so the bits order as the values do), then INT32_MAX - index (the first
// index wins a tie), then the value's sign bit.  One atomicMax per CTA finds the maximum.
__device__ __forceinline__ unsigned long long cand_key(Cand c) {
    return ((unsigned long long)__float_as_uint(c.a) << 32) |
           ((unsigned long long)(uint32_t)(INT32_MAX - c.idx) << 1) | (__float_as_uint(c.v) >> 31);
}
// the largest key of a warp's lanes: the largest high word, then the largest low word among
// the lanes that hold it
__device__ __forceinline__ unsigned long long warp_key_max(unsigned long long k) {
    const unsigned hi = (unsigned)(k >> 32), lo = (unsigned)k;
    const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
    const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? lo : 0u);
    return ((unsigned long long)mhi << 32) | mlo;
}
__device__ __forceinline__ Cand key_cand(unsigned long long k) {
    Cand c;
    c.a = __uint_as_float((uint32_t)(k >> 32));
    c.idx = INT32_MAX - (int32_t)((uint32_t)k >> 1);
    c.v = (k & 1ull) ? -c.a : c.a;
    return c;
}

// Grid-wide barrier on a monotonic arrival count: barrier number `epoch` (0, 1, ...) is passed
// when the count reaches (epoch + 1) * nblocks, so the last CTA's arrival releases the others
// (no reset, no second word) and that CTA does not wait.  Gives up after SPIN_LIMIT polls and
// reports through *timeout.  The count is cleared before each launch.
__device__ bool grid_sync(Barrier *b, unsigned nblocks, unsigned epoch, int *timeout,
                          unsigned long long *pub = nullptr, const unsigned long long *key = nullptr) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        const unsigned target = (epoch + 1u) * nblocks;
        // the CTA's maximum (a key, 0 for none) joins the global one before the CTA arrives
        if (pub && *key) atomicMax(pub, *key);
        __threadfence();
        const unsigned arrived = atomicAdd(&b->count, 1u) + 1u;
        if ((int)(arrived - target) < 0) {
            volatile unsigned *vc = &b->count;
            unsigned spins = 0;
            while ((int)(*vc - target) < 0) {
                if (++spins > SPIN_LIMIT) {
                    atomicExch(timeout, 1);
                    ok = 0;
                    break;
                }
                if (*(volatile int *)timeout) {
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

struct CleanArgs {
    const float *drt, *psf, *box;
    float *cln, *res, *cflux;
    int *cx, *cy;
    int nx, ny, pnx, pny, pmpx, pmpy;
    float gain, flux, tflux_in;
    int nsub, bsub;
    volatile int *cancel;
    Barrier *bar;
    int *status;     // [STATUS_TIMEOUT]
    float *out;      // [0] maxres [1] tflux [2] ansub (as int bits)
};

// SMEM: the CTA's slice of RES lives in shared memory for all iterations (dynamic shared
// memory of one slice) and goes to A.res once at the end; otherwise RES is read and written
// in global memory every iteration.  The arithmetic is the same either way.
template <bool SMEM>
__global__ void __launch_bounds__(CL_THREADS) k_hogbom(CleanArgs A) {
    extern __shared__ float sres[];
    const int64_t npix = (int64_t)A.nx * A.ny;
    const int64_t per = (npix + gridDim.x - 1) / gridDim.x;
    const int64_t lo = per * blockIdx.x;
    const int64_t hi = lo + per < npix ? lo + per : npix;
    const int64_t pnpix = (int64_t)A.pnx * A.pny;
    auto R = [&](int64_t k) -> float & { return SMEM ? sres[k - lo] : A.res[k]; };
    __shared__ int stop_sh;
    // the CTA's maximum of a pass as a key (cand_key; 0 for none): warps add theirs with
    // atomicMax, thread 0 adds it to the global word inside the next grid barrier
    __shared__ unsigned long long s_key;
    if (threadIdx.x == 0) s_key = 0ull;
    __syncthreads();
    // RES = DRT * BOX, and the first maximum of the slice
    Cand c{-1.0f, INT32_MAX, 0.0f};
    for (int64_t k = lo + threadIdx.x; k < hi; k += blockDim.x) {
        float r = A.box ? __fmul_rn(A.drt[k], A.box[k]) : __fmul_rn(A.drt[k], 1.0f);
        R(k) = r;
        c = better(c, Cand{fabsf(r), (int32_t)k, r});
    }
    {
        const unsigned long long wk = warp_key_max(c.a >= 0.0f ? cand_key(c) : 0ull);
        if ((threadIdx.x & 31) == 0 && wk) atomicMax(&s_key, wk);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) A.bar->stopreq[0] = (A.cancel && *A.cancel) ? 1 : 0;
    unsigned epoch = 0;
    if (!grid_sync(A.bar, gridDim.x, epoch++, &A.status[STATUS_TIMEOUT], &A.bar->best[0], &s_key)) return;
    // the maxima of successive passes take best[0], best[1], best[2] in turn: a word is read
    // after the barrier that follows its pass, and cleared by CTA 0 one pass before it is
    // used again (after every CTA has read it, before any CTA adds to it)
    int ph = 0;
    int cur = 0;
    float tflux = A.tflux_in;
    const int nabs = A.nsub < 0 ? -A.nsub : A.nsub;
    int isub;
    int stopped = 0;
    float maxres = 0.0f;
    for (isub = A.bsub; isub <= nabs; isub++) {
        // global first maximum of the last pass
        const Cand g = key_cand(__ldcg(&A.bar->best[ph % 3]));
        if (blockIdx.x == 0 && threadIdx.x == 0) A.bar->best[(ph + 2) % 3] = 0ull;
        if (threadIdx.x == 0) s_key = 0ull;  // (ordered before the warps' additions by the barrier below)
        // PIXISAMA returns 1 (index 0) when no |value| exceeds 0
        // every |value| >= 0 beats the -1 sentinel, so when nothing exceeds 0 the winner
        // is index 0 -- PIXISAMA's default of 1 (pix/pixisama.f:45)
        const int32_t ip = g.idx;
        const int pmx = 1 + ip % A.nx, pmy = 1 + ip / A.nx;
        maxres = g.v;
        if (threadIdx.x == 0) {
            int s = 0;
            if (A.nsub < 0 && maxres < 0.0f) s = 1;
            if (fabsf(maxres) <= A.flux) s = 1;
            if (((volatile int *)A.bar->stopreq)[cur]) s = 2;
            stop_sh = s;
        }
        __syncthreads();
        if (stop_sh) {
            stopped = stop_sh;
            break;
        }
        const float pntsub = __fmul_rn(A.gain, maxres);
        tflux = __fadd_rn(tflux, pntsub);
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            const int64_t ci = (int64_t)(pmy - 1) * A.nx + (pmx - 1);
            A.cln[ci] = __fadd_rn(A.cln[ci], pntsub);
            A.cflux[isub - 1] = pntsub;
            A.cx[isub - 1] = pmx;
            A.cy[isub - 1] = pmy;
        }
        const int offx = A.pmpx + pmx, offy = A.pmpy + pmy;
        Cand lc{-1.0f, INT32_MAX, 0.0f};
        // RES -= (PNTSUB*PSF(OFFX-IX, OFFY-IY))*BOX over the slice.  PSF is addressed as the
        // reference's array is, by its flat index (OFFX-IX-1) + (OFFY-IY-1)*PNX (0-based IX,
        // IY here: -2), which steps by -1 per pixel and by NX-PNX per row; when the whole
        // window's indices lie in the PSF no per-pixel check is made.  A thread visits its
        // pixels in increasing order, so a strictly larger |RES| is its first maximum.
        {
            const int nslice = (int)(hi - lo);
            int sidx = threadIdx.x;
            const int64_t k0 = lo + sidx;
            int ix0 = (int)(k0 % A.nx);
            const int iy0 = (int)(k0 / A.nx);
            int64_t flat = (int64_t)(offx - ix0 - 2) + (int64_t)(offy - iy0 - 2) * A.pnx;
            const int64_t fmin = (int64_t)(offx - (A.nx - 1) - 2) + (int64_t)(offy - (A.ny - 1) - 2) * A.pnx;
            const int64_t fmax = (int64_t)(offx - 2) + (int64_t)(offy - 2) * A.pnx;
            const bool inside = fmin >= 0 && fmax < pnpix;
            const int step = blockDim.x;
            const int64_t wrap = (int64_t)A.nx - A.pnx;
            float la = -1.0f, lv = 0.0f;
            int li = INT32_MAX;
            // CL_BATCH pixels at a time: their PSF and RES loads are issued before any is used
            for (; sidx < nslice; sidx += CL_BATCH * step) {
                float p[CL_BATCH], r0[CL_BATCH];
#pragma unroll
                for (int j = 0; j < CL_BATCH; j++) {
                    const bool in = sidx + j * step < nslice;
                    p[j] = !in ? 0.0f
                               : inside ? A.psf[flat]
                                        : ((flat >= 0 && flat < pnpix) ? A.psf[flat] : 0.0f);
                    r0[j] = in ? R(lo + sidx + j * step) : 0.0f;
                    ix0 += step;
                    flat -= step;
                    while (ix0 >= A.nx) {
                        ix0 -= A.nx;
                        flat += wrap;
                    }
                }
#pragma unroll
                for (int j = 0; j < CL_BATCH; j++) {
                    const int sj = sidx + j * step;
                    if (sj < nslice) {
                        float sub = __fmul_rn(pntsub, p[j]);
                        if (A.box) sub = __fmul_rn(sub, A.box[lo + sj]);
                        const float r = __fsub_rn(r0[j], sub);
                        R(lo + sj) = r;
                        if (fabsf(r) > la) {
                            la = fabsf(r);
                            li = (int)(lo + sj);
                            lv = r;
                        }
                    }
                }
            }
            lc = Cand{la, li, lv};
        }
        {
            const unsigned long long wk = warp_key_max(lc.a >= 0.0f ? cand_key(lc) : 0ull);
            if ((threadIdx.x & 31) == 0 && wk) atomicMax(&s_key, wk);
        }
        cur ^= 1;
        if (blockIdx.x == 0 && threadIdx.x == 0) A.bar->stopreq[cur] = (A.cancel && *A.cancel) ? 1 : 0;
        if (!grid_sync(A.bar, gridDim.x, epoch++, &A.status[STATUS_TIMEOUT], &A.bar->best[(ph + 1) % 3], &s_key))
            return;
        ph++;
    }
    if (SMEM)
        for (int64_t k = lo + threadIdx.x; k < hi; k += blockDim.x) A.res[k] = R(k);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int ansub;
        if (!stopped) {
            ansub = A.nsub;
        } else {
            ansub = isub - 1;
        }
        A.out[1] = tflux;
        A.out[2] = __int_as_float(ansub);
        A.out[3] = __int_as_float(stopped);
        if (stopped) A.out[0] = maxres;
    }
    if (!stopped) {
        // final PIXISAMA over the residual (pix/pix2drcl.f:134-138): the last pass's maximum
        if (blockIdx.x == 0 && threadIdx.x == 0) A.out[0] = key_cand(__ldcg(&A.bar->best[ph % 3])).v;
    }
}

// first strictly-largest |a| (PIXISAMA), two-level
__global__ void __launch_bounds__(CL_THREADS) k_isamax_part(const float *a, int64_t n, Cand *part) {
    Cand c{-1.0f, INT32_MAX, 0.0f};
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        c = better(c, Cand{fabsf(a[k]), (int32_t)k, a[k]});
    c = block_best(c);
    if (threadIdx.x == 0) part[blockIdx.x] = c;
}

__global__ void __launch_bounds__(CL_THREADS) k_isamax_final(const Cand *part, int nb, int64_t *out) {
    Cand c{-1.0f, INT32_MAX, 0.0f};
    for (int b = threadIdx.x; b < nb; b += blockDim.x) c = better(c, part[b]);
    c = block_best(c);
    // 1-based index of the first largest |a|, or 0 when no |a| exceeds 0
    if (threadIdx.x == 0) *out = c.a > 0.0f ? (int64_t)c.idx + 1 : 0;
}

// max value (ARRSTAT's ARRMAX) over an image
__global__ void __launch_bounds__(CL_THREADS) k_max_part(const float *a, int64_t n, float *part) {
    __shared__ float sh[32];
    float m = -INFINITY;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        m = fmaxf(m, a[k]);
    for (int d = 16; d > 0; d >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, d));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : -INFINITY;
        for (int d = 16; d > 0; d >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, d));
        if (threadIdx.x == 0) part[blockIdx.x] = m;
    }
}

__global__ void k_max_final(const float *part, int nb, float *out) {
    float m = -INFINITY;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) m = fmaxf(m, part[b]);
    for (int d = 16; d > 0; d >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, d));
    if (threadIdx.x == 0) *out = m;
}

// OUT = (1/max) * IN + 0.0 (task/uvmap.f:440 with pix/pixrscal.f)
__global__ void k_scale_inv(float *a, int64_t n, const float *maxp) {
    const float s = 1.0f / *maxp;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        a[k] = __fadd_rn(__fmul_rn(s, a[k]), 0.0f);
}

}  // namespace

int sde_isamax(sde_ctx *ctx, const float *a, int64_t n, int64_t *index_out) {
    SDE_TRY(sde_isamax0(ctx, a, n, index_out));
    if (*index_out == 0) *index_out = 1;  // PIXISAMA's default I = 1
    return SDE_OK;
}

int sde_isamax0(sde_ctx *ctx, const float *a, int64_t n, int64_t *index_out) {
    if (!ctx || !a || n <= 0 || !index_out || n > INT32_MAX) return SDE_EINVAL;
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    int nb = ctx->num_sms * 2;
    Cand *part;
    int64_t *d;
    SDE_TRY(ctx_scratch(ctx, "isa_part", sizeof(Cand) * (size_t)nb, (void **)&part));
    SDE_TRY(ctx_scratch(ctx, "isa_out", sizeof(int64_t), (void **)&d));
    k_isamax_part<<<nb, CL_THREADS, 0, ctx->stream>>>(a, n, part);
    SDE_CHECK_LAUNCH();
    k_isamax_final<<<1, CL_THREADS, 0, ctx->stream>>>(part, nb, d);
    SDE_CHECK_LAUNCH();
    SDE_CUDA_TRY(cudaMemcpyAsync(index_out, d, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    SDE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SDE_OK;
}

int sde_image_max(sde_ctx *ctx, const float *image, int64_t n, float *max_dev) {
    if (!ctx || !image || n <= 0 || !max_dev) return SDE_EINVAL;
    int nb = ctx->num_sms * 2;
    float *part;
    SDE_TRY(ctx_scratch(ctx, "max_part", sizeof(float) * (size_t)nb, (void **)&part));
    KTimer kt(ctx, "image_max");
    k_max_part<<<nb, CL_THREADS, 0, ctx->stream>>>(image, n, part);
    SDE_CHECK_LAUNCH();
    k_max_final<<<1, 32, 0, ctx->stream>>>(part, nb, max_dev);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

int sde_image_scale_by_inverse(sde_ctx *ctx, float *image, int64_t n, const float *max_dev) {
    if (!ctx || !image || n <= 0 || !max_dev) return SDE_EINVAL;
    KTimer kt(ctx, "scale_inv");
    k_scale_inv<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(image, n, max_dev);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

// The CLEAN kernels are loaded when the context is created (with CUDA's lazy module
// loading a kernel's first launch would otherwise load it, ~18 ms measured on the first
// sde_hogbom of a process), and the cooperative launch's occupancy is queried once.
int clean_preload(sde_ctx *ctx) {
    cudaFuncAttributes a;
    SDE_CUDA_TRY(cudaFuncGetAttributes(&a, k_isamax_part));
    SDE_CUDA_TRY(cudaFuncGetAttributes(&a, k_isamax_final));
    SDE_CUDA_TRY(cudaFuncGetAttributes(&a, k_max_part));
    SDE_CUDA_TRY(cudaFuncGetAttributes(&a, k_max_final));
    SDE_CUDA_TRY(cudaFuncGetAttributes(&a, k_scale_inv));
    int per_sm = 0;
    SDE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hogbom<false>, CL_THREADS, 0));
    ctx->hogbom_per_sm = per_sm;
    SDE_CUDA_TRY(cudaFuncSetAttribute(k_hogbom<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)CL_SMEM_SLICE_MAX));
    return SDE_OK;
}

int sde_hogbom(sde_ctx *ctx, const float *drt, const float *psf, const float *box, int nx, int ny,
               int pnx, int pny, float gain, int nsub, int bsub, float flux, float tflux_in,
               float *cln, float *res, float *cflux, int *cx, int *cy, volatile int *cancel_flag,
               sde_clean_result *out) {
    if (!ctx || !drt || !psf || !cln || !res || nx < 1 || ny < 1 || pnx < 1 || pny < 1 || !out ||
        (int64_t)nx * ny > INT32_MAX || bsub < 1) {
        sde_set_error("sde_hogbom: bad arguments");
        return SDE_EINVAL;
    }
    const int nabs = nsub < 0 ? -nsub : nsub;
    if (nabs >= bsub && (!cflux || !cx || !cy)) {
        sde_set_error("sde_hogbom: component arrays required");
        return SDE_EINVAL;
    }
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    // PSF peak (pix/pix2drcl.f:73-80)
    int64_t ip1;
    SDE_TRY(sde_isamax(ctx, psf, (int64_t)pnx * pny, &ip1));
    int ipeak = (int)(ip1 - 1);
    int pmpx = 1 + ipeak % pnx;
    int pmpy = 1 + (ipeak - pmpx + 1) / pnx;
    if (pmpx >= pnx) pmpx = pnx / 2;
    if (pmpy >= pny) pmpy = pny / 2;
    int per_sm = ctx->hogbom_per_sm;
    if (per_sm < 1) SDE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hogbom<false>, CL_THREADS, 0));
    if (per_sm < 1) {
        sde_set_error("sde_hogbom: kernel cannot be resident");
        return SDE_ECUDA;
    }
    int64_t npix = (int64_t)nx * ny;
    int nblocks = ctx->num_sms * (per_sm > 2 ? 2 : per_sm);
    int64_t want = (npix + 4 * CL_THREADS - 1) / (4 * CL_THREADS);  // small windows: fewer CTAs
    if (want < nblocks) nblocks = (int)(want < 1 ? 1 : want);
    // the residual in shared memory when every CTA's slice fits there and the launch stays
    // co-resident with it (windows up to ~2800^2 on GB300, two CTAs per SM)
    const size_t slice = sizeof(float) * (size_t)((npix + nblocks - 1) / nblocks);
    bool smem_res = false;
    if (slice <= CL_SMEM_SLICE_MAX) {
        int fit = 0;
        SDE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k_hogbom<true>, CL_THREADS, slice));
        smem_res = (int64_t)fit * ctx->num_sms >= nblocks;
    }
    Barrier *bar;
    float *dout;
    SDE_TRY(ctx_scratch(ctx, "cl_bar", sizeof(Barrier), (void **)&bar));
    SDE_TRY(ctx_scratch(ctx, "cl_out", 4 * sizeof(float), (void **)&dout));
    SDE_CUDA_TRY(cudaMemsetAsync(bar, 0, sizeof(Barrier), ctx->stream));
    SDE_CUDA_TRY(cudaMemsetAsync(ctx->d_status, 0, sizeof(int) * STATUS_COUNT, ctx->stream));
    CleanArgs A;
    A.drt = drt; A.psf = psf; A.box = box; A.cln = cln; A.res = res; A.cflux = cflux;
    A.cx = cx; A.cy = cy; A.nx = nx; A.ny = ny; A.pnx = pnx; A.pny = pny;
    A.pmpx = pmpx; A.pmpy = pmpy; A.gain = gain; A.flux = flux; A.tflux_in = tflux_in;
    A.nsub = nsub; A.bsub = bsub; A.cancel = cancel_flag; A.bar = bar;
    A.status = ctx->d_status; A.out = dout;
    void *args[] = {&A};
    KTimer kt(ctx, "hogbom");
    if (smem_res)
        SDE_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)k_hogbom<true>, dim3(nblocks), dim3(CL_THREADS),
                                                 args, slice, ctx->stream));
    else
        SDE_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)k_hogbom<false>, dim3(nblocks), dim3(CL_THREADS),
                                                 args, 0, ctx->stream));
    float h[4];
    SDE_CUDA_TRY(cudaMemcpyAsync(h, dout, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    SDE_CUDA_TRY(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(int) * STATUS_COUNT,
                                 cudaMemcpyDeviceToHost, ctx->stream));
    SDE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (ctx->h_status[STATUS_TIMEOUT]) {
        sde_set_error("sde_hogbom: grid barrier timed out");
        return SDE_ETIMEDOUT;
    }
    int ansub, stopped;
    memcpy(&ansub, &h[2], 4);
    memcpy(&stopped, &h[3], 4);
    out->maxres = h[0];
    out->tflux = h[1];
    out->ansub = ansub;
    if (stopped == 2) return SDE_ECANCELLED;
    return SDE_OK;
}

// ---------------------------------------------------------------------------------------
// Hogbom CLEAN without any device allocation.
//
// Some callers cannot call cudaMalloc: code that owns all device memory through its own
// allocator or a fixed arena, embedded/real-time hosts that forbid allocation after start-up,
// and serving loops that must not block on the allocator.  For them this entry point runs the
// same minor cycle as sde_hogbom on arrays the caller already holds, keeping its scratch --
// the per-CTA partial maxima of the PSF-peak search, the grid barrier with the iterations'
// maxima, the status words and the result scalars -- in one file-scope device array of fixed
// size.  That array exists on every GPU that loads the library, for the life of the process.
namespace {
constexpr int NOALLOC_MAX_CTAS = 1024;  // CTAs of the PSF-peak search and of CLEAN (~12 KB in all)
struct NoAllocScratch {
    Cand isa_part[NOALLOC_MAX_CTAS];
    int64_t isa_out;
    Barrier bar;
    int status[STATUS_COUNT];
    float out[4];
};
}  // namespace

static __device__ __align__(256) NoAllocScratch g_clean_scratch;

// Host-side copies of g_clean_scratch's device address, one per device.  The array's name in
// host code only stands in for the symbol; the address every kernel receives comes from
// cudaGetSymbolAddress, taken with that device current the first time the device is used.
// It is taken again when the device's current context has changed since (a caller's
// cudaDeviceReset destroys the primary context, and the next one loads the module, and with
// it the array, anew -- possibly at another address).
static NoAllocScratch *g_clean_scratch_dev[64];
static unsigned long long g_clean_scratch_ctx[64];
static std::mutex g_clean_scratch_mu;

// unique ID of the calling thread's current CUDA context (driver API, resolved at run time)
static int current_context_id(unsigned long long *id) {
    typedef CUresult (*GetCurrentFn)(CUcontext *);
    typedef CUresult (*GetIdFn)(CUcontext, unsigned long long *);
    static GetCurrentFn get_current = nullptr;
    static GetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void *a = nullptr, *b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) !=
                cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) !=
                cudaSuccess ||
            qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b) {
            sde_set_error("sde_hogbom_noalloc: driver context queries unavailable");
            return SDE_ECUDA;
        }
        get_current = (GetCurrentFn)a;
        get_id = (GetIdFn)b;
    }
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS || !c || get_id(c, id) != CUDA_SUCCESS) {
        sde_set_error("sde_hogbom_noalloc: no current CUDA context");
        return SDE_ECUDA;
    }
    return SDE_OK;
}

static int clean_scratch_address(int dev, NoAllocScratch **out) {
    if (dev < 0 || dev >= 64) {
        sde_set_error("sde_hogbom_noalloc: device %d out of range", dev);
        return SDE_EINVAL;
    }
    // make the device's primary context current on this thread (no allocation)
    SDE_CUDA_TRY(cudaSetDevice(dev));
    unsigned long long id = 0;
    SDE_TRY(current_context_id(&id));
    std::lock_guard<std::mutex> lk(g_clean_scratch_mu);
    if (!g_clean_scratch_dev[dev] || g_clean_scratch_ctx[dev] != id) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_clean_scratch);
        if (e != cudaSuccess || !p) {
            sde_set_error("sde_hogbom_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? SDE_ENODEV : SDE_ECUDA;
        }
        g_clean_scratch_dev[dev] = (NoAllocScratch *)p;
        g_clean_scratch_ctx[dev] = id;
    }
    *out = g_clean_scratch_dev[dev];
    return SDE_OK;
}

extern "C" int sde_hogbom_noalloc(void *stream, const float *drt, const float *psf,
                                  const float *box, int nx, int ny, int pnx, int pny, float gain,
                                  int nsub, int bsub, float flux, float tflux_in, float *cln,
                                  float *res, float *cflux, int *cx, int *cy,
                                  volatile int *cancel_flag, sde_clean_result *out) {
    if (!drt || !psf || !cln || !res || !out || nx < 1 || ny < 1 || pnx < 1 || pny < 1 || bsub < 1) {
        sde_set_error("sde_hogbom_noalloc: bad arguments");
        return SDE_EINVAL;
    }
    if ((int64_t)nx * ny > INT32_MAX || (int64_t)pnx * pny > INT32_MAX) {
        sde_set_error("sde_hogbom_noalloc: window %dx%d or PSF %dx%d exceeds 2^31-1 pixels", nx, ny,
                      pnx, pny);
        return SDE_EINVAL;
    }
    const int nabs = nsub < 0 ? -nsub : nsub;
    if (nabs >= bsub && (!cflux || !cx || !cy)) {
        sde_set_error("sde_hogbom_noalloc: component arrays required");
        return SDE_EINVAL;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, nsm = 0;
    SDE_CUDA_TRY(cudaGetDevice(&dev));
    SDE_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    NoAllocScratch *S = nullptr;
    SDE_TRY(clean_scratch_address(dev, &S));
    // PSF peak (pix/pix2drcl.f:73-80) with the partials in the static array
    int nbi = nsm * 2;
    if (nbi > NOALLOC_MAX_CTAS) nbi = NOALLOC_MAX_CTAS;
    k_isamax_part<<<nbi, CL_THREADS, 0, st>>>(psf, (int64_t)pnx * pny, S->isa_part);
    SDE_CHECK_LAUNCH();
    k_isamax_final<<<1, CL_THREADS, 0, st>>>(S->isa_part, nbi, &S->isa_out);
    SDE_CHECK_LAUNCH();
    int64_t ip1 = 0;
    SDE_CUDA_TRY(cudaMemcpyAsync(&ip1, &S->isa_out, sizeof ip1, cudaMemcpyDeviceToHost, st));
    SDE_CUDA_TRY(cudaStreamSynchronize(st));
    if (ip1 == 0) ip1 = 1;  // PIXISAMA's default I = 1
    const int ipeak = (int)(ip1 - 1);
    int pmpx = 1 + ipeak % pnx;
    int pmpy = 1 + (ipeak - pmpx + 1) / pnx;
    if (pmpx >= pnx) pmpx = pnx / 2;
    if (pmpy >= pny) pmpy = pny / 2;
    int per_sm = 0;
    SDE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hogbom<false>, CL_THREADS, 0));
    if (per_sm < 1) {
        sde_set_error("sde_hogbom_noalloc: kernel cannot be resident");
        return SDE_ECUDA;
    }
    const int64_t npix = (int64_t)nx * ny;
    int nblocks = nsm * (per_sm > 2 ? 2 : per_sm);
    const int64_t want = (npix + 4 * CL_THREADS - 1) / (4 * CL_THREADS);
    if (want < nblocks) nblocks = (int)(want < 1 ? 1 : want);
    if (nblocks > NOALLOC_MAX_CTAS) nblocks = NOALLOC_MAX_CTAS;
    // the array keeps the previous call's contents: clear what must start at zero
    SDE_CUDA_TRY(cudaMemsetAsync(&S->bar, 0, sizeof(Barrier), st));
    SDE_CUDA_TRY(cudaMemsetAsync(S->status, 0, sizeof(S->status), st));
    SDE_CUDA_TRY(cudaMemsetAsync(S->out, 0, sizeof(S->out), st));
    CleanArgs A;
    A.drt = drt; A.psf = psf; A.box = box; A.cln = cln; A.res = res; A.cflux = cflux;
    A.cx = cx; A.cy = cy; A.nx = nx; A.ny = ny; A.pnx = pnx; A.pny = pny;
    A.pmpx = pmpx; A.pmpy = pmpy; A.gain = gain; A.flux = flux; A.tflux_in = tflux_in;
    A.nsub = nsub; A.bsub = bsub; A.cancel = cancel_flag; A.bar = &S->bar;
    A.status = S->status; A.out = S->out;
    void *args[] = {&A};
    SDE_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)k_hogbom<false>, dim3(nblocks), dim3(CL_THREADS),
                                             args, 0, st));
    float h[4];
    int hs[STATUS_COUNT];
    SDE_CUDA_TRY(cudaMemcpyAsync(h, S->out, sizeof h, cudaMemcpyDeviceToHost, st));
    SDE_CUDA_TRY(cudaMemcpyAsync(hs, S->status, sizeof hs, cudaMemcpyDeviceToHost, st));
    SDE_CUDA_TRY(cudaStreamSynchronize(st));
    if (hs[STATUS_TIMEOUT]) {
        sde_set_error("sde_hogbom_noalloc: grid barrier timed out");
        return SDE_ETIMEDOUT;
    }
    int ansub, stopped;
    memcpy(&ansub, &h[2], 4);
    memcpy(&stopped, &h[3], 4);
    out->maxres = h[0];
    out->tflux = h[1];
    out->ansub = ansub;
    if (stopped == 2) return SDE_ECANCELLED;
    return SDE_OK;
}
