// weights.cu -- uniform (GRDUWT2D) and robust (GRDRUW2D) weighting, bit-exact.
//
// Pass 1 of the reference (grd/grduwt2d.f:90-115, grd/grdruw2d.f:132-159) adds WT into the
// density grid GWT(UCEN,VCEN) sequentially in FP32, in visibility order.  Here each
// visibility's cell key is computed with the reference's exact FP32/FP64 operations (no
// FMA contraction), the (key, WT) pairs are sorted stably, and one thread sums each
// cell's run in order: the same additions in the same order, so GWT is bit-identical.
// Pass 2 (grd/grduwt2d.f:118-160, grd/grdruw2d.f:196-242) is an element-wise gather.
#include <math.h>
#include <string.h>

#include "common.cuh"

namespace {

struct WParams {
    float uscale, uoffset, vscale, voffset;
    int uorigin, vorigin, nu, nv;
    double s[9];
    int doshift;
    int near_identity;  // see wcell
};

// FP32 uv -> cell of the weighting routines (grd/grduwt2d.f:92-111, grd/grdruw2d.f:198-217).
__device__ __forceinline__ bool wcell(const WParams &p, float u, float v, float w, int &uc,
                                      int &vc, float &ul, float &vl) {
    float ucell, vcell;
    // With SHIFT(2,1) = SHIFT(3,1) = SHIFT(1,2) = SHIFT(3,2) = 0 and the diagonal within
    // 2^-40 of 1 (CRDSHIFT without a shift: sin^2 + cos^2 can miss 1 by an ulp), the DOUBLE
    // ULOCAL = SHIFT(1,1)*U + 0*V + 0*W and VLOCAL lie within |U|*2^-39 of U and V, far
    // inside half a REAL ulp, so the REAL ULOCAL, VLOCAL are U and V themselves.
    if (p.doshift && !p.near_identity) {
        double du = (double)u, dv = (double)v, dw = (double)w;
        ul = __double2float_rn(__dadd_rn(__dadd_rn(__dmul_rn(p.s[0], du), __dmul_rn(p.s[1], dv)),
                                         __dmul_rn(p.s[2], dw)));
        vl = __double2float_rn(__dadd_rn(__dadd_rn(__dmul_rn(p.s[3], du), __dmul_rn(p.s[4], dv)),
                                         __dmul_rn(p.s[5], dw)));
    } else {
        ul = u;
        vl = v;
    }
    ucell = __fadd_rn(__fmul_rn(p.uscale, ul), p.uoffset);
    vcell = __fadd_rn(__fmul_rn(p.vscale, vl), p.voffset);
    if (ucell > 0.0f) {
        ucell = __fadd_rn(ucell, (float)p.uorigin);
        vcell = __fadd_rn(vcell, (float)p.vorigin);
    } else {
        ucell = __fadd_rn(-ucell, (float)p.uorigin);
        vcell = __fadd_rn(-vcell, (float)p.vorigin);
    }
    uc = nint_f(ucell);
    vc = nint_f(vcell);
    return !(uc < 1 || uc > p.nu || vc < 1 || vc > p.nv);
}

__global__ void k_wkey(WParams p, const float *__restrict__ wt, const float *__restrict__ u,
                       const float *__restrict__ v, const float *__restrict__ w, int64_t n,
                       uint32_t *keys, uint32_t *vals, unsigned long long *counts) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t valid = 0, drop = 0;
    if (i < n) {
        float wi = wt[i];
        uint32_t key = KEY_INVALID;
        if (wi > 0.0f) {
            int uc, vc;
            float ul, vl;
            if (wcell(p, u[i], v[i], w[i], uc, vc, ul, vl)) {
                key = (uint32_t)(vc - 1) * (uint32_t)p.nu + (uint32_t)(uc - 1);
                valid = 1;
            } else {
                drop = 1;
            }
        }
        keys[i] = key;
        vals[i] = __float_as_uint(wi);
    }
    // block-aggregated counters: [0] on-grid, [1] dropped (one atomic per block and counter)
    const int cv = __syncthreads_count(valid), cd = __syncthreads_count(drop);
    if (threadIdx.x == 0) {
        if (cv) atomicAdd(&counts[0], (unsigned long long)cv);
        if (cd) atomicAdd(&counts[1], (unsigned long long)cd);
    }
}

// GWT(cell) = ((0 + w1) + w2) + ... in visibility order: FP32 additions in the reference's
// order, so every cell's sum is one sequential chain.  A block stages SEG_TILE sorted entries
// (plus the one before and SEG_SHORT after) in shared memory; one thread per run head sums a
// run of at most SEG_SHORT entries from there; a longer run (dense cells hold up to ~2e5
// visibilities) is put on a list for k_segsum_long, where a warp streams it.
constexpr int SEG_SHORT = 32;
constexpr int SEG_TILE = 2048;
constexpr int SEG_T = 256;
__global__ void __launch_bounds__(SEG_T) k_segsum(const uint32_t *__restrict__ keys,
                                                  const uint32_t *__restrict__ vals,
                                                  unsigned long long *counts, float *gwt, uint32_t *longq) {
    __shared__ uint32_t sk[SEG_TILE + SEG_SHORT + 1];  // keys[base - 1 ...]
    __shared__ float sv[SEG_TILE + SEG_SHORT];          // vals[base ...]
    const int64_t nvalid = (int64_t)counts[0];
    const int64_t base = (int64_t)blockIdx.x * SEG_TILE;
    if (base >= nvalid) return;
    for (int i = threadIdx.x; i < SEG_TILE + SEG_SHORT + 1; i += SEG_T) {
        const int64_t q = base - 1 + i;
        sk[i] = q >= 0 && q < nvalid ? keys[q] : KEY_INVALID;  // valid keys are below KEY_INVALID
    }
    for (int i = threadIdx.x; i < SEG_TILE + SEG_SHORT; i += SEG_T) {
        const int64_t q = base + i;
        sv[i] = q < nvalid ? __uint_as_float(vals[q]) : 0.0f;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < SEG_TILE; j += SEG_T) {
        const int64_t p = base + j;
        if (p >= nvalid) break;
        const uint32_t k = sk[j + 1];
        if (sk[j] == k) continue;  // not the first entry of its run
        if (sk[j + 1 + SEG_SHORT] == k) {
            const unsigned long long slot = atomicAdd(&counts[2], 1ull);
            longq[slot] = (uint32_t)p;
            continue;
        }
        float s = 0.0f;
        for (int q = j; sk[q + 1] == k; q++) s = __fadd_rn(s, sv[q]);
        gwt[k] = s;
    }
}

// One warp per long run.  Lane 0 finds the run's end (galloping then binary search over the
// sorted keys), then the warp streams the run through shared memory in blocks of 256
// entries -- the next block's coalesced loads in flight while lane 0 adds the current one
// in order from 16-byte shared reads -- so the chain costs about one FADD latency per entry.
constexpr int SEG_BLK = 256;
constexpr int SEG_WARPS = 8;  // warps per block of k_segsum_long
__global__ void __launch_bounds__(SEG_WARPS * 32) k_segsum_long(
    const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals,
    unsigned long long *counts, const uint32_t *__restrict__ longq, float *gwt) {
    constexpr unsigned FULL = 0xffffffffu;
    __shared__ __align__(16) float buf[SEG_WARPS][2][SEG_BLK];
    const int64_t nvalid = (int64_t)counts[0];
    const int64_t nlong = (int64_t)counts[2];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    // runs are taken from a counter, so the warp that holds the longest run (the bound of
    // this kernel: one sequential FP32 chain) takes no other
    for (;;) {
        int64_t r = 0;
        if (lane == 0) r = (int64_t)atomicAdd(&counts[3], 1ull);
        r = __shfl_sync(FULL, r, 0);
        if (r >= nlong) break;
        const int64_t p = longq[r];
        const uint32_t k = keys[p];
        int64_t end = 0;
        if (lane == 0) {
            // keys[p + SEG_SHORT] == k (why the run is here); find the first index past the run
            int64_t lo = p + SEG_SHORT, step = 64;
            while (lo + step < nvalid && keys[lo + step] == k) {
                lo += step;
                step *= 2;
            }
            int64_t hi = lo + step < nvalid ? lo + step : nvalid;  // keys[hi] != k or hi = nvalid
            while (hi - lo > 1) {
                const int64_t mid = lo + (hi - lo) / 2;
                if (keys[mid] == k) lo = mid; else hi = mid;
            }
            end = hi;
        }
        end = __shfl_sync(FULL, end, 0);
        const int64_t len = end - p;
        const int nblk = (int)((len + SEG_BLK - 1) / SEG_BLK);
        float reg[SEG_BLK / 32];
#pragma unroll
        for (int j = 0; j < SEG_BLK / 32; j++) {
            const int64_t q = p + j * 32 + lane;
            reg[j] = q < end ? __uint_as_float(vals[q]) : 0.0f;
        }
        float s = 0.0f;
        for (int b = 0; b < nblk; b++) {
            float *cur = buf[wib][b & 1];
#pragma unroll
            for (int j = 0; j < SEG_BLK / 32; j++) cur[j * 32 + lane] = reg[j];
            __syncwarp();
            if (b + 1 < nblk) {
#pragma unroll
                for (int j = 0; j < SEG_BLK / 32; j++) {
                    const int64_t q = p + (int64_t)(b + 1) * SEG_BLK + j * 32 + lane;
                    reg[j] = q < end ? __uint_as_float(vals[q]) : 0.0f;
                }
            }
            if (lane == 0) {
                const int cnt = (int)(len - (int64_t)b * SEG_BLK < SEG_BLK ? len - (int64_t)b * SEG_BLK : SEG_BLK);
                const float4 *c4 = reinterpret_cast<const float4 *>(cur);
                if (cnt == SEG_BLK) {
#pragma unroll 8
                    for (int j = 0; j < SEG_BLK / 4; j++) {
                        const float4 x = c4[j];
                        s = __fadd_rn(s, x.x);
                        s = __fadd_rn(s, x.y);
                        s = __fadd_rn(s, x.z);
                        s = __fadd_rn(s, x.w);
                    }
                } else {
                    for (int j = 0; j < cnt; j++) s = __fadd_rn(s, cur[j]);
                }
            }
            __syncwarp();
        }
        if (lane == 0) gwt[k] = s;
    }
}

// Deterministic FP64 sums (block partials in a fixed order).
constexpr int RED_THREADS = 256;
__device__ __forceinline__ double block_sum_d(double x) {
    __shared__ double sh[RED_THREADS / 32];
    for (int d = 16; d > 0; d >>= 1) x = __dadd_rn(x, __shfl_down_sync(0xffffffffu, x, d));
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = x;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < RED_THREADS / 32; k++) r = __dadd_rn(r, sh[k]);
    return r;
}

// partial[b] = sum of weights of sorted valid entries in block b's range
__global__ void __launch_bounds__(RED_THREADS) k_sumwt_part(const uint32_t *vals,
                                                             const unsigned long long *counts,
                                                             int per_thread, double *partial) {
    int64_t nvalid = (int64_t)counts[0];
    int64_t base = ((int64_t)blockIdx.x * RED_THREADS + threadIdx.x) * per_thread;
    double s = 0.0;
    for (int k = 0; k < per_thread; k++) {
        int64_t q = base + k;
        if (q < nvalid) s = __dadd_rn(s, (double)__uint_as_float(vals[q]));
    }
    double r = block_sum_d(s);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

// partial[b] = sum over cells in block b's range of (double)(g*g), g > 0 (grd/grdruw2d.f:168-175)
__global__ void __launch_bounds__(RED_THREADS) k_sumlocwt_part(const float *gwt, int64_t ncell,
                                                                int per_thread, double *partial) {
    int64_t base = ((int64_t)blockIdx.x * RED_THREADS + threadIdx.x) * per_thread;
    double s = 0.0;
    for (int k = 0; k < per_thread; k++) {
        int64_t q = base + k;
        if (q < ncell) {
            float g = gwt[q];
            if (g > 0.0f) s = __dadd_rn(s, (double)__fmul_rn(g, g));
        }
    }
    double r = block_sum_d(s);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

// The partials in a fixed order: thread t adds partials t, t + RED_THREADS, ..., then a
// fixed tree over the threads (deterministic for a given partial count).
__global__ void __launch_bounds__(RED_THREADS) k_sum_partials(const double *partial, int n, double *out) {
    __shared__ double sh[RED_THREADS];
    double s = 0.0;
    for (int k = threadIdx.x; k < n; k += RED_THREADS) s = __dadd_rn(s, partial[k]);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int h = RED_THREADS / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) sh[threadIdx.x] = __dadd_rn(sh[threadIdx.x], sh[threadIdx.x + h]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

struct AzParams {
    int doaz;
    float r1, rbscale, rpa, pi;
    double ratio;  // SUMLOCWT / SUMWT
};

// Pass 2.  uniform: grd/grduwt2d.f:146-158; robust: grd/grdruw2d.f:225-240.
__global__ void k_newwt(WParams p, int robust, float f2, float d2, AzParams az,
                        const float *wt, const float *__restrict__ u, const float *__restrict__ v,
                        const float *__restrict__ w, const float *__restrict__ gwt, int64_t n,
                        float *newwt) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float wi = wt[i];
    if (wi <= 0.0f) return;
    int uc, vc;
    float ul, vl;
    if (!wcell(p, u[i], v[i], w[i], uc, vc, ul, vl)) {
        newwt[i] = -1.0f;
        return;
    }
    float g = gwt[(int64_t)(vc - 1) * p.nu + (uc - 1)];
    float out;
    if (!robust) {
        if (g > 0.0f) {
            if (uc == p.uorigin && vc != p.vorigin)
                out = __fdiv_rn(__fmul_rn(0.5f, wi), g);
            else
                out = __fdiv_rn(wi, g);
        } else {
            out = -1.0f;
        }
    } else {
        float ff2 = f2;
        if (az.doaz) {  // CUDA atan2f/fmodf/powf: within the CUDA math library's ulp bounds
            float t = atan2f(vl, ul);
            t = __fsub_rn(fmodf(__fadd_rn(__fsub_rn(t, az.rpa), __fmul_rn(2.5f, az.pi)), az.pi),
                          __fdiv_rn(az.pi, 2.0f));
            float r = __fsub_rn(az.r1, __fmul_rn(fabsf(t), az.rbscale));
            float tt = __fmul_rn(5.0f, powf(10.0f, -r));
            ff2 = __double2float_rn(__ddiv_rn((double)__fmul_rn(tt, tt), az.ratio));
        }
        if (g > 0.0f) {
            float den = __fadd_rn(__fmul_rn(g, ff2), d2);
            if (uc == p.uorigin && vc != p.vorigin)
                out = __fdiv_rn(__fmul_rn(0.5f, wi), den);
            else
                out = __fdiv_rn(wi, den);
        } else {
            out = -1.0f;
        }
    }
    newwt[i] = out;
}

int key_bits(int64_t maxkey) {
    int b = 1;
    while (b < 32 && ((int64_t)1 << b) <= maxkey) b++;
    return b;
}

}  // namespace

int sde_weights(sde_ctx *ctx, int rmode, const float robust[3], float ds, const float *wt,
                const float *u, const float *v, const float *w, int64_t nvis, float uscale,
                float uoffset, float vscale, float voffset, int uorigin, int vorigin, int nu,
                int nv, const double shift[9], float *newwt, float *gwt, sde_wstats *stats) {
    if (!ctx || nvis < 0 || nu <= 0 || nv <= 0 || !shift) {
        sde_set_error("sde_weights: bad arguments");
        return SDE_EINVAL;
    }
    if (rmode < 0 || rmode > 4) {
        sde_set_error("sde_weights: unrecognized RMODE %d", rmode);
        return SDE_EBADMODE;
    }
    if ((int64_t)nu * nv >= (int64_t)KEY_INVALID) {
        sde_set_error("sde_weights: grid too large");
        return SDE_EINVAL;
    }
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    WParams p;
    p.uscale = uscale; p.uoffset = uoffset; p.vscale = vscale; p.voffset = voffset;
    p.uorigin = uorigin; p.vorigin = vorigin; p.nu = nu; p.nv = nv;
    memcpy(p.s, shift, sizeof p.s);
    p.doshift = (shift[0] != 1.0) || (shift[4] != 1.0) || (shift[8] != 1.0);
    p.near_identity = shift[1] == 0.0 && shift[2] == 0.0 && shift[3] == 0.0 && shift[5] == 0.0 &&
                      fabs(shift[0] - 1.0) <= 0x1p-40 && fabs(shift[4] - 1.0) <= 0x1p-40;
    const int64_t ncell = (int64_t)nu * nv;
    if (!gwt) SDE_TRY(ctx_scratch(ctx, "w_gwt", sizeof(float) * (size_t)ncell, (void **)&gwt));
    SDE_CUDA_TRY(cudaMemsetAsync(gwt, 0, sizeof(float) * (size_t)ncell, st));
    uint32_t *keys, *vals, *ktmp, *vtmp;
    unsigned long long *counts;
    size_t nb4 = sizeof(uint32_t) * (size_t)(nvis > 0 ? nvis : 1);
    SDE_TRY(ctx_scratch(ctx, "w_keys", nb4, (void **)&keys));
    SDE_TRY(ctx_scratch(ctx, "w_vals", nb4, (void **)&vals));
    SDE_TRY(ctx_scratch(ctx, "w_ktmp", nb4, (void **)&ktmp));
    SDE_TRY(ctx_scratch(ctx, "w_vtmp", nb4, (void **)&vtmp));
    SDE_TRY(ctx_scratch(ctx, "w_counts", 64, (void **)&counts));
    SDE_CUDA_TRY(cudaMemsetAsync(counts, 0, 64, st));
    const int T = 256;
    if (nvis > 0) {
        k_wkey<<<ceil_div(nvis, T), T, 0, st>>>(p, wt, u, v, w, nvis, keys, vals, counts);
        SDE_CHECK_LAUNCH();
        SDE_TRY(launch_radix_sort_u32(ctx, keys, vals, nvis, key_bits(ncell), ktmp, vtmp));
        uint32_t *longq;
        SDE_TRY(ctx_scratch(ctx, "w_longq", sizeof(uint32_t) * (size_t)(nvis / (SEG_SHORT + 1) + 1),
                            (void **)&longq));
        k_segsum<<<ceil_div(nvis, SEG_TILE), SEG_T, 0, st>>>(keys, vals, counts, gwt, longq);
        SDE_CHECK_LAUNCH();
        k_segsum_long<<<ctx->num_sms * 4, SEG_WARPS * 32, 0, st>>>(keys, vals, counts, longq, gwt);
        SDE_CHECK_LAUNCH();
    }
    float f2 = 1.0f, d2 = 0.0f;
    AzParams az;
    memset(&az, 0, sizeof az);
    double *sums;  // [0] sumwt [1] sumlocwt
    SDE_TRY(ctx_scratch(ctx, "w_sums", 2 * sizeof(double), (void **)&sums));
    SDE_CUDA_TRY(cudaMemsetAsync(sums, 0, 2 * sizeof(double), st));
    unsigned long long hcounts[2] = {0, 0};
    double hs[2] = {0.0, 0.0};
    const int robust_mode = rmode >= 1;
    const bool need_sums = robust_mode || stats;
    if (need_sums) {
        const int per = 16;
        int nbw = ceil_div(nvis > 0 ? nvis : 1, (int64_t)RED_THREADS * per);
        int nbc = ceil_div(ncell, (int64_t)RED_THREADS * per);
        double *part;
        SDE_TRY(ctx_scratch(ctx, "w_part", sizeof(double) * (size_t)(nbw > nbc ? nbw : nbc),
                            (void **)&part));
        k_sumwt_part<<<nbw, RED_THREADS, 0, st>>>(vals, counts, per, part);
        SDE_CHECK_LAUNCH();
        k_sum_partials<<<1, RED_THREADS, 0, st>>>(part, nbw, sums);
        SDE_CHECK_LAUNCH();
        if (rmode == 1 || rmode == 3) {
            k_sumlocwt_part<<<nbc, RED_THREADS, 0, st>>>(gwt, ncell, per, part);
            SDE_CHECK_LAUNCH();
            k_sum_partials<<<1, RED_THREADS, 0, st>>>(part, nbc, sums + 1);
            SDE_CHECK_LAUNCH();
        }
        // both through the context's pinned bytes (one wait)
        SDE_CUDA_TRY(cudaMemcpyAsync(ctx->h_small, sums, sizeof hs, cudaMemcpyDeviceToHost, st));
        SDE_CUDA_TRY(cudaMemcpyAsync(ctx->h_small + sizeof hs, counts, sizeof hcounts, cudaMemcpyDeviceToHost, st));
        SDE_CUDA_TRY(cudaStreamSynchronize(st));
        memcpy(hs, ctx->h_small, sizeof hs);
        memcpy(hcounts, ctx->h_small + sizeof hs, sizeof hcounts);
    }
    // robust parameters on the host, with the reference's REAL/DOUBLE mix (grd/grdruw2d.f:106-193)
    float rob = robust ? robust[0] : 0.0f;
    if (rmode == 3) {
        rob = (robust[0] + robust[1]) / 2.0f;
        float rpa = -robust[2] + 90.0f - 90.0f;
        while (rpa < -90.0f) rpa = rpa + 180.0f;
        while (rpa > 90.0f) rpa = rpa - 180.0f;
        float pi = 4.0f * atanf(1.0f);
        rpa = rpa * pi / 180.0f;
        az.doaz = 1;
        az.r1 = robust[0];
        az.rpa = rpa;
        az.pi = pi;
        az.rbscale = (robust[0] - robust[1]) / (pi / 2.0f);
        az.ratio = hs[1] / hs[0];
    }
    if (rmode == 1 || rmode == 3) {
        float t = 5.0f * powf(10.0f, -rob);
        f2 = (float)((double)(t * t) / (hs[1] / hs[0]));
        d2 = 1.0f;
    } else if (rmode == 2) {
        f2 = rob * rob;
        d2 = 2.0f * (ds * ds);
    } else {
        f2 = 1.0f;
        d2 = 0.0f;
    }
    if (nvis > 0) {
        k_newwt<<<ceil_div(nvis, T), T, 0, st>>>(p, robust_mode, f2, d2, az, wt, u, v, w, gwt, nvis,
                                               newwt);
        SDE_CHECK_LAUNCH();
    }
    if (stats) {
        stats->ndrop = (int64_t)hcounts[1];
        stats->sumwt = hs[0];
        stats->sumlocwt = hs[1];
        stats->f2 = f2;
        stats->d2 = d2;
        SDE_CUDA_TRY(cudaStreamSynchronize(st));
    }
    return SDE_OK;
}
