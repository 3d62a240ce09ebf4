// clark.cu -- Clark CLEAN (the default algorithm of SDE's clean task): the CLARK branch of
// task/clean.f:147-205 (CRDHALF window, IMGMAKEX transfer function, IMGSUBPS beam patch and
// exterior sidelobe) and IMGCCLEA's loop (img/imgcclea.f:210-290).  A major cycle is:
//   residual *= box, its extrema (ARRSTAT)                     k_clark_stats
//   |residual| histogram of 1024 bins (PIXRABSH)               k_clark_hist
//   the list limit (PIXFLIM, ARRFLIM, EXTSIDE)                 k_clark_limit
//   the list of pixels above it, in storage order (PIX2DRLI)   k_clark_count / _scan / _emit
//   the minor cycle on the list (PIX2DRCC)                     k_clark_minor: one cluster
//   the components into the model image (PIX2DRMA)             k_clark_addcomp
//   residual = dirty - IFFT(FFT(model) * XFR) (IMGRESID)       FFTR2D passes + k_clark_cmul/_sub
// The host reads back the cycle's scalars once per major cycle for IMGCCLEA's stop test.
#include <string.h>

#include <cooperative_groups.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int CL_NB = 1024;        // histogram bins (arr/arrabshi.f:34 NB = 1024)
constexpr int CL_T = 1024;         // minor-cycle threads per CTA
constexpr int CL_CTAS = 8;         // minor-cycle CTAs: one thread-block cluster
constexpr int CL_PER = 4;          // list entries per thread held in registers
constexpr int CL_SLICE = CL_T * CL_PER;           // entries per CTA
constexpr int CL_MAXNL = CL_CTAS * CL_SLICE;      // 32768
constexpr int CL_CHUNK = 4096;     // pixels per block of the list compaction (256 x 16)

struct ClarkState {
    unsigned int smax, smin;       // ordered encodings of the signed max / min (ARRSTAT)
    unsigned int amax, amin;       // |residual| max / min (non-negative float bits)
    float base, incr, slim;
    int err;                       // 1 zero range, 2 too many points, 3 negative limit
    int anl, total;                // list length, pixels above the limit
    int pmpx, pmpy;                // beam-patch peak (1-based)
    float extside;
    int aniter;
    float maxres, tflux;
};

__device__ __forceinline__ unsigned int ord_enc(float f) {
    const unsigned int b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ord_dec(unsigned int e) {
    return __uint_as_float((e & 0x80000000u) ? (e & 0x7FFFFFFFu) : ~e);
}

__global__ void k_clark_init(ClarkState *st) {
    st->smax = 0u;
    st->smin = 0xFFFFFFFFu;
    st->amax = 0u;
    st->amin = 0x7F800000u;  // +inf
    st->err = 0;
    st->total = 0;
}

// residual *= box (pix/pixrmult.f), then ARRSTAT's max/min and PIXRABSH's |.| max/min
__global__ void k_clark_stats(float *res, const float *__restrict__ box, int64_t n, ClarkState *st) {
    float smx = -INFINITY, smn = INFINITY, amx = 0.f, amn = INFINITY;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        float v = res[k];
        if (box) {
            v = __fmul_rn(v, box[k]);
            res[k] = v;
        }
        smx = fmaxf(smx, v);
        smn = fminf(smn, v);
        amx = fmaxf(amx, fabsf(v));
        amn = fminf(amn, fabsf(v));
    }
    for (int d = 16; d > 0; d >>= 1) {
        smx = fmaxf(smx, __shfl_xor_sync(0xffffffffu, smx, d));
        smn = fminf(smn, __shfl_xor_sync(0xffffffffu, smn, d));
        amx = fmaxf(amx, __shfl_xor_sync(0xffffffffu, amx, d));
        amn = fminf(amn, __shfl_xor_sync(0xffffffffu, amn, d));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&st->smax, ord_enc(smx));
        atomicMin(&st->smin, ord_enc(smn));
        atomicMax(&st->amax, __float_as_uint(amx));
        atomicMin(&st->amin, __float_as_uint(amn));
    }
}

// pix/pixrabsh.f:30-38: BASE = min |A|, INCR = (max - min)/(NB - 1), HIST(NINT((|A|-BASE)/INCR))
// += 1.  INDEX 0 lands outside HIST(1..NB) in the reference: those values are in no bin.
__global__ void k_clark_hist(const float *__restrict__ res, int64_t n, ClarkState *st, int *hist) {
    __shared__ int h[CL_NB];
    for (int i = threadIdx.x; i < CL_NB; i += blockDim.x) h[i] = 0;
    const float amax = __uint_as_float(st->amax), amin = __uint_as_float(st->amin);
    const float base = amin, incr = __fdiv_rn(__fsub_rn(amax, amin), (float)(CL_NB - 1));
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->base = base;
        st->incr = incr;
        if (amax == amin) st->err = 1;
    }
    __syncthreads();
    if (amax != amin) {
        for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
             k += (int64_t)gridDim.x * blockDim.x) {
            const int index = (int)roundf(__fdiv_rn(__fsub_rn(fabsf(res[k]), base), incr));
            if (index >= 1 && index <= CL_NB) atomicAdd(&h[index - 1], 1);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < CL_NB; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

// pix/pixflim.f:16-30 (one warp: lane l sums bins 32l..32l+31, a suffix scan over lanes),
// arr/arrflim.f:33 FLIM = INCR*(SLIM-1) + BASE + 0.5*INCR, then img/imgcclea.f:230-236
__global__ void k_clark_limit(const int *__restrict__ hist, int nl, ClarkState *st) {
    const int l = threadIdx.x;
    int part = 0;
    for (int j = 0; j < 32; j++) part += hist[l * 32 + j];
    int suf = part;  // sum of lanes >= l
    for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_down_sync(0xffffffffu, suf, d);
        if (l + d < 32) suf += o;
    }
    // the highest bin i (1-based) whose suffix count reaches nl
    int found = 0;
    const int above = suf - part;  // lanes > l
    if (above < nl && suf >= nl) {
        int t = above;
        for (int j = 31; j >= 0; j--) {
            t += hist[l * 32 + j];
            if (t >= nl) {
                found = l * 32 + j + 1;
                break;
            }
        }
    }
    for (int d = 16; d > 0; d >>= 1) found = max(found, __shfl_xor_sync(0xffffffffu, found, d));
    if (l == 0) {
        const int slimi = found ? found + 1 : 1;
        if (slimi > CL_NB) {
            st->err = 2;  // 'Too many points'
            return;
        }
        float slim = __fadd_rn(__fadd_rn(__fmul_rn(st->incr, (float)(slimi - 1)), st->base), __fmul_rn(0.5f, st->incr));
        if (slim < 0.f) {
            st->err = 3;  // 'Limit in absolute value < 0.0'
            return;
        }
        const float mx = ord_dec(st->smax), mn = ord_dec(st->smin);
        const float maxres = fmaxf(fabsf(mx), fabsf(mn));
        st->maxres = maxres;
        slim = fmaxf(slim, fabsf(__fmul_rn(st->extside, maxres)));
        st->slim = slim;
    }
}

// pix/pix2drli.f: pixels with |A| > SLIM in storage order, the first NL of them.  Block b
// takes pixels [b*CL_CHUNK, (b+1)*CL_CHUNK), thread t 16 consecutive ones.
__global__ void __launch_bounds__(256) k_clark_count(const float *__restrict__ res, int64_t n,
                                                     const ClarkState *st, int *bcount) {
    const float slim = st->slim;
    const int64_t p0 = (int64_t)blockIdx.x * CL_CHUNK + threadIdx.x * 16;
    int c = 0;
    for (int j = 0; j < 16; j++)
        if (p0 + j < n && fabsf(res[p0 + j]) > slim) c++;
    for (int d = 16; d > 0; d >>= 1) c += __shfl_xor_sync(0xffffffffu, c, d);
    __shared__ int w[8];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int i = 0; i < 8; i++) s += w[i];
        bcount[blockIdx.x] = s;
    }
}

// exclusive scan of the block counts (one block of 1024 threads, nb <= 1024 * 16)
__global__ void k_clark_scan(int *bcount, int nb, ClarkState *st, int nl) {
    __shared__ int ws[32];
    const int t = threadIdx.x, per = (nb + 1023) / 1024;
    int loc[16];
    int s = 0;
    for (int j = 0; j < per; j++) {
        const int i = t * per + j;
        loc[j] = i < nb ? bcount[i] : 0;
        s += loc[j];
    }
    int incl = s;
    for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, incl, d);
        if ((t & 31) >= d) incl += o;
    }
    if ((t & 31) == 31) ws[t >> 5] = incl;
    __syncthreads();
    if (t < 32) {
        int v = ws[t];
        for (int d = 1; d < 32; d <<= 1) {
            const int o = __shfl_up_sync(0xffffffffu, v, d);
            if (t >= d) v += o;
        }
        ws[t] = v;
    }
    __syncthreads();
    int run = incl - s + ((t >> 5) ? ws[(t >> 5) - 1] : 0);
    for (int j = 0; j < per; j++) {
        const int i = t * per + j;
        if (i < nb) bcount[i] = run;
        run += loc[j];
    }
    if (t == 1023) {
        st->total = run;
        st->anl = run < nl ? run : nl;
    }
}

__global__ void __launch_bounds__(256) k_clark_emit(const float *__restrict__ res, int64_t n, int nx,
                                                    const ClarkState *st, const int *__restrict__ boff,
                                                    float *al, int *pl, int nl) {
    const float slim = st->slim;
    const int64_t p0 = (int64_t)blockIdx.x * CL_CHUNK + threadIdx.x * 16;
    int c = 0;
    for (int j = 0; j < 16; j++)
        if (p0 + j < n && fabsf(res[p0 + j]) > slim) c++;
    int incl = c;
    for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, incl, d);
        if ((threadIdx.x & 31) >= d) incl += o;
    }
    __shared__ int ws[8];
    if ((threadIdx.x & 31) == 31) ws[threadIdx.x >> 5] = incl;
    __syncthreads();
    int wo = 0;
    for (int i = 0; i < (int)(threadIdx.x >> 5); i++) wo += ws[i];
    int k = boff[blockIdx.x] + wo + incl - c;
    for (int j = 0; j < 16 && k < nl; j++) {
        const int64_t p = p0 + j;
        if (p < n) {
            const float v = res[p];
            if (fabsf(v) > slim) {
                al[k] = v;
                const int ix = (int)(p % nx) + 1, iy = (int)(p / nx) + 1;
                pl[k] = ix | (iy << 16);
                k++;
            }
        }
    }
}

// PIXISAMA key: larger |v| first, then the smaller list index (pix/pixisama.f: the first
// index whose |A| is strictly greater than every earlier one; 1 when all are zero)
__device__ __forceinline__ unsigned long long isama_key(float v, int i) {
    return ((unsigned long long)__float_as_uint(fabsf(v)) << 32) | (unsigned long long)(0xFFFFFFFFu - (unsigned)i);
}

// pix/pix2drcc.f:66-140 with SPEED = 1 and GSUB = BSUB on a cluster of CL_CTAS CTAs.  CTA r
// holds list entries r*CL_SLICE ..; its thread t holds CL_PER consecutive ones (storage order,
// so spatially compact) in registers, their positions in shared memory (entry (t, j) at
// spos[j*CL_T + t]), the beam patch in shared memory when it fits, and the bounding box of
// its entries: an iteration whose beam patch misses the box leaves them alone, and a thread
// rescans its local maximum only after one of its entries changed.  An iteration's argmax
// (PIXISAMA: the largest |v|, then the first index): warp shuffles, one __syncthreads, the
// CTA's best into its slot in CTA 0's shared memory, one cluster barrier, every warp reduces
// the CL_CTAS slots.  Slots alternate between two sets, so no second barrier is needed.
struct ClSlot {
    unsigned long long key;
    float val;
    int pos;
};

__device__ __forceinline__ void slot_max(unsigned long long &k, float &v, int &p, int width) {
    for (int d = width / 2; d > 0; d >>= 1) {
        const unsigned long long ok = __shfl_xor_sync(0xffffffffu, k, d);
        const float ov = __shfl_xor_sync(0xffffffffu, v, d);
        const int op = __shfl_xor_sync(0xffffffffu, p, d);
        if (ok > k) {
            k = ok;
            v = ov;
            p = op;
        }
    }
}

template <bool PSF_SMEM>
__global__ void __cluster_dims__(CL_CTAS, 1, 1) __launch_bounds__(CL_T, 1)
    k_clark_minor(const float *__restrict__ al, const int *__restrict__ pl, ClarkState *st,
                  const float *__restrict__ psf_g, int pw, int ph, float gain, int nsub, int bsub,
                  float flux, float *cl, int *cx, int *cy) {
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    extern __shared__ __align__(16) unsigned char smem[];
    int *spos = reinterpret_cast<int *>(smem);
    float *spsf = reinterpret_cast<float *>(smem + sizeof(int) * CL_SLICE);
    __shared__ unsigned long long skey[2][32];
    __shared__ float sval[2][32];
    __shared__ int spo[2][32];
    __shared__ ClSlot cslot[2][CL_CTAS];  // CTA 0's copy is the cluster's
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int anl = st->anl, base = rank * CL_SLICE;
    float v[CL_PER];
    int bx0 = 0x7FFF, bx1 = -1, by0 = 0x7FFF, by1 = -1;
#pragma unroll
    for (int j = 0; j < CL_PER; j++) {
        const int i = base + t * CL_PER + j;
        const int q = i < anl ? pl[i] : (0x7FFF | (0x7FFF << 16));  // never inside the patch
        v[j] = i < anl ? al[i] : 0.f;
        spos[j * CL_T + t] = q;
        if (i < anl) {
            const int x = q & 0xFFFF, y = q >> 16;
            bx0 = min(bx0, x);
            bx1 = max(bx1, x);
            by0 = min(by0, y);
            by1 = max(by1, y);
        }
    }
    const float *psf = psf_g;
    if (PSF_SMEM) {
        for (int k = t; k < pw * ph; k += CL_T) spsf[k] = psf_g[k];
        psf = spsf;
    }
    ClSlot *c0 = cluster.map_shared_rank(&cslot[0][0], 0);
    cluster.sync();
    const float slim = st->slim;
    const int pmpx = st->pmpx, pmpy = st->pmpy;
    float tflux = st->tflux, smn = 0.f, maxres = 0.f;
    int ansub = nsub, buf = 0;
    unsigned long long lbest = 0ull;
    float lbv = 0.f;
    int lpos = 0;
    bool rescan = true;
    // the cluster's argmax: value into *val, packed position into *pos
    auto argmax = [&](float *val, int *pos) {
        if (rescan) {
            lbest = 0ull;
            lbv = 0.f;
            lpos = 0;
#pragma unroll
            for (int j = 0; j < CL_PER; j++) {
                const unsigned long long k = isama_key(v[j], base + t * CL_PER + j);
                if (k > lbest) {
                    lbest = k;
                    lbv = v[j];
                    lpos = spos[j * CL_T + t];
                }
            }
            rescan = false;
        }
        unsigned long long k = lbest;
        float bv = lbv;
        int bp = lpos;
        slot_max(k, bv, bp, 32);
        if (lane == 0) {
            skey[buf][warp] = k;
            sval[buf][warp] = bv;
            spo[buf][warp] = bp;
        }
        __syncthreads();
        if (warp == 0) {
            k = skey[buf][lane];
            bv = sval[buf][lane];
            bp = spo[buf][lane];
            slot_max(k, bv, bp, 32);
            if (lane == 0) c0[buf * CL_CTAS + rank] = ClSlot{k, bv, bp};
        }
        cluster.sync();
        if (lane < CL_CTAS) {
            const ClSlot c = c0[buf * CL_CTAS + lane];
            k = c.key;
            bv = c.val;
            bp = c.pos;
        } else {
            k = 0ull;
            bv = 0.f;
            bp = 0;
        }
        slot_max(k, bv, bp, 32);
        buf ^= 1;
        *val = bv;
        *pos = bp;
    };
    int isub, pp = 0;
    for (isub = bsub; isub <= abs(nsub); isub++) {
        smn = __fadd_rn(smn, __fdiv_rn(1.0f, (float)isub));
        argmax(&maxres, &pp);
        if ((flux < 0.f && maxres < 0.f) || (nsub < 0 && maxres < 0.f) ||
            fabsf(maxres) <= fmaxf(__fmul_rn(slim, smn), fabsf(flux))) {
            ansub = isub - 1;
            break;
        }
        const float pntsub = __fmul_rn(gain, maxres);
        tflux = __fadd_rn(tflux, pntsub);
        const int pmx = pp & 0xFFFF, pmy = pp >> 16;
        if (rank == 0 && t == 0) {
            cl[isub - 1] = pntsub;
            cx[isub - 1] = pmx;
            cy[isub - 1] = pmy;
        }
        // entry (x, y) is updated when 1 <= offx - x <= pw and 1 <= offy - y <= ph
        const int offx = pmpx + pmx, offy = pmpy + pmy;
        if (bx1 >= offx - pw && bx0 <= offx - 1 && by1 >= offy - ph && by0 <= offy - 1) {
#pragma unroll
            for (int j = 0; j < CL_PER; j++) {
                const int q = spos[j * CL_T + t];
                const int px = offx - (q & 0xFFFF), py = offy - (q >> 16);
                if (px >= 1 && px <= pw && py >= 1 && py <= ph) {
                    v[j] = __fsub_rn(v[j], __fmul_rn(pntsub, psf[(py - 1) * pw + (px - 1)]));
                    rescan = true;
                }
            }
        }
    }
    if (isub > abs(nsub)) argmax(&maxres, &pp);  // pix/pix2drcc.f:133-135
    cluster.sync();  // no CTA leaves while another may still read CTA 0's slots
    if (rank == 0 && t == 0) {
        st->aniter = ansub;
        st->maxres = maxres;
        st->tflux = tflux;
    }
}

// pix/pix2drma.f:17-21: components RITER..ANITER added in list order (one thread keeps it)
__global__ void k_clark_addcomp(const float *cl, const int *cx, const int *cy, int riter, const ClarkState *st,
                                float *comp, int nx, int ny) {
    const int aniter = st->aniter;
    for (int i = riter; i <= aniter; i++) {
        const int ix = cx[i - 1], iy = cy[i - 1];
        if (ix >= 1 && ix <= nx && iy >= 1 && iy <= ny) {
            float *a = comp + (size_t)(iy - 1) * nx + (ix - 1);
            *a = __fadd_rn(*a, cl[i - 1]);
        }
    }
}

// pix/pixxmult.f: MVIS = MVIS * XFR, the complex product in REAL
__global__ void k_clark_cmul(float2 *g, const float2 *__restrict__ x, int nu, int nv, int pitch) {
    const int64_t n = (int64_t)nv * nu;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = k / nu, c = k % nu, o = r * pitch + c;
        const float2 a = g[o], b = x[o];
        g[o] = make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                           __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
    }
}

// pix/pixrsubt.f: RES = DRT - RES
__global__ void k_clark_sub(const float *__restrict__ drt, float *res, int64_t n) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        res[k] = __fsub_rn(drt[k], res[k]);
}

// beam-patch peak (PIXISAMA over the patch, pix/pix2drcc.f:63-66), one block; clears the
// largest |PSF| outside the patch, which k_clark_ext then takes over the whole PSF
__global__ void k_clark_patch(const float *__restrict__ spsf, int pw, ClarkState *st) {
    __shared__ unsigned long long sk[32];
    unsigned long long best = 0ull;
    for (int k = threadIdx.x; k < pw * pw; k += blockDim.x) {
        const unsigned long long key = isama_key(spsf[k], k);
        best = key > best ? key : best;
    }
    for (int d = 16; d > 0; d >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, best, d);
        best = o > best ? o : best;
    }
    if ((threadIdx.x & 31) == 0) sk[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) best = sk[w] > best ? sk[w] : best;
        const int ip = (int)(0xFFFFFFFFu - (unsigned)(best & 0xFFFFFFFFull));
        st->pmpx = 1 + ip % pw;
        st->pmpy = 1 + ip / pw;
        st->extside = 0.f;
        st->tflux = 0.f;
    }
}

// the largest |PSF| outside the patch [b0, b1]^2 (pix/pixrexts.f): blocks over rows, threads
// over columns; the maximum is order-free, so an atomic max on the float's bits (|PSF| >= 0
// orders as an unsigned integer) gives the same value as a sequential scan; NaN is skipped
// as fmaxf would skip it
__global__ void __launch_bounds__(256) k_clark_ext(const float *__restrict__ psf, int n, int b0, int b1,
                                                   ClarkState *st) {
    float ext = 0.f;
    for (int y = blockIdx.x; y < n; y += gridDim.x) {
        const bool inrows = y + 1 >= b0 && y + 1 <= b1;
        const float *row = psf + (size_t)y * n;
        for (int x = threadIdx.x; x < n; x += blockDim.x)
            if (!(inrows && x + 1 >= b0 && x + 1 <= b1)) ext = fmaxf(ext, fabsf(row[x]));
    }
    for (int d = 16; d > 0; d >>= 1) ext = fmaxf(ext, __shfl_xor_sync(0xffffffffu, ext, d));
    if ((threadIdx.x & 31) == 0 && ext > 0.f)
        atomicMax(reinterpret_cast<unsigned int *>(&st->extside), __float_as_uint(ext));
}

int fail(const char *m) {
    sde_set_error("%s", m);
    return SDE_EINVAL;
}

// IMGRESID (img/imgresid.f:13-16) on the transfer function's grid
int clark_resid(sde_ctx *ctx, const float *comp, const float *drt, const float2 *xfr, float2 *mvis, int pitch,
                float *res, int w, int n) {
    const int nu = n / 2 + 1;
    SDE_TRY(sde_grid_from_image(ctx, comp, w, w, n, n, 0, (float *)mvis, pitch));
    {
        KTimer kt(ctx, "clark_cmul");
        k_clark_cmul<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(mvis, xfr, nu, n, pitch);
        SDE_CHECK_LAUNCH();
    }
    SDE_TRY(sde_image_from_grid(ctx, (float *)mvis, pitch, w, w, n, n, 0, nullptr, res));
    KTimer kt(ctx, "clark_sub");
    k_clark_sub<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(drt, res, (int64_t)w * w);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

}  // namespace

extern "C" int sde_clark(sde_ctx *ctx, const float *dirty, const float *psf, int n, const float *box,
                         const sde_clark_params *p, float *comp, float *resid, float *cl, int *cx, int *cy,
                         sde_clark_result *out) {
    if (!ctx || !dirty || !psf || !p || !comp || !resid || !out) return fail("sde_clark: bad arguments");
    memset(out, 0, sizeof *out);
    if (n < 64 || n > 8192 || (n & (n - 1))) return fail("sde_clark: N must be a power of two, 64..8192");
    if (p->niter <= 0) return fail("sde_clark: NITER must be positive");
    if (p->numcl < 1 || p->numcl > CL_MAXNL) return fail("sde_clark: Numcl must be 1..32768");
    if (p->bpatch < 1) return fail("sde_clark: Bpatch must be positive");
    const int biter = p->biter > 0 ? p->biter : 1;
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    // window: CRDHALF with the task's BLC/TRC unset (crd/crdhalf.f:27-35)
    const int blc = n / 4 + 1, w = n / 2;
    const int64_t nw = (int64_t)w * w;
    // beam patch (img/imgsubps.f:28-33) around CRPIX = (N+1)/2 (img/imgmake.f), where
    // IMGMAKEX's phase shift ((N+1)/2 - CRPIX)/N is zero
    const int rp = (n + 1) / 2;
    const int b0 = std::max(1, rp - p->bpatch / 2 + 1), b1 = std::min(n, rp + p->bpatch / 2), pw = b1 - b0 + 1;
    const int nu = n / 2 + 1, pitch = sde_grid_pitch(nu);
    float *drt, *spsf, *al, *lcl = cl;
    float2 *xfr, *mvis;
    int *pl, *hist, *bcount, *lcx = cx, *lcy = cy;
    ClarkState *dst;
    const int nblk = (int)ceil_div(nw, (int64_t)CL_CHUNK);
    SDE_TRY(ctx_scratch(ctx, "clark_drt", sizeof(float) * (size_t)nw, (void **)&drt));
    SDE_TRY(ctx_scratch(ctx, "clark_spsf", sizeof(float) * (size_t)pw * pw, (void **)&spsf));
    SDE_TRY(ctx_scratch(ctx, "clark_al", sizeof(float) * CL_MAXNL, (void **)&al));
    SDE_TRY(ctx_scratch(ctx, "clark_pl", sizeof(int) * CL_MAXNL, (void **)&pl));
    SDE_TRY(ctx_scratch(ctx, "clark_hist", sizeof(int) * CL_NB, (void **)&hist));
    SDE_TRY(ctx_scratch(ctx, "clark_bcount", sizeof(int) * (size_t)nblk, (void **)&bcount));
    SDE_TRY(ctx_scratch(ctx, "clark_state", sizeof(ClarkState), (void **)&dst));
    SDE_TRY(ctx_scratch(ctx, "clark_xfr", sizeof(float2) * (size_t)n * pitch, (void **)&xfr));
    SDE_TRY(ctx_scratch(ctx, "clark_mvis", sizeof(float2) * (size_t)n * pitch, (void **)&mvis));
    if (!lcl) SDE_TRY(ctx_scratch(ctx, "clark_cl", sizeof(float) * (size_t)p->niter, (void **)&lcl));
    if (!lcx) SDE_TRY(ctx_scratch(ctx, "clark_cx", sizeof(int) * (size_t)p->niter, (void **)&lcx));
    if (!lcy) SDE_TRY(ctx_scratch(ctx, "clark_cy", sizeof(int) * (size_t)p->niter, (void **)&lcy));
    if (nblk > 1024 * 16) return fail("sde_clark: window too large");
    // the window of the dirty image, the beam patch, the transfer function (IMGMAKEX)
    SDE_CUDA_TRY(cudaMemcpy2DAsync(drt, sizeof(float) * w, dirty + (size_t)(blc - 1) * n + (blc - 1),
                                   sizeof(float) * n, sizeof(float) * w, w, cudaMemcpyDeviceToDevice, st));
    SDE_CUDA_TRY(cudaMemcpy2DAsync(spsf, sizeof(float) * pw, psf + (size_t)(b0 - 1) * n + (b0 - 1),
                                   sizeof(float) * n, sizeof(float) * pw, pw, cudaMemcpyDeviceToDevice, st));
    SDE_TRY(sde_grid_from_image(ctx, psf, n, n, n, n, 0, (float *)xfr, pitch));
    k_clark_patch<<<1, 1024, 0, st>>>(spsf, pw, dst);
    k_clark_ext<<<std::min(n, ctx->num_sms * 8), 256, 0, st>>>(psf, n, b0, b1, dst);
    SDE_CHECK_LAUNCH();
    // minor-cycle kernel: positions (+ beam patch when it fits) in shared memory
    const size_t sm_pos = sizeof(int) * CL_SLICE, sm_psf = sizeof(float) * (size_t)pw * pw;
    const bool psf_smem = sm_pos + sm_psf <= 200u * 1024u;
    const size_t sm = sm_pos + (psf_smem ? sm_psf : 0);
    if (psf_smem)
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_clark_minor<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    else
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_clark_minor<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    ClarkState h{};
    int riter = biter, aniter = biter - 1, rc = SDE_OK;
    float tflux = 0.f;
    SDE_TRY(clark_resid(ctx, comp, drt, xfr, mvis, pitch, resid, w, n));
    const int gsz = ctx->num_sms * 4;
    for (;;) {
        k_clark_init<<<1, 1, 0, st>>>(dst);
        SDE_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(int) * CL_NB, st));
        {
            KTimer kt(ctx, "clark_select");
            k_clark_stats<<<gsz, 256, 0, st>>>(resid, box, nw, dst);
            k_clark_hist<<<gsz, 256, 0, st>>>(resid, nw, dst, hist);
            k_clark_limit<<<1, 32, 0, st>>>(hist, p->numcl, dst);
            k_clark_count<<<nblk, 256, 0, st>>>(resid, nw, dst, bcount);
            k_clark_scan<<<1, 1024, 0, st>>>(bcount, nblk, dst, p->numcl);
            k_clark_emit<<<nblk, 256, 0, st>>>(resid, nw, w, dst, bcount, al, pl, p->numcl);
            SDE_CHECK_LAUNCH();
        }
        SDE_CUDA_TRY(cudaMemcpyAsync(&h, dst, sizeof h, cudaMemcpyDeviceToHost, st));
        SDE_CUDA_TRY(cudaStreamSynchronize(st));
        if (h.err == 1) { sde_set_error("Zero range in values"); rc = SDE_EINVAL; break; }
        if (h.err == 2) { sde_set_error("Too many points"); rc = SDE_EINVAL; break; }
        if (h.err == 3) { sde_set_error("Limit in absolute value < 0.0"); rc = SDE_EINVAL; break; }
        out->last_anl = h.anl;
        out->last_slim = h.slim;
        if (h.anl == 0) break;  // PIX2DRCC would read DRTL(1), never written: nothing to subtract
        {
            KTimer kt(ctx, "clark_minor");
            ClarkState *d = dst;
            // TFLUX carries over the cycles (img/imgcclea.f:251)
            SDE_CUDA_TRY(cudaMemcpyAsync(&d->tflux, &tflux, sizeof(float), cudaMemcpyHostToDevice, st));
            if (psf_smem)
                k_clark_minor<true><<<CL_CTAS, CL_T, sm, st>>>(al, pl, dst, spsf, pw, pw, p->gain, p->niter, riter, p->flux,
                                                         lcl, lcx, lcy);
            else
                k_clark_minor<false><<<CL_CTAS, CL_T, sm, st>>>(al, pl, dst, spsf, pw, pw, p->gain, p->niter, riter,
                                                          p->flux, lcl, lcx, lcy);
            SDE_CHECK_LAUNCH();
            k_clark_addcomp<<<1, 1, 0, st>>>(lcl, lcx, lcy, riter, dst, comp, w, w);
            SDE_CHECK_LAUNCH();
        }
        SDE_TRY(clark_resid(ctx, comp, drt, xfr, mvis, pitch, resid, w, n));
        SDE_CUDA_TRY(cudaMemcpyAsync(&h, dst, sizeof h, cudaMemcpyDeviceToHost, st));
        SDE_CUDA_TRY(cudaStreamSynchronize(st));
        aniter = h.aniter;
        tflux = h.tflux;
        if (out->ncycles < SDE_CLARK_TRACE) {
            out->t_anl[out->ncycles] = h.anl;
            out->t_aniter[out->ncycles] = aniter;
            out->t_maxres[out->ncycles] = h.maxres;
            out->t_tflux[out->ncycles] = tflux;
        }
        out->ncycles++;
        riter = aniter + 1;
        if (h.maxres <= 0.f && p->flux <= 0.f) break;
        if (!(fabsf(h.maxres) > p->flux && aniter < p->niter)) break;
    }
    out->aniter = aniter;
    out->maxres = h.maxres;
    out->tflux = tflux;
    out->extside = h.extside;
    out->window = w;
    out->blc = blc;
    return rc;
}
