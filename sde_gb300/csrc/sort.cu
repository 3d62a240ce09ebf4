// sort.cu -- device-wide scans and a stable LSD radix sort (8-bit digits).
//
// Stability matters: the weight-density counts of GRDUWT2D/GRDRUW2D are sequential FP32
// sums in visibility order (grd/grduwt2d.f:114), so the per-cell sums are reproduced
// bit-exactly by sorting (cell, weight) pairs stably and summing each cell's run in order.
#include "common.cuh"

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

struct OpAdd {
    __device__ __forceinline__ uint32_t operator()(uint32_t a, uint32_t b) const { return a + b; }
};
struct OpMax {
    __device__ __forceinline__ int32_t operator()(int32_t a, int32_t b) const { return a > b ? a : b; }
};

// Block scan of SCAN_TILE items; writes per-block aggregate to block_sums when given.
template <typename T, class Op>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_block(const T *in, T *out, int64_t n,
                                                               T *block_sums, T identity,
                                                               int inclusive) {
    __shared__ T sh[SCAN_TILE];
    __shared__ T warp_tot[SCAN_THREADS / 32];
    Op op;
    const int t = threadIdx.x;
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    for (int r = 0; r < SCAN_ITEMS; r++) {
        int64_t i = base + r * SCAN_THREADS + t;
        sh[r * SCAN_THREADS + t] = i < n ? in[i] : identity;
    }
    __syncthreads();
    T v[SCAN_ITEMS];
    T acc = identity;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = sh[t * SCAN_ITEMS + k];
        acc = op(acc, v[k]);
    }
    // warp-level inclusive scan of the thread aggregates
    const int lane = t & 31, warp = t >> 5;
    T x = acc;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x = op(y, x);
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T wv = lane < SCAN_THREADS / 32 ? warp_tot[lane] : identity;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, wv, d);
            if (lane >= d) wv = op(y, wv);
        }
        if (lane < SCAN_THREADS / 32) warp_tot[lane] = wv;
    }
    __syncthreads();
    T excl_thread = __shfl_up_sync(0xffffffffu, x, 1);
    if (lane == 0) excl_thread = identity;
    if (warp > 0) excl_thread = op(warp_tot[warp - 1], excl_thread);
    T run = excl_thread;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        T nxt = op(run, v[k]);
        sh[t * SCAN_ITEMS + k] = inclusive ? nxt : run;
        run = nxt;
    }
    if (block_sums && t == SCAN_THREADS - 1) block_sums[blockIdx.x] = run;
    __syncthreads();
    for (int r = 0; r < SCAN_ITEMS; r++) {
        int64_t i = base + r * SCAN_THREADS + t;
        if (i < n) out[i] = sh[r * SCAN_THREADS + t];
    }
}

template <typename T, class Op>
__global__ void k_scan_add(T *out, int64_t n, const T *block_prefix) {
    Op op;
    int64_t i = (int64_t)blockIdx.x * SCAN_TILE + threadIdx.x;
    T p = block_prefix[blockIdx.x];
    for (int r = 0; r < SCAN_ITEMS; r++, i += SCAN_THREADS)
        if (i < n) out[i] = op(p, out[i]);
}

template <typename T, class Op>
int scan_impl(sde_ctx *ctx, const T *in, T *out, int64_t n, T identity, int inclusive,
              int depth) {
    if (n <= 0) return SDE_OK;
    int nb = ceil_div(n, SCAN_TILE);
    if (nb == 1) {
        k_scan_block<T, Op><<<1, SCAN_THREADS, 0, ctx->stream>>>(in, out, n, nullptr, identity,
                                                                 inclusive);
        SDE_CHECK_LAUNCH();
        return SDE_OK;
    }
    char name[32];
    snprintf(name, sizeof name, "scan_bs%d", depth);
    T *bs = nullptr;
    SDE_TRY(ctx_scratch(ctx, name, sizeof(T) * (size_t)nb, (void **)&bs));
    k_scan_block<T, Op><<<nb, SCAN_THREADS, 0, ctx->stream>>>(in, out, n, bs, identity,
                                                              inclusive);
    SDE_CHECK_LAUNCH();
    // exclusive prefix of the block aggregates
    SDE_TRY((scan_impl<T, Op>(ctx, bs, bs, nb, identity, 0, depth + 1)));
    k_scan_add<T, Op><<<nb, SCAN_THREADS, 0, ctx->stream>>>(out, n, bs);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

__global__ void k_last_plus(const uint32_t *in, const uint32_t *scanned, int64_t n,
                            uint32_t *total) {
    *total = scanned[n - 1] + in[n - 1];
}

// ---------------------------------------------------------------------------------------
// Radix sort.  Each pass: per-block digit counts (k_rs_hist), one exclusive scan of the
// digit-major count table (the global start of every (digit, block) run), and a scatter
// that ranks the block's items stably in shared memory and writes each digit's run of the
// block as consecutive addresses.
constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ROUNDS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;   // items per block
constexpr int RS_WARP_ITEMS = RS_TILE / RS_WARPS;  // contiguous items per warp

template <typename K>
__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const K *keys, int64_t n, int shift,
                                                         uint32_t *hist, int nb) {
    // one count table per warp: items of one digit arrive together in the later passes
    __shared__ uint32_t h[RS_WARPS][256];
    const int t = threadIdx.x, warp = t >> 5;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) h[w][t] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RS_TILE;
    // all of the thread's loads before the first count
    K k[RS_ROUNDS];
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        const int64_t i = base + r * RS_THREADS + t;
        k[r] = i < n ? keys[i] : (K)0;
    }
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++)
        if (base + r * RS_THREADS + t < n) atomicAdd(&h[warp][(uint32_t)(k[r] >> shift) & 255u], 1u);
    __syncthreads();
    uint32_t c = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) c += h[w][t];
    hist[(int64_t)t * nb + blockIdx.x] = c;
}

// Scatter of one pass, for keys in any order: the block's RS_TILE items are ranked stably in
// shared memory (warp w ranks its RS_WARP_ITEMS consecutive items round by round; item order
// is (warp, round, lane)), and each digit's run of the block is written to consecutive
// addresses.
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter_ranked(const uint32_t *kin, const uint32_t *vin,
                                                                   uint32_t *kout, uint32_t *vout, int64_t n,
                                                                   int shift, const uint32_t *offs, int nb) {
    __shared__ uint32_t wcnt[RS_WARPS][256];  // per-warp digit counts, then the warp's offsets
    __shared__ uint32_t dstart[256];          // the digit's first position in the block
    __shared__ uint32_t gbase[256];           // the digit's first position in the output
    __shared__ uint32_t wtot[RS_WARPS];
    __shared__ uint32_t kbuf[RS_TILE], vbuf[RS_TILE];  // the block's items in (digit, item) order
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) wcnt[w][t] = 0;
    gbase[t] = offs[(int64_t)t * nb + blockIdx.x];
    const int64_t wbase = (int64_t)blockIdx.x * RS_TILE + (int64_t)warp * RS_WARP_ITEMS;
    uint32_t key[RS_ROUNDS], val[RS_ROUNDS], pos[RS_ROUNDS];
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        const int64_t i = wbase + r * 32 + lane;
        key[r] = i < n ? kin[i] : 0u;
        val[r] = i < n ? vin[i] : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        const bool valid = wbase + r * 32 + lane < n;
        const uint32_t digit = valid ? ((key[r] >> shift) & 255u) : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, digit);
        const uint32_t before = valid ? wcnt[warp][digit] : 0u;
        pos[r] = before + __popc(peers & lt);
        __syncwarp();
        if (valid && (peers & lt) == 0) wcnt[warp][digit] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // digit t: offsets of the warps' runs within the digit, and the digit's total
    {
        uint32_t acc = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) {
            const uint32_t c = wcnt[w][t];
            wcnt[w][t] = acc;
            acc += c;
        }
        // block-wide exclusive scan of the digit totals
        uint32_t x = acc;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) wtot[warp] = x;
        __syncthreads();
        uint32_t pre = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) pre += w < warp ? wtot[w] : 0u;
        dstart[t] = pre + x - acc;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        if (wbase + r * 32 + lane < n) {
            const uint32_t digit = (key[r] >> shift) & 255u;
            const uint32_t p = dstart[digit] + wcnt[warp][digit] + pos[r];
            kbuf[p] = key[r];
            vbuf[p] = val[r];
        }
    }
    __syncthreads();
    const int nblk = (int)min((int64_t)RS_TILE, n - (int64_t)blockIdx.x * RS_TILE);
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        const int p = r * RS_THREADS + t;
        if (p < nblk) {
            const uint32_t k = kbuf[p];
            const uint32_t digit = (k >> shift) & 255u;
            const uint32_t d = gbase[digit] + (uint32_t)p - dstart[digit];
            kout[d] = k;
            vout[d] = vbuf[p];
        }
    }
}

// Scatter of one pass, round by round through the block (items of one digit in a round go
// to consecutive addresses): the 64-bit keys' pass (the chunk sort, a few million items),
// whose keys and values would not fit k_rs_scatter_ranked's shared memory.
template <typename K>
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const K *kin, const uint32_t *vin,
                                                            K *kout, uint32_t *vout, int64_t n,
                                                            int shift, const uint32_t *offs,
                                                            int nb) {
    __shared__ uint32_t run[256];
    __shared__ uint32_t wcnt[RS_THREADS / 32][256];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    run[t] = offs[(int64_t)t * nb + blockIdx.x];
    const int64_t base = (int64_t)blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; r++) {
#pragma unroll
        for (int w = 0; w < RS_THREADS / 32; w++) wcnt[w][t] = 0;
        __syncthreads();
        int64_t i = base + r * RS_THREADS + t;
        bool valid = i < n;
        K key = valid ? kin[i] : (K)0;
        uint32_t val = valid ? vin[i] : 0u;
        uint32_t digit = valid ? ((uint32_t)(key >> shift) & 255u) : 256u;
        uint32_t peers = __match_any_sync(0xffffffffu, digit);
        int leader = __ffs(peers) - 1;
        uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && lane == leader) wcnt[warp][digit] = __popc(peers);
        __syncthreads();
        {
            uint32_t acc = run[t];
#pragma unroll
            for (int w = 0; w < RS_THREADS / 32; w++) {
                uint32_t c = wcnt[w][t];
                wcnt[w][t] = acc;
                acc += c;
            }
            run[t] = acc;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = wcnt[warp][digit] + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
    }
}

template <typename K>
int radix_sort(sde_ctx *ctx, K *keys, uint32_t *vals, int64_t n, int bits, K *ktmp,
               uint32_t *vtmp) {
    if (n <= 1) return SDE_OK;
    if (n >= (int64_t)0xFFFFFFFF) {
        sde_set_error("radix sort: %lld items exceeds 32-bit offsets", (long long)n);
        return SDE_EINVAL;
    }
    int nb = ceil_div(n, RS_TILE);
    uint32_t *hist = nullptr;
    SDE_TRY(ctx_scratch(ctx, "rs_hist", sizeof(uint32_t) * 256 * (size_t)nb, (void **)&hist));
    int passes = (bits + 7) / 8;
    K *src_k = keys, *dst_k = ktmp;
    uint32_t *src_v = vals, *dst_v = vtmp;
    for (int p = 0; p < passes; p++) {
        int shift = 8 * p;
        k_rs_hist<K><<<nb, RS_THREADS, 0, ctx->stream>>>(src_k, n, shift, hist, nb);
        SDE_CHECK_LAUNCH();
        SDE_TRY((scan_impl<uint32_t, OpAdd>(ctx, hist, hist, (int64_t)256 * nb, 0u, 0, 0)));
        if (sizeof(K) == 4)
            k_rs_scatter_ranked<<<nb, RS_THREADS, 0, ctx->stream>>>(
                reinterpret_cast<const uint32_t *>(src_k), src_v, reinterpret_cast<uint32_t *>(dst_k),
                dst_v, n, shift, hist, nb);
        else
            k_rs_scatter<K><<<nb, RS_THREADS, 0, ctx->stream>>>(src_k, src_v, dst_k, dst_v, n, shift,
                                                                 hist, nb);
        SDE_CHECK_LAUNCH();
        K *tk = src_k; src_k = dst_k; dst_k = tk;
        uint32_t *tv = src_v; src_v = dst_v; dst_v = tv;
    }
    if (src_k != keys) {
        SDE_CUDA_TRY(cudaMemcpyAsync(keys, src_k, sizeof(K) * (size_t)n, cudaMemcpyDeviceToDevice,
                                     ctx->stream));
        SDE_CUDA_TRY(cudaMemcpyAsync(vals, src_v, sizeof(uint32_t) * (size_t)n,
                                     cudaMemcpyDeviceToDevice, ctx->stream));
    }
    return SDE_OK;
}

}  // namespace

int launch_exclusive_scan_u32(sde_ctx *ctx, const uint32_t *in, uint32_t *out, int64_t n,
                              uint32_t *total_dev) {
    if (n <= 0) {
        if (total_dev) SDE_CUDA_TRY(cudaMemsetAsync(total_dev, 0, sizeof(uint32_t), ctx->stream));
        return SDE_OK;
    }
    if (total_dev && in == out) {
        sde_set_error("exclusive scan with total needs distinct in/out");
        return SDE_EINVAL;
    }
    SDE_TRY((scan_impl<uint32_t, OpAdd>(ctx, in, out, n, 0u, 0, 0)));
    if (total_dev) {
        k_last_plus<<<1, 1, 0, ctx->stream>>>(in, out, n, total_dev);
        SDE_CHECK_LAUNCH();
    }
    return SDE_OK;
}

int launch_inclusive_max_scan_i32(sde_ctx *ctx, const int32_t *in, int32_t *out, int64_t n) {
    return scan_impl<int32_t, OpMax>(ctx, in, out, n, (int32_t)INT32_MIN, 1, 100);
}

int launch_radix_sort_u32(sde_ctx *ctx, uint32_t *keys, uint32_t *vals, int64_t n, int bits,
                          uint32_t *keys_tmp, uint32_t *vals_tmp) {
    return radix_sort<uint32_t>(ctx, keys, vals, n, bits, keys_tmp, vals_tmp);
}

int launch_radix_sort_u64(sde_ctx *ctx, uint64_t *keys, uint32_t *vals, int64_t n, int bits,
                          uint64_t *keys_tmp, uint32_t *vals_tmp) {
    return radix_sort<uint64_t>(ctx, keys, vals, n, bits, keys_tmp, vals_tmp);
}
