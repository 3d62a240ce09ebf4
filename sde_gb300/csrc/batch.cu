// batch.cu -- many plans imaged together: the pointings of a mosaic (task/mosclean.f images
// each pointing, then forms the linear mosaic, task/mosclean.f:413-432) and batches of
// served imaging jobs.
//
// The batch owns, in one device allocation, a raw and a final grid, a PSF image and a dirty
// image per plan.  Dirty imaging of the whole batch is: one persistent gridding launch over
// the combined work-item list of all plans (k_grid_batch), one batched finalize, and per
// shape class (plans with the same grid and image size) one batched column FFT and one
// batched row c2r with grid correction and the PSF-peak normalisation of uvmap
// (task/uvmap.f:473-483).  The mosaic adds each pointing's primary-beam-weighted image and
// weight into a numerator and a denominator and divides.  Because the launch sequence of a
// batch never changes, it is captured once into a CUDA graph and replayed.
#include <algorithm>
#include <map>
#include <tuple>
#include <vector>

#include "common.cuh"

namespace {

struct MosaicPointing {
    const float *image;  // dirty image of the pointing (nx x ny, row-major)
    int nx, ny;
    int cx, cy;          // mosaic pixel of the image centre pixel ((n+1)/2, 1-based)
    float pbk;           // 4 ln2 / FWHM^2 (FWHM in pixels): PB = exp(-pbk r^2)
    float wt;            // pointing weight (SUMWT of the pointing)
    int64_t block0;      // first block of this pointing in the flattened launches
};

// Flattened over the pointings' pixels: blk[b] = the pointing of block b, 1024 pixels per
// block.  The primary beam of a pixel of pointing p and its mosaic pixel.
struct MosaicPixel {
    bool in;
    int64_t m;  // mosaic index
    float pb;
    int64_t k;  // pixel of the pointing's image
};
__device__ __forceinline__ MosaicPixel mosaic_pixel(const MosaicPointing &p, int64_t k, int mnx, int mny) {
    MosaicPixel r{false, 0, 0.f, k};
    if (k >= (int64_t)p.nx * p.ny) return r;
    const int cenx = (p.nx + 1) / 2 - 1, ceny = (p.ny + 1) / 2 - 1;
    const int iy = (int)(k / p.nx), ix = (int)(k - (int64_t)iy * p.nx);
    const int mx = p.cx - 1 + ix - cenx, my = p.cy - 1 + iy - ceny;
    if (mx < 0 || mx >= mnx || my < 0 || my >= mny) return r;
    const float dx = (float)(ix - cenx), dy = (float)(iy - ceny);
    r.in = true;
    r.m = (int64_t)my * mnx + mx;
    r.pb = expf(-p.pbk * (dx * dx + dy * dy));
    return r;
}

// den += wt PB^2 (the denominator; once per layout)
__global__ void __launch_bounds__(256) k_mosaic_den(const MosaicPointing *__restrict__ pts,
                                                    const uint16_t *__restrict__ blk, int mnx, int mny,
                                                    float *den) {
    const MosaicPointing p = pts[blk[blockIdx.x]];
    const int64_t base = (int64_t)(blockIdx.x - p.block0) * BATCH_BLOCK_CELLS;
#pragma unroll
    for (int j = 0; j < BATCH_BLOCK_CELLS / 256; j++) {
        const MosaicPixel q = mosaic_pixel(p, base + j * 256 + threadIdx.x, mnx, mny);
        if (q.in) atomicAdd(&den[q.m], p.wt * q.pb * q.pb);
    }
}

// den -> 1/den where den > clip * max(den), else 0 (in place)
__global__ void k_mosaic_invden(float *den, int64_t n, const float *__restrict__ denmax, float clip) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float d = den[k];
    den[k] = (d > 0.f && d > clip * *denmax) ? 1.0f / d : 0.f;
}

// The mosaic by gather: block = one MOS_TILE x MOS_TILE tile of the mosaic; every pixel sums
// wt PB I over the tile's pointings (in pointing order) and takes the stored 1/den.  The
// tile's pointing descriptors are staged in shared memory, and pointings are taken two at a
// time with both images' loads issued before either is added (the sum keeps pointing order).
constexpr int MOS_TILE = 64;
constexpr int MOS_STAGE = 64;  // pointings of a tile staged in shared memory
// mosaic pixel (tx, ty, k) in image p: the 0-based image pixel, false when outside the image
__device__ __forceinline__ bool mos_pix(const MosaicPointing &p, int tx, int ty, int k, int *ix, int *iy) {
    const int ox = p.cx - 1 - ((p.nx + 1) / 2 - 1), oy = p.cy - 1 - ((p.ny + 1) / 2 - 1);
    *ix = tx * MOS_TILE + (k & (MOS_TILE - 1)) - ox;
    *iy = ty * MOS_TILE + k / MOS_TILE - oy;
    return *ix >= 0 && *ix < p.nx && *iy >= 0 && *iy < p.ny;
}

// the image values of the thread's pixels (0 outside the image); loads only, so that both
// pointings' loads are in flight before any is used
__device__ __forceinline__ void mos_load(const MosaicPointing &p, int tx, int ty, float *val) {
    constexpr int PER = MOS_TILE * MOS_TILE / 256;
#pragma unroll
    for (int j = 0; j < PER; j++) {
        int ix, iy;
        val[j] = mos_pix(p, tx, ty, threadIdx.x + j * 256, &ix, &iy) ? p.image[(int64_t)iy * p.nx + ix] : 0.f;
    }
}

// acc += wt PB I over the thread's pixels inside image p
__device__ __forceinline__ void mos_add(const MosaicPointing &p, int tx, int ty, const float *val, float *acc) {
    constexpr int PER = MOS_TILE * MOS_TILE / 256;
    const int cenx = (p.nx + 1) / 2 - 1, ceny = (p.ny + 1) / 2 - 1;
#pragma unroll
    for (int j = 0; j < PER; j++) {
        int ix, iy;
        if (!mos_pix(p, tx, ty, threadIdx.x + j * 256, &ix, &iy)) continue;
        const float dx = (float)(ix - cenx), dy = (float)(iy - ceny);
        const float pb = expf(-p.pbk * (dx * dx + dy * dy));
        acc[j] += p.wt * pb * val[j];
    }
}

__global__ void __launch_bounds__(256, 3) k_mosaic_gather(const MosaicPointing *__restrict__ pts,
                                                       const int32_t *__restrict__ tstart,
                                                       const uint16_t *__restrict__ tpts, int mtx, int mnx,
                                                       int mny, const float *__restrict__ invden, float *out) {
    __shared__ MosaicPointing sp[MOS_STAGE];
    const int tx = blockIdx.x % mtx, ty = blockIdx.x / mtx;
    const int p0 = tstart[blockIdx.x], cnt = tstart[blockIdx.x + 1] - p0;
    for (int i = threadIdx.x; i < cnt && i < MOS_STAGE; i += blockDim.x) sp[i] = pts[tpts[p0 + i]];
    __syncthreads();
    constexpr int PER = MOS_TILE * MOS_TILE / 256;
    float acc[PER];
#pragma unroll
    for (int j = 0; j < PER; j++) acc[j] = 0.f;
    for (int pi = 0; pi < cnt; pi += 2) {
        const MosaicPointing pa = pi < MOS_STAGE ? sp[pi] : pts[tpts[p0 + pi]];
        float va[PER], vb[PER];
        mos_load(pa, tx, ty, va);
        if (pi + 1 < cnt) {
            const MosaicPointing pb = pi + 1 < MOS_STAGE ? sp[pi + 1] : pts[tpts[p0 + pi + 1]];
            mos_load(pb, tx, ty, vb);
            mos_add(pa, tx, ty, va, acc);
            mos_add(pb, tx, ty, vb, acc);
        } else {
            mos_add(pa, tx, ty, va, acc);
        }
    }
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const int k = threadIdx.x + j * 256;
        const int mx = tx * MOS_TILE + (k & (MOS_TILE - 1)), my = ty * MOS_TILE + k / MOS_TILE;
        if (mx >= mnx || my >= mny) continue;
        const int64_t m = (int64_t)my * mnx + mx;
        out[m] = acc[j] * invden[m];
    }
}

__global__ void k_max_batch(float *const *__restrict__ images, const int64_t *__restrict__ npix,
                                float *out) {
    // one CTA per image: max over the image (the PSF peak of uvmap, task/uvmap.f:424-441)
    const float *im = images[blockIdx.x];
    const int64_t n = npix[blockIdx.x];
    float m = -INFINITY;
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) m = fmaxf(m, im[k]);
    for (int d = 16; d > 0; d >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, d));
    __shared__ float sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < blockDim.x / 32 ? sm[threadIdx.x] : -INFINITY;
        for (int d = 16; d > 0; d >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, d));
        if (threadIdx.x == 0) out[blockIdx.x] = m;
    }
}

// max of a non-negative array, many CTAs: block maxima meet through atomicMax on the float
// bit patterns (for x >= 0 the IEEE order is the unsigned-integer order); *out starts at 0
__global__ void k_max_nonneg(const float *__restrict__ v, int64_t n, unsigned int *out) {
    float m = 0.f;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        m = fmaxf(m, v[k]);
    for (int d = 16; d > 0; d >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, d));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

}  // namespace

struct sde_batch {
    sde_ctx *ctx = nullptr;
    int n = 0;
    std::vector<sde_plan *> plans;
    std::vector<int> nx, ny;
    std::vector<float2 *> raw, grid;
    std::vector<float *> psf, image;
    float *d_peak = nullptr;                   // PSF peak per plan
    BatchPlan *d_plans = nullptr;
    int64_t *d_item_start = nullptr;
    unsigned long long *d_counter = nullptr;
    FinalizeDesc *d_fin = nullptr;
    uint16_t *d_fin_blk = nullptr;             // grid of each block of the flattened finalize
    int64_t fin_nblk = 0;                      // (plans whose shape has no fused column pass)
    std::vector<FinalizeDesc> hfin;            // host copy: the fused column passes' parameters
    int2 *d_fold = nullptr;                    // (plan, core) pairs of the compensation fold
    int64_t fold_n = 0;
    float **d_psf_ptrs = nullptr;
    int64_t *d_npix = nullptr;
    int64_t max_cells = 0;
    // raw grids: every plan's hi plane, contiguous from raw[0] (hi_bytes), then (comp) every
    // plan's compensation plane; raw_bytes covers both
    size_t raw_bytes = 0, hi_bytes = 0;
    bool comp = true;                          // compensated cross-item sums (raw_lo planes)
    bool lo_clean = false;                     // compensation planes all zero (folded)
    // shape class (fnu, nv, nx, ny, pitch) -> plan indices
    std::map<std::tuple<int, int, int, int, int>, std::vector<int>> classes;
    // mosaic
    int mnx = 0, mny = 0;
    float clip = 0.f;
    MosaicPointing *d_pts = nullptr;
    uint16_t *d_pts_blk = nullptr;             // pointing of each block of the mosaic launches
    int64_t pts_nblk = 0;
    // per MOS_TILE x MOS_TILE mosaic tile, the pointings whose image covers it (CSR)
    int mtx = 0, mty = 0;
    int32_t *d_tile_start = nullptr;
    uint16_t *d_tile_pts = nullptr;
    // num = sum wt PB I (per pass); invden = 1 / sum wt PB^2 where that sum passes the clip,
    // else 0 (fixed by the layout: computed once in sde_batch_set_mosaic)
    float *d_num = nullptr, *d_invden = nullptr, *d_denmax = nullptr, *d_mosaic = nullptr;
    // graph of sde_batch_dirty (+ mosaic)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap = nullptr;  // capture stream (the caller's may be the legacy default one)
    int graph_nodes = 0;
    int eager_runs = 0;
    std::vector<void *> allocs;
    std::vector<size_t> alloc_bytes;
    int64_t bytes = 0;
};

namespace {

int batch_alloc(sde_batch *b, void **p, size_t bytes) {
    bytes = (bytes + 255) & ~(size_t)255;
    SDE_TRY(ctx_alloc(b->ctx, p, bytes));
    b->allocs.push_back(*p);
    b->alloc_bytes.push_back(bytes);
    b->bytes += (int64_t)bytes;
    b->ctx->bytes += (int64_t)bytes;
    return SDE_OK;
}

// the launches of one gridding pass of every plan (PSF or visibilities)
// The compensation planes are written only inside the plans' marked cores and the fold
// zeroes what it adds, so after the first pass only the hi planes are cleared.  Grids of a
// shape with a fused column pass are finalized inside it (batch_fft).
int batch_grid(sde_batch *b, int psf) {
    sde_ctx *ctx = b->ctx;
    SDE_CUDA_TRY(cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned long long), ctx->stream));
    SDE_CUDA_TRY(cudaMemsetAsync(b->raw[0], 0, b->lo_clean ? b->hi_bytes : b->raw_bytes, ctx->stream));
    b->lo_clean = false;
    SDE_TRY(launch_grid_batch(ctx, psf, b->comp, b->d_plans, b->d_item_start, b->n, b->d_counter,
                              ctx->d_cft, ctx->num_sms * grid_ctas_per_sm()));
    if (b->comp) {
        SDE_TRY(launch_fold_lo_batch(ctx, b->d_plans, b->d_fold, b->fold_n));
        b->lo_clean = true;
    }
    SDE_TRY(launch_finalize_batch(ctx, b->d_fin, b->d_fin_blk, b->fin_nblk));
    return SDE_OK;
}

// grid -> image for every shape class; scale by 1/peak when peaks != NULL
int batch_fft(sde_batch *b, const std::vector<float *> &out, const float *peaks) {
    for (auto &kv : b->classes) {
        const int fnu = std::get<0>(kv.first), nv = std::get<1>(kv.first);
        const int nx = std::get<2>(kv.first), ny = std::get<3>(kv.first), pitch = std::get<4>(kv.first);
        if (fin_fused_shape(fnu / 2 + 1, nv)) {
            std::vector<FinalizeDesc> fd;
            std::vector<float *> im;
            std::vector<const float *> sc;
            for (int i : kv.second) {
                fd.push_back(b->hfin[i]);
                im.push_back(out[i]);
                sc.push_back(peaks ? peaks + i : nullptr);
            }
            SDE_TRY(fft_images_from_raw(b->ctx, (int)fd.size(), fd.data(), im.data(),
                                        peaks ? sc.data() : nullptr, nx, ny, 1));
            continue;
        }
        std::vector<float2 *> g;
        std::vector<float *> im;
        std::vector<const float *> sc;
        for (int i : kv.second) {
            g.push_back(b->grid[i]);
            im.push_back(out[i]);
            sc.push_back(peaks ? peaks + i : nullptr);
        }
        int rc = fft_images_from_grids(b->ctx, (int)g.size(), g.data(), im.data(),
                                       peaks ? sc.data() : nullptr, pitch, nx, ny, fnu, nv, 1);
        if (rc == SDE_EINVAL) {
            // no batched instance for this shape: one transform at a time
            for (size_t k = 0; k < g.size(); k++)
                SDE_TRY(sde_image_from_grid(b->ctx, (float *)g[k], pitch, nx, ny, fnu, nv, 1, sc[k],
                                            im[k]));
        } else {
            SDE_TRY(rc);
        }
    }
    return SDE_OK;
}

int batch_mosaic(sde_batch *b) {
    if (!b->d_pts) return SDE_OK;
    sde_ctx *ctx = b->ctx;
    KTimer kt(ctx, "mosaic_gather");
    k_mosaic_gather<<<(unsigned)(b->mtx * b->mty), 256, 0, ctx->stream>>>(
        b->d_pts, b->d_tile_start, b->d_tile_pts, b->mtx, b->mnx, b->mny, b->d_invden, b->d_mosaic);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

int batch_dirty_launches(sde_batch *b) {
    SDE_TRY(batch_grid(b, 0));
    SDE_TRY(batch_fft(b, b->image, b->d_peak));
    SDE_TRY(batch_mosaic(b));
    return SDE_OK;
}

void batch_drop_graph(sde_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_nodes = 0;
}

}  // namespace

extern "C" int sde_batch_create(sde_ctx *ctx, int n, sde_plan *const *plans, const int *nx,
                                const int *ny, sde_batch **out) {
    if (!ctx || n <= 0 || !plans || !nx || !ny || !out) {
        sde_set_error("sde_batch_create: bad arguments");
        return SDE_EINVAL;
    }
    if (n > 65535) {  // the flattened launches index plans with 16 bits
        sde_set_error("sde_batch_create: at most 65535 plans per batch");
        return SDE_EINVAL;
    }
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    sde_batch *b = new sde_batch();
    b->ctx = ctx;
    b->n = n;
    b->comp = ctx->compensated;
    int rc = SDE_OK;
    std::vector<BatchPlan> hp(n);
    std::vector<int64_t> start(n + 1, 0);
    std::vector<FinalizeDesc> hf(n);
    std::vector<size_t> raw_off(n), img_off(n);
    size_t raw_total = 0, img_total = 0;  // raw_total: the hi planes (the grids have the same layout)
    for (int i = 0; i < n; i++) {
        sde_plan *pl = plans[i];
        if (!pl || pl->ctx != ctx || nx[i] < 1 || ny[i] < 1) {
            sde_set_error("sde_batch_create: plan %d missing, from another context, or bad image size", i);
            delete b;
            return SDE_EINVAL;
        }
        const int fnu = 2 * (pl->spec.nu - 1), nv = pl->spec.nv;
        if (fnu < nx[i] || nv < ny[i] || (fnu & (fnu - 1)) || (nv & (nv - 1))) {
            sde_set_error("sde_batch_create: plan %d grid %dx%d does not hold a %dx%d image", i,
                          pl->spec.nu, nv, nx[i], ny[i]);
            delete b;
            return SDE_EINVAL;
        }
        if (!pl->sums_ready) {
            rc = plan_sums(pl, &pl->h_lsumwt, &pl->h_sumwt);
            if (rc != SDE_OK) {
                delete b;
                return rc;
            }
            pl->sums_ready = true;
        }
        if (pl->h_lsumwt == 0.0) {
            sde_set_error("No weight! (plan %d of the batch)", i);
            delete b;
            return SDE_ENOWEIGHT;
        }
        b->plans.push_back(pl);
        b->nx.push_back(nx[i]);
        b->ny.push_back(ny[i]);
        const size_t cells = (size_t)nv * pl->pitch;
        raw_off[i] = raw_total;
        raw_total += (cells * 8 + 255) & ~(size_t)255;
        img_off[i] = img_total;
        img_total += ((size_t)nx[i] * ny[i] * 4 + 255) & ~(size_t)255;
        b->max_cells = std::max<int64_t>(b->max_cells, (int64_t)cells);
        start[i + 1] = start[i] + pl->nitems;
        b->classes[std::make_tuple(fnu, nv, nx[i], ny[i], pl->pitch)].push_back(i);
    }
    char *rawmem = nullptr, *gridmem = nullptr, *imgmem = nullptr;
#define B_TRY(x)                              \
    do {                                      \
        rc = (x);                             \
        if (rc != SDE_OK) goto fail;          \
    } while (0)
    B_TRY(batch_alloc(b, (void **)&rawmem, raw_total * (b->comp ? 2 : 1)));
    B_TRY(batch_alloc(b, (void **)&gridmem, raw_total));
    B_TRY(batch_alloc(b, (void **)&imgmem, 2 * img_total));
    B_TRY(batch_alloc(b, (void **)&b->d_peak, sizeof(float) * n));
    B_TRY(batch_alloc(b, (void **)&b->d_plans, sizeof(BatchPlan) * n));
    B_TRY(batch_alloc(b, (void **)&b->d_item_start, sizeof(int64_t) * (n + 1)));
    B_TRY(batch_alloc(b, (void **)&b->d_counter, sizeof(unsigned long long)));
    B_TRY(batch_alloc(b, (void **)&b->d_fin, sizeof(FinalizeDesc) * n));
    for (int i = 0; i < n; i++)
        if (!fin_fused_shape(b->plans[i]->spec.nu, b->plans[i]->spec.nv))
            b->fin_nblk += ceil_div((int64_t)b->plans[i]->spec.nv * b->plans[i]->pitch, BATCH_BLOCK_CELLS);
    if (b->fin_nblk > 0)
        B_TRY(batch_alloc(b, (void **)&b->d_fin_blk, sizeof(uint16_t) * (size_t)b->fin_nblk));
    B_TRY(batch_alloc(b, (void **)&b->d_psf_ptrs, sizeof(float *) * n));
    B_TRY(batch_alloc(b, (void **)&b->d_npix, sizeof(int64_t) * n));
    b->hi_bytes = raw_total;
    b->raw_bytes = raw_total * (b->comp ? 2 : 1);
    for (int i = 0; i < n; i++) {
        sde_plan *pl = b->plans[i];
        b->raw.push_back(reinterpret_cast<float2 *>(rawmem + raw_off[i]));
        b->grid.push_back(reinterpret_cast<float2 *>(gridmem + raw_off[i]));
        b->psf.push_back(reinterpret_cast<float *>(imgmem + img_off[i]));
        b->image.push_back(reinterpret_cast<float *>(imgmem + img_total + img_off[i]));
        float2 *lo = b->comp ? reinterpret_cast<float2 *>(rawmem + raw_total + raw_off[i]) : nullptr;
        hp[i] = BatchPlan{pl->items, pl->chunks, pl->rec, b->raw[i], lo, pl->pitch, pl->ntu, pl->spec.nu,
                          pl->spec.nv};
        const float scale = (float)((double)((float)(pl->spec.nu - 1) * (float)pl->spec.nv) / pl->h_lsumwt);
        // the compensation planes are folded into raw before the finalize reads it
        hf[i] = FinalizeDesc{b->raw[i], nullptr, b->grid[i], pl->spec.nu, pl->spec.nv, pl->pitch,
                             pl->spec.uorigin, pl->spec.vorigin, pl->spec.supp, scale, 0};
    }
    {
        std::vector<int64_t> npix(n);
        for (int i = 0; i < n; i++) npix[i] = (int64_t)b->nx[i] * b->ny[i];
        std::vector<uint16_t> fblk((size_t)b->fin_nblk);
        for (int i = 0, k = 0; i < n; i++) {
            hf[i].block0 = k;
            if (fin_fused_shape(hf[i].nu, hf[i].nv)) continue;
            const int64_t nb = ceil_div((int64_t)hf[i].nv * hf[i].pitch, BATCH_BLOCK_CELLS);
            for (int64_t j = 0; j < nb; j++) fblk[(size_t)k++] = (uint16_t)i;
        }
        cudaStream_t st = ctx->stream;
        cudaError_t e = cudaSuccess;
        // the (plan, core) pairs to fold: the plans' marked cores (read back once)
        std::vector<int2> fold;
        if (b->comp) {
            for (int i = 0; i < n && e == cudaSuccess; i++) {
                const sde_plan *pl = b->plans[i];
                if (!pl->core_lo) continue;
                const int ncu = pl->ntu + 1, ncv = pl->ntv + 1;
                if (ncu > 0xFFFF || ncv > 0x7FFF) {
                    sde_set_error("sde_batch_create: plan %d grid too large for the batch fold", i);
                    rc = SDE_EINVAL;
                    goto fail;
                }
                std::vector<uint8_t> core((size_t)ncu * ncv);
                e = cudaMemcpyAsync(core.data(), pl->core_lo, core.size(), cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                for (int cv = 0; cv < ncv && e == cudaSuccess; cv++)
                    for (int cu = 0; cu < ncu; cu++)
                        if (core[(size_t)cv * ncu + cu]) fold.push_back(make_int2(i, cu | (cv << 16)));
            }
        }
        if (e == cudaSuccess && !fold.empty()) {
            b->fold_n = (int64_t)fold.size();
            rc = batch_alloc(b, (void **)&b->d_fold, sizeof(int2) * fold.size());
            if (rc != SDE_OK) goto fail;
            e = cudaMemcpyAsync(b->d_fold, fold.data(), sizeof(int2) * fold.size(), cudaMemcpyHostToDevice, st);
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_plans, hp.data(), sizeof(BatchPlan) * n, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_item_start, start.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_fin, hf.data(), sizeof(FinalizeDesc) * n, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess && !fblk.empty())
            e = cudaMemcpyAsync(b->d_fin_blk, fblk.data(), sizeof(uint16_t) * fblk.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_psf_ptrs, b->psf.data(), sizeof(float *) * n, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_npix, npix.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            sde_set_error("sde_batch_create: %s", cudaGetErrorString(e));
            rc = SDE_ECUDA;
            goto fail;
        }
    }
    b->hfin = hf;
    *out = b;
    return SDE_OK;
fail:
    for (size_t k = 0; k < b->allocs.size(); k++) ctx_free(ctx, b->allocs[k], b->alloc_bytes[k]);
    ctx->bytes -= b->bytes;
    delete b;
    return rc;
#undef B_TRY
}

extern "C" int sde_batch_destroy(sde_batch *b) {
    if (!b) return SDE_OK;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    batch_drop_graph(b);
    if (b->cap) cudaStreamDestroy(b->cap);
    for (size_t k = 0; k < b->allocs.size(); k++) ctx_free(b->ctx, b->allocs[k], b->alloc_bytes[k]);
    b->ctx->bytes -= b->bytes;
    delete b;
    return SDE_OK;
}

extern "C" int64_t sde_batch_bytes(const sde_batch *b) { return b ? b->bytes : 0; }

extern "C" int sde_batch_psf(sde_batch *b) {
    if (!b) return SDE_EINVAL;
    SDE_CUDA_TRY(cudaSetDevice(b->ctx->device));
    SDE_TRY(batch_grid(b, 1));
    SDE_TRY(batch_fft(b, b->psf, nullptr));
    k_max_batch<<<b->n, 1024, 0, b->ctx->stream>>>(b->d_psf_ptrs, b->d_npix, b->d_peak);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

extern "C" int sde_batch_set_mosaic(sde_batch *b, int mnx, int mny, const int *cx, const int *cy,
                                    const float *fwhm_px, const float *wt, float clip) {
    if (!b || mnx < 1 || mny < 1 || !cx || !cy || !fwhm_px || !wt || clip < 0.f) {
        sde_set_error("sde_batch_set_mosaic: bad arguments");
        return SDE_EINVAL;
    }
    SDE_CUDA_TRY(cudaSetDevice(b->ctx->device));
    if (b->d_pts && (b->mnx != mnx || b->mny != mny)) {
        sde_set_error("sde_batch_set_mosaic: the mosaic size is fixed once set");
        return SDE_EINVAL;
    }
    if (!b->d_pts) {
        for (int i = 0; i < b->n; i++)
            b->pts_nblk += ceil_div((int64_t)b->nx[i] * b->ny[i], BATCH_BLOCK_CELLS);
        SDE_TRY(batch_alloc(b, (void **)&b->d_pts, sizeof(MosaicPointing) * b->n));
        SDE_TRY(batch_alloc(b, (void **)&b->d_pts_blk, sizeof(uint16_t) * (size_t)b->pts_nblk));
        SDE_TRY(batch_alloc(b, (void **)&b->d_num, sizeof(float) * 2 * (size_t)mnx * mny));
        SDE_TRY(batch_alloc(b, (void **)&b->d_mosaic, sizeof(float) * (size_t)mnx * mny));
        SDE_TRY(batch_alloc(b, (void **)&b->d_denmax, sizeof(float)));
        b->d_invden = b->d_num + (size_t)mnx * mny;
    }
    std::vector<MosaicPointing> h(b->n);
    std::vector<uint16_t> pblk((size_t)b->pts_nblk);
    for (int i = 0, k = 0; i < b->n; i++) {
        if (!(fwhm_px[i] > 0.f)) {
            sde_set_error("sde_batch_set_mosaic: FWHM of pointing %d must be > 0", i);
            return SDE_EINVAL;
        }
        h[i] = MosaicPointing{b->image[i], b->nx[i], b->ny[i], cx[i], cy[i],
                              4.0f * 0.69314718f / (fwhm_px[i] * fwhm_px[i]), wt[i], k};
        const int64_t nb = ceil_div((int64_t)b->nx[i] * b->ny[i], BATCH_BLOCK_CELLS);
        for (int64_t j = 0; j < nb; j++) pblk[(size_t)k++] = (uint16_t)i;
    }
    b->mnx = mnx;
    b->mny = mny;
    b->clip = clip;
    // per mosaic tile, the pointings whose image covers it (in pointing order)
    const int mtx = (mnx + MOS_TILE - 1) / MOS_TILE, mty = (mny + MOS_TILE - 1) / MOS_TILE;
    std::vector<std::vector<uint16_t>> lists((size_t)mtx * mty);
    for (int i = 0; i < b->n; i++) {
        const int ox = cx[i] - 1 - ((b->nx[i] + 1) / 2 - 1), oy = cy[i] - 1 - ((b->ny[i] + 1) / 2 - 1);
        const int x0 = std::max(ox, 0), x1 = std::min(ox + b->nx[i], mnx);
        const int y0 = std::max(oy, 0), y1 = std::min(oy + b->ny[i], mny);
        if (x0 >= x1 || y0 >= y1) continue;
        for (int ty = y0 / MOS_TILE; ty <= (y1 - 1) / MOS_TILE; ty++)
            for (int tx = x0 / MOS_TILE; tx <= (x1 - 1) / MOS_TILE; tx++)
                lists[(size_t)ty * mtx + tx].push_back((uint16_t)i);
    }
    std::vector<int32_t> tstart(lists.size() + 1, 0);
    std::vector<uint16_t> tpts;
    for (size_t t = 0; t < lists.size(); t++) {
        tpts.insert(tpts.end(), lists[t].begin(), lists[t].end());
        tstart[t + 1] = (int32_t)tpts.size();
    }
    if (tpts.empty()) tpts.push_back(0);
    if (!b->d_tile_start) {
        SDE_TRY(batch_alloc(b, (void **)&b->d_tile_start, sizeof(int32_t) * tstart.size()));
        SDE_TRY(batch_alloc(b, (void **)&b->d_tile_pts, sizeof(uint16_t) * (size_t)b->n * mtx * mty));
    }
    b->mtx = mtx;
    b->mty = mty;
    cudaStream_t st = b->ctx->stream;
    SDE_CUDA_TRY(cudaMemcpyAsync(b->d_tile_start, tstart.data(), sizeof(int32_t) * tstart.size(), cudaMemcpyHostToDevice, st));
    SDE_CUDA_TRY(cudaMemcpyAsync(b->d_tile_pts, tpts.data(), sizeof(uint16_t) * tpts.size(), cudaMemcpyHostToDevice, st));
    SDE_CUDA_TRY(cudaMemcpyAsync(b->d_pts, h.data(), sizeof(MosaicPointing) * b->n, cudaMemcpyHostToDevice, st));
    SDE_CUDA_TRY(cudaMemcpyAsync(b->d_pts_blk, pblk.data(), sizeof(uint16_t) * pblk.size(), cudaMemcpyHostToDevice, st));
    // the denominator and its clip depend on the layout only
    const int64_t m = (int64_t)mnx * mny;
    SDE_CUDA_TRY(cudaMemsetAsync(b->d_invden, 0, sizeof(float) * (size_t)m, st));
    k_mosaic_den<<<(unsigned)b->pts_nblk, 256, 0, st>>>(b->d_pts, b->d_pts_blk, mnx, mny, b->d_invden);
    SDE_CHECK_LAUNCH();
    SDE_CUDA_TRY(cudaMemsetAsync(b->d_denmax, 0, sizeof(float), st));
    k_max_nonneg<<<b->ctx->num_sms * 4, 256, 0, st>>>(b->d_invden, m, reinterpret_cast<unsigned int *>(b->d_denmax));
    SDE_CHECK_LAUNCH();
    k_mosaic_invden<<<ceil_div(m, 256), 256, 0, st>>>(b->d_invden, m, b->d_denmax, clip);
    SDE_CHECK_LAUNCH();
    SDE_CUDA_TRY(cudaStreamSynchronize(st));
    batch_drop_graph(b);  // the captured sequence changes
    return SDE_OK;
}

extern "C" int sde_batch_dirty(sde_batch *b, int use_graph) {
    if (!b) return SDE_EINVAL;
    sde_ctx *ctx = b->ctx;
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    if (!use_graph) return batch_dirty_launches(b);
    if (!b->exec) {
        if (b->eager_runs == 0) {
            // the first run allocates the context's twiddle and correction tables; graphs
            // are captured from the second on
            SDE_TRY(batch_dirty_launches(b));
            b->eager_runs++;
            return SDE_OK;
        }
        if (!b->cap) SDE_CUDA_TRY(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
        // capture on the batch's own stream: the caller's stream may be the legacy default
        // stream, which cannot be captured; the graph is launched on the caller's stream
        SDE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        const int prof = ctx->profile;
        cudaStream_t user = ctx->stream;
        ctx->profile = 0;  // no timing events inside the graph
        ctx->stream = b->cap;
        cudaError_t e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal);
        int rc = e == cudaSuccess ? batch_dirty_launches(b) : SDE_ECUDA;
        cudaGraph_t g = nullptr;
        if (e == cudaSuccess) e = cudaStreamEndCapture(b->cap, &g);
        ctx->stream = user;
        ctx->profile = prof;
        if (rc != SDE_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) {
            sde_set_error("sde_batch_dirty: capture failed: %s", cudaGetErrorString(e));
            return SDE_ECUDA;
        }
        e = cudaGraphInstantiate(&b->exec, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            sde_set_error("sde_batch_dirty: graph instantiate: %s", cudaGetErrorString(e));
            return SDE_ECUDA;
        }
        b->graph = g;
        size_t nn = 0;
        cudaGraphGetNodes(g, nullptr, &nn);
        b->graph_nodes = (int)nn;
    }
    SDE_CUDA_TRY(cudaGraphLaunch(b->exec, ctx->stream));
    return SDE_OK;
}

// The same images through the single-plan entry points, one pointing after another
// (sde_plan_grid + sde_image_from_grid per plan): the baseline the batch is compared with.
extern "C" int sde_batch_dirty_loop(sde_batch *b) {
    if (!b) return SDE_EINVAL;
    SDE_CUDA_TRY(cudaSetDevice(b->ctx->device));
    for (int i = 0; i < b->n; i++) {
        sde_plan *pl = b->plans[i];
        SDE_TRY(sde_plan_grid(pl, SDE_GRID_VIS, (float *)b->grid[i], pl->pitch, nullptr));
        SDE_TRY(sde_image_from_grid(b->ctx, (float *)b->grid[i], pl->pitch, b->nx[i], b->ny[i],
                                    2 * (pl->spec.nu - 1), pl->spec.nv, 1, b->d_peak + i,
                                    b->image[i]));
    }
    SDE_TRY(batch_mosaic(b));
    return SDE_OK;
}

extern "C" int sde_batch_graph_nodes(const sde_batch *b) { return b ? b->graph_nodes : 0; }

extern "C" int sde_batch_image(const sde_batch *b, int i, int which, float **dev) {
    if (!b || !dev || i < -1 || i >= b->n || (i == -1 && !b->d_mosaic)) return SDE_EINVAL;
    if (i == -1) {
        *dev = b->d_mosaic;
        return SDE_OK;
    }
    *dev = which == 1 ? b->psf[i] : (which == 2 ? b->d_peak + i : b->image[i]);
    return SDE_OK;
}

extern "C" int sde_batch_read(const sde_batch *b, int i, int which, float *dst, int64_t n) {
    float *src = nullptr;
    if (!b || !dst || sde_batch_image(b, i, which, &src) != SDE_OK) {
        sde_set_error("sde_batch_read: bad arguments");
        return SDE_EINVAL;
    }
    const int64_t have = i == -1 ? (int64_t)b->mnx * b->mny
                                 : (which == 2 ? 1 : (int64_t)b->nx[i] * b->ny[i]);
    if (n != have) {
        sde_set_error("sde_batch_read: %lld floats requested, the image holds %lld", (long long)n,
                      (long long)have);
        return SDE_EINVAL;
    }
    SDE_CUDA_TRY(cudaSetDevice(b->ctx->device));
    SDE_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(float) * (size_t)n, cudaMemcpyDefault, b->ctx->stream));
    SDE_CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
    return SDE_OK;
}
