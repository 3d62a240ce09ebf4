// common.cuh -- internal declarations shared by the libsdegpu translation units.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/sde_gpu.h"

// ---------------------------------------------------------------------------------------
// Error handling: every entry point records a message and returns an SDE_E* code.
void sde_set_error(const char *fmt, ...);
#define SDE_CUDA_TRY(call)                                                                  \
    do {                                                                                    \
        cudaError_t _e = (call);                                                            \
        if (_e != cudaSuccess) {                                                            \
            sde_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(_e)); \
            return _e == cudaErrorMemoryAllocation ? SDE_ENOMEM                             \
                   : (_e == cudaErrorNoDevice || _e == cudaErrorInsufficientDriver)          \
                       ? SDE_ENODEV                                                         \
                       : SDE_ECUDA;                                                         \
        }                                                                                   \
    } while (0)
#define SDE_TRY(call)              \
    do {                           \
        int _rc = (call);          \
        if (_rc != SDE_OK) return _rc; \
    } while (0)
#define SDE_CHECK_LAUNCH() SDE_CUDA_TRY(cudaGetLastError())

// ---------------------------------------------------------------------------------------
// Geometry constants of the tiled gridder.  Tiles are TILE x TILE cells of the gridding
// frame (GRDH2D's grid before the SUPPU shift); the shared-memory copy of a tile has a
// halo of HALO = SUPP cells on every side.  A work item is a contiguous range of at most
// ITEM_MAX sorted visibilities inside one tile; a chunk is at most CHUNK_MAX visibilities
// of one cell, accumulated in registers by one thread.
constexpr int TILE = 64;
constexpr int TILE_LOG2 = 6;
constexpr int SUPP = 3;                 // 'SF' support (grd/grdcf.f:54)
constexpr int OSAMP = 128;              // oversampling (grd/grdcf.f:41)
constexpr int NTAP = 2 * SUPP + 1;      // 7
constexpr int STILE = TILE + 2 * SUPP;  // 70: shared tile edge (grid and degrid)
// The raw gridding accumulation keeps GRDH2D's raw column U (1-based, grd/grdh2d.f:177-187)
// at index U, so final column u (0-based) sits at raw index u + SUPP + 1 = u + 4 and any two
// final columns (u, u+1), u even, start on a 16-byte boundary of the raw row (TMA boxes).
constexpr int RAW_SHIFT = SUPP + 1;
// Row pitch (complex elements) of a plan's raw and final grids: a multiple of 4 (16-byte
// rows for TMA) with room for raw index NU.
inline int plan_pitch(int nu) { return (nu + 4) & ~3; }
constexpr int CFLEN = 1 + 8 * 129;      // vis/visgrid.f:105
constexpr int ITEM_MAX = 16384;        // default work-item size (sde_plan_opts.item_max)
constexpr int CHUNK_MAX = 64;           // default chunk size (sde_plan_opts.chunk_max)
constexpr int ITEM_LIMIT = 1 << 16;     // largest accepted work-item size
constexpr int CHUNK_LIMIT = 4096;       // largest accepted chunk size
constexpr uint32_t KEY_INVALID = 0xFFFFFFFFu;

// Per-visibility geometry words (sorted order):
//   gdg (uint16): du_g+64 | (dv_g+64) << 8 -- gridding sub-cell offsets (FP64 cell); the
//                 plan record carries them as tap-table byte offsets instead (taps_word);
//   gdd (uint32): taps_word(du_d, dv_d, column-in-pair) | GDD_EXCEPTION -- degridding
//                 offsets (FP32 cell); visibilities with GDD_EXCEPTION set are handled by the
//                 degridder's exception path.
__host__ __device__ inline uint16_t pack_gdg(int dug, int dvg) {
    return (uint16_t)((uint32_t)(dug + 64) | ((uint32_t)(dvg + 64) << 8));
}
constexpr uint32_t GDD_EXCEPTION = 1u << 31;

// Sub-cell offsets as byte offsets of the visibility's rows in the gridder's and degridder's
// tap tables -- u table row (du+64)*2 + column of the cell within its chunk's cell pair, 128
// bytes a row (low 16 bits); v table row dv+64, 128 bytes a row (bits 16..30) -- so that the
// lanes only add them to their table copy's address.  The plan record's second word (du_g,
// dv_g) and gdd (du_d, dv_d) hold them.
constexpr uint32_t TAPROW_BYTES = 128;
__host__ __device__ inline uint32_t taps_word(int du, int dv, uint32_t off) {
    return (((uint32_t)(du + 64) * 2u + off) * TAPROW_BYTES) | (((uint32_t)(dv + 64) * TAPROW_BYTES) << 16);
}
__host__ __device__ inline int taps_du(uint32_t g) { return (int)((g & 0xFFFFu) / (2 * TAPROW_BYTES)); }
__host__ __device__ inline int taps_dv(uint32_t g) { return (int)(((g >> 16) & 0x7FFFu) / TAPROW_BYTES); }

// Exception entries for the degridder: visibilities whose FP32 degridding cell differs
// from their FP64 gridding cell, whose conjugation flags differ, that only degrid, or that
// sit within SUPP of the v axis (reflection branch of grd/grddeh2d.f:123-158) where the
// tiled degridder cannot stand in for that branch (UORIGIN != 1, or a mirrored row
// 2*VORIGIN - v outside the grid, whose taps the reference skips).
struct DegridExc {
    uint32_t orig;     // index in the caller's order
    int32_t pos;       // sorted position in the plan, -1 if the visibility does not grid
    int32_t nuc, nvc;  // NINT(UCELL), NINT(VCELL) in GRDDEH2D's FP32 frame
    int16_t delui, delvi;
    uint8_t conj;      // USCALE*ULOCAL > 0 (grd/grddeh2d.f:189)
    uint8_t valid;     // passed GRDDEH2D's bounds (grd/grddeh2d.f:112-114)
    uint8_t gconj;     // gridding-frame conjugation of this visibility (if pos >= 0)
    uint8_t pad;
};

// The exception list is one allocation: entries, then their weights, then their
// rotations, each section starting on a 16-byte boundary.
inline size_t exc_wt_off(size_t ne) { return (sizeof(DegridExc) * ne + 15) & ~(size_t)15; }
inline size_t exc_rot_off(size_t ne) { return (exc_wt_off(ne) + 4 * ne + 15) & ~(size_t)15; }
inline size_t exc_bytes(size_t ne) { return exc_rot_off(ne) + 8 * ne; }

struct WorkItem {
    int32_t tile;      // tile id = tv * ntu + tu
    int32_t cbeg, cend;  // chunk range
    int32_t vbeg, vend;  // sorted visibility range
    int32_t dense;     // 1: the item's tile holds >= DENSE_TILE_VIS visibilities
};
// A tile this full has many work items, so its cells receive long sums across items: those
// sums are the ones compensated (sde_ctx_set_compensated).
constexpr int DENSE_TILE_VIS = 65536;

// ---------------------------------------------------------------------------------------
// Context: one device, one stream, grow-only scratch buffers, cached tables.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

struct sde_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int num_sms = 0;
    int64_t bytes = 0;                     // device bytes owned (buffers + plans)
    float *d_cf = nullptr;                 // 'SF' gridding function, CFLEN floats
    float *d_cft = nullptr;                // transposed table [129][8]
    int *d_status = nullptr;               // device status words (see STATUS_*)
    int *h_status = nullptr;               // pinned mirror
    // pinned bytes for the small device-to-host reads (counts, sums): a copy into pageable
    // memory goes through the driver's staging shared by every stream of the process
    unsigned char *h_small = nullptr;
    std::unordered_map<std::string, DevBuf> scratch;
    std::unordered_map<int, float2 *> twiddles;  // N -> exp(+-2 pi i k/N) table
    CUtensorMap *h_tmap = nullptr;
    // per-kernel CUDA-event timing (sde_ctx_profile) and launch counting
    bool profile = false;
    int64_t nlaunch = 0;
    // gridding sums across work items with TwoSum compensation (sde_ctx_set_compensated)
    bool compensated = true;
    int hogbom_per_sm = 0;            // resident k_hogbom CTAs per SM (queried at creation)
    const void *lo_clean = nullptr;  // compensation plane of the raw-grid scratch known to be zero
    struct EvPair {
        const char *name;
        cudaEvent_t a, b;
    };
    std::vector<EvPair> evq;
    std::unordered_map<std::string, std::pair<double, int64_t>> kstats;
};

// Scoped timer around one kernel launch on the context's stream: counts the launch and,
// when profiling is on, records a CUDA event pair that sde_ctx_kernel_stats resolves.
struct KTimer {
    sde_ctx *c;
    cudaEvent_t b = nullptr;
    const char *name;
    KTimer(sde_ctx *ctx, const char *n) : c(ctx), name(n) {
        c->nlaunch++;
        if (c->profile) {
            cudaEvent_t a;
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            cudaEventRecord(a, c->stream);
            c->evq.push_back({name, a, b});
        }
    }
    ~KTimer() {
        if (b) cudaEventRecord(b, c->stream);
    }
};

enum { STATUS_ERR = 0, STATUS_NOWEIGHT = 1, STATUS_TIMEOUT = 2, STATUS_COUNT = 8 };

// scratch buffer by name, grown on demand (contents undefined)
int ctx_scratch(sde_ctx *ctx, const char *name, size_t bytes, void **out);
constexpr size_t H_SMALL_BYTES = 256;
// Reads `bytes` (<= H_SMALL_BYTES) from device memory after the work queued on st, through the
// context's pinned buffer; waits for st.
int ctx_read_small(sde_ctx *ctx, cudaStream_t st, void *dst, const void *src, size_t bytes);
int ctx_alloc(sde_ctx *ctx, void **p, size_t bytes);
void ctx_free(sde_ctx *ctx, void *p, size_t bytes);
int ctx_twiddles(sde_ctx *ctx, int n, const float2 **out);

struct sde_plan {
    sde_ctx *ctx = nullptr;
    sde_gridspec spec;
    int doshift = 0;
    int pitch = 0;            // row pitch (complex elements) of grids the plan writes
    int ntu = 0, ntv = 0;     // tiles across / down
    int64_t nvis_in = 0;      // caller's count
    int64_t nvis = 0;         // gridding visibilities
    int64_t nitems = 0, nchunks = 0, nexc = 0;
    int item_max = ITEM_MAX, chunk_max = CHUNK_MAX;  // sort-bucket sizes of this plan
    // sorted, gridding-valid visibilities
    float2 *fobs = nullptr;   // observed, in the gridding frame (rotated, conjugated)
    float4 *rec = nullptr;    // {WT, gdg bits, residual re, residual im} (gridding frame):
                              // the gridder reads one 16-byte record per visibility
    float *wt = nullptr;
    uint32_t *gdd = nullptr;  // degridding offsets + cell + exception flag
    uint32_t *orig = nullptr; // caller index of each sorted visibility
    float2 *rot = nullptr;    // (cos, sin) of the phase rotation (doshift only), sorted
    uint8_t *gconj = nullptr; // gridding-frame conjugation flag, sorted
    uint2 *chunks = nullptr;  // {first vis, cell | len << 16}
    WorkItem *items = nullptr;
    DegridExc *exc = nullptr; // exception list (includes degrid-only visibilities)
    float *wt_all = nullptr;  // caller-order weights (for user-frame degridding)
    uint8_t *core_lo = nullptr;  // (ntu+1) x (ntv+1) raw-grid cores where the compensation
                                 // plane can be non-zero (dense tiles' footprints)
    int32_t *inv = nullptr;   // caller index -> position of the tiled visibilities (-1 else),
                              // built on the first caller-order degrid
    int64_t nuntouched = 0;   // caller visibilities with WT <= 0 (GRDDEH2D leaves them as they are)
    float *cf = nullptr;      // gridding function used by this plan (device, CFLEN)
    float *cft = nullptr;     // transposed table
    double *d_sums = nullptr; // [0] sum of UVWT (LSUMWT), [1] SUMWT
    double h_lsumwt = 0.0, h_sumwt = 0.0;
    bool sums_ready = false;
    int64_t bytes = 0;
};

// grid.cu internals used by api.cu
int plan_build_cft(sde_plan *pl);
int ctx_build_cft(sde_ctx *ctx);
int plan_sums(sde_plan *pl, double *lsumwt, double *sumwt);
int grid_finalize_scale(sde_ctx *ctx, const float2 *raw, const float2 *raw_lo, float2 *out, int nu, int nv, int pitch,
                        int uorigin, int vorigin, int supp, float scale);
// raw accumulation of one gridding pass; raw_lo (same shape, may be NULL) receives the
// rounding errors of the cross-item sums (compensated accumulation)
int plan_grid_raw(sde_plan *pl, int what, float2 *raw, float2 *raw_lo, bool lo_clean = false);
// Add the compensation plane into the raw grid where it can be non-zero (the plan's dense
// cores) and zero it there: afterwards raw alone is the compensated sum and raw_lo is zero.
int plan_fold_lo(sde_plan *pl, float2 *raw, float2 *raw_lo);
// Image of a gridding pass from the raw accumulation (fft.cu): finalize fused into the
// column pass where it is TMA-fed (raw_lo must then be folded, i.e. nullptr), else finalize
// into grid and the usual passes; grid receives the column-transformed grid.
int image_from_raw(sde_ctx *ctx, const float2 *raw, const float2 *raw_lo, int nu, int nv,
                   int uorigin, int vorigin, int supp, float scale, float *grid, int pitch, int nx,
                   int ny, int fnu, int correct, const float *scale_dev, float *image);

// ---- batches of plans (mosaic pointings, served jobs) -----------------------------------
// One plan as the persistent gridder sees it.
struct BatchPlan {
    const WorkItem *items;
    const uint2 *chunks;
    const float4 *rec;
    float2 *raw;
    float2 *raw_lo;  // NULL: plain FP32 sums across items
    int pitch, ntu, nu, nv;
};
// One grid of a batched finalize (Hermitian fold, shift by SUPP, GRDH2D normalisation).
struct FinalizeDesc {
    const float2 *raw;
    const float2 *raw_lo;
    float2 *out;
    int nu, nv, pitch, uorigin, vorigin, supp;
    float scale;
    int64_t block0;  // first block of this grid in the flattened launch
};
// Cells (pixels) per block of the flattened batch launches: 256 threads x 4.
constexpr int BATCH_BLOCK_CELLS = 1024;
// Pointers of up to FFT_MAXB same-shape transforms of one batched FFT launch (blockIdx.y).
constexpr int FFT_MAXB = 64;
struct FftBatch {
    float2 *grid[FFT_MAXB];
    float *image[FFT_MAXB];
    const float *scale[FFT_MAXB];
};
int clean_preload(sde_ctx *ctx);  // loads the CLEAN kernels, caches their occupancy
size_t grid_smem_bytes();
int grid_ctas_per_sm();  // resident persistent gridding CTAs per SM
// 2-D FP32 tensor map for cp.async.bulk.tensor (grid.cu): width floats x rows, row pitch in
// bytes, box box_w x box_h; out-of-range elements read as zero and are not written
int encode_tmap_f32_2d(CUtensorMap *map, const void *base, uint64_t width, uint64_t rows,
                       uint64_t row_bytes, uint32_t box_w, uint32_t box_h);
int launch_grid_batch(sde_ctx *ctx, int psf, int comp, const BatchPlan *d_plans,
                      const int64_t *d_item_start, int nplans, unsigned long long *d_counter,
                      const float *cft, int nctas);
// finalize of n grids in one flattened launch: blk[b] = the grid of block b (nblk blocks)
int launch_finalize_batch(sde_ctx *ctx, const FinalizeDesc *d_desc, const uint16_t *blk, int64_t nblk);
// compensation planes of a batch folded into their raw grids: block b folds core cores[b].y
// (cu | cv << 16) of plan cores[b].x (its raw and raw_lo)
int launch_fold_lo_batch(sde_ctx *ctx, const BatchPlan *d_plans, const int2 *cores, int64_t ncores);
int check_fft_shape(int nx, int ny, int fnu, int nv);  // SDE_EINVAL + message if unsupported
// GRDH23D / GRDDEH23 on device arrays (slowz.cu): grid [nz][nv][nu] complex, tables of
// 2*(supp+1)*osamp+1 floats, shift the host 3x3 DOUBLE matrix
int grid_h23d(sde_ctx *ctx, int64_t nvis, const float *vis, const float *wt, const float *u, const float *v,
              const float *w, float uscale, float uoffset, float vscale, float voffset, int uorigin, int vorigin,
              int psf, int nu, int nv, const float *fnu, int suppu, int osampu, const float *fnv, int suppv,
              int osampv, int nz, float cellz, float refz, const double *shift, float *grid, float *sumwt);
int degrid_h23(sde_ctx *ctx, int64_t nvis, float *vis, float *wt, const float *u, const float *v, const float *w,
               float uscale, float uoffset, float vscale, float voffset, int uorigin, int vorigin, const float *grid,
               int nu, int nv, const float *fnu, int suppu, int osampu, const float *fnv, int suppv, int osampv,
               int nz, float cellz, float refz, const double *shift, int64_t *nbad);
// GRDQH2D on device arrays (box.cu); shift is the host 3x3 DOUBLE matrix, column-major
int grid_box(sde_ctx *ctx, int64_t nvis, const float *vis, const float *wt, const float *u, const float *v,
             const float *w, float uscale, float uoffset, float vscale, float voffset, int uorigin, int vorigin,
             int psf, int nu, int nv, const double *shift, float *grid, int pitch, float *sumwt, int64_t *ngrid);
// batched images from raw accumulations (fft.cu; EINVAL when the shape has no fused path;
// fin_fused_shape says which grids have one)
bool fin_fused_shape(int nu, int nv);
int fft_images_from_raw(sde_ctx *ctx, int n, const FinalizeDesc *fd, float *const *images,
                        const float *const *scales, int nx, int ny, int correct);
// grid -> image for n same-shape grids (inverse column pass, row c2r with grid correction
// and scale 1/scales[i] when scales[i] != NULL); SDE_EINVAL if the shape has no batched form
int fft_images_from_grids(sde_ctx *ctx, int n, float2 *const *grids, float *const *images,
                          const float *const *scales, int pitch, int nx, int ny, int fnu, int nv,
                          int correct);
int plan_inverse(sde_plan *pl);
int plan_degrid(sde_plan *pl, const float *grid, int pitch, int mode, float2 *vis_out,
                float *wt_out, unsigned long long *nbad_dev);
int plan_scatter_residual(sde_plan *pl, float2 *dst);
int plan_set_vis_dev(sde_plan *pl, const float2 *vis_user);
int sde_isamax0(sde_ctx *ctx, const float *a, int64_t n, int64_t *index_out);

// ---------------------------------------------------------------------------------------
// Kernels shared across translation units (host-side launchers).
int launch_radix_sort_u32(sde_ctx *ctx, uint32_t *keys, uint32_t *vals, int64_t n, int bits,
                          uint32_t *keys_tmp, uint32_t *vals_tmp);
int launch_radix_sort_u64(sde_ctx *ctx, uint64_t *keys, uint32_t *vals, int64_t n, int bits,
                          uint64_t *keys_tmp, uint32_t *vals_tmp);
int launch_exclusive_scan_u32(sde_ctx *ctx, const uint32_t *in, uint32_t *out, int64_t n,
                              uint32_t *total_dev);
int launch_inclusive_max_scan_i32(sde_ctx *ctx, const int32_t *in, int32_t *out, int64_t n);


// host restatement of the 'SF' tables (grd/grdcf.f, grd/grdsf.f, grd/grdccf.f)
double sf_grdsf(double nu);
void sf_cf_table(float *cf);
void sf_ccf_table(float *ccf, int ccflen);
int fftpwr2(int i);

// ---------------------------------------------------------------------------------------
// Device helpers.
__device__ __forceinline__ int nint_f(float x) { return (int)roundf(x); }   // half away
__device__ __forceinline__ int nint_d(double x) { return (int)round(x); }

// TwoSum (Knuth): the rounding error of fl(a + b), exactly, in round-to-nearest
__device__ __forceinline__ float two_sum_err(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float ap = __fsub_rn(s, bp);
    return __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}

__device__ __forceinline__ void red_add_f2(float2 *addr, float2 v) {
    asm volatile("red.relaxed.gpu.global.add.v2.f32 [%0], {%1, %2};" ::"l"(addr), "f"(v.x),
                 "f"(v.y)
                 : "memory");
}

// Ask the TMA unit to pull elements [first, last) of an array into L2 (no registers, no
// completion to wait for).  The byte range is shrunk to 16-byte boundaries (the rule of
// cp.async.bulk.prefetch.L2), so it never reaches outside the array; the elements cut off
// at either end are simply not prefetched.
__device__ __forceinline__ void prefetch_l2_range(const void *base, int64_t first, int64_t last,
                                                  int esize) {
    uintptr_t a = (reinterpret_cast<uintptr_t>(base) + (uintptr_t)(first * esize) + 15) & ~(uintptr_t)15;
    const uintptr_t b = (reinterpret_cast<uintptr_t>(base) + (uintptr_t)(last * esize)) & ~(uintptr_t)15;
    while (a < b) {
        const uint32_t n = (uint32_t)(b - a < 16384 ? b - a : 16384);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"(n) : "memory");
        a += n;
    }
}

// The residual half of a plan record.
__device__ __forceinline__ float2 *rec_res(float4 *rec, int64_t p) {
    return reinterpret_cast<float2 *>(rec + p) + 1;
}
__device__ __forceinline__ float2 rec_res(const float4 *rec, int64_t p) {
    return reinterpret_cast<const float2 *>(rec + p)[1];
}

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }
