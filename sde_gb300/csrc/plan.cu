// plan.cu -- builds a resident, tile- and chunk-sorted visibility set (sde_plan).
//
// For every visibility the plan evaluates, once, the cell placement that GRDH2D uses (FP64,
// grd/grdh2d.f:114-166) and the one GRDDEH2D uses (FP32 cell from FP64 coordinates,
// grd/grddeh2d.f:92-118), with the reference's results: its exact operations, or FP32
// arithmetic whose error bound decides the same roundings (geom.cuh).  Visibilities are
// then sorted by (uv tile, cell), split into same-cell chunks of <= CHUNK_MAX, and the
// chunks of each work item are ordered by (7x7 colour class, chunk index, cell) so that
// the 32 chunks a warp flushes at once never overlap; the plan stores the visibilities in
// that chunk order, so a team's concurrent chunks read one contiguous range.  The observed
// visibilities are stored already rotated/conjugated into the gridding frame (FVIS of
// grd/grdh2d.f:125-143), so the per-cycle kernels carry no FP64 or trigonometric work.
#include <math.h>
#include <string.h>

#include "common.cuh"
#include "geom.cuh"

namespace {

using namespace sde_geom;

constexpr int LENBIN_BITS = 3;  // coarse length bins above the colour class in the chunk order

// Bit 0 of a caller-order degridding word (a table byte offset, a multiple of 128, is even
// there) carries the gridding-frame conjugation (the plan's own words leave it clear).
constexpr uint32_t GDD_GCONJ_U = 1u;
static_assert(TAPROW_BYTES % 2 == 0, "bit 0 of a degridding word is free");

// A visibility's plan data in caller order, one 32-byte sector: the plan record {WT, the
// gridder's tap-table offsets, observed value in the gridding frame}, the degridding word
// (with the gridding-frame conjugation in bit 0), the rotation and, for an exception, its
// place in the exception list.  The gather into sorted
// order reads one sector per visibility.
struct __align__(32) PlanRecU {
    float4 rec;
    uint32_t gdd;
    float rc, rs;
    uint32_t exc_slot;  // the visibility's place in the exception list (exceptions only)
};

// Per visibility (caller order): gridding key, the PlanRecU sector and, for an exception, its
// entry in the exception list,
// from both routines' geometry (geom_vis).
__global__ void k_plan_geom(GParams p, const float *__restrict__ u, const float *__restrict__ v,
                            const float *__restrict__ w, const float2 *__restrict__ vis,
                            const float *__restrict__ wt, int64_t n, uint32_t *keys,
                            uint32_t *vals, PlanRecU *rec_u, uint32_t *exc_list,
                            unsigned long long *counts) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t nvalid = 0, nexc = 0;
    const float wi = i < n ? wt[i] : 0.0f;
    if (i < n) {
        uint32_t key = KEY_INVALID, pdd = 0, tw = 0;
        float2 f = make_float2(0.f, 0.f), r = make_float2(1.f, 0.f);
        uint8_t gc = 0;
        if (wi > 0.0f) {
            const float2 vv = vis[i];
            const GGeo g = geom_vis(p, u[i], v[i], w[i], vv.x, vv.y);
            const DGeo &dg = g.dg;
            gc = g.gc ? 1 : 0;
            r = make_float2(g.rc, g.rs);
            const int nuc = g.nuc, nvc = g.nvc;
            const bool gvalid = g.sane && !(nuc + 2 * p.supp > p.nu) && !(nvc + p.supp > p.nv) && !(nvc - p.supp < 1);
            if (gvalid) {
                const int dug = g.dug, dvg = g.dvg;
                int ucen = nuc + p.supp, vcen = nvc;  // 1-based, gridding frame
                int tu = (ucen - 1) >> TILE_LOG2, lu = (ucen - 1) & (TILE - 1);
                int tv = (vcen - 1) >> TILE_LOG2, lv = (vcen - 1) & (TILE - 1);
                key = ((uint32_t)(tv * p.ntu + tu) << 12) | ((uint32_t)lv << 6) | (uint32_t)lu;
                // GRDDEH2D's reflection branch (NUD <= SUPP) reads conj(G(-u, 2*VORIGIN - v))
                // left of the v axis; the tiled degridder holds those values in the u = 0
                // tile's halo, so the branch stays in the tiled path when every mirrored
                // row lies inside the grid (else the reference skips taps: exception)
                const bool refl_tiled = p.uorigin == 1 && 2 * p.vorigin - (dg.nvd + p.supp) >= 1 &&
                                        2 * p.vorigin - (dg.nvd - p.supp) <= p.nv;
                bool exc = !dg.valid || dg.nud != nuc || dg.nvd != nvc ||
                           (dg.nud <= p.supp && !refl_tiled) || dg.conj != (gc != 0);
                // column of the cell within its chunk's cell pair (chunks start on even lu)
                const uint32_t off = (uint32_t)lu & 1u;
                tw = taps_word(dug, dvg, off);
                pdd = exc ? (taps_word(0, 0, off) | GDD_EXCEPTION) : taps_word(dg.dui, dg.dvi, off);
                nvalid = 1;
                nexc = exc;
                f = make_float2(g.fr, g.fi);
            } else {
                nexc = 1;  // degrid-only or degrid-invalid: exception path
            }
        }
        keys[i] = key;
        vals[i] = (uint32_t)i;
        PlanRecU pr;
        pr.rec = make_float4(wi, __uint_as_float(tw), f.x, f.y);
        pr.gdd = pdd | (gc ? GDD_GCONJ_U : 0u);
        pr.rc = r.x;
        pr.rs = r.y;
        pr.exc_slot = 0;
        // GRDDEH2D's exception path takes the visibilities with WT > 0 that do not grid or
        // whose degridding cell is not the gridding cell: appended to the list (a few in 10^4;
        // the list's order does not matter, each is degridded on its own)
        if (wi > 0.0f && (key == KEY_INVALID || (pdd & GDD_EXCEPTION) != 0)) {
            pr.exc_slot = (uint32_t)atomicAdd(&counts[3], 1ull);
            exc_list[pr.exc_slot] = (uint32_t)i;
        }
        rec_u[i] = pr;
    }
    // block-aggregated counters (one atomic per block and counter: per-warp atomics on three
    // addresses serialise in L2 at this visibility count)
    const int cv = __syncthreads_count(nvalid), ce = __syncthreads_count(nexc);
    const int ct = __syncthreads_count(i < n && wi > 0.0f);
    if (threadIdx.x == 0) {
        if (cv) atomicAdd(&counts[0], (unsigned long long)cv);
        if (ce) atomicAdd(&counts[1], (unsigned long long)ce);
        if (ct) atomicAdd(&counts[2], (unsigned long long)ct);
    }
}

// Gather the per-visibility data into the plan's order (one 32-byte sector read per
// visibility), one warp per chunk: chunk c's visibilities, at [st, st + length) in the sort's
// order, go to [cpos[c], cpos[c] + length) -- the chunk order, the order the kernels take
// them -- and the chunk's start moves there.  An exception that also grids learns its
// position here.
__global__ void __launch_bounds__(256) k_plan_gather(const uint32_t *__restrict__ perm,
                                                     const uint32_t *__restrict__ cpos, int64_t nchunks,
                                                     uint2 *chunks, const PlanRecU *__restrict__ rec_u,
                                                     float2 *fobs,
                                                     float4 *rec, float *wt, uint32_t *gdd, uint32_t *orig,
                                                     float2 *rot, uint8_t *gconj, DegridExc *exc) {
    const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= nchunks) return;
    const uint2 ch = chunks[c];
    const uint32_t st = ch.x, len = ch.y >> 16, to = cpos[c];
    for (uint32_t k = lane; k < len; k += 32) {
        const uint32_t i = perm[st + k];
        const int64_t p = (int64_t)to + k;
        const PlanRecU pr = rec_u[i];
        const float4 r = pr.rec;
        const uint32_t d = pr.gdd;
        rec[p] = r;
        fobs[p] = make_float2(r.z, r.w);
        wt[p] = r.x;
        gdd[p] = d & ~GDD_GCONJ_U;
        orig[p] = i;
        gconj[p] = (d & GDD_GCONJ_U) ? 1 : 0;
        if (rot) rot[p] = make_float2(pr.rc, pr.rs);
        if ((d & GDD_EXCEPTION) && exc) exc[pr.exc_slot].pos = (int32_t)p;
    }
    __syncwarp();  // every lane has read the chunk record
    if (lane == 0) chunks[c] = make_uint2(to, ch.y);
}

// The exception list's entries, one thread per exception (pos is set by k_plan_gather for the
// exceptions that also grid).
__global__ void k_exc_write(GParams p, const float *__restrict__ u, const float *__restrict__ v,
                            const float *__restrict__ w, const float *__restrict__ wt,
                            const PlanRecU *__restrict__ rec_u, const uint32_t *__restrict__ exc_list,
                            int64_t nexc, DegridExc *exc, float *exc_wt, float2 *exc_rot) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nexc) return;
    const uint32_t i = exc_list[s];
    DGeo g = p.fast ? degrid_geom_fast(p, u[i], v[i]) : degrid_geom(p, u[i], v[i], w[i]);
    DegridExc e;
    e.orig = i;
    e.pos = -1;
    e.nuc = g.nud;
    e.nvc = g.nvd;
    e.delui = (int16_t)g.dui;
    e.delvi = (int16_t)g.dvi;
    e.conj = g.conj;
    e.valid = g.valid;
    e.gconj = (rec_u[i].gdd & GDD_GCONJ_U) ? 1 : 0;
    e.pad = 0;
    exc[s] = e;
    exc_wt[s] = wt[i];
    exc_rot[s] = make_float2(g.rc, g.rs);
}

// Runs, work items and chunks from the sorted keys.  A run is one cell pair of one tile
// (equal key >> 1); a tile's visibilities split into work items at every item_max from the
// tile's first one; a run's part within one item (a piece) splits into chunks of chunk_max
// from the piece's start.  Chunks and items are numbered in position order.
__global__ void k_run_heads(const uint32_t *__restrict__ keys, const unsigned long long *counts,
                            int64_t n, uint32_t *head) {
    const int64_t nv = (int64_t)counts[0];
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    head[q] = q < nv && (q == 0 || (keys[q - 1] >> 1) != (keys[q] >> 1));
}

__global__ void k_run_compact(const uint32_t *__restrict__ head, const uint32_t *__restrict__ ridx,
                              const unsigned long long *counts, uint32_t *rstart) {
    const int64_t nv = (int64_t)counts[0];
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nv && head[q]) rstart[ridx[q]] = (uint32_t)q;
}

// a run that starts a tile: its start (the tile's first visibility), else -1, for a max-scan
__global__ void k_run_tilehead(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ rstart,
                               int64_t nruns, int32_t *tstart) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nruns) return;
    const uint32_t rs = rstart[r];
    const bool th = r == 0 || (keys[rstart[r - 1]] >> 12) != (keys[rs] >> 12);
    tstart[r] = th ? (int32_t)rs : -1;
}

// the run's chunks and item heads (an item head is a position ts + k*item_max of the run)
__global__ void k_run_counts(const uint32_t *__restrict__ rstart, const int32_t *__restrict__ tstart,
                             int64_t nruns, int64_t nvalid, int item_max, int chunk_max, uint32_t *nch,
                             uint32_t *nih) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nruns) return;
    const int64_t rs = rstart[r], re = r + 1 < nruns ? (int64_t)rstart[r + 1] : nvalid, ts = tstart[r];
    uint32_t c = 0, h = 0;
    for (int64_t a = rs; a < re;) {
        const int64_t is = ts + (a - ts) / item_max * item_max;
        h += is == a;
        const int64_t b = min(re, is + item_max);
        c += (uint32_t)((b - a + chunk_max - 1) / chunk_max);
        a = b;
    }
    nch[r] = c;
    nih[r] = h;
}

// the run's chunk records (sort key, index, start) and the items that start in it
__global__ void k_run_emit(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ rstart,
                           const int32_t *__restrict__ tstart, int64_t nruns, int64_t nvalid,
                           const uint32_t *__restrict__ cbase, const uint32_t *__restrict__ ibase,
                           int item_max, int chunk_max, int lbits, int jbits, uint64_t *ckey,
                           uint32_t *cval, uint32_t *cstart, WorkItem *items) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nruns) return;
    const int64_t rs = rstart[r], re = r + 1 < nruns ? (int64_t)rstart[r + 1] : nvalid, ts = tstart[r];
    const uint32_t k = keys[rs];
    const uint32_t cell = k & 4094u, lu = cell & 63u, lv = cell >> 6;  // pair's even cell
    const uint32_t color = ((lu >> 1) & 3u) * 7u + (lv % 7u);
    uint32_t c = cbase[r], nit = ibase[r];  // items started before the run's current piece
    for (int64_t a = rs; a < re;) {
        const int64_t is = ts + (a - ts) / item_max * item_max;
        if (is == a) {
            WorkItem wi;
            wi.tile = (int32_t)(k >> 12);
            wi.cbeg = wi.cend = 0;
            wi.vbeg = (int32_t)a;
            wi.vend = 0;
            wi.dense = 0;
            items[nit++] = wi;
        }
        const uint64_t it = nit - 1;
        const int64_t b = min(re, is + item_max);
        uint32_t j = 0;
        for (int64_t q = a; q < b; q += chunk_max, j++, c++) {
            ckey[c] = (it << (LENBIN_BITS + 6 + lbits + jbits + 12)) |
                      ((uint64_t)color << (lbits + jbits + 12)) | ((uint64_t)j << 12) | cell;
            cval[c] = c;
            cstart[c] = (uint32_t)q;
        }
        a = b;
    }
}

// Length class (CHUNK_MAX - length) of each chunk, above the chunk index in its sort key,
// and a coarse length bin (LENBIN_BITS, longest first) above the colour class: the 8 chunks
// a warp of the gridder or degridder takes together have similar lengths (the warp runs to
// its longest), and mostly one colour.  On the large single field the lanes do useful work
// in 94% of the warps' visibility slots with 8 bins, 81% with the colour class alone above
// the length (a simulation of both orders on its chunks; measured: gridder 0.82 -> 0.75 ms).
__global__ void k_chunk_len(const uint32_t *__restrict__ cstart, int64_t nchunks, int64_t nvalid,
                            int chunk_max, int lshift, int bshift, uint64_t *ckey) {
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const uint32_t en = c + 1 < nchunks ? cstart[c + 1] : (uint32_t)nvalid;
    const uint32_t len = en - cstart[c];
    const int cls = chunk_max - (int)len;
    const int nbin = 1 << LENBIN_BITS;
    const int bin = min(cls * nbin / chunk_max, nbin - 1);
    ckey[c] |= ((uint64_t)cls << lshift) | ((uint64_t)bin << bshift);
}

__global__ void k_chunk_final(const uint64_t *__restrict__ ckey, const uint32_t *__restrict__ cval,
                              const uint32_t *__restrict__ cstart, const uint32_t *__restrict__ keys,
                              int64_t nchunks, int64_t nvalid, int shift_item, uint2 *chunks,
                              uint32_t *clen, WorkItem *items) {
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    uint32_t orig = cval[c];
    uint32_t st = cstart[orig];
    uint32_t en = (int64_t)orig + 1 < nchunks ? cstart[orig + 1] : (uint32_t)nvalid;
    uint32_t cell = keys[st] & 4094u;
    chunks[c] = make_uint2(st, cell | ((en - st) << 16));
    clen[c] = en - st;
    uint32_t it = (uint32_t)(ckey[c] >> shift_item);
    if (c == 0 || (uint32_t)(ckey[c - 1] >> shift_item) != it) items[it].cbeg = (int32_t)c;
    if (c == nchunks - 1 || (uint32_t)(ckey[c + 1] >> shift_item) != it) items[it].cend = (int32_t)(c + 1);
}

// a work item's first visibility: its first chunk's (new) start
__global__ void k_item_vbeg(const uint2 *__restrict__ chunks, int64_t nitems, WorkItem *items) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nitems) return;
    items[t].vbeg = (int32_t)chunks[items[t].cbeg].x;
}

// dense flag of each work item: its tile's items (contiguous, sorted by tile) together
// hold >= DENSE_TILE_VIS visibilities
// Raw-grid cores of the compensation plane: the footprint of a tile (tu, tv) (its 64x64
// cells and 3-cell halo, raw rows [64 tv - 3, 64 tv + 67), raw indices [64 tu - 2,
// 64 tu + 68)) lies in cores (tu, tv), (tu+1, tv), (tu, tv+1), (tu+1, tv+1), where core
// (cu, cv) is raw rows [64 cv - 3, 64 cv + 61) x raw indices [64 cu - 2, 64 cu + 62).
__global__ void k_core_lo(const WorkItem *items, int64_t nitems, int ntu, uint8_t *core) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nitems || !items[t].dense) return;
    const int tu = items[t].tile % ntu, tv = items[t].tile / ntu, ncu = ntu + 1;
    core[tv * ncu + tu] = 1;
    core[tv * ncu + tu + 1] = 1;
    core[(tv + 1) * ncu + tu] = 1;
    core[(tv + 1) * ncu + tu + 1] = 1;
}

__global__ void k_item_dense(WorkItem *items, int64_t nitems) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nitems) return;
    const int32_t tile = items[t].tile;
    int64_t lo = 0, hi = t;  // first item of the tile
    while (lo < hi) {
        const int64_t mid = (lo + hi) / 2;
        if (items[mid].tile < tile) lo = mid + 1; else hi = mid;
    }
    const int64_t first = lo;
    lo = t;
    hi = nitems;  // one past the last item of the tile
    while (lo < hi) {
        const int64_t mid = (lo + hi) / 2;
        if (items[mid].tile <= tile) lo = mid + 1; else hi = mid;
    }
    items[t].dense = (int64_t)items[lo - 1].vend - items[first].vbeg >= DENSE_TILE_VIS;
}

__global__ void k_item_vend(WorkItem *items, int64_t nitems, int64_t nvalid) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nitems) return;
    items[t].vend = t + 1 < nitems ? items[t + 1].vbeg : (int32_t)nvalid;
}

int bits_for(int64_t maxval) {
    int b = 1;
    while (b < 63 && ((int64_t)1 << b) <= maxval) b++;
    return b;
}

}  // namespace

int sde_grid_pitch(int nu) { return (nu + 3) & ~3; }

int64_t sde_plan_nvis(const sde_plan *plan) { return plan ? plan->nvis : 0; }
int64_t sde_plan_bytes(const sde_plan *plan) { return plan ? plan->bytes : 0; }
int sde_plan_stats(const sde_plan *plan, int64_t *nitems, int64_t *nchunks, int64_t *nexc) {
    if (!plan) return SDE_EINVAL;
    if (nitems) *nitems = plan->nitems;
    if (nchunks) *nchunks = plan->nchunks;
    if (nexc) *nexc = plan->nexc;
    return SDE_OK;
}

static int plan_alloc(sde_plan *pl, void **p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    int rc = ctx_alloc(pl->ctx, p, bytes);
    if (rc == SDE_OK) pl->bytes += (int64_t)bytes;
    return rc;
}

int sde_plan_destroy(sde_plan *pl) {
    if (!pl) return SDE_OK;
    sde_ctx *ctx = pl->ctx;
    cudaSetDevice(ctx->device);
    // stream-ordered frees: after the plan's last use on the context's stream
    void *ptrs[] = {pl->fobs, pl->rec, pl->wt, pl->gdd, pl->orig, pl->rot, pl->gconj, pl->chunks,
                    pl->items, pl->exc, pl->wt_all, pl->cf, pl->cft, pl->d_sums, pl->inv, pl->core_lo};
    for (void *p : ptrs) ctx_free(ctx, p, 0);
    ctx->bytes -= pl->bytes;
    delete pl;
    return SDE_OK;
}

// Upload (or alias) caller arrays; builds everything described at the top of the file.
int sde_plan_create(sde_ctx *ctx, const sde_gridspec *spec, int64_t nvis, const float *u,
                    const float *v, const float *w, const float *vis, const float *wt,
                    int where, sde_plan **out) {
    return sde_plan_create_opts(ctx, spec, nvis, u, v, w, vis, wt, where, nullptr, out);
}

int sde_plan_create_opts(sde_ctx *ctx, const sde_gridspec *spec, int64_t nvis, const float *u,
                         const float *v, const float *w, const float *vis, const float *wt,
                         int where, const sde_plan_opts *opts, sde_plan **out) {
    if (!ctx || !spec || !out || nvis < 0 || (nvis > 0 && (!u || !v || !w || !vis || !wt))) {
        sde_set_error("sde_plan_create: bad arguments");
        return SDE_EINVAL;
    }
    const int item_max = opts && opts->item_max > 0 ? opts->item_max : ITEM_MAX;
    const int chunk_max = opts && opts->chunk_max > 0 ? opts->chunk_max : CHUNK_MAX;
    if (item_max > ITEM_LIMIT || chunk_max > CHUNK_LIMIT || chunk_max > item_max) {
        sde_set_error("sde_plan_create: work item %d / chunk %d out of range (item <= %d, "
                      "chunk <= %d, chunk <= item)", item_max, chunk_max, ITEM_LIMIT, CHUNK_LIMIT);
        return SDE_EINVAL;
    }
    if (spec->supp != SUPP || spec->osamp != OSAMP) {
        sde_set_error("sde_plan_create: support %d / oversampling %d unsupported (SF needs 3/128)",
                      spec->supp, spec->osamp);
        return SDE_EINVAL;
    }
    if (spec->nu < 2 * SUPP + 1 || spec->nv < 2 * SUPP + 1 || nvis >= (int64_t)0x7FFFFFFF) {
        sde_set_error("sde_plan_create: grid %dx%d / %lld visibilities out of range", spec->nu,
                      spec->nv, (long long)nvis);
        return SDE_EINVAL;
    }
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    sde_plan *pl = new sde_plan();
    pl->ctx = ctx;
    pl->spec = *spec;
    pl->doshift = (spec->shift[0] != 1.0) || (spec->shift[4] != 1.0) || (spec->shift[8] != 1.0);
    pl->pitch = plan_pitch(spec->nu);
    pl->ntu = (spec->nu + TILE - 1) / TILE;
    pl->ntv = (spec->nv + TILE - 1) / TILE;
    pl->nvis_in = nvis;
    pl->item_max = item_max;
    pl->chunk_max = chunk_max;
    int rc = SDE_OK;
#define PL_TRY(x)                      \
    do {                               \
        rc = (x);                      \
        if (rc != SDE_OK) goto fail;   \
    } while (0)
#define PL_CUDA(x)                                                                   \
    do {                                                                             \
        cudaError_t _e = (x);                                                        \
        if (_e != cudaSuccess) {                                                     \
            sde_set_error("plan: %s: %s", #x, cudaGetErrorString(_e));               \
            rc = _e == cudaErrorMemoryAllocation ? SDE_ENOMEM : SDE_ECUDA;           \
            goto fail;                                                               \
        }                                                                            \
    } while (0)
    {
        const size_t n = (size_t)(nvis > 0 ? nvis : 1);
        const float *du = u, *dv = v, *dw = w, *dwt = wt;
        const float2 *dvis = (const float2 *)vis;
        if (where == SDE_HOST && nvis > 0) {
            float *bu, *bv, *bw, *bwt;
            float2 *bvis;
            PL_TRY(ctx_scratch(ctx, "pl_u", 4 * n, (void **)&bu));
            PL_TRY(ctx_scratch(ctx, "pl_v", 4 * n, (void **)&bv));
            PL_TRY(ctx_scratch(ctx, "pl_w", 4 * n, (void **)&bw));
            PL_TRY(ctx_scratch(ctx, "pl_wt", 4 * n, (void **)&bwt));
            PL_TRY(ctx_scratch(ctx, "pl_vis", 8 * n, (void **)&bvis));
            PL_CUDA(cudaMemcpyAsync(bu, u, 4 * n, cudaMemcpyHostToDevice, st));
            PL_CUDA(cudaMemcpyAsync(bv, v, 4 * n, cudaMemcpyHostToDevice, st));
            PL_CUDA(cudaMemcpyAsync(bw, w, 4 * n, cudaMemcpyHostToDevice, st));
            PL_CUDA(cudaMemcpyAsync(bwt, wt, 4 * n, cudaMemcpyHostToDevice, st));
            PL_CUDA(cudaMemcpyAsync(bvis, vis, 8 * n, cudaMemcpyHostToDevice, st));
            du = bu; dv = bv; dw = bw; dwt = bwt; dvis = bvis;
        }
        GParams gp;
        gp.uscale = spec->uscale; gp.uoffset = spec->uoffset;
        gp.vscale = spec->vscale; gp.voffset = spec->voffset;
        gp.uorigin = spec->uorigin; gp.vorigin = spec->vorigin;
        gp.nu = spec->nu; gp.nv = spec->nv; gp.supp = spec->supp; gp.osamp = spec->osamp;
        memcpy(gp.s, spec->shift, sizeof gp.s);
        gp.doshift = pl->doshift;
        gp.identity = 1;
        for (int k = 0; k < 9; k++)
            if (spec->shift[k] != ((k % 4) == 0 ? 1.0 : 0.0)) gp.identity = 0;
        gp.diagonal = 1;
        for (int k = 0; k < 9; k++)
            if (k % 4 != 0 && spec->shift[k] != 0.0) gp.diagonal = 0;
        gp.fast = gp.identity && spec->uoffset == 0.0f && spec->voffset == 0.0f;
        gp.near_id = gp.diagonal && fabs(spec->shift[0] - 1.0) <= 0x1p-50 && fabs(spec->shift[4] - 1.0) <= 0x1p-50 &&
                     spec->uoffset == 0.0f && spec->voffset == 0.0f && spec->osamp >= 1 && spec->osamp <= 65536;
        gp.ntu = pl->ntu;
        gp.twopi = (double)(8.0f * atanf(1.0f));  // TWOPI = 8 * ATAN(1.0), REAL (grdh2d.f:91)

        uint32_t *keys, *vals, *ktmp, *vtmp, *exc_list;
        PlanRecU *rec_u;
        unsigned long long *counts;
        PL_TRY(ctx_scratch(ctx, "pl_keys", 4 * n, (void **)&keys));
        PL_TRY(ctx_scratch(ctx, "pl_vals", 4 * n, (void **)&vals));
        PL_TRY(ctx_scratch(ctx, "pl_ktmp", 4 * n, (void **)&ktmp));
        PL_TRY(ctx_scratch(ctx, "pl_vtmp", 4 * n, (void **)&vtmp));
        PL_TRY(ctx_scratch(ctx, "pl_exclist", 4 * n, (void **)&exc_list));
        PL_TRY(ctx_scratch(ctx, "pl_rec", sizeof(PlanRecU) * n, (void **)&rec_u));
        PL_TRY(ctx_scratch(ctx, "pl_counts", 64, (void **)&counts));
        PL_CUDA(cudaMemsetAsync(counts, 0, 64, st));
        const int T = 256;
        if (nvis > 0) {
            k_plan_geom<<<ceil_div(nvis, T), T, 0, st>>>(gp, du, dv, dw, dvis, dwt, nvis, keys, vals,
                                                       rec_u, exc_list, counts);
            PL_CUDA(cudaGetLastError());
        }
        int64_t ntiles = (int64_t)pl->ntu * pl->ntv;
        int kbits = bits_for((ntiles << 12) + 1);
        if (kbits > 32) {
            sde_set_error("plan: grid too large for 32-bit tile keys");
            rc = SDE_EINVAL;
            goto fail;
        }
        if (nvis > 0) PL_TRY(launch_radix_sort_u32(ctx, keys, vals, nvis, kbits, ktmp, vtmp));
        // run heads of the sorted keys (0 past the gridded visibilities) and their count, read
        // back with the visibility counts: one wait for both
        uint32_t *head, *ridx, *tot;
        PL_TRY(ctx_scratch(ctx, "pl_runhead", 4 * n, (void **)&head));
        PL_TRY(ctx_scratch(ctx, "pl_runidx", 4 * n, (void **)&ridx));
        PL_TRY(ctx_scratch(ctx, "pl_tot", 16, (void **)&tot));
        if (nvis > 0) {
            k_run_heads<<<ceil_div(nvis, T), T, 0, st>>>(keys, counts, nvis, head);
            PL_CUDA(cudaGetLastError());
            PL_TRY(launch_exclusive_scan_u32(ctx, head, ridx, nvis, tot));
        } else {
            PL_CUDA(cudaMemsetAsync(tot, 0, 16, st));
        }
        unsigned long long hc[3] = {0, 0, 0};
        uint32_t hruns = 0;
        PL_CUDA(cudaMemcpyAsync(ctx->h_small, counts, sizeof hc, cudaMemcpyDeviceToHost, st));
        PL_CUDA(cudaMemcpyAsync(ctx->h_small + sizeof hc, tot, sizeof hruns, cudaMemcpyDeviceToHost, st));
        PL_CUDA(cudaStreamSynchronize(st));
        memcpy(hc, ctx->h_small, sizeof hc);
        memcpy(&hruns, ctx->h_small + sizeof hc, sizeof hruns);
        const int64_t nvalid = (int64_t)hc[0], nexc = (int64_t)hc[1];
        pl->nuntouched = nvis - (int64_t)hc[2];
        pl->nvis = nvalid;
        pl->nexc = nexc;
        const size_t nv1 = (size_t)(nvalid > 0 ? nvalid : 1);
        PL_TRY(plan_alloc(pl, (void **)&pl->fobs, 8 * nv1));
        PL_TRY(plan_alloc(pl, (void **)&pl->rec, 16 * nv1));
        PL_TRY(plan_alloc(pl, (void **)&pl->wt, 4 * nv1));
        PL_TRY(plan_alloc(pl, (void **)&pl->gdd, 4 * nv1));
        PL_TRY(plan_alloc(pl, (void **)&pl->orig, 4 * nv1));
        PL_TRY(plan_alloc(pl, (void **)&pl->gconj, nv1));
        if (pl->doshift) PL_TRY(plan_alloc(pl, (void **)&pl->rot, 8 * nv1));
        PL_TRY(plan_alloc(pl, (void **)&pl->d_sums, 4 * sizeof(double)));
        // exception list (also carries the GRDDEH2D geometry of non-gridding visibilities);
        // the gather below fills in the sorted positions
        size_t ne1 = (size_t)(nexc > 0 ? nexc : 1);
        PL_TRY(plan_alloc(pl, (void **)&pl->exc, exc_bytes(ne1)));
        if (nexc > 0) {
            float *exc_wt = (float *)((char *)pl->exc + exc_wt_off(ne1));
            float2 *exc_rot = (float2 *)((char *)pl->exc + exc_rot_off(ne1));
            k_exc_write<<<ceil_div(nexc, T), T, 0, st>>>(gp, du, dv, dw, dwt, rec_u, exc_list, nexc, pl->exc,
                                                       exc_wt, exc_rot);
            PL_CUDA(cudaGetLastError());
        }
        // runs, chunks, work items
        if (nvalid > 0) {
            const int64_t nruns = hruns;
            uint32_t *rstart, *nch, *nih, *cbase, *ibase;
            int32_t *tstart;
            PL_TRY(ctx_scratch(ctx, "pl_rstart", 4 * (size_t)nruns, (void **)&rstart));
            PL_TRY(ctx_scratch(ctx, "pl_tstart", 4 * (size_t)nruns, (void **)&tstart));
            PL_TRY(ctx_scratch(ctx, "pl_nch", 4 * (size_t)nruns, (void **)&nch));
            PL_TRY(ctx_scratch(ctx, "pl_nih", 4 * (size_t)nruns, (void **)&nih));
            PL_TRY(ctx_scratch(ctx, "pl_cbase", 4 * (size_t)nruns, (void **)&cbase));
            PL_TRY(ctx_scratch(ctx, "pl_ibase", 4 * (size_t)nruns, (void **)&ibase));
            k_run_compact<<<ceil_div(nvalid, T), T, 0, st>>>(head, ridx, counts, rstart);
            PL_CUDA(cudaGetLastError());
            k_run_tilehead<<<ceil_div(nruns, T), T, 0, st>>>(keys, rstart, nruns, tstart);
            PL_CUDA(cudaGetLastError());
            PL_TRY(launch_inclusive_max_scan_i32(ctx, tstart, tstart, nruns));
            k_run_counts<<<ceil_div(nruns, T), T, 0, st>>>(rstart, tstart, nruns, nvalid, pl->item_max,
                                                         pl->chunk_max, nch, nih);
            PL_CUDA(cudaGetLastError());
            PL_TRY(launch_exclusive_scan_u32(ctx, nih, ibase, nruns, tot + 1));
            PL_TRY(launch_exclusive_scan_u32(ctx, nch, cbase, nruns, tot + 2));
            uint32_t htot[2];
            PL_TRY(ctx_read_small(ctx, st, htot, tot + 1, sizeof htot));
            const int64_t nitems = htot[0], nchunks = htot[1];
            pl->nitems = nitems;
            pl->nchunks = nchunks;
            PL_TRY(plan_alloc(pl, (void **)&pl->items, sizeof(WorkItem) * (size_t)nitems));
            PL_TRY(plan_alloc(pl, (void **)&pl->chunks, sizeof(uint2) * (size_t)nchunks));
            uint64_t *ckey, *cktmp;
            uint32_t *cval, *cvtmp, *cstart;
            PL_TRY(ctx_scratch(ctx, "pl_ckey", 8 * (size_t)nchunks, (void **)&ckey));
            PL_TRY(ctx_scratch(ctx, "pl_cktmp", 8 * (size_t)nchunks, (void **)&cktmp));
            PL_TRY(ctx_scratch(ctx, "pl_cval", 4 * (size_t)nchunks, (void **)&cval));
            PL_TRY(ctx_scratch(ctx, "pl_cvtmp", 4 * (size_t)nchunks, (void **)&cvtmp));
            PL_TRY(ctx_scratch(ctx, "pl_cstart", 4 * (size_t)nchunks, (void **)&cstart));
            const int jbits = bits_for(pl->item_max / pl->chunk_max);
            const int lbits = bits_for(pl->chunk_max - 1);
            k_run_emit<<<ceil_div(nruns, T), T, 0, st>>>(keys, rstart, tstart, nruns, nvalid, cbase, ibase,
                                                       pl->item_max, pl->chunk_max, lbits, jbits, ckey,
                                                       cval, cstart, pl->items);
            PL_CUDA(cudaGetLastError());
            k_chunk_len<<<ceil_div(nchunks, T), T, 0, st>>>(cstart, nchunks, nvalid, pl->chunk_max,
                                                          jbits + 12, 6 + lbits + jbits + 12, ckey);
            PL_CUDA(cudaGetLastError());
            const int shift_item = LENBIN_BITS + 6 + lbits + jbits + 12;
            const int cbits = shift_item + bits_for(nitems);
            PL_TRY(launch_radix_sort_u64(ctx, ckey, cval, nchunks, cbits, cktmp, cvtmp));
            uint32_t *clen, *cpos;
            PL_TRY(ctx_scratch(ctx, "pl_clen", 4 * (size_t)nchunks, (void **)&clen));
            PL_TRY(ctx_scratch(ctx, "pl_cpos", 4 * (size_t)nchunks, (void **)&cpos));
            k_chunk_final<<<ceil_div(nchunks, T), T, 0, st>>>(ckey, cval, cstart, keys, nchunks,
                                                            nvalid, shift_item, pl->chunks, clen,
                                                            pl->items);
            PL_CUDA(cudaGetLastError());
            // chunk order: each chunk's new start, then one gather of the caller-order sectors
            PL_TRY(launch_exclusive_scan_u32(ctx, clen, cpos, nchunks, nullptr));
            k_plan_gather<<<ceil_div(nchunks, T / 32), T, 0, st>>>(vals, cpos, nchunks, pl->chunks, rec_u,
                                                                 pl->fobs, pl->rec, pl->wt, pl->gdd,
                                                                 pl->orig, pl->rot, pl->gconj,
                                                                 nexc > 0 ? pl->exc : nullptr);
            PL_CUDA(cudaGetLastError());
            k_item_vbeg<<<ceil_div(nitems, T), T, 0, st>>>(pl->chunks, nitems, pl->items);
            PL_CUDA(cudaGetLastError());
            k_item_vend<<<ceil_div(nitems, T), T, 0, st>>>(pl->items, nitems, nvalid);
            PL_CUDA(cudaGetLastError());
            k_item_dense<<<ceil_div(nitems, T), T, 0, st>>>(pl->items, nitems);
            PL_CUDA(cudaGetLastError());
            const size_t ncore = (size_t)(pl->ntu + 1) * (pl->ntv + 1);
            PL_TRY(plan_alloc(pl, (void **)&pl->core_lo, ncore));
            PL_CUDA(cudaMemsetAsync(pl->core_lo, 0, ncore, st));
            k_core_lo<<<ceil_div(nitems, T), T, 0, st>>>(pl->items, nitems, pl->ntu, pl->core_lo);
            PL_CUDA(cudaGetLastError());
        }
        // gridding function: the context's 'SF' table
        PL_TRY(plan_alloc(pl, (void **)&pl->cf, sizeof(float) * CFLEN));
        PL_TRY(plan_alloc(pl, (void **)&pl->cft, sizeof(float) * 129 * 8));
        PL_CUDA(cudaMemcpyAsync(pl->cf, ctx->d_cf, sizeof(float) * CFLEN, cudaMemcpyDeviceToDevice, st));
        PL_CUDA(cudaMemcpyAsync(pl->cft, ctx->d_cft, sizeof(float) * 129 * 8, cudaMemcpyDeviceToDevice, st));
    }
    ctx->bytes += pl->bytes;
    *out = pl;
    return SDE_OK;
fail:
    ctx->bytes += pl->bytes;
    sde_plan_destroy(pl);
    return rc;
#undef PL_TRY
#undef PL_CUDA
}
