// grid.cu -- tiled gridding (GRDH2D) and degridding (GRDDEH2D) over a sde_plan.
//
// Both kernels are persistent: one CTA per SM of TEAMS teams of 256 threads; a team takes
// work items (<= ITEM_MAX visibilities of one 64x64-cell tile) from an atomic counter.
//
// Gridding: a team keeps its item's tile plus a 3-cell halo in shared memory.  A 4-lane
// group owns a chunk (<= CHUNK_MAX visibilities of one cell pair) and accumulates the
// chunk's 7x8 complex footprint in registers (two columns per lane), then adds it into the
// shared tile once; the chunk order (length bin, colour class, length class, chunk index,
// cell) gives the 8 chunks of a warp mostly disjoint cells and similar lengths.  The shared
// tile is then reduced into the raw grid in HBM with vector red.global.add (only the cells
// the item touched).
//
// Degridding: a team stages the model grid's tile (+halo) into shared memory with a single
// TMA 2-D bulk copy, then a 4-lane group per chunk interpolates the chunk's visibilities
// from a register copy of the chunk cell's 7x8 neighbourhood (two columns per lane) and
// reduces the lanes' partial sums with shuffles.
#include <math.h>
#include <string.h>

#include "common.cuh"

namespace {

// ---------------------------------------------------------------------------------------
// Gridding (GRDH2D's 7x7 accumulation, grd/grdh2d.f:168-189).
//
// A chunk holds visibilities of one cell pair (lu0, lu0+1); its footprint is a 7-row x
// 8-column window.  A 4-lane group owns a chunk: lane q holds window columns q and q+4 over
// the 7 rows in registers (14 complex sums) for the whole chunk and adds them into the
// work item's shared tile once, at the end (shared-memory atomics: the 8 chunks of a warp
// share a colour class, so their windows do not overlap).  The group's lanes load four
// consecutive records at a time (one 64-byte run) and exchange weight x value and the
// offset word by shuffle.
//
// A CTA is TEAMS independent teams of 256 threads, one CTA per SM, persistent: the teams
// share one copy of the tap tables (filled once) and each team owns a shared tile, takes
// work items from an atomic counter and synchronises with its own named barrier, so a
// team waiting at its item's end does not hold the others.  The tables are laid out so
// that no read has a bank conflict:
//   v table: per offset row d (0..128) 4 copies of the 7 v taps (+ a zero), 32 bytes each
//     in a 128-byte row; group g reads copy g mod 4, so the 4 groups of a half-warp read
//     4 different 32-byte octets (measured on GB300 with a probe of this access pattern: a
//     128-bit shared load of 4-lane groups takes the minimum 2 wavefronts this way, and
//     3.5 with 2 copies in 64-byte rows);
//   u table: per (d, column-in-pair off) row 4 copies of the 4 pairs (t'_q, t'_{q+4}),
//     t'_j = tap j - off for window column j (zero outside 0..6); lane q of group g reads
//     pair q of copy g mod 4: the 4 groups of a half-warp (the unit of a 64-bit load) read
//     the 4 different 32-byte octets of one 128-byte row (2 wavefronts, the minimum).
constexpr int TEAMS = 3;
constexpr int TEAM_THREADS = 256;
constexpr int GRID_THREADS = TEAMS * TEAM_THREADS;
constexpr int GLANES = 4;                          // lanes per chunk
constexpr int GGROUPS = TEAM_THREADS / GLANES;     // chunks in flight per team
constexpr int VT_ROW = 32;                         // floats per v-table row (4 copies x 8)
static_assert(VT_ROW * 4 == TAPROW_BYTES, "the plan record's v-table offsets");
constexpr int VT_FLOATS = 129 * VT_ROW;
constexpr int UT_ROW = 32;                         // floats per u-table row (4 copies x 4 pairs)
static_assert(UT_ROW * 4 == TAPROW_BYTES, "the plan record's u-table offsets");
constexpr int UT_FLOATS = 2 * 129 * UT_ROW;
constexpr int GTAB_FLOATS = VT_FLOATS + UT_FLOATS;
constexpr int GTILE_FLOATS = 2 * STILE * STILE;    // a team's tile: re and im planes
constexpr int NPAIR = (NTAP + 1) / 2;              // window rows taken in pairs

// cft_g[d * 8 + a] = tap a (0..6) of offset row d; cft_g[d * 8 + 7] = 0
__device__ __forceinline__ void fill_tap_tables(const float *__restrict__ cft_g, float *vt, float *ut) {
    for (int k = threadIdx.x; k < VT_FLOATS; k += blockDim.x)
        vt[k] = cft_g[(k / VT_ROW) * 8 + (k & 7)];
    for (int k = threadIdx.x; k < UT_FLOATS; k += blockDim.x) {
        const int r = k / UT_ROW, d = r >> 1, off = r & 1, e = k & 7;  // e: pair e/2, half e&1
        const int a = (e >> 1) + 4 * (e & 1) - off;
        ut[k] = a >= 0 && a < NTAP ? cft_g[d * 8 + a] : 0.f;
    }
}

// the team's named barrier (0 is __syncthreads)
__device__ __forceinline__ void team_sync(int team) {
    asm volatile("bar.sync %0, %1;" ::"r"(team + 1), "r"(TEAM_THREADS) : "memory");
}

// 1 on every thread of the team when pred holds on all of them
__device__ __forceinline__ int team_and(int team, int pred) {
    int r;
    asm volatile(
        "{ .reg .pred pi, po; setp.ne.s32 pi, %1, 0; bar.red.and.pred po, %2, %3, pi;"
        " selp.s32 %0, 1, 0, po; }"
        : "=r"(r)
        : "r"(pred), "r"(team + 1), "r"(TEAM_THREADS)
        : "memory");
    return r;
}

// Grid one work item: its chunks into the team's shared tile (planar re/im planes, zero on
// entry), then the touched cells into the raw grid.  Reading the tile back zeroes it, so
// the next item starts from a clean tile once the team barrier after the flush has passed.
template <bool PSF, bool COMP>
__device__ __forceinline__ void grid_item(const WorkItem &it, const uint2 *__restrict__ chunks,
                                          const float4 *__restrict__ rec, const float *vt,
                                          const float *ut, float *tre, float *tim, float2 *raw,
                                          float2 *raw_lo, int pitch, int ntu, int nu, int nv,
                                          int tid, int team) {
    // Every lane of a warp runs the same number of chunk rounds and visibility steps (the
    // warp's longest chunk; shorter chunks read zero-weight records, whose offset word 0
    // reads table row 0), so full-warp shuffles are safe.
    const int q = tid & (GLANES - 1);
    const int grp = tid / GLANES;
    const int gbase = threadIdx.x & (32 - GLANES);  // lane of q = 0 in this group
    const float *vcopy = vt + (grp & 3) * 8;
    const float *ucopy = ut + (grp & 3) * 8 + 2 * q;
    constexpr uint32_t FULL = 0xffffffffu;
    const int rounds = (it.cend - it.cbeg + GGROUPS - 1) / GGROUPS;
    for (int rr = 0; rr < rounds; rr++) {
        const int c = it.cbeg + rr * GGROUPS + grp;
        const bool live = c < it.cend;
        const uint2 ch = live ? chunks[c] : make_uint2(0u, 0u);
        const int start = (int)ch.x, cell = (int)(ch.y & 4095u), len = live ? (int)(ch.y >> 16) : 0;
        const int lu = cell & 63, lv = cell >> 6;
        int wlen = len;
#pragma unroll
        for (int d = GLANES; d < 32; d <<= 1) wlen = max(wlen, __shfl_xor_sync(FULL, wlen, d));
        // window rows in pairs (0,1) (2,3) (4,5) (6,-): one packed FMA (__ffma2_rn, two
        // round-to-nearest FMAs) per pair; the v-table row's zero fills the seventh pair's
        // second half
        float2 A0r[NPAIR], A0i[NPAIR], A1r[NPAIR], A1i[NPAIR];
#pragma unroll
        for (int p = 0; p < NPAIR; p++) {
            A0r[p] = make_float2(0.f, 0.f);
            A1r[p] = make_float2(0.f, 0.f);
            if (!PSF) {
                A0i[p] = make_float2(0.f, 0.f);
                A1i[p] = make_float2(0.f, 0.f);
            }
        }
        const float4 *pr = rec + start;
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        float4 cur = q < len ? pr[q] : zero;
        for (int k = 0; k < wlen; k += GLANES) {
            const float4 nxt = k + GLANES + q < len ? pr[k + GLANES + q] : zero;
            const uint32_t gq = __float_as_uint(cur.y);
            const float frq = PSF ? cur.x : cur.x * cur.z, fiq = PSF ? 0.f : cur.x * cur.w;
#pragma unroll
            for (int u = 0; u < GLANES; u++) {
                const uint32_t g = __shfl_sync(FULL, gq, gbase + u);
                const float fr = __shfl_sync(FULL, frq, gbase + u);
                const float fi = PSF ? 0.f : __shfl_sync(FULL, fiq, gbase + u);
                const float2 gu = *reinterpret_cast<const float2 *>(
                    reinterpret_cast<const char *>(ucopy) + (g & 0xFFFFu));
                const float4 *vr = reinterpret_cast<const float4 *>(reinterpret_cast<const char *>(vcopy) + (g >> 16));
                const float4 v0 = vr[0], v1 = vr[1];
                const float2 P[NPAIR] = {make_float2(v0.x, v0.y), make_float2(v0.z, v0.w),
                                         make_float2(v1.x, v1.y), make_float2(v1.z, v1.w)};
                const float h0r = gu.x * fr, h1r = gu.y * fr;
                const float2 H0r = make_float2(h0r, h0r), H1r = make_float2(h1r, h1r);
#pragma unroll
                for (int p = 0; p < NPAIR; p++) {
                    A0r[p] = __ffma2_rn(P[p], H0r, A0r[p]);
                    A1r[p] = __ffma2_rn(P[p], H1r, A1r[p]);
                }
                if (!PSF) {
                    const float h0i = gu.x * fi, h1i = gu.y * fi;
                    const float2 H0i = make_float2(h0i, h0i), H1i = make_float2(h1i, h1i);
#pragma unroll
                    for (int p = 0; p < NPAIR; p++) {
                        A0i[p] = __ffma2_rn(P[p], H0i, A0i[p]);
                        A1i[p] = __ffma2_rn(P[p], H1i, A1i[p]);
                    }
                }
            }
            cur = nxt;
        }
        if (!live) continue;
#pragma unroll
        for (int b = 0; b < NTAP; b++) {
            float *rr_ = &tre[(lv + b) * STILE + lu + q];
            float *ri = &tim[(lv + b) * STILE + lu + q];
            const int p = b >> 1;
            atomicAdd(rr_, (b & 1) ? A0r[p].y : A0r[p].x);
            if (!PSF) atomicAdd(ri, (b & 1) ? A0i[p].y : A0i[p].x);
            atomicAdd(rr_ + 4, (b & 1) ? A1r[p].y : A1r[p].x);
            if (!PSF) atomicAdd(ri + 4, (b & 1) ? A1i[p].y : A1i[p].x);
        }
    }
    team_sync(team);
    const int tu = it.tile % ntu, tv = it.tile / ntu;
    // flush FLUSH_B cells per thread at a time, so that the compensated path keeps FLUSH_B
    // returning atomics in flight instead of waiting on each
    constexpr int FLUSH_B = 4;
    for (int k0 = tid; k0 < STILE * STILE; k0 += FLUSH_B * TEAM_THREADS) {
        float2 val[FLUSH_B];
        int64_t gi[FLUSH_B];
#pragma unroll
        for (int j = 0; j < FLUSH_B; j++) {
            const int k = k0 + j * TEAM_THREADS;
            gi[j] = -1;
            val[j] = make_float2(0.f, 0.f);
            if (k >= STILE * STILE) continue;
            val[j] = make_float2(tre[k], tim[k]);
            if (val[j].x == 0.f && val[j].y == 0.f) continue;
            tre[k] = 0.f;
            tim[k] = 0.f;
            const int r = k / STILE, cc = k - r * STILE;
            // GRDH2D's 0-based raw cell; stored at raw index gu0 + 1 (RAW_SHIFT = SUPP + 1)
            const int gv0 = tv * TILE + r - SUPP, gu0 = tu * TILE + cc - SUPP;
            if (gv0 < 0 || gv0 >= nv || gu0 < 0 || gu0 >= nu) continue;
            gi[j] = (int64_t)gv0 * pitch + gu0 + 1;
        }
        if (COMP && it.dense) {
            // compensated sum across items (dense tiles, many items per cell): the atomic
            // returns the value it added to, so the rounding error of the stored sum is
            // exact (TwoSum) and goes to raw_lo
            float2 old[FLUSH_B];
#pragma unroll
            for (int j = 0; j < FLUSH_B; j++)
                if (gi[j] >= 0) old[j] = atomicAdd(&raw[gi[j]], val[j]);
#pragma unroll
            for (int j = 0; j < FLUSH_B; j++)
                if (gi[j] >= 0)
                    red_add_f2(&raw_lo[gi[j]], make_float2(two_sum_err(old[j].x, val[j].x),
                                                           two_sum_err(old[j].y, val[j].y)));
        } else {
#pragma unroll
            for (int j = 0; j < FLUSH_B; j++)
                if (gi[j] >= 0) red_add_f2(&raw[gi[j]], val[j]);
        }
    }
}

// Persistent gridding of one plan: every team takes work items from an atomic counter
// until the list is exhausted.
template <bool PSF, bool COMP>
__global__ void __launch_bounds__(GRID_THREADS, 1)
    k_grid(const WorkItem *__restrict__ items, int64_t nitems, unsigned long long *counter,
           const uint2 *__restrict__ chunks, const float4 *__restrict__ rec,
           const float *__restrict__ cft_g, float2 *raw, float2 *raw_lo, int pitch, int ntu, int nu,
           int nv) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *vt = reinterpret_cast<float *>(smem_raw);
    float *ut = vt + VT_FLOATS;
    const int team = threadIdx.x / TEAM_THREADS, tid = threadIdx.x % TEAM_THREADS;
    float *tre = ut + UT_FLOATS + team * GTILE_FLOATS;
    float *tim = tre + STILE * STILE;
    __shared__ long long s_next[TEAMS];
    for (int k = tid; k < STILE * STILE; k += TEAM_THREADS) {
        tre[k] = 0.f;
        tim[k] = 0.f;
    }
    fill_tap_tables(cft_g, vt, ut);
    __syncthreads();
    for (;;) {
        if (tid == 0) s_next[team] = (long long)atomicAdd(counter, 1ull);
        team_sync(team);
        const long long n = s_next[team];
        if (n >= nitems) break;
        const WorkItem it = items[n];
        if (tid == 0) {
            // the item's chunk list and records stream into L2 while the first chunks run
            prefetch_l2_range(chunks, it.cbeg, it.cend, 8);
            prefetch_l2_range(rec, it.vbeg, it.vend, 16);
        }
        grid_item<PSF, COMP>(it, chunks, rec, vt, ut, tre, tim, raw, raw_lo, pitch, ntu, nu, nv, tid, team);
        team_sync(team);
    }
}

// Persistent gridding of many plans (a mosaic's pointings, a batch of served jobs): the
// same, over the combined work-item list of all plans (item_start[p] = first combined index
// of plan p).  One launch grids every plan.
template <bool PSF, bool COMP>
__global__ void __launch_bounds__(GRID_THREADS, 1)
    k_grid_batch(const BatchPlan *__restrict__ plans, const int64_t *__restrict__ item_start,
                 int nplans, unsigned long long *counter, const float *__restrict__ cft_g) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *vt = reinterpret_cast<float *>(smem_raw);
    float *ut = vt + VT_FLOATS;
    const int team = threadIdx.x / TEAM_THREADS, tid = threadIdx.x % TEAM_THREADS;
    float *tre = ut + UT_FLOATS + team * GTILE_FLOATS;
    float *tim = tre + STILE * STILE;
    __shared__ long long s_next[TEAMS];
    __shared__ int s_plan[TEAMS];
    for (int k = tid; k < STILE * STILE; k += TEAM_THREADS) {
        tre[k] = 0.f;
        tim[k] = 0.f;
    }
    fill_tap_tables(cft_g, vt, ut);
    __syncthreads();
    const int64_t total = item_start[nplans];
    for (;;) {
        if (tid == 0) {
            const long long n = (long long)atomicAdd(counter, 1ull);
            int p = 0;
            if (n < total)
                while (p + 1 < nplans && item_start[p + 1] <= n) p++;
            s_next[team] = n;
            s_plan[team] = p;
        }
        team_sync(team);
        const long long n = s_next[team];
        if (n >= total) break;
        const BatchPlan P = plans[s_plan[team]];
        const WorkItem it = P.items[n - item_start[s_plan[team]]];
        if (tid == 0) {
            prefetch_l2_range(P.chunks, it.cbeg, it.cend, 8);
            prefetch_l2_range(P.rec, it.vbeg, it.vend, 16);
        }
        grid_item<PSF, COMP>(it, P.chunks, P.rec, vt, ut, tre, tim, P.raw, P.raw_lo, P.pitch, P.ntu,
                             P.nu, P.nv, tid, team);
        team_sync(team);
    }
}

// Plan-invariant sums: LSUMWT = sum of UVWT (grd/grdh2d.f:185) and SUMWT (grd/grdh2d.f:157).
// A visibility's UVWT sum over its 7x7 taps is W * SU * SV, SU and SV the sums of its u and v
// tap rows (REAL, in tap order, once per row).  Each thread sums its visibilities as
// float-float pairs (exact products by FMA, TwoSum additions: ~2^-44 relative), and the
// partial sums meet in DOUBLE: FP64 arithmetic per visibility is the slow path on this GPU.
constexpr int RED_T = 256;
__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float x) {
    const float s = __fadd_rn(hi, x);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    hi = s;
    lo = __fadd_rn(lo, e);
}
__global__ void __launch_bounds__(RED_T) k_plan_sums(const float4 *__restrict__ rec,
                                                      const float *__restrict__ cft, int64_t n,
                                                      double *partial) {
    __shared__ double sh[2][RED_T / 32];
    __shared__ float rowsum[129];
    for (int d = threadIdx.x; d < 129; d += RED_T) {
        float t = 0.f;
        for (int a = 0; a < NTAP; a++) t = __fadd_rn(t, cft[d * 8 + a]);
        rowsum[d] = t;
    }
    __syncthreads();
    float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f;
    for (int64_t p = (int64_t)blockIdx.x * RED_T + threadIdx.x; p < n; p += (int64_t)gridDim.x * RED_T) {
        const float2 wgp = reinterpret_cast<const float2 *>(rec + p)[0];
        const uint32_t g = __float_as_uint(wgp.y);
        const float su = rowsum[taps_du(g)], sv = rowsum[taps_dv(g)], w = wgp.x;
        // W*SU exactly as ph + pl, then (ph + pl)*SV as th + tl
        const float ph = __fmul_rn(w, su), pl = __fmaf_rn(w, su, -ph);
        const float th = __fmul_rn(ph, sv);
        const float tl = __fmaf_rn(pl, sv, __fmaf_rn(ph, sv, -th));
        two_sum_acc(h0, l0, th);
        l0 = __fadd_rn(l0, tl);
        two_sum_acc(h1, l1, w);
    }
    double s0 = (double)h0 + (double)l0, s1 = (double)h1 + (double)l1;
    for (int d = 16; d > 0; d >>= 1) {
        s0 += __shfl_down_sync(0xffffffffu, s0, d);
        s1 += __shfl_down_sync(0xffffffffu, s1, d);
    }
    if ((threadIdx.x & 31) == 0) {
        sh[0][threadIdx.x >> 5] = s0;
        sh[1][threadIdx.x >> 5] = s1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int k = 0; k < RED_T / 32; k++) {
            a += sh[0][k];
            b += sh[1][k];
        }
        partial[2 * blockIdx.x] = a;
        partial[2 * blockIdx.x + 1] = b;
    }
}

// The partial pairs summed in a fixed order by one block: thread t takes partials t, t+256,
// ..., then a fixed tree over the threads (deterministic for a given partial count).
__global__ void __launch_bounds__(RED_T) k_sum_pairs(const double *partial, int n, double *out) {
    __shared__ double sh[2][RED_T];
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < n; k += RED_T) {
        a += partial[2 * k];
        b += partial[2 * k + 1];
    }
    sh[0][threadIdx.x] = a;
    sh[1][threadIdx.x] = b;
    __syncthreads();
    for (int s = RED_T / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + s];
            sh[1][threadIdx.x] += sh[1][threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sh[0][0];
        out[1] = sh[1][0];
    }
}

// Transposed gridding-function table: cft[d][a] = CF(CFOFFSET + (d-64) + OSAMP*(a-SUPP)).
__global__ void k_build_cft(const float *cf, float *cft) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= 129) return;
    const int center = (SUPP + 1) * OSAMP;  // CFOFFSET - 1 (0-based)
    for (int a = 0; a < 8; a++)
        cft[d * 8 + a] = a < NTAP ? cf[center + (d - 64) + OSAMP * (a - SUPP)] : 0.f;
}

// ---------------------------------------------------------------------------------------
// Symmetrise, shift left by SUPPU and normalise (grd/grdh2d.f:202-226).  raw and out are
// [nv][pitch] complex; out(u,v) = scale * R'(u+SUPP, v) for u <= NU-SUPP, else 0, where R'
// adds conj(R(UC-k, 2VC-v)) into columns UC+k, k = 0..SUPP, UC = UORIGIN+SUPP.
// One cell of the final GRDH2D grid from the raw accumulation (index idx of [nv][pitch]).
__device__ __forceinline__ float2 raw_at(const float2 *__restrict__ raw,
                                         const float2 *__restrict__ raw_lo, int64_t i) {
    float2 r = raw[i];
    if (raw_lo) {
        const float2 e = raw_lo[i];
        r.x = r.x + e.x;
        r.y = r.y + e.y;
    }
    return r;
}

__device__ __forceinline__ float2 finalize_cell(const float2 *__restrict__ raw,
                                                const float2 *__restrict__ raw_lo, int64_t idx,
                                                int nu, int nv, int pitch, int uorigin,
                                                int vorigin, int supp, float scale) {
    const int v0 = (int)(idx / pitch), u0 = (int)(idx - (int64_t)v0 * pitch);
    if (u0 >= nu) return make_float2(0.f, 0.f);
    const int u1 = u0 + 1, v1 = v0 + 1;  // 1-based
    float2 r = make_float2(0.f, 0.f);
    if (u1 <= nu - supp) {
        const int U = u1 + supp;            // GRDH2D's raw column (1-based) = raw index
        r = raw_at(raw, raw_lo, (int64_t)v0 * pitch + U);
        const int UC = uorigin + supp, VC = vorigin;
        const int k = U - UC;
        if (k >= 0 && k <= supp) {
            const int dvv = v1 - VC;
            const int vm = 2 * VC - v1;
            if (dvv >= -(nv / 2) + 1 && dvv <= nv / 2 - 1 && vm >= 1 && vm <= nv) {
                const float2 m = raw_at(raw, raw_lo, (int64_t)(vm - 1) * pitch + (UC - k));
                r.x = r.x + m.x;
                r.y = r.y - m.y;
            }
        }
        r.x *= scale;
        r.y *= scale;
    }
    return r;
}

// The compensation plane folded into the raw grid over one marked core (see k_core_lo):
// raw = raw + lo where lo != 0 (the add finalize would do), lo = 0.  A core row is 32 pairs
// of cells starting at an even raw index (16-byte aligned: the pitch is a multiple of 4);
// each thread loads 8 pairs before touching any.
__device__ __forceinline__ void fold_core(float2 *raw, float2 *raw_lo, int cu, int cv, int nv, int pitch) {
    const int r0 = cv * TILE - SUPP, i0 = cu * TILE - (SUPP - 1);
    float4 *raw4 = reinterpret_cast<float4 *>(raw);
    float4 *lo4 = reinterpret_cast<float4 *>(raw_lo);
    constexpr int PAIRS = TILE * TILE / 2 / 256;  // 8
    float4 e[PAIRS];
    int64_t q[PAIRS];
#pragma unroll
    for (int j = 0; j < PAIRS; j++) {
        const int k = threadIdx.x + j * 256;
        const int r = r0 + (k >> 5), i = i0 + 2 * (k & 31);
        q[j] = -1;
        e[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (r < 0 || r >= nv || i < 0 || i >= pitch) continue;
        q[j] = ((int64_t)r * pitch + i) >> 1;
        e[j] = lo4[q[j]];
    }
#pragma unroll
    for (int j = 0; j < PAIRS; j++) {
        if (q[j] < 0 || (e[j].x == 0.f && e[j].y == 0.f && e[j].z == 0.f && e[j].w == 0.f)) continue;
        float4 h = raw4[q[j]];
        h.x = h.x + e[j].x;
        h.y = h.y + e[j].y;
        h.z = h.z + e[j].z;
        h.w = h.w + e[j].w;
        raw4[q[j]] = h;
        lo4[q[j]] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

__global__ void __launch_bounds__(256) k_fold_lo(float2 *raw, float2 *raw_lo, const uint8_t *__restrict__ core,
                                                 int ncu, int nv, int pitch) {
    if (!core[blockIdx.x]) return;
    fold_core(raw, raw_lo, blockIdx.x % ncu, blockIdx.x / ncu, nv, pitch);
}

// the marked cores of many grids, one block per (grid, core) pair of the list
__global__ void __launch_bounds__(256) k_fold_lo_batch(const BatchPlan *__restrict__ d,
                                                       const int2 *__restrict__ cores) {
    const int2 c = cores[blockIdx.x];
    const BatchPlan &p = d[c.x];
    fold_core(p.raw, p.raw_lo, c.y & 0xFFFF, c.y >> 16, p.nv, p.pitch);
}

__global__ void k_finalize(const float2 *__restrict__ raw, const float2 *__restrict__ raw_lo,
                           float2 *__restrict__ out, int nu, int nv, int pitch, int uorigin,
                           int vorigin, int supp, float scale) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)nv * pitch) return;
    out[idx] = finalize_cell(raw, raw_lo, idx, nu, nv, pitch, uorigin, vorigin, supp, scale);
}

// finalize of many grids: blockIdx.y picks the grid, blocks past its size return
__global__ void __launch_bounds__(256) k_finalize_batch(const FinalizeDesc *__restrict__ d,
                                                         const uint16_t *__restrict__ blk) {
    const FinalizeDesc f = d[blk[blockIdx.x]];
    const int64_t base = (int64_t)(blockIdx.x - f.block0) * BATCH_BLOCK_CELLS;
    const int64_t ncell = (int64_t)f.nv * f.pitch;
#pragma unroll
    for (int j = 0; j < BATCH_BLOCK_CELLS / 256; j++) {
        const int64_t idx = base + j * 256 + threadIdx.x;
        if (idx < ncell)
            f.out[idx] = finalize_cell(f.raw, f.raw_lo, idx, f.nu, f.nv, f.pitch, f.uorigin,
                                       f.vorigin, f.supp, f.scale);
    }
}

// ---------------------------------------------------------------------------------------
// Degridding (GRDDEH2D, grd/grddeh2d.f:119-193).
//
// Persistent, TEAMS teams of 256 threads per CTA and one CTA per SM, like the gridder: the
// CTA fills the gridder's tap tables and the tap row sums once; each team takes work items
// from an atomic counter and stages the item's model tile + halo in its own shared buffer
// with one TMA 2-D bulk load (cp.async.bulk.tensor, the team's mbarrier, bounded wait).  A
// 4-lane group owns a chunk (the chunk's visibilities lie in one cell pair -- their
// degridding cell is their gridding cell -- or carry GDD_EXCEPTION and are skipped here):
// lane q holds columns q and q+4 of the pair's 7x8 neighbourhood window in registers, read
// once per chunk, and for each visibility forms sum_b gv[b] G[b][col] per column, then the u
// tap of that column times that: a partial sum over its columns.  Four visibilities'
// partials are reduced across the group with a transposing butterfly (6 shuffles per
// lane), after which lane q owns visibility q of the four and finishes it: divide by
// (sum gu)(sum gv) (row sums in the same order as a plain loop), subtract from the observed
// value or stage it for the caller's order.
constexpr int DG_THREADS = GRID_THREADS;
constexpr int DG_GROUPS = TEAM_THREADS / 4;        // chunks in flight per team
constexpr int DG_TILE_FLOATS = STILE * STILE * 2;  // 9800 floats, 39200 B
constexpr uint32_t DG_TX_BYTES = DG_TILE_FLOATS * 4;
constexpr size_t DG_TILE_STRIDE = (DG_TX_BYTES + 127) / 128 * 128;  // TMA destinations: 128-byte aligned

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

constexpr int DG_PREFETCH = 4096;                  // visibilities prefetched into L2 per item
constexpr int RSUM_FLOATS = 132;                    // 129 row sums, padded
constexpr size_t DG_VT_OFF = (size_t)TEAMS * DG_TILE_STRIDE;
constexpr size_t DG_UT_OFF = DG_VT_OFF + sizeof(float) * VT_FLOATS;
constexpr size_t DG_RSUM_OFF = DG_UT_OFF + sizeof(float) * UT_FLOATS;
constexpr size_t DG_BAR_OFF = DG_RSUM_OFF + sizeof(float) * RSUM_FLOATS;
static_assert(DG_TILE_STRIDE % 128 == 0 && DG_VT_OFF % 16 == 0 && DG_UT_OFF % 16 == 0 &&
                  DG_BAR_OFF % 8 == 0, "layout");

// mode 0: residual update in the gridding frame; mode 1: caller-order output (user frame).
template <int MODE>
__global__ void __launch_bounds__(DG_THREADS, 1)
    k_degrid(const __grid_constant__ CUtensorMap tmap, const WorkItem *__restrict__ items,
             int64_t nitems, unsigned long long *counter, const uint2 *__restrict__ chunks,
             const uint32_t *__restrict__ gdd, const float *__restrict__ cft_g,
             const float2 *__restrict__ fobs, float4 *rec, const uint8_t *__restrict__ gconj,
             const float2 *__restrict__ rot, const float *__restrict__ wt, float4 *stage, int ntu,
             const float2 *__restrict__ grid, int pitch, int nv, int vorigin, int refl,
             int *status) {
    extern __shared__ __align__(128) unsigned char smem_dg[];
    const int team = threadIdx.x / TEAM_THREADS, tid = threadIdx.x % TEAM_THREADS;
    float2 *tile = reinterpret_cast<float2 *>(smem_dg + (size_t)team * DG_TILE_STRIDE);
    float *vt = reinterpret_cast<float *>(smem_dg + DG_VT_OFF);
    float *ut = reinterpret_cast<float *>(smem_dg + DG_UT_OFF);
    float *rsum = reinterpret_cast<float *>(smem_dg + DG_RSUM_OFF);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_dg + DG_BAR_OFF) + team;
    __shared__ long long s_next[TEAMS];
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    fill_tap_tables(cft_g, vt, ut);
    // reciprocal tap-row sums: GRDDEH2D's SUMWT is (sum of u taps)(sum of v taps)
    for (int d = threadIdx.x; d < 129; d += DG_THREADS) {
        float sacc = 0.f;
#pragma unroll
        for (int a = 0; a < NTAP; a++) sacc += cft_g[d * 8 + a];
        rsum[d] = 1.0f / sacc;
    }
    __syncthreads();
    const int q = tid & 3;
    const bool hi2 = (q & 2) != 0, hi1 = (q & 1) != 0;
    const int grp = tid >> 2;
    const int gbase = threadIdx.x & 28;  // lane of q = 0 in this group
    const float *vcopy = vt + (grp & 3) * 8;
    const float *ucopy = ut + (grp & 3) * 8 + 2 * q;
    constexpr uint32_t FULL = 0xffffffffu;
    constexpr uint32_t GDD_PAD = 0u;  // table row 0: harmless reads for the padding lanes
    for (uint32_t iter = 0;; iter++) {
        if (tid == 0) s_next[team] = (long long)atomicAdd(counter, 1ull);
        team_sync(team);  // also: the team's reads of its previous tile are done
        const long long n = s_next[team];
        if (n >= nitems) break;
        const WorkItem it = items[n];
        const int tu = it.tile % ntu, tv = it.tile / ntu;
        if (tid == 0) {
            // the previous item's generic-proxy writes to the tile (reflection halo) are
            // ordered before this async-proxy write
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            // box origin: columns tu*64-6 (complex) -> float x = 2*(tu*64-6), rows tv*64-3
            const int x = 2 * (tu * TILE - 2 * SUPP), y = tv * TILE - SUPP;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                         "r"(DG_TX_BYTES));
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(tile)),
                "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(x), "r"(y), "r"(smem_u32(bar))
                : "memory");
            prefetch_l2_range(chunks, it.cbeg, it.cend, 8);
            // the first DG_PREFETCH visibilities' words only: whole items of all resident
            // teams would not fit in L2 together (measured: the full range evicts what it
            // fetched)
            const int pf_end = min(it.vend, it.vbeg + DG_PREFETCH);
            prefetch_l2_range(gdd, it.vbeg, pf_end, 4);
            if (MODE == 0) prefetch_l2_range(fobs, it.vbeg, pf_end, 8);
        }
        {
            uint32_t done = 0;
            const uint32_t parity = iter & 1u;
            for (int spin = 0; spin < (1 << 24) && !done; spin++) {
                asm volatile(
                    "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;"
                    " selp.u32 %0, 1, 0, p; }"
                    : "=r"(done)
                    : "r"(smem_u32(bar)), "r"(parity)
                    : "memory");
            }
            if (!team_and(team, done != 0)) {
                if (tid == 0) atomicExch(&status[STATUS_TIMEOUT], 1);
                return;
            }
        }
        if (refl && tu == 0) {
            // GRDDEH2D's reflection branch (grd/grddeh2d.f:123-158) in the tile: halo columns
            // 3..5 stand for u = -3..-1 (left of the v axis; TMA filled them with zeros) and
            // receive conj(G(-u, 2*VORIGIN - v)), the values that branch reads there
            for (int k = tid; k < STILE * SUPP; k += TEAM_THREADS) {
                const int r = k / SUPP, c = SUPP + k % SUPP;    // c = 2*SUPP + u
                const int vm = 2 * vorigin - (tv * TILE - SUPP + r + 1);  // mirrored 1-based row
                float2 val = make_float2(0.f, 0.f);
                if (vm >= 1 && vm <= nv) {
                    const float2 gm = grid[(int64_t)(vm - 1) * pitch + (2 * SUPP - c)];
                    val = make_float2(gm.x, -gm.y);
                }
                tile[r * STILE + c] = val;
            }
            team_sync(team);
        }
        // Every lane of a warp runs the same number of group iterations (the loop bounds are
        // per item), so the shuffles below always see all 32 lanes.
        const int ngroups_iter = (it.cend - it.cbeg + DG_GROUPS - 1) / DG_GROUPS;
        for (int gi = 0; gi < ngroups_iter; gi++) {
            const int c = it.cbeg + gi * DG_GROUPS + grp;
            const bool live = c < it.cend;
            const uint2 ch = live ? chunks[c] : make_uint2(0u, 0u);
            const int start = (int)ch.x, len = live ? (int)(ch.y >> 16) : 0;
            const int cell = (int)(ch.y & 4095u), lu = cell & 63, lv = cell >> 6;
            float2 G0[NTAP], G1[NTAP];
#pragma unroll
            for (int b = 0; b < NTAP; b++) {
                const float2 *row = &tile[(lv + b) * STILE + lu];
                G0[b] = row[q];
                G1[b] = row[q + 4];
            }
            // the warp iterates to the longest chunk among its 8 groups
            int wlen = len;
#pragma unroll
            for (int d = 4; d < 32; d <<= 1) wlen = max(wlen, __shfl_xor_sync(FULL, wlen, d));
            // lane q loads the offset word and observed value of visibility q of the next
            // batch (one coalesced load per group); the group shares the words by shuffle
            uint32_t gqn = q < len ? gdd[start + q] : GDD_PAD;
            float2 obn = make_float2(0.f, 0.f);
            if (MODE == 0 && q < len) obn = fobs[start + q];
            for (int k = 0; k < wlen; k += 4) {
                const int pq = start + k + q;
                const bool mine = k + q < len;
                const float2 ob = obn;
                const uint32_t gq = gqn;
                if (k + 4 + q < len) {
                    gqn = gdd[pq + 4];
                    if (MODE == 0) obn = fobs[pq + 4];
                }
                float pr[4], pim[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const uint32_t g = __shfl_sync(FULL, gq, gbase + u);
                    const float2 gu = *reinterpret_cast<const float2 *>(
                        reinterpret_cast<const char *>(ucopy) + (g & 0xFFFFu));
                    const float4 *vr = reinterpret_cast<const float4 *>(
                        reinterpret_cast<const char *>(vcopy) + ((g >> 16) & 0x7FFFu));
                    const float4 v0 = vr[0], v1 = vr[1];
                    const float gv[NTAP] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z};
                    float c0r = 0.f, c0i = 0.f, c1r = 0.f, c1i = 0.f;
#pragma unroll
                    for (int b = 0; b < NTAP; b++) {
                        c0r = fmaf(gv[b], G0[b].x, c0r);
                        c0i = fmaf(gv[b], G0[b].y, c0i);
                        c1r = fmaf(gv[b], G1[b].x, c1r);
                        c1i = fmaf(gv[b], G1[b].y, c1i);
                    }
                    pr[u] = fmaf(gu.y, c1r, gu.x * c0r);
                    pim[u] = fmaf(gu.y, c1i, gu.x * c0i);
                }
                // butterfly over lane bit 1: keep visibilities {0,1} (or {2,3}), pass the others
                float k0r = hi2 ? pr[2] : pr[0], k0i = hi2 ? pim[2] : pim[0];
                float k1r = hi2 ? pr[3] : pr[1], k1i = hi2 ? pim[3] : pim[1];
                const float s0r = hi2 ? pr[0] : pr[2], s0i = hi2 ? pim[0] : pim[2];
                const float s1r = hi2 ? pr[1] : pr[3], s1i = hi2 ? pim[1] : pim[3];
                k0r += __shfl_xor_sync(FULL, s0r, 2);
                k0i += __shfl_xor_sync(FULL, s0i, 2);
                k1r += __shfl_xor_sync(FULL, s1r, 2);
                k1i += __shfl_xor_sync(FULL, s1i, 2);
                // butterfly over lane bit 0: keep visibility q
                float tr = hi1 ? k1r : k0r, ti = hi1 ? k1i : k0i;
                tr += __shfl_xor_sync(FULL, hi1 ? k0r : k1r, 1);
                ti += __shfl_xor_sync(FULL, hi1 ? k0i : k1i, 1);
                if (!mine || (gq & GDD_EXCEPTION)) continue;
                const float inv = rsum[taps_du(gq)] * rsum[taps_dv(gq)];
                float mr = tr * inv, mi = ti * inv;
                if (MODE == 0) {
                    *rec_res(rec, pq) = make_float2(ob.x - mr, ob.y - mi);
                } else {
                    // caller's frame, staged in plan order (k_gather_user puts it in the
                    // caller's order with coalesced writes)
                    if (gconj[pq]) mi = -mi;
                    float2 vv = make_float2(mr, mi);
                    if (rot) {
                        const float2 rt = rot[pq];
                        vv = make_float2(mr * rt.x - mi * rt.y, mr * rt.y + mi * rt.x);
                    }
                    stage[pq] = make_float4(vv.x, vv.y, wt[pq], 0.f);
                }
            }
        }
    }
}

// Caller index -> plan position of the visibilities the tiled degridder handles (-1 for
// the others: exceptions, visibilities outside the plan).
__global__ void k_plan_inverse(const uint32_t *__restrict__ orig, const uint32_t *__restrict__ gdd,
                               int64_t n, int32_t *inv) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    if (!(gdd[p] & GDD_EXCEPTION)) inv[orig[p]] = (int32_t)p;
}

// Caller-order output of the tiled degridder: coalesced writes, one 16-byte gather each.
__global__ void k_gather_user(const int32_t *__restrict__ inv, const float4 *__restrict__ stage,
                              int64_t n, float2 *vis_out, float *wt_out) {
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int32_t p = inv[o];
    if (p < 0) return;
    const float4 s = stage[p];
    vis_out[o] = make_float2(s.x, s.y);
    wt_out[o] = s.z;
}

// Exception path: GRDDEH2D's taps and weights (the axis-reflection branch,
// grd/grddeh2d.f:123-158, and the plain branch, :163-173), reading the grid from HBM.  One
// warp per exception: lane l < 49 evaluates tap (offu, offv) = (l/7 - SUPP, l%7 - SUPP) and
// the warp sums the products and weights by shuffles.  A mirrored row outside the grid,
// which the reference's reflection loop reads without a bounds check (undefined there),
// is left out of both sums.
constexpr int EXC_THREADS = 128;
template <int MODE>
__global__ void __launch_bounds__(EXC_THREADS)
    k_degrid_exc(const DegridExc *__restrict__ exc, const float *__restrict__ exc_wt,
                 const float2 *__restrict__ exc_rot, int64_t nexc,
                 const float2 *__restrict__ grid, int pitch, int nu, int nv,
                 int uorigin, int vorigin, const float *__restrict__ cf,
                 int doshift, const float2 *__restrict__ fobs, float4 *rec,
                 float2 *vis_out, float *wt_out, unsigned long long *nbad) {
    const int64_t t = ((int64_t)blockIdx.x * EXC_THREADS + threadIdx.x) >> 5;  // per warp
    const int lane = threadIdx.x & 31;
    if (t >= nexc) return;
    const DegridExc e = exc[t];
    if (MODE == 0 && e.pos < 0) return;
    const float w0 = exc_wt[t];
    float vr = 0.f, vi = 0.f;
    bool ok = false;
    if (e.valid) {
        const int cfo = (SUPP + 1) * OSAMP + 1;
        const int ucen = e.nuc - uorigin, vcen = e.nvc - vorigin;
        const bool axis = e.nuc <= SUPP;
        float pr = 0.f, pi = 0.f, pw = 0.f;
        for (int l = lane; l < NTAP * NTAP; l += 32) {
            const int offu = l / NTAP - SUPP, offv = l % NTAP - SUPP;
            const int delu = e.delui + OSAMP * offu + cfo, delv = e.delvi + OSAMP * offv + cfo;
            const float uvwt = __fmul_rn(cf[delu - 1], cf[delv - 1]);
            int ui = uorigin + ucen + offu, vint = vorigin + vcen + offv;
            bool cj = false;
            if (axis && ucen + offu != 0) {
                const int us = (ucen + offu) >= 0 ? 1 : -1;
                ui = uorigin + us * (ucen + offu);
                vint = vorigin + us * (vcen + offv);
                cj = us < 0;
            }
            if (axis && (ui < 1 || ui > nu || vint < 1 || vint > nv)) continue;
            float2 f = grid[(int64_t)(vint - 1) * pitch + (ui - 1)];
            if (cj) f.y = -f.y;
            pr = __fadd_rn(pr, __fmul_rn(f.x, uvwt));
            pi = __fadd_rn(pi, __fmul_rn(f.y, uvwt));
            pw = __fadd_rn(pw, uvwt);
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            pr += __shfl_xor_sync(0xffffffffu, pr, d);
            pi += __shfl_xor_sync(0xffffffffu, pi, d);
            pw += __shfl_xor_sync(0xffffffffu, pw, d);
        }
        if (pw > 0.0f) {
            vr = __fdiv_rn(pr, pw);
            vi = __fdiv_rn(pi, pw);
            ok = true;
        } else if (MODE == 1 && lane == 0) {
            atomicAdd(nbad, 1ull);
        }
        if (e.conj) vi = -vi;
        const float2 rt = exc_rot[t];
        const float xr = __fsub_rn(__fmul_rn(vr, rt.x), __fmul_rn(vi, rt.y));
        const float xi = __fadd_rn(__fmul_rn(vr, rt.y), __fmul_rn(vi, rt.x));
        vr = xr;
        vi = xi;
    }
    if (lane != 0) return;
    if (MODE == 1) {
        vis_out[e.orig] = make_float2(vr, vi);
        wt_out[e.orig] = ok ? fabsf(w0) : -w0;
        if (!ok) atomicAdd(nbad + 1, 1ull);  // WT left negated: the caller's WT changes
    } else {
        // model in the gridding frame: rotate by (c, -s) when the plan rotates, conjugate
        float mr = vr, mi = vi;
        if (doshift) {
            const float2 rt = exc_rot[t];
            mr = vr * rt.x + vi * rt.y;
            mi = -vr * rt.y + vi * rt.x;
        }
        if (e.gconj) mi = -mi;
        const float2 o = fobs[e.pos];
        *rec_res(rec, e.pos) = make_float2(o.x - mr, o.y - mi);
    }
}

// residual back to the caller's frame and order: V = conj?(F) * (c, s), the inverse of
// F = conj?(V * (c, -s)) applied when the plan was built
__global__ void k_scatter_vis(const float4 *__restrict__ rec, const uint32_t *__restrict__ orig,
                              const uint8_t *__restrict__ gconj, const float2 *__restrict__ rot,
                              int64_t n, float2 *dst) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float2 f = rec_res(rec, p);
    if (gconj[p]) f.y = -f.y;
    if (rot) {
        const float2 r = rot[p];
        f = make_float2(f.x * r.x - f.y * r.y, f.x * r.y + f.y * r.x);
    }
    dst[orig[p]] = f;
}

// frame transform of the caller's visibilities into the plan's residual (sde_plan_set_vis)
__global__ void k_set_vis(const float2 *__restrict__ vis_user, const uint32_t *__restrict__ orig,
                          const uint8_t *__restrict__ gconj, const float2 *__restrict__ rot,
                          int64_t n, float2 *fobs, float4 *rec) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float2 v = vis_user[orig[p]];
    float fr = v.x, fi = v.y;
    if (rot) {
        const float2 r = rot[p];  // FVIS = VIS * (c, -s)
        fr = __fsub_rn(__fmul_rn(v.x, r.x), __fmul_rn(v.y, -r.y));
        fi = __fadd_rn(__fmul_rn(v.x, -r.y), __fmul_rn(v.y, r.x));
    }
    if (gconj[p]) fi = -fi;
    fobs[p] = make_float2(fr, fi);
    *rec_res(rec, p) = make_float2(fr, fi);
}

int make_grid_tmap(CUtensorMap *map, const float *grid, int pitch, int nv) {
    return encode_tmap_f32_2d(map, grid, (uint64_t)pitch * 2, (uint64_t)nv, (uint64_t)pitch * 8,
                              STILE * 2, STILE);
}

size_t grid_smem() { return sizeof(float) * (GTAB_FLOATS + TEAMS * GTILE_FLOATS); }
size_t degrid_smem() { return DG_BAR_OFF + 8 * TEAMS; }

}  // namespace

// A 2-D FP32 tensor map (width floats x rows, row pitch in bytes, box box_w x box_h) for
// cp.async.bulk.tensor; out-of-range elements read as zero and are not written.
int encode_tmap_f32_2d(CUtensorMap *map, const void *base, uint64_t width, uint64_t rows,
                       uint64_t row_bytes, uint32_t box_w, uint32_t box_h) {
    typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                      const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                      const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                      CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                         cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
            sde_set_error("cuTensorMapEncodeTiled unavailable");
            return SDE_ECUDA;
        }
        fn = (EncodeTiledFn)p;
    }
    if (((uintptr_t)base & 15u) != 0 || row_bytes % 16 != 0 || (box_w * 4) % 16 != 0) {
        sde_set_error("array not 16-byte aligned for TMA");
        return SDE_EINVAL;
    }
    cuuint64_t dims[2] = {(cuuint64_t)width, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)row_bytes};
    cuuint32_t box[2] = {box_w, box_h};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(base), dims, strides,
                    box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        sde_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return SDE_ECUDA;
    }
    return SDE_OK;
}

// ---------------------------------------------------------------------------------------
int plan_build_cft(sde_plan *pl) {
    k_build_cft<<<1, 160, 0, pl->ctx->stream>>>(pl->cf, pl->cft);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

int ctx_build_cft(sde_ctx *ctx) {
    k_build_cft<<<1, 160, 0, ctx->stream>>>(ctx->d_cf, ctx->d_cft);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

// LSUMWT and SUMWT of the plan (host doubles), computed once.
int plan_sums(sde_plan *pl, double *lsumwt, double *sumwt) {
    sde_ctx *ctx = pl->ctx;
    if (pl->nvis == 0) {
        *lsumwt = 0.0;
        *sumwt = 0.0;
        return SDE_OK;
    }
    const int nb = (int)std::min<int64_t>(ctx->num_sms * 4, ceil_div(pl->nvis, RED_T));
    double *part;
    SDE_TRY(ctx_scratch(ctx, "gs_part", sizeof(double) * 2 * (size_t)(ctx->num_sms * 4), (void **)&part));
    KTimer kt(ctx, "plan_sums");
    k_plan_sums<<<nb, RED_T, 0, ctx->stream>>>(pl->rec, pl->cft, pl->nvis, part);
    SDE_CHECK_LAUNCH();
    k_sum_pairs<<<1, RED_T, 0, ctx->stream>>>(part, nb, pl->d_sums);
    SDE_CHECK_LAUNCH();
    double h[2];
    SDE_TRY(ctx_read_small(ctx, ctx->stream, h, pl->d_sums, sizeof h));
    *lsumwt = h[0];
    *sumwt = h[1];
    return SDE_OK;
}

int grid_finalize_scale(sde_ctx *ctx, const float2 *raw, const float2 *raw_lo, float2 *out, int nu,
                        int nv, int pitch, int uorigin, int vorigin, int supp, float scale) {
    int64_t n = (int64_t)nv * pitch;
    KTimer kt(ctx, "finalize");
    k_finalize<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(raw, raw_lo, out, nu, nv, pitch, uorigin,
                                                          vorigin, supp, scale);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

size_t grid_smem_bytes() { return grid_smem(); }
int grid_ctas_per_sm() { return 1; }

int launch_grid_batch(sde_ctx *ctx, int psf, int comp, const BatchPlan *d_plans,
                      const int64_t *d_item_start, int nplans, unsigned long long *d_counter,
                      const float *cft, int nctas) {
    static bool attr = false;
    if (!attr) {
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_grid_batch<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)grid_smem()));
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_grid_batch<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)grid_smem()));
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_grid_batch<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)grid_smem()));
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_grid_batch<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)grid_smem()));
        attr = true;
    }
    KTimer kt(ctx, psf ? "grid_batch_psf" : "grid_batch");
    const dim3 g((unsigned)nctas), b(GRID_THREADS);
    if (psf && comp)
        k_grid_batch<true, true><<<g, b, grid_smem(), ctx->stream>>>(d_plans, d_item_start, nplans, d_counter, cft);
    else if (psf)
        k_grid_batch<true, false><<<g, b, grid_smem(), ctx->stream>>>(d_plans, d_item_start, nplans, d_counter, cft);
    else if (comp)
        k_grid_batch<false, true><<<g, b, grid_smem(), ctx->stream>>>(d_plans, d_item_start, nplans, d_counter, cft);
    else
        k_grid_batch<false, false><<<g, b, grid_smem(), ctx->stream>>>(d_plans, d_item_start, nplans, d_counter, cft);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

int launch_finalize_batch(sde_ctx *ctx, const FinalizeDesc *d_desc, const uint16_t *blk, int64_t nblk) {
    if (nblk <= 0) return SDE_OK;
    KTimer kt(ctx, "finalize_batch");
    k_finalize_batch<<<(unsigned)nblk, 256, 0, ctx->stream>>>(d_desc, blk);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

int launch_fold_lo_batch(sde_ctx *ctx, const BatchPlan *d_plans, const int2 *cores, int64_t ncores) {
    if (ncores <= 0) return SDE_OK;
    KTimer kt(ctx, "fold_lo_batch");
    k_fold_lo_batch<<<(unsigned)ncores, 256, 0, ctx->stream>>>(d_plans, cores);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

int plan_grid_raw(sde_plan *pl, int what, float2 *raw, float2 *raw_lo, bool lo_clean) {
    sde_ctx *ctx = pl->ctx;
    const int nu = pl->spec.nu, nv = pl->spec.nv;
    SDE_CUDA_TRY(cudaMemsetAsync(raw, 0, sizeof(float2) * (size_t)nv * pl->pitch, ctx->stream));
    if (raw_lo && !lo_clean)
        SDE_CUDA_TRY(cudaMemsetAsync(raw_lo, 0, sizeof(float2) * (size_t)nv * pl->pitch, ctx->stream));
    if (pl->nitems == 0) return SDE_OK;
    static bool attr = false;
    if (!attr) {
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_grid<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)grid_smem()));
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_grid<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)grid_smem()));
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_grid<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)grid_smem()));
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_grid<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)grid_smem()));
        attr = true;
    }
    unsigned long long *counter;
    SDE_TRY(ctx_scratch(ctx, "grid_counter", sizeof(unsigned long long), (void **)&counter));
    SDE_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), ctx->stream));
    KTimer kt(ctx, what == SDE_GRID_PSF ? "grid_psf" : "grid");
    const int64_t want = (int64_t)ctx->num_sms;
    const dim3 g((unsigned)(pl->nitems < want ? pl->nitems : want)), b(GRID_THREADS);
    const size_t sm = grid_smem();
    cudaStream_t st = ctx->stream;
    const int64_t ni = pl->nitems;
    if (what == SDE_GRID_PSF && raw_lo)
        k_grid<true, true><<<g, b, sm, st>>>(pl->items, ni, counter, pl->chunks, pl->rec, pl->cft, raw, raw_lo, pl->pitch, pl->ntu, nu, nv);
    else if (what == SDE_GRID_PSF)
        k_grid<true, false><<<g, b, sm, st>>>(pl->items, ni, counter, pl->chunks, pl->rec, pl->cft, raw, raw_lo, pl->pitch, pl->ntu, nu, nv);
    else if (raw_lo)
        k_grid<false, true><<<g, b, sm, st>>>(pl->items, ni, counter, pl->chunks, pl->rec, pl->cft, raw, raw_lo, pl->pitch, pl->ntu, nu, nv);
    else
        k_grid<false, false><<<g, b, sm, st>>>(pl->items, ni, counter, pl->chunks, pl->rec, pl->cft, raw, raw_lo, pl->pitch, pl->ntu, nu, nv);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

// The caller -> plan permutation of the tiled visibilities, built on first use.
int plan_inverse(sde_plan *pl) {
    if (pl->inv || pl->nvis_in == 0) return SDE_OK;
    sde_ctx *ctx = pl->ctx;
    int32_t *inv = nullptr;
    SDE_TRY(ctx_alloc(ctx, (void **)&inv, sizeof(int32_t) * (size_t)pl->nvis_in));
    pl->bytes += (int64_t)(sizeof(int32_t) * (size_t)pl->nvis_in);
    ctx->bytes += (int64_t)(sizeof(int32_t) * (size_t)pl->nvis_in);
    SDE_CUDA_TRY(cudaMemsetAsync(inv, 0xFF, sizeof(int32_t) * (size_t)pl->nvis_in, ctx->stream));
    if (pl->nvis > 0) {
        k_plan_inverse<<<ceil_div(pl->nvis, 256), 256, 0, ctx->stream>>>(pl->orig, pl->gdd, pl->nvis, inv);
        SDE_CHECK_LAUNCH();
    }
    pl->inv = inv;
    return SDE_OK;
}

int plan_fold_lo(sde_plan *pl, float2 *raw, float2 *raw_lo) {
    if (!raw_lo || !pl->core_lo) return SDE_OK;
    sde_ctx *ctx = pl->ctx;
    KTimer kt(ctx, "fold_lo");
    const int ncu = pl->ntu + 1, ncv = pl->ntv + 1;
    k_fold_lo<<<ncu * ncv, 256, 0, ctx->stream>>>(raw, raw_lo, pl->core_lo, ncu, pl->spec.nv, pl->pitch);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

// mode 0: residual update; mode 1: caller-order output
int plan_degrid(sde_plan *pl, const float *grid, int pitch, int mode, float2 *vis_out,
                float *wt_out, unsigned long long *nbad_dev) {
    sde_ctx *ctx = pl->ctx;
    const int nu = pl->spec.nu, nv = pl->spec.nv;
    static bool attr = false;
    if (!attr) {
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_degrid<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)degrid_smem()));
        SDE_CUDA_TRY(cudaFuncSetAttribute(k_degrid<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)degrid_smem()));
        attr = true;
    }
    float4 *stage = nullptr;
    if (mode == 1 && pl->nitems > 0) {
        SDE_TRY(ctx_scratch(ctx, "dg_stage", sizeof(float4) * (size_t)pl->nvis, (void **)&stage));
        SDE_TRY(plan_inverse(pl));
    }
    if (pl->nitems > 0) {
        CUtensorMap map;
        SDE_TRY(make_grid_tmap(&map, grid, pitch, nv));
        unsigned long long *counter;
        SDE_TRY(ctx_scratch(ctx, "degrid_counter", sizeof(unsigned long long), (void **)&counter));
        SDE_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), ctx->stream));
        const int64_t want = (int64_t)ctx->num_sms;
        const unsigned nb = (unsigned)(pl->nitems < want ? pl->nitems : want);
        KTimer kt(ctx, "degrid");
        if (mode == 0)
            k_degrid<0><<<nb, DG_THREADS, degrid_smem(), ctx->stream>>>(
                map, pl->items, pl->nitems, counter, pl->chunks, pl->gdd, pl->cft, pl->fobs, pl->rec,
                pl->gconj, pl->rot, pl->wt, nullptr, pl->ntu, (const float2 *)grid, pitch, nv,
                pl->spec.vorigin, (int)(pl->spec.uorigin == 1), ctx->d_status);
        else
            k_degrid<1><<<nb, DG_THREADS, degrid_smem(), ctx->stream>>>(
                map, pl->items, pl->nitems, counter, pl->chunks, pl->gdd, pl->cft, pl->fobs, pl->rec,
                pl->gconj, pl->rot, pl->wt, stage, pl->ntu, (const float2 *)grid, pitch, nv,
                pl->spec.vorigin, (int)(pl->spec.uorigin == 1), ctx->d_status);
        SDE_CHECK_LAUNCH();
        if (mode == 1) {
            KTimer kg(ctx, "gather_user");
            k_gather_user<<<ceil_div(pl->nvis_in, 256), 256, 0, ctx->stream>>>(
                pl->inv, stage, pl->nvis_in, vis_out, wt_out);
            SDE_CHECK_LAUNCH();
        }
    }
    if (pl->nexc > 0) {
        size_t ne1 = (size_t)pl->nexc;
        const float *exc_wt = (const float *)((const char *)pl->exc + exc_wt_off(ne1));
        const float2 *exc_rot = (const float2 *)((const char *)pl->exc + exc_rot_off(ne1));
        const int64_t nb = ceil_div(pl->nexc * 32, EXC_THREADS);
        const int T = EXC_THREADS;
        KTimer kt(ctx, "degrid_exc");
        if (mode == 0)
            k_degrid_exc<0><<<nb, T, 0, ctx->stream>>>(
                pl->exc, exc_wt, exc_rot, pl->nexc, (const float2 *)grid, pitch, nu, nv,
                pl->spec.uorigin, pl->spec.vorigin, pl->cf, pl->doshift, pl->fobs, pl->rec,
                vis_out, wt_out, nbad_dev);
        else
            k_degrid_exc<1><<<nb, T, 0, ctx->stream>>>(
                pl->exc, exc_wt, exc_rot, pl->nexc, (const float2 *)grid, pitch, nu, nv,
                pl->spec.uorigin, pl->spec.vorigin, pl->cf, pl->doshift, pl->fobs, pl->rec,
                vis_out, wt_out, nbad_dev);
        SDE_CHECK_LAUNCH();
    }
    return SDE_OK;
}

int plan_scatter_residual(sde_plan *pl, float2 *dst) {
    if (pl->nvis == 0) return SDE_OK;
    KTimer kt(pl->ctx, "scatter_vis");
    k_scatter_vis<<<ceil_div(pl->nvis, 256), 256, 0, pl->ctx->stream>>>(
        pl->rec, pl->orig, pl->gconj, pl->rot, pl->nvis, dst);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

int plan_set_vis_dev(sde_plan *pl, const float2 *vis_user) {
    if (pl->nvis == 0) return SDE_OK;
    KTimer kt(pl->ctx, "set_vis");
    k_set_vis<<<ceil_div(pl->nvis, 256), 256, 0, pl->ctx->stream>>>(vis_user, pl->orig, pl->gconj,
                                                                  pl->rot, pl->nvis, pl->fobs,
                                                                  pl->rec);
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}
