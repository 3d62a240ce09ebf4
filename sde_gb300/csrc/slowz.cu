// slowz.cu -- the slow-Z ("3-D with a slow w axis") gridder and degridder VISGRID/VISDEGRI
// call for images whose third axis is N----SIN: GRDH23D (grd/grdh23d.f) and GRDDEH23
// (grd/grddeh23.f).  Each visibility's 2-D window (the prolate-spheroidal table, support
// SUPP, oversampling OSAMP) is applied on NZ planes, plane iz rotated by
// exp(-i TWOPI WLOCAL DTOR CELLZ (iz - REFZ)).
//   gridding:   one thread per visibility adds its NZ x (2S+1)^2 taps into a raw cube by
//               atomics (FP32 sums in no fixed order); k_h23_final applies GRDH23D's
//               Hermitian fold, the shift left by SUPPU and (NU-1)NV NZ/LSUMWT as a gather.
//   degridding: one thread per visibility sums its taps in the reference's loop order, with
//               the reference's per-branch operation order.
#include <math.h>

#include "common.cuh"

namespace {

struct H23Geom {
    float uscale, uoffset, vscale, voffset, cellz, refz, twopi, dtor;
    int uorigin, vorigin, nu, nv, nz, suppu, osampu, suppv, osampv, psf;
    double s[9];  // SHIFT(3,3), column-major
};

struct H23Sums {
    double sumwt, lsumwt;
};

// ULOCAL/VLOCAL/WLOCAL: DOUBLE products summed left to right, stored REAL
__device__ __forceinline__ void h23_local(const H23Geom &g, float u, float v, float w, float *ul, float *vl,
                                          float *wl) {
    const double uu = u, vv = v, ww = w;
    *ul = (float)__dadd_rn(__dadd_rn(__dmul_rn(g.s[0], uu), __dmul_rn(g.s[1], vv)), __dmul_rn(g.s[2], ww));
    *vl = (float)__dadd_rn(__dadd_rn(__dmul_rn(g.s[3], uu), __dmul_rn(g.s[4], vv)), __dmul_rn(g.s[5], ww));
    *wl = (float)__dadd_rn(__dadd_rn(__dmul_rn(g.s[6], uu), __dmul_rn(g.s[7], vv)), __dmul_rn(g.s[8], ww));
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                       __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(__fmul_rn(a.x, s), __fmul_rn(a.y, s)); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)); }

// the plane rotation -TWOPI * WLOCAL * DTOR * CELLZ * (FLOAT(IZ) - REFZ), left to right
__device__ __forceinline__ float h23_plane_phase(const H23Geom &g, float wl, int iz) {
    return __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(-g.twopi, wl), g.dtor), g.cellz), __fsub_rn((float)iz, g.refz));
}

// grd/grdh23d.f:54-103
__global__ void k_h23_grid(const float2 *__restrict__ vis, const float *__restrict__ wt, const float *__restrict__ u,
                           const float *__restrict__ v, const float *__restrict__ w, int64_t nvis, H23Geom g,
                           const float *__restrict__ fnu, const float *__restrict__ fnv, float2 *raw, H23Sums *sums) {
    double sw = 0.0, lw = 0.0;
    const int cfou = (g.suppu + 1) * g.osampu + 1, cfov = (g.suppv + 1) * g.osampv + 1;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nvis; k += (int64_t)gridDim.x * blockDim.x) {
        const float wk = wt[k];
        if (!(wk > 0.f)) continue;
        sw += wk;
        float ul, vl, wl;
        h23_local(g, u[k], v[k], w[k], &ul, &vl, &wl);
        const float ph = __fmul_rn(g.twopi, __fsub_rn(wl, w[k]));
        float2 f = cmul(vis ? vis[k] : make_float2(0.f, 0.f), make_float2(cosf(ph), -sinf(ph)));
        float uc = __fadd_rn(__fmul_rn(g.uscale, ul), g.uoffset), vc = __fadd_rn(__fmul_rn(g.vscale, vl), g.voffset);
        if (uc > 0.f) {
            f.y = -f.y;
            uc = __fadd_rn(uc, (float)g.uorigin);
            vc = __fadd_rn(vc, (float)g.vorigin);
        } else {
            uc = __fadd_rn(-uc, (float)g.uorigin);
            vc = __fadd_rn(-vc, (float)g.vorigin);
            wl = -wl;
        }
        if (g.psf) f = make_float2(1.f, 0.f);
        const int nuc = (int)lroundf(uc), nvc = (int)lroundf(vc);
        if (nuc + 2 * g.suppu > g.nu || nvc + g.suppv > g.nv || nvc - g.suppv < 1) continue;
        const int delui = (int)lroundf(__fmul_rn((float)g.osampu, __fsub_rn((float)nuc, uc)));
        const int delvi = (int)lroundf(__fmul_rn((float)g.osampv, __fsub_rn((float)nvc, vc)));
        const int uz = nuc + g.suppu;
        for (int iz = 1; iz <= g.nz; iz++) {
            const float p = h23_plane_phase(g, wl, iz);
            const float2 rf = cmul(f, make_float2(cosf(p), -sinf(p)));
            float2 *plane = raw + (size_t)(iz - 1) * g.nv * g.nu;
            for (int ov = -g.suppv; ov <= g.suppv; ov++) {
                const float gv = fnv[delvi + g.osampv * ov + cfov - 1];
                const int vg = nvc + ov;
                for (int ou = -g.suppu; ou <= g.suppu; ou++) {
                    const float uvwt = __fmul_rn(__fmul_rn(wk, fnu[delui + g.osampu * ou + cfou - 1]), gv);
                    const int ug = uz + ou;
                    if (ug < 1 || ug > g.nu) continue;  // the bound tests above keep every tap inside
                    float2 *c = plane + (size_t)(vg - 1) * g.nu + (ug - 1);
                    atomicAdd(&c->x, __fmul_rn(uvwt, rf.x));
                    atomicAdd(&c->y, __fmul_rn(uvwt, rf.y));
                    lw += uvwt;
                }
            }
        }
    }
    for (int d = 16; d > 0; d >>= 1) {
        sw += __shfl_xor_sync(0xffffffffu, sw, d);
        lw += __shfl_xor_sync(0xffffffffu, lw, d);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&sums->sumwt, sw);
        atomicAdd(&sums->lsumwt, lw);
    }
}

// grd/grdh23d.f:109-145 as a gather: out(u, v, z) = S * F(u + SUPPU, v, z), F the raw cube
// after the fold of the left margin into u > 0 and of the u = 0 column about VORIGIN
__global__ void k_h23_final(const float2 *__restrict__ raw, H23Geom g, const H23Sums *sums, float2 *out) {
    const float scale = __fdiv_rn(__fmul_rn(__fmul_rn((float)(g.nu - 1), (float)g.nv), (float)g.nz), (float)sums->lsumwt);
    const int64_t n = (int64_t)g.nu * g.nv * g.nz;
    const int uz = g.uorigin + g.suppu, vz = g.vorigin, h = g.nv / 2;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int ucol = (int)(k % g.nu) + 1;
        const int64_t rz = k / g.nu;
        const int vr = (int)(rz % g.nv) + 1;
        const int64_t z = rz / g.nv;
        if (ucol > g.nu - g.suppu) {
            out[k] = make_float2(0.f, 0.f);
            continue;
        }
        const float2 *plane = raw + (size_t)z * g.nv * g.nu;
        auto at = [&](int c, int r) { return plane[(size_t)(r - 1) * g.nu + (c - 1)]; };
        const int c = ucol + g.suppu, d = vr - vz;
        float2 val = at(c, vr);
        if (c > uz && c <= uz + g.suppu && d >= -h + 1 && d <= h - 1) {
            const int mc = uz - (c - uz), mr = vz - d;
            if (mc >= 1 && mr >= 1 && mr <= g.nv) {
                const float2 m = at(mc, mr);
                val = make_float2(__fadd_rn(val.x, m.x), __fsub_rn(val.y, m.y));
            }
        } else if (c == uz && d >= 0 && d <= h - 1) {
            if (vz - d >= 1) {
                const float2 m = at(uz, vz - d);
                val = make_float2(__fadd_rn(val.x, m.x), __fsub_rn(val.y, m.y));
            }
        } else if (c == uz && d < 0 && -d <= h - 1) {
            // GVIS(UZ, VZ-OFF) = CONJG(GVIS(UZ, VZ+OFF) + CONJG(GVIS(UZ, VZ-OFF)))
            if (vz - d <= g.nv) {
                const float2 p = at(uz, vz - d);
                val = make_float2(__fadd_rn(p.x, val.x), -__fsub_rn(p.y, val.y));
            }
        }
        out[k] = make_float2(__fmul_rn(scale, val.x), __fmul_rn(scale, val.y));
    }
}

// grd/grddeh23.f:45-183, one thread per visibility in the reference's loop order
__global__ void k_deh23(float2 *vis, float *wt, const float *__restrict__ u, const float *__restrict__ v,
                        const float *__restrict__ w, int64_t nvis, H23Geom g, const float *__restrict__ fnu,
                        const float *__restrict__ fnv, const float2 *__restrict__ grid, unsigned long long *nbad) {
    const int cfou = (g.suppu + 1) * g.osampu + 1, cfov = (g.suppv + 1) * g.osampv + 1;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nvis; k += (int64_t)gridDim.x * blockDim.x) {
        const float wk = wt[k];
        if (!(wk > 0.f)) continue;
        float2 acc = make_float2(0.f, 0.f);
        float sumwt = 0.f;
        float ul, vl, wl;
        h23_local(g, u[k], v[k], w[k], &ul, &vl, &wl);
        const float ph = __fmul_rn(g.twopi, __fsub_rn(wl, w[k]));
        const float2 rot = make_float2(cosf(ph), sinf(ph));
        float uc = __fadd_rn(__fmul_rn(g.uscale, ul), g.uoffset), vc = __fadd_rn(__fmul_rn(g.vscale, vl), g.voffset);
        if (uc > 0.f) {
            uc = __fadd_rn(uc, (float)g.uorigin);
            vc = __fadd_rn(vc, (float)g.vorigin);
        } else {
            uc = __fadd_rn(-uc, (float)g.uorigin);
            vc = __fadd_rn(-vc, (float)g.vorigin);
            wl = -wl;
        }
        const int nuc = (int)lroundf(uc), nvc = (int)lroundf(vc);
        // VIS = 0 and WT negated before the bound tests: points outside the grid end so, and
        // are not counted as failed (grd/grddeh23.f:47-49, 74-76)
        wt[k] = -wk;
        if (nuc + g.suppu > g.nu || nvc + g.suppv > g.nv || nvc - g.suppv < 1) {
            vis[k] = make_float2(0.f, 0.f);
            continue;
        }
        const int delui = (int)lroundf(__fmul_rn((float)g.osampu, __fsub_rn((float)nuc, uc)));
        const int delvi = (int)lroundf(__fmul_rn((float)g.osampv, __fsub_rn((float)nvc, vc)));
        const int ucen = nuc - g.uorigin, vcen = nvc - g.vorigin;
        auto gat = [&](int ui, int vi, int iz) -> float2 {
            if (ui < 1 || ui > g.nu || vi < 1 || vi > g.nv) return make_float2(0.f, 0.f);
            return grid[((size_t)(iz - 1) * g.nv + (vi - 1)) * g.nu + (ui - 1)];
        };
        auto crotz = [&](int iz) {
            const float p = h23_plane_phase(g, wl, iz);
            return make_float2(cosf(p), sinf(p));
        };
        if (nuc <= g.suppu) {
            for (int ou = -g.suppu; ou <= g.suppu; ou++) {
                const float gu = fnu[delui + g.osampu * ou + cfou - 1];
                if (ucen != -ou) {
                    const int us = (ucen + ou) > 0 ? 1 : -1;
                    const int ui = g.uorigin + us * (ucen + ou);
                    for (int ov = -g.suppv; ov <= g.suppv; ov++) {
                        const int vi = g.vorigin + us * (vcen + ov);
                        const float uvwt = __fmul_rn(gu, fnv[delvi + g.osampv * ov + cfov - 1]);
                        sumwt = __fadd_rn(sumwt, uvwt);
                        for (int iz = 1; iz <= g.nz; iz++) {
                            float2 f = gat(ui, vi, iz);
                            if (us < 0) f.y = -f.y;
                            acc = cadd(acc, cscale(cmul(f, crotz(iz)), uvwt));
                        }
                    }
                } else {
                    for (int ov = -g.suppv; ov <= g.suppv; ov++) {
                        const int vi = g.vorigin + (vcen + ov);
                        const float uvwt = __fmul_rn(gu, fnv[delvi + g.osampv * ov + cfov - 1]);
                        sumwt = __fadd_rn(sumwt, uvwt);
                        for (int iz = 1; iz <= g.nz; iz++)
                            acc = cadd(acc, cmul(cscale(gat(g.uorigin, vi, iz), uvwt), crotz(iz)));
                    }
                }
            }
        } else {
            for (int ov = -g.suppv; ov <= g.suppv; ov++) {
                const float gv = fnv[delvi + g.osampv * ov + cfov - 1];
                const int vi = g.vorigin + vcen + ov;
                for (int ou = -g.suppu; ou <= g.suppu; ou++) {
                    const int ui = g.uorigin + ucen + ou;
                    const float uvwt = __fmul_rn(fnu[delui + g.osampu * ou + cfou - 1], gv);
                    sumwt = __fadd_rn(sumwt, uvwt);
                    for (int iz = 1; iz <= g.nz; iz++)
                        acc = cadd(acc, cmul(cscale(gat(ui, vi, iz), uvwt), crotz(iz)));
                }
            }
        }
        if (sumwt > 0.f) {
            acc = make_float2(__fdiv_rn(acc.x, sumwt), __fdiv_rn(acc.y, sumwt));
            wt[k] = wk;
        } else {
            atomicAdd(nbad, 1ull);
            acc = make_float2(0.f, 0.f);
        }
        if (__fmul_rn(g.uscale, ul) > 0.f) acc.y = -acc.y;
        vis[k] = cmul(acc, rot);
    }
}

H23Geom make_geom(float uscale, float uoffset, float vscale, float voffset, int uorigin, int vorigin, int nu, int nv,
                  int nz, int suppu, int osampu, int suppv, int osampv, float cellz, float refz, const double *shift,
                  int psf) {
    H23Geom g{};
    g.uscale = uscale;
    g.uoffset = uoffset;
    g.vscale = vscale;
    g.voffset = voffset;
    g.uorigin = uorigin;
    g.vorigin = vorigin;
    g.nu = nu;
    g.nv = nv;
    g.nz = nz;
    g.suppu = suppu;
    g.osampu = osampu;
    g.suppv = suppv;
    g.osampv = osampv;
    g.cellz = cellz;
    g.refz = refz;
    g.twopi = 8.0f * atanf(1.0f);
    g.dtor = g.twopi / 360.0f;
    g.psf = psf;
    for (int i = 0; i < 9; i++) g.s[i] = shift[i];
    return g;
}

}  // namespace

// GRDH23D on device arrays: the NZ-plane grid [nz][nv][nu] complex is written to grid
int grid_h23d(sde_ctx *ctx, int64_t nvis, const float *vis, const float *wt, const float *u, const float *v,
              const float *w, float uscale, float uoffset, float vscale, float voffset, int uorigin, int vorigin,
              int psf, int nu, int nv, const float *fnu, int suppu, int osampu, const float *fnv, int suppv,
              int osampv, int nz, float cellz, float refz, const double *shift, float *grid, float *sumwt) {
    cudaStream_t st = ctx->stream;
    const H23Geom g = make_geom(uscale, uoffset, vscale, voffset, uorigin, vorigin, nu, nv, nz, suppu, osampu, suppv,
                                osampv, cellz, refz, shift, psf);
    const size_t cells = (size_t)nu * nv * nz;
    float2 *raw;
    H23Sums *sums;
    SDE_TRY(ctx_scratch(ctx, "h23_raw", sizeof(float2) * cells, (void **)&raw));
    SDE_TRY(ctx_scratch(ctx, "h23_sums", sizeof(H23Sums), (void **)&sums));
    SDE_CUDA_TRY(cudaMemsetAsync(raw, 0, sizeof(float2) * cells, st));
    SDE_CUDA_TRY(cudaMemsetAsync(sums, 0, sizeof(H23Sums), st));
    {
        KTimer kt(ctx, "h23_grid");
        const unsigned nb = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(nvis, (int64_t)128),
                                                                              (int64_t)ctx->num_sms * 16));
        k_h23_grid<<<nb, 128, 0, st>>>(reinterpret_cast<const float2 *>(vis), wt, u, v, w, nvis, g, fnu, fnv, raw, sums);
        SDE_CHECK_LAUNCH();
    }
    H23Sums h{};
    SDE_CUDA_TRY(cudaMemcpyAsync(&h, sums, sizeof h, cudaMemcpyDeviceToHost, st));
    SDE_CUDA_TRY(cudaStreamSynchronize(st));
    if (sumwt) *sumwt = (float)h.sumwt;
    if (h.lsumwt == 0.0) {
        sde_set_error("No weight!");  // grd/grdh23d.f:104-106: the grid stays as gridded
        SDE_CUDA_TRY(cudaMemcpyAsync(grid, raw, sizeof(float2) * cells, cudaMemcpyDeviceToDevice, st));
        return SDE_ENOWEIGHT;
    }
    k_h23_final<<<ctx->num_sms * 8, 256, 0, st>>>(raw, g, sums, reinterpret_cast<float2 *>(grid));
    SDE_CHECK_LAUNCH();
    return SDE_OK;
}

// GRDDEH23 on device arrays; *nbad = points not degridded (their WT negated)
int degrid_h23(sde_ctx *ctx, int64_t nvis, float *vis, float *wt, const float *u, const float *v, const float *w,
               float uscale, float uoffset, float vscale, float voffset, int uorigin, int vorigin, const float *grid,
               int nu, int nv, const float *fnu, int suppu, int osampu, const float *fnv, int suppv, int osampv,
               int nz, float cellz, float refz, const double *shift, int64_t *nbad) {
    cudaStream_t st = ctx->stream;
    const H23Geom g = make_geom(uscale, uoffset, vscale, voffset, uorigin, vorigin, nu, nv, nz, suppu, osampu, suppv,
                                osampv, cellz, refz, shift, 0);
    unsigned long long *dn;
    SDE_TRY(ctx_scratch(ctx, "h23_nbad", sizeof(unsigned long long), (void **)&dn));
    SDE_CUDA_TRY(cudaMemsetAsync(dn, 0, sizeof(unsigned long long), st));
    {
        KTimer kt(ctx, "h23_degrid");
        const unsigned nb = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(nvis, (int64_t)128),
                                                                              (int64_t)ctx->num_sms * 16));
        k_deh23<<<nb, 128, 0, st>>>(reinterpret_cast<float2 *>(vis), wt, u, v, w, nvis, g, fnu, fnv,
                                    reinterpret_cast<const float2 *>(grid), dn);
        SDE_CHECK_LAUNCH();
    }
    unsigned long long h = 0;
    SDE_CUDA_TRY(cudaMemcpyAsync(&h, dn, sizeof h, cudaMemcpyDeviceToHost, st));
    SDE_CUDA_TRY(cudaStreamSynchronize(st));
    if (nbad) *nbad = (int64_t)h;
    return SDE_OK;
}
