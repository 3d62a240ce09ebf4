// uruwt.cu -- ungridded robust weighting, uvmap's "slow weighting" (GridWeights = F,
// task/uvmap.f:283-290): GRDURUWT (grd/grduruwt.f) with its default GRDURUW2
// (grd/grduruw2.f).  Each visibility's new weight comes from the summed weight of the
// visibilities (either conjugation) inside an ellipse of radii IDELT/(WTFOV SQRT(PI)) around
// it, then the robust formula WT/(WTSUM F2 + D2).
// The reference finds neighbours through a bin plane of linked lists whose structure is fixed
// by the order of insertion (a bin's head is also overwritten by visibilities whose conjugate
// lands there, so a conjugate bin's list is the tail of another bin's list, and each node
// carries the running weight sum of the rest of its list).  That O(N) build runs on the host
// in the reference's order; the search -- the bins of each visibility's ellipse in (J, I)
// order, whole-list sums where a bin is inside, list walks where it is cut -- runs on the GPU,
// one thread per visibility summing in the reference's order, so WTSUM is the reference's
// REAL sum bit for bit.
#include <math.h>
#include <string.h>

#include <vector>

#include "common.cuh"

namespace {

struct UruGeom {
    int nu, nv, uorigin, vorigin, doshift;
    float du, dv, uscale, vscale, urad, vrad, ur2, vr2;
    double s[9];
};

// U0/V0: DOUBLE products summed left to right, stored REAL (grd/grduruw2.f:145-152); no
// contraction into FMA on either side (the host build passes -ffp-contract=off)
__host__ __device__ inline void uru_local(const UruGeom &g, float u, float v, float w, float *u0, float *v0) {
    if (g.doshift) {
        const double uu = u, vv = v, ww = w;
#ifdef __CUDA_ARCH__
        *u0 = (float)__dadd_rn(__dadd_rn(__dmul_rn(g.s[0], uu), __dmul_rn(g.s[1], vv)), __dmul_rn(g.s[2], ww));
        *v0 = (float)__dadd_rn(__dadd_rn(__dmul_rn(g.s[3], uu), __dmul_rn(g.s[4], vv)), __dmul_rn(g.s[5], ww));
#else
        *u0 = (float)(g.s[0] * uu + g.s[1] * vv + g.s[2] * ww);
        *v0 = (float)(g.s[3] * uu + g.s[4] * vv + g.s[5] * ww);
#endif
    } else {
        *u0 = u;
        *v0 = v;
    }
}

// UTLGINT (utl/utlgint.f): the greatest integer <= f
__host__ __device__ inline int utlgint(float f) {
    if (f >= 0.f) return (int)f;
    const int i = (int)f;
    return ((float)i == f) ? i : i - 1;
}

// ((A)**2/UR2 + (B)**2/VR2), REAL
__device__ __forceinline__ float ell(float a, float b, float ur2, float vr2) {
    return __fadd_rn(__fdiv_rn(__fmul_rn(a, a), ur2), __fdiv_rn(__fmul_rn(b, b), vr2));
}

// grd/grduruw2.f:262-390 for every visibility with WT > 0: NEWWT = WTSUM
__global__ void k_uru_search(const float *__restrict__ u, const float *__restrict__ v, const float *__restrict__ w,
                             const float *__restrict__ wt, int nvis, UruGeom g, const int *__restrict__ head,
                             const int *__restrict__ links, const float *__restrict__ bsum, float *newwt,
                             int *zero_flag) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nvis || !(wt[k] > 0.f)) return;
    float u0, v0;
    uru_local(g, u[k], v[k], w[k], &u0, &v0);
    if (u0 < 0.f) {
        u0 = -u0;
        v0 = -v0;
    }
    int ub = utlgint(__fmul_rn(__fsub_rn(u0, g.urad), g.uscale)) + g.uorigin + 1;
    int ub1 = utlgint(__fmul_rn(__fadd_rn(u0, g.urad), g.uscale)) + g.uorigin + 1;
    int vb = utlgint(__fmul_rn(__fsub_rn(v0, g.vrad), g.vscale)) + g.vorigin + 1;
    int vb1 = utlgint(__fmul_rn(__fadd_rn(v0, g.vrad), g.vscale)) + g.vorigin + 1;
    ub = max(1, min(g.nu, ub));
    ub1 = max(1, min(g.nu, ub1));
    vb = max(1, min(g.nv, vb));
    vb1 = max(1, min(g.nv, vb1));
    const float ur2 = g.ur2, vr2 = g.vr2, du = g.du, dv = g.dv;
    float wtsum = 0.f;
    for (int j = vb; j <= vb1; j++) {
        for (int i = ub; i <= ub1; i++) {
            const int h = head[(size_t)(j - 1) * g.nu + (i - 1)];
            if (h == 0) continue;
            // the bin's upper right corner
            const float UB = __fmul_rn((float)(i - g.uorigin - 1), du), VB = __fmul_rn((float)(j - g.vorigin), dv);
            const float a0 = __fsub_rn(UB, u0), a1 = __fsub_rn(__fadd_rn(UB, du), u0);
            const float b0 = __fsub_rn(VB, v0), b1 = __fsub_rn(__fsub_rn(VB, dv), v0);
            int take = 0;  // 1: whole list (GO TO 205); -1: skip (GO TO 210); 0: walk the list
            if (__fadd_rn(UB, du) < u0) {
                if (__fsub_rn(VB, dv) > v0) {
                    if (ell(a0, b0, ur2, vr2) <= 1.f) take = 1;
                    else if (ell(a1, b1, ur2, vr2) >= 1.f) take = -1;
                } else if (VB < v0) {
                    if (ell(a0, b1, ur2, vr2) <= 1.f) take = 1;
                    else if (ell(a1, b0, ur2, vr2) >= 1.f) take = -1;
                } else {
                    if (ell(a0, b0, ur2, vr2) <= 1.f && ell(a0, b1, ur2, vr2) <= 1.f) take = 1;
                }
            } else if (UB > u0) {
                if (__fsub_rn(VB, dv) > v0) {
                    if (ell(a1, b0, ur2, vr2) <= 1.f) take = 1;
                    else if (ell(a0, b1, ur2, vr2) >= 1.f) take = -1;
                } else if (VB < v0) {
                    if (ell(a1, b1, ur2, vr2) <= 1.f) take = 1;
                    else if (ell(a0, b0, ur2, vr2) >= 1.f) take = -1;
                } else {
                    if (ell(a1, b0, ur2, vr2) <= 1.f && ell(a1, b1, ur2, vr2) <= 1.f) take = 1;
                }
            } else {
                if (__fsub_rn(VB, dv) > v0) {
                    if (ell(a0, b0, ur2, vr2) <= 1.f && ell(a1, b0, ur2, vr2) <= 1.f) take = 1;
                } else if (VB < v0) {
                    if (ell(a0, b1, ur2, vr2) <= 1.f && ell(a1, b1, ur2, vr2) <= 1.f) take = 1;
                } else {
                    if (ell(a0, b0, ur2, vr2) <= 1.f && ell(a1, b0, ur2, vr2) <= 1.f &&
                        ell(a1, b1, ur2, vr2) <= 1.f && ell(a0, b1, ur2, vr2) <= 1.f)
                        take = 1;
                }
            }
            if (take < 0) continue;
            if (take > 0) {
                wtsum = __fadd_rn(wtsum, bsum[h - 1]);
                continue;
            }
            const bool posbin = i > g.uorigin;
            for (int l = h; l != 0; l = links[l - 1]) {
                float ut, vt;
                uru_local(g, u[l - 1], v[l - 1], w[l - 1], &ut, &vt);
                if (posbin ? (ut < 0.f) : (ut > 0.f)) {
                    ut = -ut;
                    vt = -vt;
                }
                if (ell(__fsub_rn(ut, u0), __fsub_rn(vt, v0), ur2, vr2) < 1.f) wtsum = __fadd_rn(wtsum, wt[l - 1]);
            }
        }
    }
    if (wtsum == 0.f) atomicExch(zero_flag, 1);
    newwt[k] = wtsum;
}

// grd/grduruw2.f:436-439: NEWWT = WT / (NEWWT * F2 + D2) where WT > 0; elsewhere NEWWT keeps
// the input weight it was given before the binning (dropped points included)
__global__ void k_uru_apply(const float *__restrict__ wt, int nvis, float f2, float d2, float *newwt) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nvis) return;
    const float w = wt[k];
    if (w > 0.f) newwt[k] = __fdiv_rn(w, __fadd_rn(__fmul_rn(newwt[k], f2), d2));
}

int fail(const char *m) {
    sde_set_error("%s", m);
    return SDE_EINVAL;
}

}  // namespace

extern "C" int sde_weights_ungridded(sde_ctx *ctx, int64_t nvis64, const float *u, const float *v, const float *w,
                                     const float *wt_in, float idelt_u, float idelt_v, float wtfov, int rmode,
                                     const float *robust, float ds, const double *shift, int nbu, int nbv,
                                     float *newwt, sde_uruwt_stats *st) {
    if (!ctx || nvis64 < 0 || (nvis64 > 0 && (!u || !v || !w || !wt_in || !newwt)) || !shift)
        return fail("sde_weights_ungridded: bad arguments");
    if (nvis64 >= (int64_t)1 << 31) return fail("sde_weights_ungridded: at most 2^31-1 visibilities");
    if (rmode < 1 || rmode > 3) return fail("Unrecognized RMODE");  // NORM 1, ABS 2, NONE 3
    const int nvis = (int)nvis64;
    // WT as GRDURUW2 sees it: points off the binning plane become -1 (grd/grduruw2.f:219-221)
    std::vector<float> wtv(wt_in, wt_in + nvis);
    float *wt = wtv.data();
    sde_uruwt_stats stats{};
    UruGeom g{};
    for (int i = 0; i < 9; i++) g.s[i] = shift[i];
    g.doshift = shift[0] != 1.0 || shift[4] != 1.0 || shift[8] != 1.0;
    // grd/grduruwt.f:178-179, PI = 3.1415927 (REAL)
    const float pi = 3.1415927f;
    g.urad = fabsf(idelt_u / (wtfov * sqrtf(pi)));
    g.vrad = fabsf(idelt_v / (wtfov * sqrtf(pi)));
    float umax = -1.f, vmax = -1.f;
    for (int k = 0; k < nvis; k++) {
        if (!(wt[k] > 0.f)) continue;
        float u0, v0;
        uru_local(g, u[k], v[k], w[k], &u0, &v0);
        if (fabsf(u0) > umax) umax = fabsf(u0);
        if (fabsf(v0) > vmax) vmax = fabsf(v0);
    }
    const float bineps = 0.1f;
    if (nbu <= 0) {
        // GRDEUSZ0 (grd/grdeusz0.f:58-64), UTLLINT = least integer >= f
        auto utllint = [](float f) {
            const int i = (int)f;
            return f >= 0.f ? (((float)i == f) ? i : i + 1) : i;
        };
        const float opt = 7.6f;
        const int nun = utllint(opt + bineps), nup = utllint(opt * umax / g.urad + bineps);
        int nvb = 2 * utllint(opt * vmax / g.vrad + bineps);
        nbu = std::min(1000, nun + nup);
        nbv = std::min(2000, nvb);
    }
    if (nbv <= 0) nbv = 2 * nbu;  // grd/grduruwt.f:148
    if (nbu < 2 || nbv < 2) return fail("Bad size for binning array");
    g.nu = nbu;
    g.nv = nbv;
    g.ur2 = g.urad * g.urad;
    g.vr2 = g.vrad * g.vrad;
    // origin and bin sizes (grd/grduruw2.f:172-190)
    int uo;
    for (uo = 1; uo <= nbu - 1; uo++) {
        g.du = umax / ((float)(nbu - uo) - bineps);
        if (((float)uo - bineps) * g.du > g.urad) break;
    }
    if (uo > nbu - 1) uo = nbu - 1;
    if (g.urad / g.du + bineps > (float)uo && (nbu - uo) > uo) return fail("Problems with binsize calcs");
    g.uorigin = uo;
    g.vorigin = nbv / 2;
    g.dv = vmax / ((float)g.vorigin - bineps);
    g.uscale = 1.0f / g.du;
    g.vscale = 1.0f / g.dv;
    // the bin plane of linked lists, in the reference's insertion order (grd/grduruw2.f:197-240)
    std::vector<int> head((size_t)nbu * nbv, 0), links((size_t)nvis, 0);
    std::vector<float> bsum((size_t)nvis, 0.f);
    for (int k = 0; k < nvis; k++) {
        newwt[k] = wt[k];
        if (!(wt[k] > 0.f)) continue;
        float u0, v0;
        uru_local(g, u[k], v[k], w[k], &u0, &v0);
        float uc = g.uscale * u0, vc = g.vscale * v0;
        if (uc < 0.f) {
            uc = -uc;
            vc = -vc;
        }
        const int ub = utlgint(uc) + g.uorigin + 1, vb = utlgint(vc) + g.vorigin + 1;
        const int ub1 = utlgint(-uc) + g.uorigin + 1, vb1 = utlgint(-vc) + g.vorigin + 1;
        if (ub < 1 || ub > nbu || vb < 1 || vb > nbv) {
            stats.ndrop++;
            wt[k] = -1.0f;
            continue;
        }
        int &hd = head[(size_t)(vb - 1) * nbu + (ub - 1)];
        const int l = hd;
        hd = k + 1;
        links[(size_t)k] = l;
        if (ub1 >= 1 && ub1 <= nbu && vb1 >= 1 && vb1 <= nbv) head[(size_t)(vb1 - 1) * nbu + (ub1 - 1)] = k + 1;
        bsum[(size_t)k] = l == 0 ? wt[k] : wt[k] + bsum[(size_t)l - 1];
    }
    stats.nbu = nbu;
    stats.nbv = nbv;
    stats.uradius = g.urad;
    stats.vradius = g.vrad;
    // the search on the device
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t stm = ctx->stream;
    const size_t n1 = (size_t)(nvis > 0 ? nvis : 1);
    float *d;
    int *dh, *dflag;
    SDE_TRY(ctx_scratch(ctx, "uru_f", sizeof(float) * n1 * 6, (void **)&d));
    SDE_TRY(ctx_scratch(ctx, "uru_i", sizeof(int) * ((size_t)nbu * nbv + n1 + 1), (void **)&dh));
    float *du = d, *dv = d + n1, *dw = d + 2 * n1, *dwt = d + 3 * n1, *dbs = d + 4 * n1, *dnw = d + 5 * n1;
    int *dl = dh + (size_t)nbu * nbv;
    dflag = dl + n1;
    const cudaMemcpyKind h2d = cudaMemcpyHostToDevice;
    if (nvis > 0) {
        SDE_CUDA_TRY(cudaMemcpyAsync(du, u, sizeof(float) * nvis, h2d, stm));
        SDE_CUDA_TRY(cudaMemcpyAsync(dv, v, sizeof(float) * nvis, h2d, stm));
        SDE_CUDA_TRY(cudaMemcpyAsync(dw, w, sizeof(float) * nvis, h2d, stm));
        SDE_CUDA_TRY(cudaMemcpyAsync(dwt, wt, sizeof(float) * nvis, h2d, stm));
        SDE_CUDA_TRY(cudaMemcpyAsync(dbs, bsum.data(), sizeof(float) * nvis, h2d, stm));
        SDE_CUDA_TRY(cudaMemcpyAsync(dl, links.data(), sizeof(int) * nvis, h2d, stm));
        SDE_CUDA_TRY(cudaMemcpyAsync(dnw, newwt, sizeof(float) * nvis, h2d, stm));  // NEWWT = WT
    }
    SDE_CUDA_TRY(cudaMemcpyAsync(dh, head.data(), sizeof(int) * head.size(), h2d, stm));
    SDE_CUDA_TRY(cudaMemsetAsync(dflag, 0, sizeof(int), stm));
    if (nvis > 0) {
        KTimer kt(ctx, "uru_search");
        k_uru_search<<<(unsigned)ceil_div(nvis, 128), 128, 0, stm>>>(du, dv, dw, dwt, nvis, g, dh, dl, dbs, dnw, dflag);
        SDE_CHECK_LAUNCH();
    }
    std::vector<float> sums((size_t)nvis);
    int flag = 0;
    if (nvis > 0) SDE_CUDA_TRY(cudaMemcpyAsync(sums.data(), dnw, sizeof(float) * nvis, cudaMemcpyDeviceToHost, stm));
    SDE_CUDA_TRY(cudaMemcpyAsync(&flag, dflag, sizeof(int), cudaMemcpyDeviceToHost, stm));
    SDE_CUDA_TRY(cudaStreamSynchronize(stm));
    if (flag) return fail("Zero WTSUM");
    // SUMLOCWT in DOUBLE in visibility order, then F2, D2 (grd/grduruw2.f:380-382, 422-434)
    double sumloc = 0.0;
    int64_t nsel = 0;
    for (int k = 0; k < nvis; k++)
        if (wt[k] > 0.f) {
            sumloc += sums[(size_t)k];
            nsel++;
        }
    float f2 = 1.f, d2 = 0.f;
    if (rmode == 1) {
        const float t = 5.0f * powf(10.0f, -robust[0]);
        f2 = (float)((double)(t * t) / (sumloc / (double)nsel));
        d2 = 1.f;
    } else if (rmode == 2) {
        f2 = robust[0] * robust[0];
        d2 = 2.0f * ds * ds;
    }
    if (nvis > 0) {
        k_uru_apply<<<(unsigned)ceil_div(nvis, 256), 256, 0, stm>>>(dwt, nvis, f2, d2, dnw);
        SDE_CHECK_LAUNCH();
        SDE_CUDA_TRY(cudaMemcpyAsync(newwt, dnw, sizeof(float) * nvis, cudaMemcpyDeviceToHost, stm));
        SDE_CUDA_TRY(cudaStreamSynchronize(stm));
    }
    stats.sumlocwt = sumloc;
    stats.nsel = nsel;
    stats.f2 = f2;
    stats.d2 = d2;
    if (st) *st = stats;
    if (stats.ndrop > 0) {  // grd/grduruw2.f:243-247
        char m[96];
        snprintf(m, sizeof m, "Warning:%7lld points dropped off the binning grid", (long long)stats.ndrop);
        msgput_(m, "W", strlen(m), 1);
    }
    return SDE_OK;
}
