// model.cu -- MODIMG2D (mod/modimg2d.f, called by MODIMG, mod/modimg.f, for vismodel's and
// the imaging tasks' component models): point, Gaussian, disk, rectangle, sphere, shell and
// power-law components added into an image.  One thread per pixel walks the components in
// order, so each pixel's FP32 sum has the reference's order; the per-component constants
// (RNORM, FACT, COS/SIN of the position angle) are the reference's REAL expressions evaluated
// once on the host, and the per-pixel arithmetic uses round-to-nearest intrinsics (no FMA
// contraction), so results differ from the reference only where CUDA's expf/powf round
// differently in the last place.  A shell's normalisation (a sum over all pixels) is one
// block per shell, in double.
#include <math.h>
#include <string.h>

#include <vector>

#include "common.cuh"

namespace {

enum { M_POIN = 0, M_GAUS, M_DISK, M_RECT, M_SPHE, M_SHEL, M_PLOR };

struct ModelComp {
    int type, px, py;  // px, py: the point's 1-based pixel (POIN)
    float flux, ra, dec, bmaj, bmin, rnorm, fact, cospa, sinpa, dr;
};

__device__ __forceinline__ void comp_offsets(const ModelComp &c, int ix, int iy, float refx, float deltx,
                                             float refy, float delty, float *qa, float *qb, float *dmaj,
                                             float *dmin) {
    const float dy = __fsub_rn(__fmul_rn(__fsub_rn((float)iy, refy), delty), c.dec);
    const float dx = __fsub_rn(__fmul_rn(__fsub_rn((float)ix, refx), deltx), c.ra);
    *dmaj = __fadd_rn(__fmul_rn(dx, c.sinpa), __fmul_rn(dy, c.cospa));
    *dmin = __fadd_rn(__fmul_rn(-dx, c.cospa), __fmul_rn(dy, c.sinpa));
    *qa = __fdiv_rn(*dmaj, c.bmaj);
    *qb = __fdiv_rn(*dmin, c.bmin);
}

// the shell term (mod/modimg2d.f:178-201) as (numerator, denominator); (0, 1) outside.  The
// normalisation adds num/den, the image RNORM*num/den, i.e. (RNORM*num)/den.
__device__ __forceinline__ float2 shell_term(const ModelComp &c, float qa, float qb) {
    const float r = __fsqrt_rn(__fmul_rn(4.0f, __fadd_rn(__fmul_rn(qa, qa), __fmul_rn(qb, qb))));
    const float h = __fdiv_rn(c.dr, 2.0f);
    float rmin = __fsub_rn(r, h);
    if (!(rmin < 1.0f)) return make_float2(0.f, 1.f);
    rmin = fmaxf(rmin, 0.f);
    const float rmax = __fadd_rn(r, h), rmax1 = fminf(rmax, 1.0f);
    if (!(rmax > rmin)) return make_float2(0.f, 1.f);
    const float num = __fsub_rn(__fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(rmin, rmin))),
                                __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(rmax1, rmax1))));
    const float pi = 3.14159265358979323846f;
    const float den = __fmul_rn(__fmul_rn(__fmul_rn(2.0f, pi), pi),
                                __fsub_rn(__fmul_rn(rmax, rmax), __fmul_rn(rmin, rmin)));
    return make_float2(num, den);
}

// RNORM of each shell: FLUX / (sum of the shell term over all pixels), block c for shell c
__global__ void k_shell_norm(ModelComp *comps, const int *shells, int nx, int ny, float refx, float deltx,
                             float refy, float delty) {
    ModelComp &c = comps[shells[blockIdx.x]];
    double s = 0.0;
    for (int64_t p = threadIdx.x; p < (int64_t)nx * ny; p += blockDim.x) {
        float qa, qb, dmaj, dmin;
        comp_offsets(c, (int)(p % nx) + 1, (int)(p / nx) + 1, refx, deltx, refy, delty, &qa, &qb, &dmaj, &dmin);
        const float2 q = shell_term(c, qa, qb);
        s += __fdiv_rn(q.x, q.y);
    }
    __shared__ double ws[32];
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += ws[w];
        c.rnorm = __fdiv_rn(c.flux, (float)t);
    }
}

__global__ void k_model_image(const ModelComp *__restrict__ comps, int ncomp, int nx, int ny, float refx,
                              float deltx, float refy, float delty, float *image) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (int64_t)nx * ny) return;
    const int ix = (int)(p % nx) + 1, iy = (int)(p / nx) + 1;
    float a = image[p];
    for (int k = 0; k < ncomp; k++) {
        const ModelComp c = comps[k];
        if (c.type == M_POIN) {
            if (ix == c.px && iy == c.py) a = __fadd_rn(a, c.flux);
            continue;
        }
        float qa, qb, dmaj, dmin;
        comp_offsets(c, ix, iy, refx, deltx, refy, delty, &qa, &qb, &dmaj, &dmin);
        const float r = __fadd_rn(__fmul_rn(qa, qa), __fmul_rn(qb, qb));
        switch (c.type) {
            case M_GAUS:
                a = __fadd_rn(a, __fmul_rn(__fmul_rn(c.flux, c.rnorm), expf(__fmul_rn(-c.fact, r))));
                break;
            case M_DISK:
                if (r < 0.25f) a = __fadd_rn(a, c.rnorm);
                break;
            case M_RECT:
                if (fabsf(dmaj) < __fmul_rn(0.5f, c.bmaj) && fabsf(dmin) < __fmul_rn(0.5f, c.bmin))
                    a = __fadd_rn(a, __fmul_rn(c.flux, c.rnorm));
                break;
            case M_SPHE:
                if (r < 0.25f) a = __fadd_rn(a, __fmul_rn(c.rnorm, __fsqrt_rn(__fsub_rn(1.0f, __fmul_rn(4.0f, r)))));
                break;
            case M_SHEL: {
                const float2 q = shell_term(c, qa, qb);
                if (q.x != 0.f) a = __fadd_rn(a, __fdiv_rn(__fmul_rn(c.rnorm, q.x), q.y));
                break;
            }
            default:  // PLOR
                a = __fadd_rn(a, __fmul_rn(__fmul_rn(c.flux, c.rnorm),
                                           powf(__fadd_rn(__fmul_rn(c.fact, __fmul_rn(r, 4.0f)), 1.0f), -1.5f)));
                break;
        }
    }
    image[p] = a;
}

int fail(const char *m) {
    sde_set_error("%s", m);
    return SDE_EINVAL;
}

}  // namespace

extern "C" int sde_model_image(sde_ctx *ctx, int ncomp, const char *types, const float *flux, const float *ra,
                               const float *dec, const float *bmaj, const float *bmin, const float *bpa, int nx,
                               int ny, float refx, float deltx, float refy, float delty, float *image) {
    if (!ctx || ncomp < 0 || nx < 1 || ny < 1 || !image || (ncomp > 0 && (!types || !flux || !ra || !dec)))
        return fail("sde_model_image: bad arguments");
    // mod/modimg2d.f:31-38
    if (deltx == 0.0f) return fail("Zero increment in X");
    if (delty == 0.0f) return fail("Zero increment in Y");
    if (ncomp == 0) return SDE_OK;
    static const char *names[] = {"POIN", "GAUS", "DISK", "RECT", "SPHE", "SHEL", "PLOR"};
    const float pi = 3.14159265358979323846f;
    std::vector<ModelComp> h((size_t)ncomp);
    std::vector<int> shells;
    for (int k = 0; k < ncomp; k++) {
        ModelComp c{};
        c.type = -1;
        for (int t = 0; t < 7; t++)
            if (strncmp(types + 4 * (size_t)k, names[t], 4) == 0) c.type = t;
        if (c.type < 0) {
            sde_set_error("Unknown model type %.4s for component %4d", types + 4 * (size_t)k, k + 1);
            return SDE_EINVAL;
        }
        c.flux = flux[k];
        c.ra = ra[k];
        c.dec = dec[k];
        if (c.type == M_POIN) {
            // IX = NINT(REFX + RA/DELTX) (mod/modimg2d.f:41-42)
            c.px = (int)lroundf(refx + ra[k] / deltx);
            c.py = (int)lroundf(refy + dec[k] / delty);
            h[(size_t)k] = c;
            continue;
        }
        if (!bmaj || !bmin || !bpa) return fail("sde_model_image: bad arguments");
        if (bmaj[k] == 0.0f) return fail("Major axis zero");
        if (bmin[k] == 0.0f) return fail("Minor axis zero");
        c.bmaj = bmaj[k];
        c.bmin = bmin[k];
        c.cospa = cosf(pi * bpa[k] / 180.0f);
        c.sinpa = sinf(pi * bpa[k] / 180.0f);
        switch (c.type) {
            case M_GAUS:
                c.rnorm = 1.0f / fabsf((atanf(1.0f) / logf(2.0f)) * c.bmaj * c.bmin / (deltx * delty));
                c.fact = 4.0f * logf(2.0f);
                break;
            case M_DISK:
                c.rnorm = c.flux / fabsf(atanf(1.0f) * c.bmaj * c.bmin / (deltx * delty));
                break;
            case M_RECT:
                c.rnorm = 1.0f / fabsf(c.bmaj * c.bmin / (deltx * delty));
                break;
            case M_SPHE:
                c.rnorm = c.flux * fabsf(4.0f * 1.5f * deltx * delty / (pi * c.bmaj * c.bmin));
                break;
            case M_SHEL:
                c.dr = 2.0f * sqrtf(fabsf(deltx * delty) / (c.bmaj * c.bmin));
                shells.push_back(k);
                break;
            default:  // PLOR
                c.fact = powf(4.0f, 1.0f / 3.0f) - 1.0f;
                c.rnorm = fabsf(deltx * delty) * c.fact / (atanf(1.0f) * 2.0f * c.bmaj * c.bmin);
                break;
        }
        h[(size_t)k] = c;
    }
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    ModelComp *d;
    int *dsh = nullptr;
    SDE_TRY(ctx_scratch(ctx, "model_comps", sizeof(ModelComp) * (size_t)ncomp, (void **)&d));
    SDE_CUDA_TRY(cudaMemcpyAsync(d, h.data(), sizeof(ModelComp) * (size_t)ncomp, cudaMemcpyHostToDevice, st));
    if (!shells.empty()) {
        SDE_TRY(ctx_scratch(ctx, "model_shells", sizeof(int) * shells.size(), (void **)&dsh));
        SDE_CUDA_TRY(cudaMemcpyAsync(dsh, shells.data(), sizeof(int) * shells.size(), cudaMemcpyHostToDevice, st));
        k_shell_norm<<<(unsigned)shells.size(), 1024, 0, st>>>(d, dsh, nx, ny, refx, deltx, refy, delty);
        SDE_CHECK_LAUNCH();
    }
    KTimer kt(ctx, "model_image");
    const int64_t npix = (int64_t)nx * ny;
    k_model_image<<<(unsigned)ceil_div(npix, (int64_t)256), 256, 0, st>>>(d, ncomp, nx, ny, refx, deltx, refy, delty,
                                                                        image);
    SDE_CHECK_LAUNCH();
    // the host arrays h and shells go out of scope: finish their (pageable) uploads first
    SDE_CUDA_TRY(cudaStreamSynchronize(st));
    return SDE_OK;
}

// ---------------------------------------------------------------------------------------
// IMGDOUBL (img/imgdoubl.f:56-86) with PIXRPAD (pix/pixrpad.f:38-62) for 2-D images: the
// image placed in a zeroed px x py array, px = FFTPWR2(2 nx) (1 for a one-pixel axis), with
// left margin LSHIFT = NINT(px/2 - RPIX) per axis, so the reference pixel moves to
// RPIX + LSHIFT.  One thread per output pixel reads its source pixel or writes zero: every
// output element written once, coalesced.
namespace {
__global__ void k_image_pad(const float *__restrict__ in, int nx, int ny, int lsx, int lsy,
                            float *__restrict__ out, int px, int py) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (int64_t)px * py) return;
    const int jy = (int)(k / px), jx = (int)(k - (int64_t)jy * px);  // 0-based output pixel
    const int ix = jx - lsx, iy = jy - lsy;                          // 0-based source pixel
    out[k] = (ix >= 0 && ix < nx && iy >= 0 && iy < ny) ? in[(int64_t)iy * nx + ix] : 0.0f;
}
}  // namespace

extern "C" int sde_image_double(sde_ctx *ctx, const float *in, int nx, int ny, float rpix_x,
                                float rpix_y, float *out, int px, int py, float *rpix_out) {
    if (!ctx || !in || !out || nx < 1 || ny < 1) {
        sde_set_error("sde_image_double: bad arguments");
        return SDE_EINVAL;
    }
    const int n[2] = {nx, ny};
    const float rp[2] = {rpix_x, rpix_y};
    int pn[2], ls[2];
    for (int a = 0; a < 2; a++) {
        if (n[a] > 1) {
            if (n[a] > (1 << 29)) {
                sde_set_error("sde_image_double: axis of %d pixels too long", n[a]);
                return SDE_EINVAL;
            }
            pn[a] = fftpwr2(2 * n[a]);
            // NINT(REAL(P/2) - RPIX): REAL arithmetic, half away from zero
            const float d = (float)(pn[a] / 2) - rp[a];
            ls[a] = (int)(d >= 0.0f ? floorf(d + 0.5f) : -floorf(-d + 0.5f));
        } else {
            pn[a] = 1;
            ls[a] = 0;
        }
    }
    if (px != pn[0] || py != pn[1]) {
        sde_set_error("sde_image_double: output must be %d x %d (FFTPWR2 of twice each axis)", pn[0], pn[1]);
        return SDE_EINVAL;
    }
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    const int64_t np = (int64_t)px * py;
    KTimer kt(ctx, "image_pad");
    k_image_pad<<<(unsigned)ceil_div(np, (int64_t)256), 256, 0, ctx->stream>>>(in, nx, ny, ls[0], ls[1], out, px, py);
    SDE_CHECK_LAUNCH();
    if (rpix_out) {
        rpix_out[0] = rpix_x + (float)ls[0];
        rpix_out[1] = rpix_y + (float)ls[1];
    }
    return SDE_OK;
}
