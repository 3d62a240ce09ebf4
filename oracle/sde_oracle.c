/*
 * sde_oracle.c -- CPU restatement of SDE's imaging hot path.  TEST INFRASTRUCTURE ONLY:
 * the product library never links, loads or calls this code.  See sde_oracle.h for the
 * conventions.  Every routine cites the Fortran file and lines (timcornwell/sde,
 * source/ tree) whose arithmetic it follows, statement by statement.
 *
 * Build: gcc -O2 -ffp-contract=off -fno-fast-math -fPIC -shared (oracle/Makefile).
 */
#include "sde_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define F2(a, i, j, ld) ((a)[((i)-1) + (size_t)((j)-1) * (size_t)(ld)]) /* 1-based col-major */

int orc_nint_f(float x) { return (int)lroundf(x); }  /* Fortran NINT: half away from zero */
int orc_nint_d(double x) { return (int)lround(x); }

/* fft/fftpwr2.f:28-39 */
int orc_fftpwr2(int i) {
    if (i < 1) return 1;
    int lg = orc_nint_f(logf((float)i) / logf(2.0f));
    int p = 1;
    for (int k = 0; k < lg; k++) p *= 2;
    while (p < i) p *= 2;
    return p;
}

/* grd/grdsf.f:46-73: prolate spheroidal m=6, alpha=1 rational approximation */
double orc_grdsf(double nu) {
    static const double P[2][5] = {
        {8.203343e-2, -3.644705e-1, 6.278660e-1, -5.335581e-1, 2.312756e-1},
        {4.028559e-3, -3.697768e-2, 1.021332e-1, -1.201436e-1, 6.412774e-2}};
    static const double Q[2][3] = {{1.0000000e0, 8.212018e-1, 2.078043e-1},
                                   {1.0000000e0, 9.599102e-1, 2.918724e-1}};
    int part;
    double nuend;
    if (nu >= 0.0 && nu < 0.75) {
        part = 0;
        nuend = 0.75;
    } else if (nu >= 0.75 && nu <= 1.00) {
        part = 1;
        nuend = 1.00;
    } else {
        return 0.0;
    }
    double top = P[part][0];
    double delnusq = nu * nu - nuend * nuend;
    for (int k = 1; k <= 4; k++) top = top + P[part][k] * pow(delnusq, (double)k);
    double bot = Q[part][0];
    for (int k = 1; k <= 2; k++) bot = bot + Q[part][k] * pow(delnusq, (double)k);
    return (bot != 0.0) ? top / bot : 0.0;
}

/* grd/grdcf.f:41-90.  code_sf: 1 = 'SF', 0 = 'BOX'.  cf must hold 1+8*129 floats
 * (vis/visgrid.f CFLEN); CF(CFOFFSET+I) == cf[CFOFFSET-1+I]. */
void orc_grdcf(int code_sf, float *cf, int *cfsupp, int *cfosamp) {
    int osamp = 128, supp, off;
    if (!code_sf) {
        supp = 1;
        off = (supp + 1) * osamp + 1;
        for (int i = 0; i <= osamp / 2; i++) {
            cf[off - 1 + i] = 1.0f;
            cf[off - 1 - i] = 1.0f;
        }
        for (int i = osamp / 2 + 1; i <= 2 * osamp; i++) {
            cf[off - 1 + i] = 0.0f;
            cf[off - 1 - i] = 0.0f;
        }
    } else {
        supp = 3;
        off = (supp + 1) * osamp + 1;
        for (int i = 0; i <= supp * osamp; i++) {
            double nu = (double)i / (double)(supp * osamp);
            cf[off - 1 + i] = (float)((1 - pow(nu, 2.0)) * orc_grdsf(nu));
            cf[off - 1 - i] = cf[off - 1 + i];
        }
        for (int i = supp * osamp + 1; i <= (supp + 1) * osamp; i++) {
            cf[off - 1 + i] = 0.0f;
            cf[off - 1 - i] = 0.0f;
        }
    }
    float sum = 0.0f;
    for (int i = -(supp + 1) * osamp; i <= (supp + 1) * osamp; i++) sum = sum + cf[off - 1 + i];
    for (int i = -(supp + 1) * osamp; i <= (supp + 1) * osamp; i++)
        cf[off - 1 + i] = cf[off - 1 + i] / sum;
    *cfsupp = supp;
    *cfosamp = osamp;
}

/* grd/grdccf.f:48-52 ('SF' branch); 'BOX' (grd/grdccf.f:42-47) uses SINC(0.5*PI*NU). */
void orc_grdccf(int code_sf, float *ccf, int ccflen) {
    if (code_sf) {
        for (int i = 1; i <= ccflen; i++) {
            double nu = (double)(i - 1) / (double)(ccflen - 1);
            ccf[i - 1] = (float)orc_grdsf(nu);
        }
    } else {
        const float PI = 3.141592554f;
        ccf[0] = 1.0f;
        for (int i = 2; i <= ccflen; i++) {
            double nu = (double)(i - 1) / (double)(ccflen - 1);
            float x = 0.5f * PI * (float)nu;
            ccf[i - 1] = sinf(x) / x;
        }
    }
}

/* crd/crdshift.f:95-160.  shift is SHIFT(3,3) column-major: SHIFT(I,J) = shift[(I-1)+3(J-1)] */
void orc_crdshift(double vra_deg, double vdec_deg, double ira_deg, double idec_deg,
                  float vrota3_deg, double *shift) {
    double dtor = 4.0 * atan(1.0) / 180.0;
    double rao = dtor * vra_deg, deco = dtor * vdec_deg;
    double ra = dtor * ira_deg, dec = dtor * idec_deg;
    double T[3][3]; /* T[i][j] == TMAT(i+1, j+1) */
    T[0][0] = cos(ra - rao);
    T[1][0] = sin(ra - rao) * sin(deco);
    T[2][0] = -sin(ra - rao) * cos(deco);
    T[0][1] = -sin(ra - rao) * sin(dec);
    T[1][1] = cos(ra - rao) * sin(dec) * sin(deco) + cos(dec) * cos(deco);
    T[2][1] = -cos(ra - rao) * cos(deco) * sin(dec) + cos(dec) * sin(deco);
    T[0][2] = sin(ra - rao) * cos(dec);
    T[1][2] = -cos(ra - rao) * sin(deco) * cos(dec) + sin(dec) * cos(deco);
    T[2][2] = cos(ra - rao) * cos(dec) * cos(deco) + sin(dec) * sin(deco);
    float rota = (float)(dtor * vrota3_deg); /* REAL ROTA */
    if (rota != 0.0f) {
        double R[3][3], S[3][3];
        R[0][0] = cos(rota); R[0][1] = sin(rota); R[0][2] = 0.0;
        R[1][0] = -sin(rota); R[1][1] = cos(rota); R[1][2] = 0.0;
        R[2][0] = 0.0; R[2][1] = 0.0; R[2][2] = 1.0;
        for (int j = 0; j < 3; j++)
            for (int i = 0; i < 3; i++) {
                S[i][j] = 0.0;
                for (int k = 0; k < 3; k++) S[i][j] = S[i][j] + T[k][j] * R[i][k];
            }
        for (int j = 0; j < 3; j++)
            for (int i = 0; i < 3; i++) {
                double s = 0.0;
                for (int k = 0; k < 3; k++) s = s + R[j][k] * S[i][k];
                shift[i + 3 * j] = s;
            }
    } else {
        for (int j = 0; j < 3; j++)
            for (int i = 0; i < 3; i++) shift[i + 3 * j] = T[i][j];
    }
}

#define SH(i, j) shift[((i)-1) + 3 * ((j)-1)]

static int doshift_of(const double *shift) {
    return (SH(1, 1) != 1.0) || (SH(2, 2) != 1.0) || (SH(3, 3) != 1.0);
}

/* FP32 uv -> cell for the weighting routines: grd/grduwt2d.f:92-111 (and grd/grdruw2d.f:134-153).
 * Returns 0 and the 1-based cell if on the grid, else -1. */
static int wcell(const float *u, const float *v, const float *w, int i, float uscale,
                 float uoffset, float vscale, float voffset, int uorigin, int vorigin,
                 const double *shift, int doshift, int nu, int nv, int *ucen, int *vcen,
                 float *ulocal_out, float *vlocal_out) {
    float ucell, vcell, ulocal, vlocal;
    if (doshift) {
        ulocal = (float)(SH(1, 1) * (double)u[i] + SH(2, 1) * (double)v[i] + SH(3, 1) * (double)w[i]);
        vlocal = (float)(SH(1, 2) * (double)u[i] + SH(2, 2) * (double)v[i] + SH(3, 2) * (double)w[i]);
        ucell = uscale * ulocal + uoffset;
        vcell = vscale * vlocal + voffset;
    } else {
        ulocal = u[i];
        vlocal = v[i];
        ucell = uscale * u[i] + uoffset;
        vcell = vscale * v[i] + voffset;
    }
    if (ucell > 0.0f) {
        ucell = ucell + (float)uorigin;
        vcell = vcell + (float)vorigin;
    } else {
        ucell = -ucell + (float)uorigin;
        vcell = -vcell + (float)vorigin;
    }
    *ucen = orc_nint_f(ucell);
    *vcen = orc_nint_f(vcell);
    if (ulocal_out) *ulocal_out = ulocal;
    if (vlocal_out) *vlocal_out = vlocal;
    if (*ucen < 1 || *ucen > nu || *vcen < 1 || *vcen > nv) return -1;
    return 0;
}

/* grd/grduwt2d.f:75-167 (uniform weighting, pass 1 density count then pass 2 NEWWT).
 * newwt may alias wt, as in GRDUWT (grd/grduwt.f:122). */
void orc_grduwt2d(const float *wt, const float *u, const float *v, const float *w, int nvis,
                  float uscale, float uoffset, float vscale, float voffset, int uorigin,
                  int vorigin, float *newwt, float *gwt, int nu, int nv, const double *shift,
                  int *ndrop) {
    for (size_t k = 0; k < (size_t)nu * nv; k++) gwt[k] = 0.0f;
    int doshift = doshift_of(shift);
    for (int i = 0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        int uc, vc;
        if (wcell(u, v, w, i, uscale, uoffset, vscale, voffset, uorigin, vorigin, shift, doshift,
                  nu, nv, &uc, &vc, NULL, NULL))
            continue;
        F2(gwt, uc, vc, nu) = F2(gwt, uc, vc, nu) + wt[i];
    }
    int nd = 0;
    for (int i = 0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        int uc, vc;
        if (wcell(u, v, w, i, uscale, uoffset, vscale, voffset, uorigin, vorigin, shift, doshift,
                  nu, nv, &uc, &vc, NULL, NULL)) {
            newwt[i] = -1.0f;
            nd++;
            continue;
        }
        float g = F2(gwt, uc, vc, nu);
        if (g > 0.0f) {
            if (uc == uorigin) {
                if (vc == vorigin)
                    newwt[i] = wt[i] / g;
                else
                    newwt[i] = 0.5f * wt[i] / g;
            } else {
                newwt[i] = wt[i] / g;
            }
        } else {
            newwt[i] = -1.0f;
        }
    }
    if (ndrop) *ndrop = nd;
}

/* grd/grdruw2d.f:97-242 (robust weighting).  rmode: "NORM", "ABS", "NONE", "AZ-NORM". */
int orc_grdruw2d(const float *wt, const float *u, const float *v, const float *w, int nvis,
                 float uscale, float uoffset, float vscale, float voffset, int uorigin,
                 int vorigin, float *newwt, float *gwt, int nu, int nv, const double *shift,
                 const char *rmode, const float *robust, float ds, int *ndrop,
                 double *sumwt_out, double *sumlocwt_out, float *f2_out) {
    for (size_t k = 0; k < (size_t)nu * nv; k++) gwt[k] = 0.0f;
    int doshift = doshift_of(shift);
    int doaz = (strncmp(rmode, "AZ", 2) == 0);
    float rob, rpa = 0.0f, rbscale = 0.0f, pi = 0.0f;
    if (doaz) {
        rob = (robust[0] + robust[1]) / 2.0f;
        rpa = -robust[2] + 90.0f - 90.0f;
        while (rpa < -90.0f) rpa = rpa + 180.0f;
        while (rpa > 90.0f) rpa = rpa - 180.0f;
        pi = 4.0f * atanf(1.0f);
        rpa = rpa * pi / 180.0f;
        rbscale = (robust[0] - robust[1]) / (pi / 2.0f);
    } else {
        rob = robust[0];
    }
    double sumwt = 0.0;
    for (int i = 0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        int uc, vc;
        if (wcell(u, v, w, i, uscale, uoffset, vscale, voffset, uorigin, vorigin, shift, doshift,
                  nu, nv, &uc, &vc, NULL, NULL))
            continue;
        F2(gwt, uc, vc, nu) = F2(gwt, uc, vc, nu) + wt[i];
        sumwt = sumwt + (double)wt[i];
    }
    float f2, d2;
    double sumlocwt = 0.0;
    if (!strcmp(rmode, "NORM") || !strcmp(rmode, "AZ-NORM")) {
        for (int vg = 1; vg <= nv; vg++)
            for (int ug = 1; ug <= nu; ug++) {
                float g = F2(gwt, ug, vg, nu);
                if (g > 0.0f) sumlocwt = sumlocwt + (double)(g * g);
            }
        float t = 5.0f * powf(10.0f, -rob);
        f2 = (float)((double)(t * t) / (sumlocwt / sumwt));
        d2 = 1.0f;
    } else if (!strcmp(rmode, "ABS")) {
        f2 = rob * rob;
        d2 = 2.0f * (ds * ds);
    } else if (!strcmp(rmode, "NONE")) {
        f2 = 1.0f;
        d2 = 0.0f;
    } else {
        return ORC_EBADMODE;
    }
    if (sumwt_out) *sumwt_out = sumwt;
    if (sumlocwt_out) *sumlocwt_out = sumlocwt;
    if (f2_out) *f2_out = f2;
    int nd = 0;
    for (int i = 0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        int uc, vc;
        float ul, vl;
        if (wcell(u, v, w, i, uscale, uoffset, vscale, voffset, uorigin, vorigin, shift, doshift,
                  nu, nv, &uc, &vc, &ul, &vl)) {
            newwt[i] = -1.0f;
            nd++;
            continue;
        }
        if (doaz) {
            float t = atan2f(vl, ul);
            t = fmodf(t - rpa + 2.5f * pi, pi) - pi / 2.0f;
            float r = robust[0] - fabsf(t) * rbscale;
            float tt = 5.0f * powf(10.0f, -r);
            f2 = (float)((double)(tt * tt) / (sumlocwt / sumwt));
        }
        float g = F2(gwt, uc, vc, nu);
        if (g > 0.0f) {
            if (uc == uorigin && vc != vorigin)
                newwt[i] = 0.5f * wt[i] / (g * f2 + d2);
            else
                newwt[i] = wt[i] / (g * f2 + d2);
        } else {
            newwt[i] = -1.0f;
        }
    }
    if (ndrop) *ndrop = nd;
    return ORC_OK;
}

/* grd/grdh2d.f:89-226 -- the 2-D gridder (shifted by SUPPU, symmetrised, normalised).
 * Written as three parts -- zero the grid, accumulate visibilities i0..i1-1 in order
 * (grdh2d.f:110-189), finalize (grdh2d.f:195-226) -- so that a caller may split the
 * visibility loop into consecutive ranges and get the grid of one pass over all of them. */
#define GRE(uu, vv) gvis[2 * (((size_t)(uu)-1) + (size_t)((vv)-1) * (size_t)nu)]
#define GIM(uu, vv) gvis[2 * (((size_t)(uu)-1) + (size_t)((vv)-1) * (size_t)nu) + 1]
void orc_grdh2d_acc(const float *vis, const float *wt, const float *u, const float *v,
                    const float *w, int i0, int nvis, float uscale, float uoffset, float vscale,
                    float voffset, int uorigin, int vorigin, float *gvis, int psf, int nu, int nv,
                    const float *gridfnu, int suppu, int osampu, const float *gridfnv, int suppv,
                    int osampv, const double *shift, float *sumwt_acc, double *lsumwt_acc) {
    const double twopi = (double)(8.0f * atanf(1.0f));
    const int cfoffset = (suppu + 1) * osampu + 1;
    const int doshift = doshift_of(shift);
    double lsumwt = *lsumwt_acc;
    float swt = *sumwt_acc;
    for (int i = i0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        double ug = (double)u[i], vg = (double)v[i], wg = (double)w[i];
        double ucell, vcell;
        float fr, fi;
        if (doshift) {
            double ul = SH(1, 1) * ug + SH(2, 1) * vg + SH(3, 1) * wg;
            double vl = SH(1, 2) * ug + SH(2, 2) * vg + SH(3, 2) * wg;
            double wl = SH(1, 3) * ug + SH(2, 3) * vg + SH(3, 3) * wg;
            double phase = twopi * (wl - wg);
            float c = (float)cos(phase), s = (float)(-sin(phase));
            float a = vis[2 * i], b = vis[2 * i + 1];
            fr = a * c - b * s;
            fi = a * s + b * c;
            ucell = (double)uscale * ul + (double)uoffset;
            vcell = (double)vscale * vl + (double)voffset;
        } else {
            fr = vis[2 * i];
            fi = vis[2 * i + 1];
            ucell = (double)uscale * ug + (double)uoffset;
            vcell = (double)vscale * vg + (double)voffset;
        }
        if (ucell > 0.0) {
            fi = -fi;
            ucell = ucell + (double)(float)uorigin;
            vcell = vcell + (double)(float)vorigin;
        } else {
            ucell = -ucell + (double)(float)uorigin;
            vcell = -vcell + (double)(float)vorigin;
        }
        if (psf) {
            fr = 1.0f;
            fi = 0.0f;
        }
        int nuc = orc_nint_d(ucell), nvc = orc_nint_d(vcell);
        if (nuc + 2 * suppu > nu) continue;
        if (nvc + suppv > nv) continue;
        if (nvc - suppv < 1) continue;
        swt = swt + wt[i];
        int delui = orc_nint_d((double)osampu * ((double)(float)nuc - ucell)) + cfoffset;
        int delvi = orc_nint_d((double)osampv * ((double)(float)nvc - vcell)) + cfoffset;
        int ucen = nuc + suppu, vcen = nvc;
        for (int offv = -suppv; offv <= suppv; offv++) {
            int delv = delvi + osampv * offv;
            int vgrid = vcen + offv;
            for (int offu = -suppu; offu <= suppu; offu++) {
                int delu = delui + osampu * offu;
                int ugrid = ucen + offu;
                double uvwt = (double)(wt[i] * gridfnu[delu - 1] * gridfnv[delv - 1]);
                GRE(ugrid, vgrid) = (float)((double)GRE(ugrid, vgrid) + uvwt * (double)fr);
                GIM(ugrid, vgrid) = (float)((double)GIM(ugrid, vgrid) + uvwt * (double)fi);
                lsumwt = lsumwt + uvwt;
            }
        }
    }
    *sumwt_acc = swt;
    *lsumwt_acc = lsumwt;
}

int orc_grdh2d_end(float *gvis, int nu, int nv, int uorigin, int vorigin, int suppu,
                   double lsumwt) {
    if (lsumwt == 0.0) return ORC_ENOWEIGHT;
    /* Symmetrize: grd/grdh2d.f:202-214 */
    int ucen = uorigin + suppu, vcen = vorigin;
    for (int offv = -nv / 2 + 1; offv <= nv / 2 - 1; offv++)
        for (int offu = 1; offu <= suppu; offu++) {
            GRE(ucen + offu, vcen + offv) = GRE(ucen + offu, vcen + offv) + GRE(ucen - offu, vcen - offv);
            GIM(ucen + offu, vcen + offv) = GIM(ucen + offu, vcen + offv) - GIM(ucen - offu, vcen - offv);
        }
    for (int offv = 0; offv <= nv / 2 - 1; offv++) {
        GRE(ucen, vcen + offv) = GRE(ucen, vcen + offv) + GRE(ucen, vcen - offv);
        GIM(ucen, vcen + offv) = GIM(ucen, vcen + offv) - GIM(ucen, vcen - offv);
        GRE(ucen, vcen - offv) = GRE(ucen, vcen + offv);
        GIM(ucen, vcen - offv) = -GIM(ucen, vcen + offv);
    }
    /* Shift left and normalize: grd/grdh2d.f:218-226 */
    double scale = (double)((float)(nu - 1) * (float)nv) / lsumwt;
    for (int vg = 1; vg <= nv; vg++) {
        for (int ug = 1; ug <= nu - suppu; ug++) {
            GRE(ug, vg) = (float)(scale * (double)GRE(ug + suppu, vg));
            GIM(ug, vg) = (float)(scale * (double)GIM(ug + suppu, vg));
        }
        for (int ug = nu - suppu + 1; ug <= nu; ug++) {
            GRE(ug, vg) = 0.0f;
            GIM(ug, vg) = 0.0f;
        }
    }
    return ORC_OK;
}
#undef GRE
#undef GIM

int orc_grdh2d(const float *vis, const float *wt, const float *u, const float *v, const float *w,
               int nvis, float uscale, float uoffset, float vscale, float voffset, int uorigin,
               int vorigin, float *gvis, int psf, int nu, int nv, const float *gridfnu, int suppu,
               int osampu, const float *gridfnv, int suppv, int osampv, const double *shift,
               float *sumwt, double *lsumwt_out) {
    for (size_t k = 0; k < 2 * (size_t)nu * nv; k++) gvis[k] = 0.0f;
    double lsumwt = 0.0;
    float swt = 0.0f;
    orc_grdh2d_acc(vis, wt, u, v, w, 0, nvis, uscale, uoffset, vscale, voffset, uorigin, vorigin,
                   gvis, psf, nu, nv, gridfnu, suppu, osampu, gridfnv, suppv, osampv, shift, &swt,
                   &lsumwt);
    if (sumwt) *sumwt = swt;
    if (lsumwt_out) *lsumwt_out = lsumwt;
    return orc_grdh2d_end(gvis, nu, nv, uorigin, vorigin, suppu, lsumwt);
}

/* grd/grddeh2d.f:77-200 -- the 2-D degridder. */
void orc_grddeh2d(float *vis, float *wt, const float *u, const float *v, const float *w, int nvis,
                  float uscale, float uoffset, float vscale, float voffset, int uorigin,
                  int vorigin, const float *gvis, int nu, int nv, const float *intfnu, int suppu,
                  int osampu, const float *intfnv, int suppv, int osampv, const double *shift,
                  int *nbad_out) {
    const double twopi = (double)(8.0f * atanf(1.0f));
    const int cfoffset = (suppu + 1) * osampu + 1;
    int nbad = 0;
#define GR(uu, vv) gvis[2 * (((size_t)(uu)-1) + (size_t)((vv)-1) * (size_t)nu)]
#define GI(uu, vv) gvis[2 * (((size_t)(uu)-1) + (size_t)((vv)-1) * (size_t)nu) + 1]
    for (int i = 0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        float vr = 0.0f, vi = 0.0f, sumwt = 0.0f;
        vis[2 * i] = 0.0f;
        vis[2 * i + 1] = 0.0f;
        wt[i] = -wt[i];
        double ug = (double)u[i], vg = (double)v[i], wg = (double)w[i];
        double ul = SH(1, 1) * ug + SH(2, 1) * vg + SH(3, 1) * wg;
        double vl = SH(1, 2) * ug + SH(2, 2) * vg + SH(3, 2) * wg;
        double wl = SH(1, 3) * ug + SH(2, 3) * vg + SH(3, 3) * wg;
        double phase = twopi * (wl - wg);
        float rc = (float)cos(phase), rs = (float)sin(phase);
        float ucell = (float)((double)uscale * ul + (double)uoffset);
        float vcell = (float)((double)vscale * vl + (double)voffset);
        if (ucell > 0.0f) {
            ucell = ucell + (float)uorigin;
            vcell = vcell + (float)vorigin;
        } else {
            ucell = -ucell + (float)uorigin;
            vcell = -vcell + (float)vorigin;
        }
        int nuc = orc_nint_f(ucell), nvc = orc_nint_f(vcell);
        if (nuc + suppu > nu) continue;
        if (nvc + suppv > nv) continue;
        if (nvc - suppv < 1) continue;
        int delui = orc_nint_f((float)osampu * ((float)nuc - ucell));
        int delvi = orc_nint_f((float)osampv * ((float)nvc - vcell));
        int ucen = nuc - uorigin, vcen = nvc - vorigin;
        if (nuc <= suppu) {
            for (int offu = -suppu; offu <= suppu; offu++) {
                if (ucen != -offu) {
                    int usign = (ucen + offu) >= 0 ? 1 : -1;
                    int delu = delui + osampu * offu + cfoffset;
                    int uint_ = uorigin + usign * (ucen + offu);
                    for (int offv = -suppv; offv <= suppv; offv++) {
                        int delv = delvi + osampv * offv + cfoffset;
                        int vint = vorigin + usign * (vcen + offv);
                        float uvwt = intfnu[delu - 1] * intfnv[delv - 1];
                        float fr = GR(uint_, vint), fi = GI(uint_, vint);
                        if (usign <= 0) fi = -fi;
                        vr = vr + fr * uvwt;
                        vi = vi + fi * uvwt;
                        sumwt = sumwt + uvwt;
                    }
                } else {
                    int delu = delui + osampu * offu + cfoffset;
                    int uint_ = uorigin;
                    for (int offv = -suppv; offv <= suppv; offv++) {
                        int delv = delvi + osampv * offv + cfoffset;
                        int vint = vorigin + (vcen + offv);
                        float uvwt = intfnu[delu - 1] * intfnv[delv - 1];
                        vr = vr + GR(uint_, vint) * uvwt;
                        vi = vi + GI(uint_, vint) * uvwt;
                        sumwt = sumwt + uvwt;
                    }
                }
            }
        } else {
            for (int offv = -suppv; offv <= suppv; offv++) {
                int delv = delvi + osampv * offv + cfoffset;
                int vint = vorigin + vcen + offv;
                for (int offu = -suppu; offu <= suppu; offu++) {
                    int delu = delui + osampu * offu + cfoffset;
                    int uint_ = uorigin + ucen + offu;
                    float uvwt = intfnu[delu - 1] * intfnv[delv - 1];
                    vr = vr + GR(uint_, vint) * uvwt;
                    vi = vi + GI(uint_, vint) * uvwt;
                    sumwt = sumwt + uvwt;
                }
            }
        }
        if (sumwt > 0.0f) {
            vr = vr / sumwt;
            vi = vi / sumwt;
            wt[i] = fabsf(wt[i]);
        } else {
            nbad++;
            vr = 0.0f;
            vi = 0.0f;
        }
        if ((double)uscale * ul > 0.0) vi = -vi;
        vis[2 * i] = vr * rc - vi * rs;
        vis[2 * i + 1] = vr * rs + vi * rc;
    }
#undef GR
#undef GI
    if (nbad_out) *nbad_out = nbad;
}

/* fft/fftx.f:84-275 -- radix-2 complex FFT with quarter-length tables (Newman/AIPS). */
void orc_fftx(float *x, float *wk, int m, int isig) {
#define X1(i) x[2 * ((i)-1)]
#define X2(i) x[2 * ((i)-1) + 1]
#define W1(i) wk[2 * ((i)-1)]
#define W2(i) wk[2 * ((i)-1) + 1]
    float arg = (float)m;
    int n = (int)(logf(arg) / logf(2.0f) + 0.1f);
    int m4 = m / 4, nm2 = n - 2;
    float tpi = 8.0f * atanf(1.0f);
    tpi = tpi / (float)m;
    float *C = (float *)malloc(sizeof(float) * (size_t)(m4 > 0 ? m4 : 1));
    float *S = (float *)malloc(sizeof(float) * (size_t)(m4 > 0 ? m4 : 1));
    int *ibitrv = (int *)malloc(sizeof(int) * (size_t)m);
    for (int i = 1; i <= m4; i++) {
        arg = tpi * (float)(i - 1);
        C[i - 1] = cosf(arg);
        S[i - 1] = sinf(arg);
    }
    for (int i = 1; i <= m4; i++) {
        int i1 = i - 1, j = 0;
        for (int k = 1; k <= nm2; k++) {
            int l = i1 / 2;
            j = i1 + 2 * (j - l);
            i1 = l;
        }
        j = j + 1;
        if (i >= j) continue;
        float xt = C[i - 1]; C[i - 1] = C[j - 1]; C[j - 1] = xt;
        xt = S[i - 1]; S[i - 1] = S[j - 1]; S[j - 1] = xt;
    }
    for (int i = 1; i <= m; i++) {
        int i1 = i - 1, j = 0;
        for (int k = 1; k <= n; k++) {
            int l = i1 / 2;
            j = i1 + 2 * (j - l);
            i1 = l;
        }
        ibitrv[i - 1] = j + 1;
    }
    if (isig == -1) {
        for (int i = 1; i <= m; i++) { W1(i) = X1(i); W2(i) = X2(i); }
    } else {
        for (int i = 1; i <= m; i++) { W1(i) = X1(i); W2(i) = -X2(i); }
    }
    for (int mstep = 1; mstep <= n; mstep++) {
        int isep = 1 << (n - mstep);
        int isep4 = isep * 4;
        int itimes = 1 << (mstep - 1);
        if (itimes <= isep) {
            for (int i = 1; i <= itimes; i++) {
                int isepi1 = 2 * (i - 1) * isep;
                int ii = (i + 1) / 2;
                int ji1 = isepi1 + 1;
                int ji = ji1 + isep;
                float c = C[ii - 1], s = S[ii - 1];
                if (i != 2 * (i / 2)) {
                    for (int j = 1; j <= isep; j++) {
                        float ar = W1(ji) * c - W2(ji) * s;
                        float ai = W1(ji) * s + W2(ji) * c;
                        W1(ji) = W1(ji1) - ar;
                        W2(ji) = W2(ji1) - ai;
                        W1(ji1) = W1(ji1) + ar;
                        W2(ji1) = W2(ji1) + ai;
                        ji1++;
                        ji++;
                    }
                } else {
                    for (int j = 1; j <= isep; j++) {
                        float ar = W1(ji) * s + W2(ji) * c;
                        float ai = W1(ji) * c - W2(ji) * s;
                        W1(ji) = W1(ji1) + ar;
                        W2(ji) = W2(ji1) - ai;
                        W1(ji1) = W1(ji1) - ar;
                        W2(ji1) = W2(ji1) + ai;
                        ji1++;
                        ji++;
                    }
                }
            }
        } else {
            for (int j = 1; j <= isep; j++) {
                int ii = 1, ji1 = j, ji = ji1 + isep;
                for (int i = 1; i <= itimes; i += 2) {
                    float c = C[ii - 1], s = S[ii - 1];
                    float ar = W1(ji) * c - W2(ji) * s;
                    float ai = W1(ji) * s + W2(ji) * c;
                    W1(ji) = W1(ji1) - ar;
                    W2(ji) = W2(ji1) - ai;
                    W1(ji1) = W1(ji1) + ar;
                    W2(ji1) = W2(ji1) + ai;
                    ii++;
                    ji1 += isep4;
                    ji += isep4;
                }
                ii = 1;
                ji1 = j + 2 * isep;
                ji = ji1 + isep;
                for (int i = 2; i <= itimes; i += 2) {
                    float c = C[ii - 1], s = S[ii - 1];
                    float ar = W1(ji) * s + W2(ji) * c;
                    float ai = W1(ji) * c - W2(ji) * s;
                    W1(ji) = W1(ji1) + ar;
                    W2(ji) = W2(ji1) - ai;
                    W1(ji1) = W1(ji1) - ar;
                    W2(ji1) = W2(ji1) + ai;
                    ii++;
                    ji1 += isep4;
                    ji += isep4;
                }
            }
        }
    }
    if (isig == -1) {
        for (int i = 1; i <= m; i++) { int ii = ibitrv[i - 1]; X1(i) = W1(ii); X2(i) = W2(ii); }
    } else {
        for (int i = 1; i <= m; i++) { int ii = ibitrv[i - 1]; X1(i) = W1(ii); X2(i) = -W2(ii); }
    }
    if (isig == -1) {
        for (int i = 1; i <= m; i++) {
            X1(i) = X1(i) / (float)m;
            X2(i) = X2(i) / (float)m;
        }
    }
    free(C);
    free(S);
    free(ibitrv);
#undef X1
#undef X2
#undef W1
#undef W2
}

/* fft/fftx1d.f:57-92 (power-of-two branch) */
void orc_fftx1d(float *xarray, float *xwork, float *xwork2, int nx, int dir) {
    int icen = (nx + 1) / 2, ioff = nx - icen + 1;
    for (int ix = 1; ix <= icen - 1; ix++) {
        xwork2[2 * (ix + ioff - 1)] = xarray[2 * (ix - 1)];
        xwork2[2 * (ix + ioff - 1) + 1] = xarray[2 * (ix - 1) + 1];
    }
    ioff = -icen + 1;
    for (int ix = icen; ix <= nx; ix++) {
        xwork2[2 * (ix + ioff - 1)] = xarray[2 * (ix - 1)];
        xwork2[2 * (ix + ioff - 1) + 1] = xarray[2 * (ix - 1) + 1];
    }
    orc_fftx(xwork2, xwork, nx, dir);
    ioff = nx - icen + 1;
    for (int ix = 1; ix <= icen - 1; ix++) {
        xarray[2 * (ix - 1)] = xwork2[2 * (ix + ioff - 1)];
        xarray[2 * (ix - 1) + 1] = xwork2[2 * (ix + ioff - 1) + 1];
    }
    ioff = -icen + 1;
    for (int ix = icen; ix <= nx; ix++) {
        xarray[2 * (ix - 1)] = xwork2[2 * (ix + ioff - 1)];
        xarray[2 * (ix - 1) + 1] = xwork2[2 * (ix + ioff - 1) + 1];
    }
}

/* fft/fftr.f:80-176 (non-Cray branch): real FFT via a half-length complex FFT. */
void orc_fftr(float *R, float *C, float *work, int n, int f) {
#define RR(i) R[(i)-1]
#define CC(i) C[(i)-1]
    if (n <= 0) return;
    const float twopi = 6.2831852f;
    int h = n / 2, q = h / 2;
    float *tablr = (float *)malloc(sizeof(float) * (size_t)(q + 1));
    float *tabli = (float *)malloc(sizeof(float) * (size_t)(q + 1));
    float phas0 = -twopi / 4.0f, dphas = -twopi / (float)n;
    for (int loop = 1; loop <= q; loop++) {
        float phase = phas0 + (float)loop * dphas;
        tablr[loop] = cosf(phase);
        tabli[loop] = sinf(phase);
    }
    if (f >= 0) {
        for (int loop = 1; loop <= n; loop++) CC(loop) = RR(loop);
        orc_fftx(C, work, h, f);
        for (int loop = 1; loop <= q; loop++) {
            float sumr = CC(1 + 2 * loop) + CC(1 + 2 * (h - loop));
            float sumi = CC(2 + 2 * loop) - CC(2 + 2 * (h - loop));
            float diffr = CC(1 + 2 * loop) - CC(1 + 2 * (h - loop));
            float diffi = CC(2 + 2 * loop) + CC(2 + 2 * (h - loop));
            CC(1 + 2 * loop) = sumr + (tablr[loop] * diffr - tabli[loop] * diffi);
            CC(2 + 2 * loop) = sumi + (tabli[loop] * diffr + tablr[loop] * diffi);
            CC(1 + 2 * (h - loop)) = sumr - (tablr[loop] * diffr - tabli[loop] * diffi);
            CC(2 + 2 * (h - loop)) = -sumi + (tabli[loop] * diffr + tablr[loop] * diffi);
        }
        float tempr = 2.0f * (CC(1) + CC(2));
        CC(2) = 2.0f * (CC(1) - CC(2));
        CC(1) = tempr;
        for (int loop = 1; loop <= n; loop++) CC(loop) = 0.5f * CC(loop);
        CC(n + 1) = CC(2);
        CC(n + 2) = 0.0f;
        CC(2) = 0.0f;
    } else {
        for (int loop = 1; loop <= n; loop++) RR(loop) = CC(loop);
        RR(2) = CC(n + 1);
        RR(n + 1) = 0.0f;
        RR(n + 2) = 0.0f;
        for (int loop = 1; loop <= q; loop++) {
            float sumr = RR(1 + 2 * loop) + RR(1 + 2 * (h - loop));
            float sumi = RR(2 + 2 * loop) - RR(2 + 2 * (h - loop));
            float diffr = RR(1 + 2 * loop) - RR(1 + 2 * (h - loop));
            float diffi = RR(2 + 2 * loop) + RR(2 + 2 * (h - loop));
            RR(1 + 2 * loop) = sumr + (tablr[loop] * diffr + tabli[loop] * diffi);
            RR(2 + 2 * loop) = sumi - (tabli[loop] * diffr - tablr[loop] * diffi);
            RR(1 + 2 * (h - loop)) = sumr - (tablr[loop] * diffr + tabli[loop] * diffi);
            RR(2 + 2 * (h - loop)) = -sumi - (tabli[loop] * diffr - tablr[loop] * diffi);
        }
        float tempr = RR(1) + RR(2);
        RR(2) = RR(1) - RR(2);
        RR(1) = tempr;
        orc_fftx(R, work, h, f);
        for (int loop = 1; loop <= n; loop++) RR(loop) = 0.5f * RR(loop);
    }
    free(tablr);
    free(tabli);
#undef RR
#undef CC
}

/* fft/fftr1d.f:63-109 (power-of-two branch).  rwork needs nx+2 floats, xwork nx/2 complex. */
void orc_fftr1d(float *rarray, float *xarray, float *rwork, float *xwork, int nx, int dir) {
    int icen = (nx + 1) / 2;
    if (dir > 0) {
        int ioff = nx - icen + 1;
        for (int ix = 1; ix <= icen - 1; ix++) rwork[ix + ioff - 1] = rarray[ix - 1];
        ioff = -icen + 1;
        for (int ix = icen; ix <= nx; ix++) rwork[ix + ioff - 1] = rarray[ix - 1];
        orc_fftr(rwork, xarray, xwork, nx, dir);
    } else {
        orc_fftr(rwork, xarray, xwork, nx, dir);
        int ioff = nx - icen + 1;
        for (int ix = 1; ix <= icen - 1; ix++) rarray[ix - 1] = rwork[ix + ioff - 1];
        ioff = -icen + 1;
        for (int ix = icen; ix <= nx; ix++) rarray[ix - 1] = rwork[ix + ioff - 1];
    }
}

/* fft/fftr1d2.f:41-84 */
void orc_fftr1d2(float *rarray, float *xarray, float *xwork, float *xwork2, float *rwork,
                 int nx, int fnu, int dir) {
    if (dir > 0) {
        if (fnu > nx) {
            int ioff = (fnu - nx) / 2;
            for (int ix = 1; ix <= fnu; ix++) rwork[ix - 1] = 0.0f;
            for (int ix = 1; ix <= nx; ix++) rwork[ioff + ix - 1] = rarray[ix - 1];
        } else {
            for (int ix = 1; ix <= nx; ix++) rwork[ix - 1] = rarray[ix - 1];
        }
        orc_fftr1d(rwork, xarray, xwork, xwork2, fnu, dir);
    } else {
        orc_fftr1d(rwork, xarray, xwork, xwork2, fnu, dir);
        if (fnu == nx) {
            for (int ix = 1; ix <= nx; ix++) rarray[ix - 1] = rwork[ix - 1];
        } else {
            int ioff = (fnu - nx) / 2;
            for (int ix = 1; ix <= nx; ix++) rarray[ix - 1] = rwork[ioff + ix - 1];
        }
    }
}

/* fft/fftr2d.f:46-97.  rarray [ny][nx] real, xarray [nv][fnu/2+1] complex. */
void orc_fftr2d(float *rarray, float *xarray, int nx, int ny, int fnu, int nv, int dir) {
    int nu = fnu / 2 + 1, fny = nv;
    int ibegy = (fny + 1) / 2 - (ny + 1) / 2 + 1;
    int iendy = (fny + 1) / 2 + ny / 2;
    int maxn = (fnu > nv ? fnu : nv) + 8;
    float *work = (float *)calloc(2 * (size_t)maxn, sizeof(float));
    float *work2 = (float *)calloc(2 * (size_t)maxn, sizeof(float));
    float *rwork = (float *)calloc(2 * (size_t)maxn, sizeof(float));
#define XA(ix, iy) (xarray + 2 * (((size_t)(ix)-1) + (size_t)((iy)-1) * (size_t)nu))
    if (dir > 0) {
        for (int iy = 1; iy <= ibegy - 1; iy++)
            for (int ix = 1; ix <= nu; ix++) { XA(ix, iy)[0] = 0.0f; XA(ix, iy)[1] = 0.0f; }
        for (int iy = 1; iy <= ny; iy++)
            orc_fftr1d2(rarray + (size_t)(iy - 1) * nx, XA(1, iy + ibegy - 1), work, work2, rwork,
                        nx, fnu, dir);
        for (int iy = iendy + 1; iy <= fny; iy++)
            for (int ix = 1; ix <= nu; ix++) { XA(ix, iy)[0] = 0.0f; XA(ix, iy)[1] = 0.0f; }
        for (int ix = 1; ix <= nu; ix++) {
            for (int iy = 1; iy <= fny; iy++) { work2[2 * (iy - 1)] = XA(ix, iy)[0]; work2[2 * (iy - 1) + 1] = XA(ix, iy)[1]; }
            orc_fftx1d(work2, work, rwork, fny, dir);
            for (int iy = 1; iy <= fny; iy++) { XA(ix, iy)[0] = work2[2 * (iy - 1)]; XA(ix, iy)[1] = work2[2 * (iy - 1) + 1]; }
        }
    } else {
        for (int ix = 1; ix <= nu; ix++) {
            for (int iy = 1; iy <= fny; iy++) { work2[2 * (iy - 1)] = XA(ix, iy)[0]; work2[2 * (iy - 1) + 1] = XA(ix, iy)[1]; }
            orc_fftx1d(work2, work, rwork, fny, dir);
            for (int iy = 1; iy <= fny; iy++) { XA(ix, iy)[0] = work2[2 * (iy - 1)]; XA(ix, iy)[1] = work2[2 * (iy - 1) + 1]; }
        }
        for (int iy = 1; iy <= ny; iy++)
            orc_fftr1d2(rarray + (size_t)(iy - 1) * nx, XA(1, iy + ibegy - 1), work, work2, rwork,
                        nx, fnu, dir);
    }
#undef XA
    free(work);
    free(work2);
    free(rwork);
}

/* pix/pixcor2d.f:44-68 */
void orc_pixcor2d(const float *in, int nx, int ny, const float *cf, int cflen, int correct,
                  float *out, float cenx, float ceny) {
    int fnx = orc_fftpwr2(nx), fny = orc_fftpwr2(ny);
    float scalex = (float)(cflen - 1) * 2.0f / (float)fnx;
    float scaley = (float)(cflen - 1) * 2.0f / (float)fny;
    for (int iy = 1; iy <= ny; iy++) {
        int icfy = 1 + abs(orc_nint_f(scaley * ((float)iy - ceny)));
        for (int ix = 1; ix <= nx; ix++) {
            int icfx = 1 + abs(orc_nint_f(scalex * ((float)ix - cenx)));
            size_t k = (size_t)(ix - 1) + (size_t)(iy - 1) * nx;
            if (correct)
                out[k] = in[k] / (cf[icfx - 1] * cf[icfy - 1]);
            else
                out[k] = cf[icfx - 1] * cf[icfy - 1] * in[k];
        }
    }
}

/* pix/pixisama.f:45-53 -- first index of strictly greatest |A|, 1-based; I if none */
int orc_pixisama(int n, const float *a, int i) {
    int r = i;
    float maxval = 0.0f;
    for (int j = 1; j <= n; j++) {
        if (fabsf(a[j - 1]) > maxval) {
            maxval = fabsf(a[j - 1]);
            r = j;
        }
    }
    return r;
}

/* pix/pix2drcl.f:67-142 -- Hogbom CLEAN minor cycle.  A PSF read whose flat
 * column-major offset falls outside the PSF array reads 0 (the reference reads
 * whatever memory follows; no caller in the reference does that). */
void orc_pix2drcl(const float *drt, const float *psf, const float *box, int nx, int ny, int pnx,
                  int pny, float gain, int nsub, int bsub, float flux, float *cln, float *res,
                  int *ansub, float *maxres, float *tflux, float *cflux, int *cx, int *cy) {
    const size_t npix = (size_t)nx * ny, pnpix = (size_t)pnx * pny;
    for (size_t k = 0; k < npix; k++) res[k] = drt[k] * box[k];
    int ipeak = orc_pixisama(pnx * pny, psf, 1) - 1;
    int pmpx = 1 + ipeak % pnx;
    int pmpy = 1 + (ipeak - pmpx + 1) / pnx;
    if (pmpx >= pnx) pmpx = pnx / 2;
    if (pmpy >= pny) pmpy = pny / 2;
    int isub, pmx, pmy;
    float mres = 0.0f;
    int nabs = nsub < 0 ? -nsub : nsub;
    for (isub = bsub; isub <= nabs; isub++) {
        ipeak = orc_pixisama(nx * ny, res, 1) - 1;
        pmx = 1 + ipeak % nx;
        pmy = 1 + (ipeak - pmx + 1) / nx;
        mres = res[(size_t)(pmx - 1) + (size_t)(pmy - 1) * nx];
        if (nsub < 0 && mres < 0.0f) goto stopped;
        if (fabsf(mres) <= flux) goto stopped;
        float pntsub = gain * mres;
        *tflux = *tflux + pntsub;
        cln[(size_t)(pmx - 1) + (size_t)(pmy - 1) * nx] += pntsub;
        cflux[isub - 1] = pntsub;
        cx[isub - 1] = pmx;
        cy[isub - 1] = pmy;
        int offx = pmpx + pmx, offy = pmpy + pmy;
        for (int iy = 1; iy <= ny; iy++)
            for (int ix = 1; ix <= nx; ix++) {
                long long flat = (long long)(offx - ix - 1) + (long long)(offy - iy - 1) * pnx;
                float p = (flat >= 0 && (size_t)flat < pnpix) ? psf[flat] : 0.0f;
                size_t k = (size_t)(ix - 1) + (size_t)(iy - 1) * nx;
                res[k] = res[k] - (pntsub * p * box[k]);
            }
    }
    *ansub = nsub;
    ipeak = orc_pixisama(nx * ny, res, 1) - 1;
    pmx = 1 + ipeak % nx;
    pmy = 1 + (ipeak - pmx + 1) / nx;
    *maxres = res[(size_t)(pmx - 1) + (size_t)(pmy - 1) * nx];
    return;
stopped:
    *ansub = isub - 1;
    *maxres = mres;
}

/* pix/pixrscal.f: OUT(I) = SCALE * IN(I) + OFFSET */
void orc_pixrscal(const float *in, float scale, float offset, float *out, int64_t n) {
    for (int64_t i = 0; i < n; i++) out[i] = scale * in[i] + offset;
}

/* ---------------------------------------------------------------------------------------
 * Task-level drivers.
 * img/imgmake.f (CDELT = -/+ CELLSIZE/3600, CRPIX = (N+1)/2), fft/fftconja.f:159-163 and
 * fft/fftconj.f (FNU = pow2(N), NU = FNU/2+1, CDELT = 1/(D2R*WIDTH), RPIX = 1, (NV+1)/2),
 * vis/visgrid.f:148-153 (USCALE = 1/CDELT, UORIGIN = NINT(RPIX)). */
void orc_make_geom(const orc_uvmap_params *p, orc_geom *g) {
    const float PI = 3.141592654f;
    const float D2R = PI / 180.0f;
    int n = p->imsize;
    float delt_ra = -p->cellsize / 3600.0f, delt_dec = p->cellsize / 3600.0f;
    g->nx = n;
    g->ny = n;
    g->fnu = orc_fftpwr2(n);
    g->nu = g->fnu / 2 + 1;
    g->nv = orc_fftpwr2(n);
    float width_u = (float)orc_fftpwr2(n) * delt_ra;
    float width_v = (float)orc_fftpwr2(n) * delt_dec;
    float cdelt_u = 1.0f / (D2R * width_u);
    float cdelt_v = 1.0f / (D2R * width_v);
    g->uscale = 1.0f / cdelt_u;
    g->vscale = 1.0f / cdelt_v;
    g->uorigin = 1;
    g->vorigin = orc_nint_f((float)((g->nv + 1) / 2));
    g->cenx = (float)((n + 1) / 2);
    g->ceny = (float)((n + 1) / 2);
    double ira = p->vra + (double)(p->shift_ra / 3600.0f);
    double idec = p->vdec + (double)(p->shift_dec / 3600.0f);
    orc_crdshift(p->vra, p->vdec, ira, idec, 0.0f, g->shift);
}

static void image_from_grid(const orc_geom *g, float *grid, float *image, const float *ccf,
                            int ccflen) {
    orc_fftr2d(image, grid, g->nx, g->ny, g->fnu, g->nv, -1);
    orc_pixcor2d(image, g->nx, g->ny, ccf, ccflen, 1, image, g->cenx, g->ceny);
}

/* task/uvmap.f:212-314 (weighting), 414-491 (PSF + dirty, PSF-peak normalisation). */
int orc_uvmap(const orc_uvmap_params *p, int nvis, const float *u, const float *v,
              const float *w, const float *vis, float *wt, float *dirty, float *psf,
              float *maxpsf_out, float *sumwt_psf) {
    orc_geom g;
    orc_make_geom(p, &g);
    size_t ncell = (size_t)g.nu * g.nv;
    float *grid = (float *)malloc(2 * ncell * sizeof(float));
    int rc = ORC_OK;
    if (p->fov != 0.0f) {
        /* CDELT of the XFR axes is 1/uscale; GRDUWT/GRDRUWT use WTFOV/CDELT (grd/grduwt.f:115). */
        float cdelt_u = 1.0f / g.uscale, cdelt_v = 1.0f / g.vscale;
        float us = p->fov / cdelt_u, vs = p->fov / cdelt_v;
        if (p->rmode == 0) {
            orc_grduwt2d(wt, u, v, w, nvis, us, 0.0f, vs, 0.0f, g.uorigin, g.vorigin, wt, grid,
                         g.nu, g.nv, g.shift, NULL);
        } else {
            static const char *modes[] = {"NONE", "NORM", "ABS", "AZ-NORM"};
            rc = orc_grdruw2d(wt, u, v, w, nvis, us, 0.0f, vs, 0.0f, g.uorigin, g.vorigin, wt,
                              grid, g.nu, g.nv, g.shift, modes[p->rmode], p->robust, p->ds, NULL,
                              NULL, NULL, NULL);
            if (rc) goto done;
        }
    }
    float cf[1 + 8 * 129];
    int supp, osamp;
    orc_grdcf(1, cf, &supp, &osamp);
    int ccflen = 1 + orc_fftpwr2(g.nx > g.ny ? g.nx : g.ny) / 2;
    float *ccf = (float *)malloc(sizeof(float) * (size_t)ccflen);
    orc_grdccf(1, ccf, ccflen);
    float sumwt;
    rc = orc_grdh2d(vis, wt, u, v, w, nvis, g.uscale, 0.0f, g.vscale, 0.0f, g.uorigin, g.vorigin,
                    grid, 1, g.nu, g.nv, cf, supp, osamp, cf, supp, osamp, g.shift, &sumwt, NULL);
    if (rc) { free(ccf); goto done; }
    if (sumwt_psf) *sumwt_psf = sumwt;
    image_from_grid(&g, grid, psf, ccf, ccflen);
    size_t npix = (size_t)g.nx * g.ny;
    float maxpsf = psf[0];
    for (size_t k = 1; k < npix; k++)
        if (psf[k] > maxpsf) maxpsf = psf[k];
    if (maxpsf_out) *maxpsf_out = maxpsf;
    if (maxpsf == 0.0f) { rc = ORC_EBADARG; free(ccf); goto done; }
    orc_pixrscal(psf, 1.0f / maxpsf, 0.0f, psf, (int64_t)npix);
    rc = orc_grdh2d(vis, wt, u, v, w, nvis, g.uscale, 0.0f, g.vscale, 0.0f, g.uorigin, g.vorigin,
                    grid, 0, g.nu, g.nv, cf, supp, osamp, cf, supp, osamp, g.shift, &sumwt, NULL);
    if (rc) { free(ccf); goto done; }
    image_from_grid(&g, grid, dirty, ccf, ccflen);
    orc_pixrscal(dirty, 1.0f / maxpsf, 0.0f, dirty, (int64_t)npix);
    free(ccf);
done:
    free(grid);
    return rc;
}

/* task/vismodel.f:70-73: IMGGRIDC(CORRECT) -> IMGFFT (r2c, DIR +1) -> VISDEGRI. */
int orc_vismodel(const orc_uvmap_params *p, int nvis, const float *u, const float *v,
                 const float *w, float *vis, float *wt, const float *image) {
    orc_geom g;
    orc_make_geom(p, &g);
    size_t npix = (size_t)g.nx * g.ny;
    float *img = (float *)malloc(npix * sizeof(float));
    float *grid = (float *)malloc(2 * (size_t)g.nu * g.nv * sizeof(float));
    int ccflen = 1 + orc_fftpwr2(g.nx > g.ny ? g.nx : g.ny) / 2;
    float *ccf = (float *)malloc(sizeof(float) * (size_t)ccflen);
    orc_grdccf(1, ccf, ccflen);
    orc_pixcor2d(image, g.nx, g.ny, ccf, ccflen, 1, img, g.cenx, g.ceny);
    orc_fftr2d(img, grid, g.nx, g.ny, g.fnu, g.nv, +1);
    float cf[1 + 8 * 129];
    int supp, osamp;
    orc_grdcf(1, cf, &supp, &osamp);
    orc_grddeh2d(vis, wt, u, v, w, nvis, g.uscale, 0.0f, g.vscale, 0.0f, g.uorigin, g.vorigin,
                 grid, g.nu, g.nv, cf, supp, osamp, cf, supp, osamp, g.shift, NULL);
    free(img);
    free(grid);
    free(ccf);
    return ORC_OK;
}

/* ---------------------------------------------------------------------------------------
 * FP64 oracle: the gridder, inverse FFT and grid correction of the same algorithm carried
 * in double precision (convolution-function table kept at its REAL values, since it is
 * part of the algorithm's definition).  Used to state every result's error vs FP64. */
int orc64_grdh2d(const float *vis, const float *wt, const float *u, const float *v,
                 const float *w, int nvis, const orc_geom *g, int psf, double *gvis) {
    float cf[1 + 8 * 129];
    int supp, osamp;
    orc_grdcf(1, cf, &supp, &osamp);
    const double *shift = g->shift;
    const int nu = g->nu, nv = g->nv;
    const double twopi = 2.0 * M_PI;
    const int cfoffset = (supp + 1) * osamp + 1;
    const int doshift = doshift_of(shift);
    memset(gvis, 0, 2 * (size_t)nu * nv * sizeof(double));
    double lsumwt = 0.0;
#define GRE(uu, vv) gvis[2 * (((size_t)(uu)-1) + (size_t)((vv)-1) * (size_t)nu)]
#define GIM(uu, vv) gvis[2 * (((size_t)(uu)-1) + (size_t)((vv)-1) * (size_t)nu) + 1]
    for (int i = 0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        double ug = u[i], vg = v[i], wg = w[i], ucell, vcell, fr, fi;
        if (doshift) {
            double ul = SH(1, 1) * ug + SH(2, 1) * vg + SH(3, 1) * wg;
            double vl = SH(1, 2) * ug + SH(2, 2) * vg + SH(3, 2) * wg;
            double wl = SH(1, 3) * ug + SH(2, 3) * vg + SH(3, 3) * wg;
            double ph = twopi * (wl - wg), c = cos(ph), s = -sin(ph);
            double a = vis[2 * i], b = vis[2 * i + 1];
            fr = a * c - b * s;
            fi = a * s + b * c;
            ucell = (double)g->uscale * ul;
            vcell = (double)g->vscale * vl;
        } else {
            fr = vis[2 * i];
            fi = vis[2 * i + 1];
            ucell = (double)g->uscale * ug;
            vcell = (double)g->vscale * vg;
        }
        if (ucell > 0.0) {
            fi = -fi;
            ucell += g->uorigin;
            vcell += g->vorigin;
        } else {
            ucell = -ucell + g->uorigin;
            vcell = -vcell + g->vorigin;
        }
        if (psf) { fr = 1.0; fi = 0.0; }
        int nuc = orc_nint_d(ucell), nvc = orc_nint_d(vcell);
        if (nuc + 2 * supp > nu || nvc + supp > nv || nvc - supp < 1) continue;
        int delui = orc_nint_d((double)osamp * ((double)nuc - ucell)) + cfoffset;
        int delvi = orc_nint_d((double)osamp * ((double)nvc - vcell)) + cfoffset;
        for (int offv = -supp; offv <= supp; offv++)
            for (int offu = -supp; offu <= supp; offu++) {
                double uvwt = (double)wt[i] * (double)cf[delui + osamp * offu - 1] *
                              (double)cf[delvi + osamp * offv - 1];
                GRE(nuc + supp + offu, nvc + offv) += uvwt * fr;
                GIM(nuc + supp + offu, nvc + offv) += uvwt * fi;
                lsumwt += uvwt;
            }
    }
    if (lsumwt == 0.0) return ORC_ENOWEIGHT;
    int ucen = g->uorigin + supp, vcen = g->vorigin;
    for (int offv = -nv / 2 + 1; offv <= nv / 2 - 1; offv++)
        for (int offu = 1; offu <= supp; offu++) {
            GRE(ucen + offu, vcen + offv) += GRE(ucen - offu, vcen - offv);
            GIM(ucen + offu, vcen + offv) -= GIM(ucen - offu, vcen - offv);
        }
    for (int offv = 0; offv <= nv / 2 - 1; offv++) {
        GRE(ucen, vcen + offv) += GRE(ucen, vcen - offv);
        GIM(ucen, vcen + offv) -= GIM(ucen, vcen - offv);
        GRE(ucen, vcen - offv) = GRE(ucen, vcen + offv);
        GIM(ucen, vcen - offv) = -GIM(ucen, vcen + offv);
    }
    double scale = (double)(nu - 1) * (double)nv / lsumwt;
    for (int vg = 1; vg <= nv; vg++) {
        for (int ug = 1; ug <= nu - supp; ug++) {
            GRE(ug, vg) = scale * GRE(ug + supp, vg);
            GIM(ug, vg) = scale * GIM(ug + supp, vg);
        }
        for (int ug = nu - supp + 1; ug <= nu; ug++) { GRE(ug, vg) = 0.0; GIM(ug, vg) = 0.0; }
    }
#undef GRE
#undef GIM
    return ORC_OK;
}

/* in-place radix-2 complex FFT in double, x[k] <- sum_j x[j] exp(sgn*2*pi*i*j*k/n) */
static void fft64(double *x, int n, int sgn) {
    for (int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double t0 = x[2 * i], t1 = x[2 * i + 1];
            x[2 * i] = x[2 * j]; x[2 * i + 1] = x[2 * j + 1];
            x[2 * j] = t0; x[2 * j + 1] = t1;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        double ang = sgn * 2.0 * M_PI / len;
        for (int i = 0; i < n; i += len)
            for (int k = 0; k < len / 2; k++) {
                double wr = cos(ang * k), wi = sin(ang * k);
                double *a = x + 2 * (i + k), *b = x + 2 * (i + k + len / 2);
                double tr = b[0] * wr - b[1] * wi, ti = b[0] * wi + b[1] * wr;
                b[0] = a[0] - tr; b[1] = a[1] - ti;
                a[0] += tr; a[1] += ti;
            }
    }
}

/* Inverse (DIR = -1) transform of fft/fftr2d.f in double.  The reference's FFTX with
 * ISIG = -1 computes sum_j x_j exp(+2 pi i jk/M)/M, FFTX1D/FFTR1D shift the centre by
 * (N+1)/2-1 on both sides, and FFTR's c2r (FFTX of length N/2 then x0.5) gives
 * r_n = (1/N) sum over the Hermitian extension of C_k exp(+2 pi i kn/N), reading only the
 * real parts of C_1 and C_{N/2+1}. */
void orc64_fftr2d_inv(const double *xarray, double *image, int nx, int ny, int fnu, int nv) {
    int nu = fnu / 2 + 1;
    double *col = (double *)malloc(2 * (size_t)nv * sizeof(double));
    double *xt = (double *)malloc(2 * (size_t)nu * nv * sizeof(double));
    int icv = (nv + 1) / 2, cv = icv - 1;
    for (int ix = 0; ix < nu; ix++) {
        for (int j = 0; j < nv; j++) { /* packed: xw[j] = x[(j + cv) mod nv] */
            int src = (j + cv) % nv;
            col[2 * j] = xarray[2 * ((size_t)src * nu + ix)];
            col[2 * j + 1] = xarray[2 * ((size_t)src * nu + ix) + 1];
        }
        fft64(col, nv, +1);
        for (int j = 0; j < nv; j++) {
            int dst = (j + cv) % nv;
            xt[2 * ((size_t)dst * nu + ix)] = col[2 * j] / nv;
            xt[2 * ((size_t)dst * nu + ix) + 1] = col[2 * j + 1] / nv;
        }
    }
    free(col);
    double *row = (double *)malloc(2 * (size_t)fnu * sizeof(double));
    int icu = (fnu + 1) / 2, cu = icu - 1;
    int ibegy = (nv + 1) / 2 - (ny + 1) / 2 + 1;
    for (int iy = 0; iy < ny; iy++) {
        const double *xr = xt + 2 * (size_t)(iy + ibegy - 1) * nu;
        for (int k = 0; k < fnu; k++) {
            double re, im;
            if (k == 0) { re = xr[0]; im = 0.0; }
            else if (k == fnu / 2) { re = xr[2 * k]; im = 0.0; }
            else if (k < fnu / 2) { re = xr[2 * k]; im = xr[2 * k + 1]; }
            else { re = xr[2 * (fnu - k)]; im = -xr[2 * (fnu - k) + 1]; }
            row[2 * k] = re;
            row[2 * k + 1] = im;
        }
        fft64(row, fnu, +1);
        int ioff = (fnu - nx) / 2;
        for (int ix = 0; ix < nx; ix++) {
            int n = ((ix + ioff) - cu + fnu) % fnu; /* rarray(ix) = r[(ix - cu) mod fnu] */
            image[(size_t)iy * nx + ix] = row[2 * n] / fnu;
        }
    }
    free(row);
    free(xt);
}

void orc64_uvmap_image(const orc_geom *g, int nvis, const float *u, const float *v,
                       const float *w, const float *vis, const float *wt, int psf,
                       double *image) {
    double *grid = (double *)malloc(2 * (size_t)g->nu * g->nv * sizeof(double));
    if (orc64_grdh2d(vis, wt, u, v, w, nvis, g, psf, grid) != ORC_OK) {
        memset(image, 0, sizeof(double) * (size_t)g->nx * g->ny);
        free(grid);
        return;
    }
    orc64_fftr2d_inv(grid, image, g->nx, g->ny, g->fnu, g->nv);
    free(grid);
    int ccflen = 1 + orc_fftpwr2(g->nx > g->ny ? g->nx : g->ny) / 2;
    int fnx = orc_fftpwr2(g->nx), fny = orc_fftpwr2(g->ny);
    double sx = (double)(ccflen - 1) * 2.0 / fnx, sy = (double)(ccflen - 1) * 2.0 / fny;
    for (int iy = 1; iy <= g->ny; iy++) {
        int icy = 1 + abs(orc_nint_d(sy * (iy - g->ceny)));
        double cy = orc_grdsf((double)(icy - 1) / (double)(ccflen - 1));
        for (int ix = 1; ix <= g->nx; ix++) {
            int icx = 1 + abs(orc_nint_d(sx * (ix - g->cenx)));
            double cx = orc_grdsf((double)(icx - 1) / (double)(ccflen - 1));
            image[(size_t)(iy - 1) * g->nx + (ix - 1)] /= (cx * cy);
        }
    }
}

/* Direct Fourier sum of the weighted visibilities onto the image pixels (the idea of the
 * reference's VISDFT, vis/visdft.f), with the same sign and centre conventions as the
 * gridded path: I(ix,iy) = sum_k wt_k Re{V_k exp(2 pi i (u_k l + v_k m))}, l = (ix-cenx)*dl.
 * Sign of l follows CDELT(RA) < 0.  Normalised so that the PSF peak is 1 (psf=1). */
void orc64_dft_image(const orc_geom *g, int nvis, const float *u, const float *v,
                     const float *vis, const float *wt, int psf, double *image) {
    double dl = -1.0 / ((double)g->uscale * g->fnu);
    double dm = -1.0 / ((double)g->vscale * g->nv);
    double wsum = 0.0;
    for (int k = 0; k < nvis; k++)
        if (wt[k] > 0.0f) wsum += wt[k];
    for (int iy = 1; iy <= g->ny; iy++) {
        double m = (iy - g->ceny) * dm;
        for (int ix = 1; ix <= g->nx; ix++) {
            double l = (ix - g->cenx) * dl, s = 0.0;
            for (int k = 0; k < nvis; k++) {
                if (wt[k] <= 0.0f) continue;
                double ph = 2.0 * M_PI * ((double)u[k] * l + (double)v[k] * m);
                double vr = psf ? 1.0 : vis[2 * k], vi = psf ? 0.0 : vis[2 * k + 1];
                s += wt[k] * (vr * cos(ph) - vi * sin(ph));
            }
            image[(size_t)(iy - 1) * g->nx + (ix - 1)] = s / wsum;
        }
    }
}

/* ---------------------------------------------------------------------------------------
 * Clark CLEAN: the CLARK branch of task/clean.f:147-205 (CRDHALF window, IMGMAKEX,
 * IMGSUBPS) and IMGCCLEA's major/minor cycle loop (img/imgcclea.f:210-290).
 */

/* crd/crdhalf.f:21-41 with the task's BLC = TRC unset: the inner half of an axis */
static void orc_crdhalf_axis(int n, int *blc, int *trc) {
    int b = 1, t = 1;
    if (n > 1) {
        b = n / 4 + 1;
        t = 3 * n / 4;
        int idel = t - b + 1 < n / 2 ? t - b + 1 : n / 2;
        t = b + idel - 1;
    }
    *blc = b;
    *trc = t;
}

/* pix/pixrabsh.f:18-40.  INDEX = NINT((|A|-BASE)/INCR) is 0 for values near the minimum;
 * the reference then writes HIST(0), outside HIST(1..NB): those values are in no bin. */
static int orc_pixrabsh(const float *a, int64_t n, int nb, int *hist, float *base, float *incr) {
    float amax = fabsf(a[0]), amin = amax;
    for (int64_t i = 0; i < n; i++) {
        float x = fabsf(a[i]);
        amax = amax > x ? amax : x;
        amin = amin < x ? amin : x;
    }
    if (amax == amin) return -1; /* 'Zero range in values' */
    for (int i = 0; i < nb; i++) hist[i] = 0;
    *base = amin;
    *incr = (amax - amin) / (float)(nb - 1);
    for (int64_t i = 0; i < n; i++) {
        int index = orc_nint_f((fabsf(a[i]) - *base) / *incr);
        if (index >= 1 && index <= nb) hist[index - 1]++;
    }
    return 0;
}

/* pix/pixflim.f:16-30; -2 = 'Too many points' */
static int orc_pixflim(const int *hist, int nb, int nl, int *slim) {
    int ntotal = 0;
    *slim = 1;
    for (int i = nb; i >= 1; i--) {
        ntotal += hist[i - 1];
        if (ntotal >= nl) {
            *slim = i + 1;
            break;
        }
    }
    return *slim > nb ? -2 : 0;
}

/* pix/pix2drli.f:17-31: pixels with |A| > SLIM in storage order, at most NL */
static int orc_pix2drli(const float *a, int nx, int ny, float slim, float *al, int *xl, int *yl, int nl) {
    int anl = 0;
    for (int iy = 1; iy <= ny; iy++)
        for (int ix = 1; ix <= nx; ix++) {
            float v = a[(size_t)(iy - 1) * nx + (ix - 1)];
            if (fabsf(v) > slim) {
                al[anl] = v;
                xl[anl] = ix;
                yl[anl] = iy;
                anl++;
                if (anl >= nl) return anl;
            }
        }
    return anl;
}

/* pix/pix2drcc.f:66-140 with SPEED = 1 and GSUB = BSUB (IMGCCLEA's call); cl/cx/cy are
 * 1-based component lists (index ISUB - 1).  Returns ANSUB. */
static int orc_pix2drcc(float *drtl, const int *xl, const int *yl, int nl, const float *psf, int pnx,
                        int pny, float gain, int nsub, int bsub, float flux, float slim, float *cl,
                        int *cx, int *cy, float *maxres, float *tflux) {
    int ipeak = orc_pixisama(pnx * pny, psf, 1) - 1;
    int pmpx = 1 + ipeak % pnx;
    int pmpy = 1 + (ipeak - pmpx + 1) / pnx;
    float smn = 0.0f;
    int isub;
    for (isub = bsub; isub <= abs(nsub); isub++) {
        smn = smn + 1.0f / (float)isub; /* FLOAT(ISUB)**SPEED with SPEED = 1.0 */
        int ip = orc_pixisama(nl, drtl, 1);
        int pmx = xl[ip - 1], pmy = yl[ip - 1];
        *maxres = drtl[ip - 1];
        if (flux < 0.0f && *maxres < 0.0f) return isub - 1;
        if (nsub < 0 && *maxres < 0.0f) return isub - 1;
        float lim = slim * smn;
        if (fabsf(flux) > lim) lim = fabsf(flux);
        if (fabsf(*maxres) <= lim) return isub - 1;
        float pntsub = gain * *maxres;
        *tflux = *tflux + pntsub;
        cl[isub - 1] = pntsub;
        cx[isub - 1] = pmx;
        cy[isub - 1] = pmy;
        int offx = pmpx + pmx, offy = pmpy + pmy;
        for (int i = 0; i < nl; i++) {
            int px = offx - xl[i], py = offy - yl[i];
            if (px >= 1 && px <= pnx && py >= 1 && py <= pny)
                drtl[i] = drtl[i] - pntsub * psf[(size_t)(py - 1) * pnx + (px - 1)];
        }
    }
    int ip = orc_pixisama(nl, drtl, 1);
    *maxres = drtl[ip - 1];
    return nsub;
}

/* img/imgresid.f:13-16: RES = DRT - IMGFFT(IMGFFT(MODEL) * XFR) on the transfer
 * function's grid (fnu x nv), PIXXMULT's complex product in REAL */
static void orc_imgresid(const float *model, const float *drt, const float *xfr, float *res, int nx,
                         int ny, int fnu, int nv, float *mvis) {
    const size_t nxf = (size_t)(fnu / 2 + 1) * nv;
    orc_fftr2d((float *)model, mvis, nx, ny, fnu, nv, +1);
    for (size_t k = 0; k < nxf; k++) {
        float a = mvis[2 * k], b = mvis[2 * k + 1], c = xfr[2 * k], d = xfr[2 * k + 1];
        mvis[2 * k] = a * c - b * d;
        mvis[2 * k + 1] = a * d + b * c;
    }
    orc_fftr2d(res, mvis, nx, ny, fnu, nv, -1);
    for (size_t k = 0; k < (size_t)nx * ny; k++) res[k] = drt[k] - res[k];
}

int orc_clark(const float *dirty, const float *psf, int n, const float *box, const orc_clark_params *p,
              float *comp, float *resid, float *cl, int *cx, int *cy, orc_clark_result *r) {
    memset(r, 0, sizeof *r);
    if (n < 4 || (n & (n - 1)) || p->niter <= 0 || p->numcl <= 0 || p->bpatch <= 0) return -10;
    /* window (task/clean.f:146-157) */
    int blc, trc;
    orc_crdhalf_axis(n, &blc, &trc);
    const int w = trc - blc + 1;
    const size_t nw = (size_t)w * w;
    float *drt = (float *)malloc(sizeof(float) * nw);
    for (int y = 0; y < w; y++)
        for (int x = 0; x < w; x++) drt[(size_t)y * w + x] = dirty[(size_t)(y + blc - 1) * n + (x + blc - 1)];
    /* XFR (img/imgmakex.f: IMGFFT, then ARRPHASE by ((N+1)/2 - CRPIX)/N = 0 for CRPIX = (N+1)/2) */
    const int fnu = n, nv = n, nu = n / 2 + 1;
    float *xfr = (float *)malloc(sizeof(float) * 2 * (size_t)nu * nv);
    float *mvis = (float *)malloc(sizeof(float) * 2 * (size_t)nu * nv);
    orc_fftr2d((float *)psf, xfr, n, n, fnu, nv, +1);
    /* beam patch and exterior sidelobe (img/imgsubps.f:28-33, pix/pixrexts.f) */
    const int rp = (n + 1) / 2, bp = p->bpatch;
    int pb0 = rp - bp / 2 + 1, pb1 = rp + bp / 2;
    if (pb0 < 1) pb0 = 1;
    if (pb1 > n) pb1 = n;
    const int pw = pb1 - pb0 + 1;
    float *spsf = (float *)malloc(sizeof(float) * (size_t)pw * pw);
    float ext = 0.0f;
    for (int y = 1; y <= n; y++)
        for (int x = 1; x <= n; x++) {
            float v = psf[(size_t)(y - 1) * n + (x - 1)];
            if (x >= pb0 && x <= pb1 && y >= pb0 && y <= pb1)
                spsf[(size_t)(y - pb0) * pw + (x - pb0)] = v;
            else if (fabsf(v) > ext)
                ext = fabsf(v);
        }
    r->extside = ext;
    /* lists */
    const int nl = p->numcl, nb = 1024;
    float *al = (float *)malloc(sizeof(float) * nl);
    int *xl = (int *)malloc(sizeof(int) * nl), *yl = (int *)malloc(sizeof(int) * nl);
    int *hist = (int *)malloc(sizeof(int) * nb);
    int rc = 0, riter = 1, aniter = 0;
    float maxres = 0.0f, tflux = 0.0f;
    orc_imgresid(comp, drt, xfr, resid, w, w, fnu, nv, mvis);
    for (;;) {
        if (box)
            for (size_t k = 0; k < nw; k++) resid[k] = resid[k] * box[k];
        float amax = resid[0], amin = resid[0];
        for (size_t k = 0; k < nw; k++) {
            if (resid[k] > amax) amax = resid[k];
            if (resid[k] < amin) amin = resid[k];
        }
        maxres = fabsf(amax) > fabsf(amin) ? fabsf(amax) : fabsf(amin);
        float base, incr;
        int slimi;
        if ((rc = orc_pixrabsh(resid, (int64_t)nw, nb, hist, &base, &incr)) != 0) break;
        if ((rc = orc_pixflim(hist, nb, nl, &slimi)) != 0) break;
        float slim = incr * (float)(slimi - 1) + base + 0.5f * incr;
        if (slim < 0.0f) {
            rc = -3; /* 'Limit in absolute value < 0.0' */
            break;
        }
        float es = fabsf(ext * maxres);
        slim = slim > es ? slim : es;
        int anl = orc_pix2drli(resid, w, w, slim, al, xl, yl, nl);
        r->last_anl = anl;
        r->last_slim = slim;
        if (anl == 0) {
            /* PIX2DRCC would read DRTL(1), never written: stop with nothing subtracted */
            aniter = riter - 1;
            break;
        }
        aniter = orc_pix2drcc(al, xl, yl, anl, spsf, pw, pw, p->gain, p->niter, riter, p->flux, slim, cl, cx, cy,
                              &maxres, &tflux);
        /* pix/pix2drma.f:17-21 */
        for (int i = riter; i <= aniter; i++) {
            int ix = cx[i - 1], iy = cy[i - 1];
            if (ix >= 1 && ix <= w && iy >= 1 && iy <= w)
                comp[(size_t)(iy - 1) * w + (ix - 1)] = comp[(size_t)(iy - 1) * w + (ix - 1)] + cl[i - 1];
        }
        riter = aniter + 1;
        orc_imgresid(comp, drt, xfr, resid, w, w, fnu, nv, mvis);
        if (r->ncycles < ORC_CLARK_TRACE) {
            r->t_anl[r->ncycles] = anl;
            r->t_aniter[r->ncycles] = aniter;
            r->t_maxres[r->ncycles] = maxres;
            r->t_tflux[r->ncycles] = tflux;
        }
        r->ncycles++;
        if (maxres <= 0.0f && p->flux <= 0.0f) break;
        if (!(fabsf(maxres) > p->flux && aniter < abs(p->niter))) break;
    }
    r->aniter = aniter;
    r->maxres = maxres;
    r->tflux = tflux;
    r->window = w;
    r->blc = blc;
    free(drt);
    free(xfr);
    free(mvis);
    free(spsf);
    free(al);
    free(xl);
    free(yl);
    free(hist);
    return rc;
}

/* ---------------------------------------------------------------------------------------
 * Direct Fourier transforms of uvmap's and vismodel's DFT options.
 */

/* vis/visdft3d.f:24-77 for a 2-D image (NZ = 1, REFZ = 1): dirty and PSF by the reference's
 * FP32 rotation recurrence (CFACTXYZ *= CROTX along x, CFACTYZ *= CROTY along y).
 * refx/refy 1-based reference pixel, deltx/delty in degrees.  Returns -1 ('No valid data'). */
int orc_visdft2d(const float *vis, int nvis, const float *wt, const float *u, const float *v, float *image,
                 float *psf, int nx, int ny, float refx, float deltx, float refy, float delty) {
    const float cf = 2.0f * (4.0f * atanf(1.0f)) * (4.0f * atanf(1.0f)) / 180.0f;
    for (size_t k = 0; k < (size_t)nx * ny; k++) image[k] = psf[k] = 0.0f;
    float rnorm = 0.0f;
    for (int i = 0; i < nvis; i++)
        if (wt[i] > 0.0f) rnorm = rnorm + wt[i];
    if (!(rnorm > 0.0f)) return -1;
    rnorm = 1.0f / rnorm;
    for (int i = 0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        /* the z term vanishes: W * DELTZ * (1 - REFZ) with REFZ = 1 */
        float phase = cf * (u[i] * deltx * (1.0f - refx) + v[i] * delty * (1.0f - refy));
        float fr = rnorm * wt[i] * cosf(phase), fi = rnorm * wt[i] * -sinf(phase);
        phase = cf * u[i] * deltx;
        const float rxr = cosf(phase), rxi = -sinf(phase);
        phase = cf * v[i] * delty;
        const float ryr = cosf(phase), ryi = -sinf(phase);
        const float vr = vis[2 * i], vi = vis[2 * i + 1];
        for (int iy = 0; iy < ny; iy++) {
            float xr = fr, xi = fi;
            for (int ix = 0; ix < nx; ix++) {
                const size_t o = (size_t)iy * nx + ix;
                image[o] = image[o] + (vr * xr - vi * xi);
                psf[o] = psf[o] + xr;
                const float tr = xr * rxr - xi * rxi, ti = xr * rxi + xi * rxr;
                xr = tr;
                xi = ti;
            }
            const float tr = fr * ryr - fi * ryi, ti = fr * ryi + fi * ryr;
            fr = tr;
            fi = ti;
        }
    }
    return 0;
}

/* img/imgdft2d.f:21-42: model image -> visibilities by the same recurrence (sign +);
 * points with WT <= 0 keep their VIS */
void orc_imgdft2d(const float *image, int nx, int ny, float refx, float deltx, float refy, float delty,
                  float *vis, int nvis, const float *wt, const float *u, const float *v) {
    const float cf = (8.0f * atanf(1.0f)) * (8.0f * atanf(1.0f)) / 360.0f;
    for (int i = 0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        float sr = 0.0f, si = 0.0f;
        float phase = cf * (u[i] * deltx * (1.0f - refx) + v[i] * delty * (1.0f - refy));
        float fr = cosf(phase), fi = sinf(phase);
        phase = cf * u[i] * deltx;
        const float rxr = cosf(phase), rxi = sinf(phase);
        phase = cf * v[i] * delty;
        const float ryr = cosf(phase), ryi = sinf(phase);
        for (int iy = 0; iy < ny; iy++) {
            float xr = fr, xi = fi;
            for (int ix = 0; ix < nx; ix++) {
                const float a = image[(size_t)iy * nx + ix];
                sr = sr + a * xr;
                si = si + a * xi;
                const float tr = xr * rxr - xi * rxi, ti = xr * rxi + xi * rxr;
                xr = tr;
                xi = ti;
            }
            const float tr = fr * ryr - fi * ryi, ti = fr * ryi + fi * ryr;
            fr = tr;
            fi = ti;
        }
        vis[2 * i] = sr;
        vis[2 * i + 1] = si;
    }
}

/* the same two transforms in FP64 with exact phases (the accuracy reference) */
int orc64_visdft2d(const float *vis, int nvis, const float *wt, const float *u, const float *v, double *image,
                   double *psf, int nx, int ny, double refx, double deltx, double refy, double delty) {
    const double d2r = M_PI / 180.0;
    double rn = 0.0;
    for (int i = 0; i < nvis; i++)
        if (wt[i] > 0.0f) rn += wt[i];
    if (!(rn > 0.0)) return -1;
    for (size_t k = 0; k < (size_t)nx * ny; k++) image[k] = psf[k] = 0.0;
    for (int i = 0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        const double c = wt[i] / rn;
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++) {
                const double ph = -2.0 * M_PI * d2r * ((double)u[i] * deltx * (ix + 1 - refx) +
                                                       (double)v[i] * delty * (iy + 1 - refy));
                const size_t o = (size_t)iy * nx + ix;
                image[o] += c * ((double)vis[2 * i] * cos(ph) - (double)vis[2 * i + 1] * sin(ph));
                psf[o] += c * cos(ph);
            }
    }
    return 0;
}

void orc64_imgdft2d(const float *image, int nx, int ny, double refx, double deltx, double refy, double delty,
                    double *vis, int nvis, const float *wt, const float *u, const float *v) {
    const double d2r = M_PI / 180.0;
    for (int i = 0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        double sr = 0.0, si = 0.0;
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++) {
                const double a = image[(size_t)iy * nx + ix];
                if (a == 0.0) continue;
                const double ph = 2.0 * M_PI * d2r * ((double)u[i] * deltx * (ix + 1 - refx) +
                                                      (double)v[i] * delty * (iy + 1 - refy));
                sr += a * cos(ph);
                si += a * sin(ph);
            }
        vis[2 * i] = sr;
        vis[2 * i + 1] = si;
    }
}

/* mod/modimg2d.f:29-232: components added into an image.  type: 0 POIN, 1 GAUS, 2 DISK,
 * 3 RECT, 4 SPHE, 5 SHEL, 6 PLOR; ra/dec offsets and deltx/delty in arcsec (MODIMG passes
 * 3600 * CDELT).  Returns 0, or -1 zero increment, -2 zero axis, -3 unknown type. */
int orc_modimg2d(int ncomp, const int *type, const float *flux, const float *ra, const float *dec,
                 const float *bmaj, const float *bmin, const float *bpa, float *image, int nx, int ny,
                 float refx, float deltx, float refy, float delty) {
    const float pi = 3.14159265358979323846f;
    if (deltx == 0.0f || delty == 0.0f) return -1;
    for (int c = 0; c < ncomp; c++) {
        const int t = type[c];
        if (t < 0 || t > 6) return -3;
        if (t == 0) {
            int ix = orc_nint_f(refx + ra[c] / deltx), iy = orc_nint_f(refy + dec[c] / delty);
            if (ix >= 1 && ix <= nx && iy >= 1 && iy <= ny) image[(size_t)(iy - 1) * nx + ix - 1] += flux[c];
            continue;
        }
        if (bmaj[c] == 0.0f || bmin[c] == 0.0f) return -2;
        const float cospa = cosf(pi * bpa[c] / 180.0f), sinpa = sinf(pi * bpa[c] / 180.0f);
        float rnorm = 0.0f, fact = 0.0f, dr = 0.0f;
        if (t == 1) {
            rnorm = (atanf(1.0f) / logf(2.0f)) * bmaj[c] * bmin[c] / (deltx * delty);
            rnorm = 1.0f / fabsf(rnorm);
            fact = 4.0f * logf(2.0f);
        } else if (t == 2) {
            rnorm = atanf(1.0f) * bmaj[c] * bmin[c] / (deltx * delty);
            rnorm = flux[c] / fabsf(rnorm);
        } else if (t == 3) {
            rnorm = bmaj[c] * bmin[c] / (deltx * delty);
            rnorm = 1.0f / fabsf(rnorm);
        } else if (t == 4) {
            rnorm = 4.0f * 1.5f * deltx * delty / (pi * bmaj[c] * bmin[c]);
            rnorm = flux[c] * fabsf(rnorm);
        } else if (t == 5) {
            dr = 2.0f * sqrtf(fabsf(deltx * delty) / (bmaj[c] * bmin[c]));
        } else {
            fact = powf(4.0f, 1.0f / 3.0f) - 1.0f;
            rnorm = fabsf(deltx * delty) * fact / (atanf(1.0f) * 2.0f * bmaj[c] * bmin[c]);
        }
        for (int pass = (t == 5 ? 0 : 1); pass < 2; pass++) {
            for (int iy = 1; iy <= ny; iy++) {
                const float dy = ((float)iy - refy) * delty - dec[c];
                for (int ix = 1; ix <= nx; ix++) {
                    const float dx = ((float)ix - refx) * deltx - ra[c];
                    const float dmaj = dx * sinpa + dy * cospa;
                    const float dmin = -dx * cospa + dy * sinpa;
                    float *a = image + (size_t)(iy - 1) * nx + ix - 1;
                    const float qa = dmaj / bmaj[c], qb = dmin / bmin[c];
                    if (t == 1) {
                        const float r = qa * qa + qb * qb;
                        *a = *a + flux[c] * rnorm * expf(-fact * r);
                    } else if (t == 2) {
                        if (qa * qa + qb * qb < 0.25f) *a = *a + rnorm;
                    } else if (t == 3) {
                        if (fabsf(dmaj) < 0.5f * bmaj[c] && fabsf(dmin) < 0.5f * bmin[c]) *a = *a + flux[c] * rnorm;
                    } else if (t == 4) {
                        const float r = qa * qa + qb * qb;
                        if (r < 0.25f) *a = *a + rnorm * sqrtf(1.0f - 4.0f * r);
                    } else if (t == 5) {
                        const float r = sqrtf(4.0f * (qa * qa + qb * qb));
                        float rmin = r - dr / 2.0f;
                        if (r - dr / 2.0f < 1.0f) {
                            rmin = rmin > 0.0f ? rmin : 0.0f;
                            const float rmax = r + dr / 2.0f, rmax1 = rmax < 1.0f ? rmax : 1.0f;
                            if (rmax > rmin) {
                                const float num = sqrtf(1.0f - rmin * rmin) - sqrtf(1.0f - rmax1 * rmax1);
                                const float den = 2 * pi * pi * (rmax * rmax - rmin * rmin);
                                if (pass == 0) rnorm = rnorm + num / den;
                                else *a = *a + rnorm * num / den;
                            }
                        }
                    } else {
                        const float r = (qa * qa + qb * qb) * 4.0f;
                        *a = *a + flux[c] * rnorm * powf(fact * r + 1.0f, -1.5f);
                    }
                }
            }
            if (t == 5 && pass == 0) rnorm = flux[c] / rnorm;
        }
    }
    return 0;
}

/* grd/grdqh2d.f:64-133 -- 'BOX' gridding: nearest cell, sequential REAL sums in visibility
 * order; gvis [nv][nu] complex; shift DOUBLE 3x3 column-major.  Returns -1 'No weight!'
 * (grid left folded and unnormalised). */
int orc_grdqh2d(const float *vis, const float *wt, const float *u, const float *v, const float *w, int nvis,
                float uscale, float uoffset, float vscale, float voffset, int uorigin, int vorigin, float *gvis,
                int psf, int nu, int nv, const double *shift, float *sumwt) {
    const float twopi = 8.0f * atanf(1.0f);
    for (size_t k = 0; k < (size_t)2 * nu * nv; k++) gvis[k] = 0.0f;
    float lsumwt = 0.0f;
    *sumwt = 0.0f;
    for (int i = 0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        const float ul = (float)(shift[0] * u[i] + shift[1] * v[i] + shift[2] * w[i]);
        const float vl = (float)(shift[3] * u[i] + shift[4] * v[i] + shift[5] * w[i]);
        const float wl = (float)(shift[6] * u[i] + shift[7] * v[i] + shift[8] * w[i]);
        const float phase = twopi * (wl - w[i]);
        const float c = cosf(phase), s = -sinf(phase);
        float fr = vis[2 * i] * c - vis[2 * i + 1] * s, fi = vis[2 * i] * s + vis[2 * i + 1] * c;
        float ucell = uscale * ul + uoffset, vcell = vscale * vl + voffset;
        *sumwt = *sumwt + wt[i];
        if (ucell > 0.0f) {
            fi = -fi;
            ucell = ucell + (float)uorigin;
            vcell = vcell + (float)vorigin;
        } else {
            ucell = -ucell + (float)uorigin;
            vcell = -vcell + (float)vorigin;
        }
        if (psf) {
            fr = 1.0f;
            fi = 0.0f;
        }
        const int ug = orc_nint_f(ucell) + 1, vg = orc_nint_f(vcell);
        if (ug < 1 || ug > nu || vg < 1 || vg > nv) continue;
        float *g = gvis + 2 * ((size_t)(vg - 1) * nu + (ug - 1));
        g[0] = g[0] + wt[i] * fr;
        g[1] = g[1] + wt[i] * fi;
        lsumwt = lsumwt + wt[i];
    }
    const int uz = uorigin + 1, vz = vorigin;
    for (int off = 0; off <= nv / 2 - 1; off++) {
        if (vz + off > nv || vz - off < 1) continue;
        float *p = gvis + 2 * ((size_t)(vz + off - 1) * nu + (uz - 1));
        float *m = gvis + 2 * ((size_t)(vz - off - 1) * nu + (uz - 1));
        p[0] = p[0] + m[0];
        p[1] = p[1] - m[1];
        m[0] = p[0];
        m[1] = -p[1];
    }
    if (lsumwt == 0.0f) return -1;
    lsumwt = (float)(nu - 1) * (float)nv / lsumwt;
    for (int vg = 0; vg < nv; vg++) {
        float *row = gvis + 2 * (size_t)vg * nu;
        for (int ug = 0; ug < nu - 1; ug++) {
            row[2 * ug] = lsumwt * row[2 * ug + 2];
            row[2 * ug + 1] = lsumwt * row[2 * ug + 3];
        }
        row[2 * (nu - 1)] = 0.0f;
        row[2 * (nu - 1) + 1] = 0.0f;
    }
    return 0;
}

/* grd/grdh23d.f:39-147 -- slow-Z gridding: gvis [nz][nv][nu] complex; tables of
 * 2*(supp+1)*osamp+1 floats.  Returns -1 'No weight!' (grid left unfolded). */
int orc_grdh23d(const float *vis, const float *wt, const float *u, const float *v, const float *w, int nvis,
                float uscale, float uoffset, float vscale, float voffset, int uorigin, int vorigin, float *gvis,
                int psf, int nu, int nv, const float *fnu, int suppu, int osampu, const float *fnv, int suppv,
                int osampv, int nz, float cellz, float refz, const double *shift, float *sumwt) {
    const float twopi = 8.0f * atanf(1.0f), dtor = twopi / 360.0f;
    const int cfou = (suppu + 1) * osampu + 1, cfov = (suppv + 1) * osampv + 1;
#define G3(uu, vv, zz) (gvis + 2 * (((size_t)(zz) - 1) * nv * nu + ((size_t)(vv) - 1) * nu + ((uu) - 1)))
    for (size_t k = 0; k < (size_t)2 * nu * nv * nz; k++) gvis[k] = 0.0f;
    float lsumwt = 0.0f;
    *sumwt = 0.0f;
    for (int i = 0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        *sumwt = *sumwt + wt[i];
        const float ul = (float)(shift[0] * u[i] + shift[1] * v[i] + shift[2] * w[i]);
        const float vl = (float)(shift[3] * u[i] + shift[4] * v[i] + shift[5] * w[i]);
        float wl = (float)(shift[6] * u[i] + shift[7] * v[i] + shift[8] * w[i]);
        float phase = twopi * (wl - w[i]);
        float c = cosf(phase), s = -sinf(phase);
        float fr = vis[2 * i] * c - vis[2 * i + 1] * s, fi = vis[2 * i] * s + vis[2 * i + 1] * c;
        float ucell = uscale * ul + uoffset, vcell = vscale * vl + voffset;
        if (ucell > 0.0f) {
            fi = -fi;
            ucell = ucell + (float)uorigin;
            vcell = vcell + (float)vorigin;
        } else {
            ucell = -ucell + (float)uorigin;
            vcell = -vcell + (float)vorigin;
            wl = -wl;
        }
        if (psf) {
            fr = 1.0f;
            fi = 0.0f;
        }
        const int nuc = orc_nint_f(ucell), nvc = orc_nint_f(vcell);
        if (nuc + 2 * suppu > nu || nvc + suppv > nv || nvc - suppv < 1) continue;
        const int delui = orc_nint_f((float)osampu * ((float)nuc - ucell));
        const int delvi = orc_nint_f((float)osampv * ((float)nvc - vcell));
        const int uzero = nuc + suppu, vzero = nvc;
        for (int iz = 1; iz <= nz; iz++) {
            phase = -twopi * wl * dtor * cellz * ((float)iz - refz);
            c = cosf(phase);
            s = -sinf(phase);
            const float rr = fr * c - fi * s, ri = fr * s + fi * c;
            for (int ov = -suppv; ov <= suppv; ov++) {
                const int delv = delvi + osampv * ov + cfov;
                for (int ou = -suppu; ou <= suppu; ou++) {
                    const int delu = delui + osampu * ou + cfou;
                    const float uvwt = wt[i] * fnu[delu - 1] * fnv[delv - 1];
                    float *g = G3(uzero + ou, vzero + ov, iz);
                    g[0] = g[0] + uvwt * rr;
                    g[1] = g[1] + uvwt * ri;
                    lsumwt = lsumwt + uvwt;
                }
            }
        }
    }
    if (lsumwt == 0.0f) return -1;
    const int uz = uorigin + suppu, vz = vorigin;
    for (int iz = 1; iz <= nz; iz++)
        for (int ov = -nv / 2 + 1; ov <= nv / 2 - 1; ov++)
            for (int ou = 1; ou <= suppu; ou++) {
                if (vz + ov < 1 || vz + ov > nv || vz - ov < 1 || vz - ov > nv || uz - ou < 1) continue;
                float *a = G3(uz + ou, vz + ov, iz), *b = G3(uz - ou, vz - ov, iz);
                a[0] = a[0] + b[0];
                a[1] = a[1] - b[1];
            }
    for (int iz = 1; iz <= nz; iz++)
        for (int ov = 0; ov <= nv / 2 - 1; ov++) {
            if (vz + ov > nv || vz - ov < 1) continue;
            float *a = G3(uz, vz + ov, iz), *b = G3(uz, vz - ov, iz);
            a[0] = a[0] + b[0];
            a[1] = a[1] - b[1];
            b[0] = a[0];
            b[1] = -a[1];
        }
    lsumwt = (float)(nu - 1) * (float)nv * (float)nz / lsumwt;
    for (int iz = 1; iz <= nz; iz++)
        for (int vg = 1; vg <= nv; vg++) {
            for (int ug = 1; ug <= nu - suppu; ug++) {
                float *a = G3(ug, vg, iz), *b = G3(ug + suppu, vg, iz);
                a[0] = lsumwt * b[0];
                a[1] = lsumwt * b[1];
            }
            for (int ug = nu - suppu + 1; ug <= nu; ug++) G3(ug, vg, iz)[0] = G3(ug, vg, iz)[1] = 0.0f;
        }
#undef G3
    return 0;
}

/* grd/grddeh23.f:45-190 -- slow-Z degridding in the reference's loop and operation order;
 * reads outside the grid (the reference's mirrored rows) read 0.  Returns NBAD. */
int orc_grddeh23(float *vis, float *wt, const float *u, const float *v, const float *w, int nvis, float uscale,
                 float uoffset, float vscale, float voffset, int uorigin, int vorigin, const float *gvis, int nu,
                 int nv, const float *fnu, int suppu, int osampu, const float *fnv, int suppv, int osampv, int nz,
                 float cellz, float refz, const double *shift) {
    const float twopi = 8.0f * atanf(1.0f), dtor = twopi / 360.0f;
    const int cfou = (suppu + 1) * osampu + 1, cfov = (suppv + 1) * osampv + 1;
    int nbad = 0;
    float *crr = (float *)malloc(sizeof(float) * nz), *cri = (float *)malloc(sizeof(float) * nz);
    for (int i = 0; i < nvis; i++) {
        if (wt[i] <= 0.0f) continue;
        float ar = 0.0f, ai = 0.0f, sumwt = 0.0f;
        vis[2 * i] = vis[2 * i + 1] = 0.0f;
        wt[i] = -wt[i];
        const float ul = (float)(shift[0] * u[i] + shift[1] * v[i] + shift[2] * w[i]);
        const float vl = (float)(shift[3] * u[i] + shift[4] * v[i] + shift[5] * w[i]);
        float wl = (float)(shift[6] * u[i] + shift[7] * v[i] + shift[8] * w[i]);
        float phase = twopi * (wl - w[i]);
        const float rotr = cosf(phase), roti = sinf(phase);
        float ucell = uscale * ul + uoffset, vcell = vscale * vl + voffset;
        if (ucell > 0.0f) {
            ucell = ucell + (float)uorigin;
            vcell = vcell + (float)vorigin;
        } else {
            ucell = -ucell + (float)uorigin;
            vcell = -vcell + (float)vorigin;
            wl = -wl;
        }
        const int nuc = orc_nint_f(ucell), nvc = orc_nint_f(vcell);
        if (nuc + suppu > nu || nvc + suppv > nv || nvc - suppv < 1) continue;
        const int delui = orc_nint_f((float)osampu * ((float)nuc - ucell));
        const int delvi = orc_nint_f((float)osampv * ((float)nvc - vcell));
        const int ucen = nuc - uorigin, vcen = nvc - vorigin;
        for (int iz = 1; iz <= nz; iz++) {
            phase = -twopi * wl * dtor * cellz * ((float)iz - refz);
            crr[iz - 1] = cosf(phase);
            cri[iz - 1] = sinf(phase);
        }
#define GAT(uu, vv, zz, R, I)                                                                              \
    do {                                                                                                   \
        if ((uu) < 1 || (uu) > nu || (vv) < 1 || (vv) > nv) {                                              \
            R = 0.0f;                                                                                      \
            I = 0.0f;                                                                                      \
        } else {                                                                                           \
            const float *q_ = gvis + 2 * (((size_t)(zz) - 1) * nv * nu + ((size_t)(vv) - 1) * nu + ((uu) - 1)); \
            R = q_[0];                                                                                     \
            I = q_[1];                                                                                     \
        }                                                                                                  \
    } while (0)
        if (nuc <= suppu) {
            for (int ou = -suppu; ou <= suppu; ou++) {
                const int delu = delui + osampu * ou + cfou;
                if (ucen != -ou) {
                    const int us = (ucen + ou) >= 0 ? 1 : -1;
                    const int ui = uorigin + us * (ucen + ou);
                    for (int ov = -suppv; ov <= suppv; ov++) {
                        const int delv = delvi + osampv * ov + cfov;
                        const int vi = vorigin + us * (vcen + ov);
                        const float uvwt = fnu[delu - 1] * fnv[delv - 1];
                        sumwt = sumwt + uvwt;
                        for (int iz = 1; iz <= nz; iz++) {
                            float gr, gi;
                            GAT(ui, vi, iz, gr, gi);
                            if (us < 0) gi = -gi;
                            const float pr = gr * crr[iz - 1] - gi * cri[iz - 1], pi_ = gr * cri[iz - 1] + gi * crr[iz - 1];
                            ar = ar + pr * uvwt;
                            ai = ai + pi_ * uvwt;
                        }
                    }
                } else {
                    for (int ov = -suppv; ov <= suppv; ov++) {
                        const int delv = delvi + osampv * ov + cfov;
                        const int vi = vorigin + (vcen + ov);
                        const float uvwt = fnu[delu - 1] * fnv[delv - 1];
                        sumwt = sumwt + uvwt;
                        for (int iz = 1; iz <= nz; iz++) {
                            float gr, gi;
                            GAT(uorigin, vi, iz, gr, gi);
                            gr = gr * uvwt;
                            gi = gi * uvwt;
                            ar = ar + (gr * crr[iz - 1] - gi * cri[iz - 1]);
                            ai = ai + (gr * cri[iz - 1] + gi * crr[iz - 1]);
                        }
                    }
                }
            }
        } else {
            for (int ov = -suppv; ov <= suppv; ov++) {
                const int delv = delvi + osampv * ov + cfov;
                const int vi = vorigin + vcen + ov;
                for (int ou = -suppu; ou <= suppu; ou++) {
                    const int delu = delui + osampu * ou + cfou;
                    const int ui = uorigin + ucen + ou;
                    const float uvwt = fnu[delu - 1] * fnv[delv - 1];
                    sumwt = sumwt + uvwt;
                    for (int iz = 1; iz <= nz; iz++) {
                        float gr, gi;
                        GAT(ui, vi, iz, gr, gi);
                        gr = gr * uvwt;
                        gi = gi * uvwt;
                        ar = ar + (gr * crr[iz - 1] - gi * cri[iz - 1]);
                        ai = ai + (gr * cri[iz - 1] + gi * crr[iz - 1]);
                    }
                }
            }
        }
#undef GAT
        if (sumwt > 0.0f) {
            ar = ar / sumwt;
            ai = ai / sumwt;
            wt[i] = fabsf(wt[i]);
        } else {
            nbad++;
            ar = ai = 0.0f;
        }
        if (uscale * ul > 0.0f) ai = -ai;
        vis[2 * i] = ar * rotr - ai * roti;
        vis[2 * i + 1] = ar * roti + ai * rotr;
    }
    free(crr);
    free(cri);
    return nbad;
}

/* ---------------------------------------------------------------------------------------
 * GRDURUWT (grd/grduruwt.f) with GRDURUW2 (grd/grduruw2.f): ungridded robust weighting.
 */
static int orc_utlgint(float f) { /* utl/utlgint.f */
    if (f >= 0.0f) return (int)f;
    int i = (int)f;
    return ((float)i == f) ? i : i - 1;
}
static int orc_utllint(float f) { /* utl/utllint.f */
    int i = (int)f;
    if (f >= 0.0f) return ((float)i == f) ? i : i + 1;
    return i;
}

/* rmode 1 NORM, 2 ABS, 3 NONE; nbu/nbv <= 0: GRDEUSZ0's estimate.  newwt: the weights
 * GRDURUWT leaves (ARRCOPY of NEWWT).  Returns 0, -1 zero WTSUM, -2 bad bin size, -3 bin
 * calculation, -4 bad RMODE.  stats (7): nbu, nbv, ndrop, nsel, uradius, vradius, f2. */
int orc_grduruwt(const float *u, const float *v, const float *w, const float *wt_in, int nvis, float idelt_u,
                 float idelt_v, float wtfov, int rmode, float robust, float ds, const double *shift, int nbu,
                 int nbv, float *newwt, double *stats) {
    const float pi = 3.1415927f, bineps = 0.1f;
    if (rmode < 1 || rmode > 3) return -4;
    float *wt = (float *)malloc(sizeof(float) * (nvis > 0 ? nvis : 1));
    memcpy(wt, wt_in, sizeof(float) * (size_t)nvis);
    const float urad = fabsf(idelt_u / (wtfov * sqrtf(pi))), vrad = fabsf(idelt_v / (wtfov * sqrtf(pi)));
    const int doshift = shift[0] != 1.0 || shift[4] != 1.0 || shift[8] != 1.0;
#define ORC_LOCAL(k, U0, V0)                                                          \
    do {                                                                              \
        if (doshift) {                                                                \
            U0 = (float)(shift[0] * u[k] + shift[1] * v[k] + shift[2] * w[k]);        \
            V0 = (float)(shift[3] * u[k] + shift[4] * v[k] + shift[5] * w[k]);        \
        } else {                                                                      \
            U0 = u[k];                                                                \
            V0 = v[k];                                                                \
        }                                                                             \
    } while (0)
    float umax = -1.0f, vmax = -1.0f;
    for (int k = 0; k < nvis; k++) {
        if (wt[k] <= 0.0f) continue;
        float u0, v0;
        ORC_LOCAL(k, u0, v0);
        if (fabsf(u0) > umax) umax = fabsf(u0);
        if (fabsf(v0) > vmax) vmax = fabsf(v0);
    }
    if (nbu <= 0) { /* grd/grdeusz0.f:58-64 */
        int nun = orc_utllint(7.6f + bineps), nup = orc_utllint(7.6f * umax / urad + bineps);
        int nvb = 2 * orc_utllint(7.6f * vmax / vrad + bineps);
        nbu = nun + nup < 1000 ? nun + nup : 1000;
        nbv = nvb < 2000 ? nvb : 2000;
    }
    if (nbv <= 0) nbv = 2 * nbu;
    if (nbu < 2 || nbv < 2) {
        free(wt);
        return -2;
    }
    int uorigin;
    float du = 0.0f;
    for (uorigin = 1; uorigin <= nbu - 1; uorigin++) {
        du = umax / ((float)(nbu - uorigin) - bineps);
        if (((float)uorigin - bineps) * du > urad) break;
    }
    if (uorigin > nbu - 1) uorigin = nbu - 1;
    if (urad / du + bineps > (float)uorigin && (nbu - uorigin) > uorigin) {
        free(wt);
        return -3;
    }
    const int vorigin = nbv / 2;
    const float dv = vmax / ((float)vorigin - bineps), uscale = 1.0f / du, vscale = 1.0f / dv;
    const float ur2 = urad * urad, vr2 = vrad * vrad;
    int *head = (int *)calloc((size_t)nbu * nbv, sizeof(int));
    int *links = (int *)calloc((size_t)(nvis > 0 ? nvis : 1), sizeof(int));
    float *bsum = (float *)calloc((size_t)(nvis > 0 ? nvis : 1), sizeof(float));
    long long ndrop = 0;
#define HEAD(i, j) head[((size_t)(j) - 1) * nbu + ((i) - 1)]
    for (int k = 0; k < nvis; k++) {
        newwt[k] = wt[k];
        if (wt[k] <= 0.0f) continue;
        float u0, v0;
        ORC_LOCAL(k, u0, v0);
        float uc = uscale * u0, vc = vscale * v0;
        if (uc < 0.0f) {
            uc = -uc;
            vc = -vc;
        }
        int ub = orc_utlgint(uc) + uorigin + 1, vb = orc_utlgint(vc) + vorigin + 1;
        int ub1 = orc_utlgint(-uc) + uorigin + 1, vb1 = orc_utlgint(-vc) + vorigin + 1;
        if (ub < 1 || ub > nbu || vb < 1 || vb > nbv) {
            ndrop++;
            wt[k] = -1.0f;
        } else {
            int l = HEAD(ub, vb);
            HEAD(ub, vb) = k + 1;
            links[k] = l;
            if (ub1 >= 1 && ub1 <= nbu && vb1 >= 1 && vb1 <= nbv) HEAD(ub1, vb1) = k + 1;
            bsum[k] = l == 0 ? wt[k] : wt[k] + bsum[l - 1];
        }
    }
#define ELL(a, b) ((a) * (a) / ur2 + (b) * (b) / vr2)
    double sumloc = 0.0;
    long long nsel = 0;
    int rc = 0;
    for (int k = 0; k < nvis && rc == 0; k++) {
        if (wt[k] <= 0.0f) continue;
        float u0, v0;
        ORC_LOCAL(k, u0, v0);
        if (u0 < 0.0f) {
            u0 = -u0;
            v0 = -v0;
        }
        int ub = orc_utlgint((u0 - urad) * uscale) + uorigin + 1, ub1 = orc_utlgint((u0 + urad) * uscale) + uorigin + 1;
        int vb = orc_utlgint((v0 - vrad) * vscale) + vorigin + 1, vb1 = orc_utlgint((v0 + vrad) * vscale) + vorigin + 1;
        ub = ub < 1 ? 1 : (ub > nbu ? nbu : ub);
        ub1 = ub1 < 1 ? 1 : (ub1 > nbu ? nbu : ub1);
        vb = vb < 1 ? 1 : (vb > nbv ? nbv : vb);
        vb1 = vb1 < 1 ? 1 : (vb1 > nbv ? nbv : vb1);
        float wtsum = 0.0f;
        for (int j = vb; j <= vb1; j++)
            for (int i = ub; i <= ub1; i++) {
                if (HEAD(i, j) == 0) continue;
                const float UB = (float)(i - uorigin - 1) * du, VB = (float)(j - vorigin) * dv;
                int take = 0;
                if (UB + du < u0) {
                    if (VB - dv > v0) {
                        if (ELL(UB - u0, VB - v0) <= 1.0f) take = 1;
                        else if (ELL(UB + du - u0, VB - dv - v0) >= 1.0f) take = -1;
                    } else if (VB < v0) {
                        if (ELL(UB - u0, VB - dv - v0) <= 1.0f) take = 1;
                        else if (ELL(UB + du - u0, VB - v0) >= 1.0f) take = -1;
                    } else if (ELL(UB - u0, VB - v0) <= 1.0f && ELL(UB - u0, VB - dv - v0) <= 1.0f) {
                        take = 1;
                    }
                } else if (UB > u0) {
                    if (VB - dv > v0) {
                        if (ELL(UB + du - u0, VB - v0) <= 1.0f) take = 1;
                        else if (ELL(UB - u0, VB - dv - v0) >= 1.0f) take = -1;
                    } else if (VB < v0) {
                        if (ELL(UB + du - u0, VB - dv - v0) <= 1.0f) take = 1;
                        else if (ELL(UB - u0, VB - v0) >= 1.0f) take = -1;
                    } else if (ELL(UB + du - u0, VB - v0) <= 1.0f && ELL(UB + du - u0, VB - dv - v0) <= 1.0f) {
                        take = 1;
                    }
                } else {
                    if (VB - dv > v0) {
                        if (ELL(UB - u0, VB - v0) <= 1.0f && ELL(UB + du - u0, VB - v0) <= 1.0f) take = 1;
                    } else if (VB < v0) {
                        if (ELL(UB - u0, VB - dv - v0) <= 1.0f && ELL(UB + du - u0, VB - dv - v0) <= 1.0f) take = 1;
                    } else if (ELL(UB - u0, VB - v0) <= 1.0f && ELL(UB + du - u0, VB - v0) <= 1.0f &&
                               ELL(UB + du - u0, VB - dv - v0) <= 1.0f && ELL(UB - u0, VB - dv - v0) <= 1.0f) {
                        take = 1;
                    }
                }
                if (take < 0) continue;
                if (take > 0) {
                    wtsum = wtsum + bsum[HEAD(i, j) - 1];
                    continue;
                }
                const int posbin = i > uorigin;
                for (int l = HEAD(i, j); l != 0; l = links[l - 1]) {
                    float ut, vt;
                    ORC_LOCAL(l - 1, ut, vt);
                    if (posbin ? ut < 0.0f : ut > 0.0f) {
                        ut = -ut;
                        vt = -vt;
                    }
                    if (ELL(ut - u0, vt - v0) < 1.0f) wtsum = wtsum + wt[l - 1];
                }
            }
        if (wtsum == 0.0f) {
            rc = -1;
            break;
        }
        newwt[k] = wtsum;
        sumloc += wtsum;
        nsel++;
    }
#undef ELL
#undef HEAD
#undef ORC_LOCAL
    float f2 = 1.0f, d2 = 0.0f;
    if (rc == 0) {
        if (rmode == 1) {
            const float t = 5.0f * powf(10.0f, -robust);
            f2 = (float)((double)(t * t) / (sumloc / (double)nsel));
            d2 = 1.0f;
        } else if (rmode == 2) {
            f2 = robust * robust;
            d2 = 2.0f * (ds * ds);
        }
        for (int k = 0; k < nvis; k++)
            if (wt[k] > 0.0f) newwt[k] = wt[k] / (newwt[k] * f2 + d2);
    }
    if (stats) {
        stats[0] = nbu;
        stats[1] = nbv;
        stats[2] = (double)ndrop;
        stats[3] = (double)nsel;
        stats[4] = urad;
        stats[5] = vrad;
        stats[6] = f2;
    }
    free(wt);
    free(head);
    free(links);
    free(bsum);
    return rc;
}

/* ---------------------------------------------------------------------------------------
 * Threaded FP64 oracle for full-size images (64.7 M visibilities at 4096^2): the same
 * gridder, inverse transform and correction as orc64_uvmap_image, split over host threads.
 * Gridding: thread t owns the grid rows of 64-row bands b with b mod T == t and scans every
 * visibility, adding only the taps of its rows, so each cell still sums its contributions
 * in visibility order -- the grid equals the serial orc64_grdh2d's bit for bit.  LSUMWT is
 * summed by one more thread in the serial loop's order.  Columns and rows of the transform
 * are independent and split over threads. */
#include <pthread.h>

typedef struct {
    const orc_geom *g;
    const float *vis, *wt, *u, *v, *w;
    int nvis, psf, t, nt;
    const float *cf;
    int supp, osamp;
    double *gvis;
    double lsumwt;
} g64_job;

/* the per-visibility geometry of orc64_grdh2d; returns 0 when the point is skipped */
static int g64_cell(const g64_job *J, int i, double *fr, double *fi, int *nuc, int *nvc, int *delui,
                    int *delvi) {
    const orc_geom *g = J->g;
    const double *shift = g->shift;
    const int cfoffset = (J->supp + 1) * J->osamp + 1;
    if (J->wt[i] <= 0.0f) return 0;
    double ug = J->u[i], vg = J->v[i], wg = J->w[i], ucell, vcell;
    if (doshift_of(shift)) {
        double ul = SH(1, 1) * ug + SH(2, 1) * vg + SH(3, 1) * wg;
        double vl = SH(1, 2) * ug + SH(2, 2) * vg + SH(3, 2) * wg;
        double wl = SH(1, 3) * ug + SH(2, 3) * vg + SH(3, 3) * wg;
        double ph = 2.0 * M_PI * (wl - wg), c = cos(ph), s = -sin(ph);
        double a = J->vis[2 * i], b = J->vis[2 * i + 1];
        *fr = a * c - b * s;
        *fi = a * s + b * c;
        ucell = (double)g->uscale * ul;
        vcell = (double)g->vscale * vl;
    } else {
        *fr = J->vis[2 * i];
        *fi = J->vis[2 * i + 1];
        ucell = (double)g->uscale * ug;
        vcell = (double)g->vscale * vg;
    }
    if (ucell > 0.0) {
        *fi = -*fi;
        ucell += g->uorigin;
        vcell += g->vorigin;
    } else {
        ucell = -ucell + g->uorigin;
        vcell = -vcell + g->vorigin;
    }
    if (J->psf) { *fr = 1.0; *fi = 0.0; }
    *nuc = orc_nint_d(ucell);
    *nvc = orc_nint_d(vcell);
    if (*nuc + 2 * J->supp > g->nu || *nvc + J->supp > g->nv || *nvc - J->supp < 1) return 0;
    *delui = orc_nint_d((double)J->osamp * ((double)*nuc - ucell)) + cfoffset;
    *delvi = orc_nint_d((double)J->osamp * ((double)*nvc - vcell)) + cfoffset;
    return 1;
}

static void *g64_rows(void *arg) {
    g64_job *J = (g64_job *)arg;
    const int nu = J->g->nu, supp = J->supp, osamp = J->osamp;
    const float *cf = J->cf;
    for (int i = 0; i < J->nvis; i++) {
        double fr, fi;
        int nuc, nvc, delui, delvi;
        if (!g64_cell(J, i, &fr, &fi, &nuc, &nvc, &delui, &delvi)) continue;
        if (J->t == J->nt) { /* the LSUMWT thread */
            for (int offv = -supp; offv <= supp; offv++)
                for (int offu = -supp; offu <= supp; offu++)
                    J->lsumwt += (double)J->wt[i] * (double)cf[delui + osamp * offu - 1] *
                                 (double)cf[delvi + osamp * offv - 1];
            continue;
        }
        for (int offv = -supp; offv <= supp; offv++) {
            const int vv = nvc + offv;
            if (((vv - 1) / 64) % J->nt != J->t) continue;
            double *row = J->gvis + 2 * (size_t)(vv - 1) * (size_t)nu;
            for (int offu = -supp; offu <= supp; offu++) {
                double uvwt = (double)J->wt[i] * (double)cf[delui + osamp * offu - 1] *
                              (double)cf[delvi + osamp * offv - 1];
                const size_t k = (size_t)(nuc + supp + offu - 1);
                row[2 * k] += uvwt * fr;
                row[2 * k + 1] += uvwt * fi;
            }
        }
    }
    return NULL;
}

typedef struct {
    const double *x;
    double *xt, *image;
    int nx, ny, fnu, nv, t, nt, phase;
} f64_job;

static void *f64_part(void *arg) {
    f64_job *J = (f64_job *)arg;
    const int nu = J->fnu / 2 + 1, nv = J->nv, fnu = J->fnu;
    if (J->phase == 0) { /* columns */
        double *col = (double *)malloc(2 * (size_t)nv * sizeof(double));
        const int cv = (nv + 1) / 2 - 1;
        for (int ix = J->t; ix < nu; ix += J->nt) {
            for (int j = 0; j < nv; j++) {
                int src = (j + cv) % nv;
                col[2 * j] = J->x[2 * ((size_t)src * nu + ix)];
                col[2 * j + 1] = J->x[2 * ((size_t)src * nu + ix) + 1];
            }
            fft64(col, nv, +1);
            for (int j = 0; j < nv; j++) {
                int dst = (j + cv) % nv;
                J->xt[2 * ((size_t)dst * nu + ix)] = col[2 * j] / nv;
                J->xt[2 * ((size_t)dst * nu + ix) + 1] = col[2 * j + 1] / nv;
            }
        }
        free(col);
    } else { /* rows */
        double *row = (double *)malloc(2 * (size_t)fnu * sizeof(double));
        const int cu = (fnu + 1) / 2 - 1;
        const int ibegy = (nv + 1) / 2 - (J->ny + 1) / 2 + 1;
        for (int iy = J->t; iy < J->ny; iy += J->nt) {
            const double *xr = J->xt + 2 * (size_t)(iy + ibegy - 1) * nu;
            for (int k = 0; k < fnu; k++) {
                double re, im;
                if (k == 0) { re = xr[0]; im = 0.0; }
                else if (k == fnu / 2) { re = xr[2 * k]; im = 0.0; }
                else if (k < fnu / 2) { re = xr[2 * k]; im = xr[2 * k + 1]; }
                else { re = xr[2 * (fnu - k)]; im = -xr[2 * (fnu - k) + 1]; }
                row[2 * k] = re;
                row[2 * k + 1] = im;
            }
            fft64(row, fnu, +1);
            const int ioff = (fnu - J->nx) / 2;
            for (int ix = 0; ix < J->nx; ix++) {
                int n = ((ix + ioff) - cu + fnu) % fnu;
                J->image[(size_t)iy * J->nx + ix] = row[2 * n] / fnu;
            }
        }
        free(row);
    }
    return NULL;
}

void orc64_uvmap_image_mt(const orc_geom *g, int nvis, const float *u, const float *v,
                          const float *w, const float *vis, const float *wt, int psf,
                          double *image, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    const int nu = g->nu, nv = g->nv;
    double *gvis = (double *)calloc(2 * (size_t)nu * nv, sizeof(double));
    float cf[1 + 8 * 129];
    int supp, osamp;
    orc_grdcf(1, cf, &supp, &osamp);
    g64_job *jobs = (g64_job *)calloc((size_t)nthreads + 1, sizeof(g64_job));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads + 1, sizeof(pthread_t));
    for (int t = 0; t <= nthreads; t++) {
        g64_job J = {g, vis, wt, u, v, w, nvis, psf, t, nthreads, cf, supp, osamp, gvis, 0.0};
        jobs[t] = J;
        pthread_create(&th[t], NULL, g64_rows, &jobs[t]);
    }
    for (int t = 0; t <= nthreads; t++) pthread_join(th[t], NULL);
    const double lsumwt = jobs[nthreads].lsumwt;
    if (lsumwt == 0.0) {
        memset(image, 0, sizeof(double) * (size_t)g->nx * g->ny);
        free(gvis); free(jobs); free(th);
        return;
    }
    /* symmetrise, shift left by SUPPU and normalise: orc64_grdh2d's serial tail */
#define GRE(uu, vv) gvis[2 * (((size_t)(uu)-1) + (size_t)((vv)-1) * (size_t)nu)]
#define GIM(uu, vv) gvis[2 * (((size_t)(uu)-1) + (size_t)((vv)-1) * (size_t)nu) + 1]
    int ucen = g->uorigin + supp, vcen = g->vorigin;
    for (int offv = -nv / 2 + 1; offv <= nv / 2 - 1; offv++)
        for (int offu = 1; offu <= supp; offu++) {
            GRE(ucen + offu, vcen + offv) += GRE(ucen - offu, vcen - offv);
            GIM(ucen + offu, vcen + offv) -= GIM(ucen - offu, vcen - offv);
        }
    for (int offv = 0; offv <= nv / 2 - 1; offv++) {
        GRE(ucen, vcen + offv) += GRE(ucen, vcen - offv);
        GIM(ucen, vcen + offv) -= GIM(ucen, vcen - offv);
        GRE(ucen, vcen - offv) = GRE(ucen, vcen + offv);
        GIM(ucen, vcen - offv) = -GIM(ucen, vcen + offv);
    }
    double scale = (double)(nu - 1) * (double)nv / lsumwt;
    for (int vg = 1; vg <= nv; vg++) {
        for (int ug = 1; ug <= nu - supp; ug++) {
            GRE(ug, vg) = scale * GRE(ug + supp, vg);
            GIM(ug, vg) = scale * GIM(ug + supp, vg);
        }
        for (int ug = nu - supp + 1; ug <= nu; ug++) { GRE(ug, vg) = 0.0; GIM(ug, vg) = 0.0; }
    }
#undef GRE
#undef GIM
    double *xt = (double *)malloc(2 * (size_t)nu * nv * sizeof(double));
    f64_job *fj = (f64_job *)calloc((size_t)nthreads, sizeof(f64_job));
    for (int phase = 0; phase < 2; phase++) {
        for (int t = 0; t < nthreads; t++) {
            f64_job J = {gvis, xt, image, g->nx, g->ny, g->fnu, nv, t, nthreads, phase};
            fj[t] = J;
            pthread_create(&th[t], NULL, f64_part, &fj[t]);
        }
        for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    }
    free(xt);
    free(gvis);
    free(fj);
    free(jobs);
    free(th);
    int ccflen = 1 + orc_fftpwr2(g->nx > g->ny ? g->nx : g->ny) / 2;
    int fnx = orc_fftpwr2(g->nx), fny = orc_fftpwr2(g->ny);
    double sx = (double)(ccflen - 1) * 2.0 / fnx, sy = (double)(ccflen - 1) * 2.0 / fny;
    for (int iy = 1; iy <= g->ny; iy++) {
        int icy = 1 + abs(orc_nint_d(sy * (iy - g->ceny)));
        double cy = orc_grdsf((double)(icy - 1) / (double)(ccflen - 1));
        for (int ix = 1; ix <= g->nx; ix++) {
            int icx = 1 + abs(orc_nint_d(sx * (ix - g->cenx)));
            double cx = orc_grdsf((double)(icx - 1) / (double)(ccflen - 1));
            image[(size_t)(iy - 1) * g->nx + (ix - 1)] /= (cx * cy);
        }
    }
}

/* Visibilities of point sources, V = sum_k S_k exp(+2 pi i (u l_k + v m_k)) in double, stored
 * complex64 -- the benchmark's synthetic sky for the CPU runs (the sign of SDE's direct
 * transform, vis/visdftp2.f:101-107), on nthreads host threads over contiguous ranges. */
typedef struct {
    int64_t i0, i1;
    const float *u, *v;
    int nsrc;
    const double *flux, *l, *m;
    float *out;
} pv_job;

static void *pv_part(void *arg) {
    pv_job *J = (pv_job *)arg;
    const double tp = 2.0 * M_PI;
    for (int64_t i = J->i0; i < J->i1; i++) {
        double re = 0.0, im = 0.0, uu = J->u[i], vv = J->v[i];
        for (int k = 0; k < J->nsrc; k++) {
            double ph = tp * (uu * J->l[k] + vv * J->m[k]);
            re += J->flux[k] * cos(ph);
            im += J->flux[k] * sin(ph);
        }
        J->out[2 * i] = (float)re;
        J->out[2 * i + 1] = (float)im;
    }
    return NULL;
}

void orc_point_vis_mt(int64_t n, const float *u, const float *v, int nsrc, const double *flux,
                      const double *l, const double *m, float *out, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    pv_job jobs[256];
    for (int t = 0; t < nthreads; t++) {
        pv_job J = {n * t / nthreads, n * (t + 1) / nthreads, u, v, nsrc, flux, l, m, out};
        jobs[t] = J;
        pthread_create(&th[t], NULL, pv_part, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

/* img/imgdoubl.f:56-86 with pix/pixrpad.f:38-62 (2-D): the image placed in a zeroed P x P'
 * array, P = FFTPWR2(2N) on each axis longer than one pixel, with left margin
 * LSHIFT = NINT(P/2 - RPIX) (P/2 an INTEGER division, RPIX REAL), so that the reference
 * pixel moves to RPIX + LSHIFT.  out must hold px*py floats; returns the new RPIX. */
void orc_imgdoubl(const float *in, int nx, int ny, float rpix_x, float rpix_y, float *out, int *px,
                  int *py, float *rpix_x_out, float *rpix_y_out) {
    int pn[2], ls[2];
    const int n[2] = {nx, ny};
    const float rp[2] = {rpix_x, rpix_y};
    for (int a = 0; a < 2; a++) {
        if (n[a] > 1) {
            pn[a] = orc_fftpwr2(2 * n[a]);
            if (pn[a] < 1) pn[a] = 1;
            ls[a] = orc_nint_f((float)(pn[a] / 2) - rp[a]);
        } else {
            pn[a] = 1;
            ls[a] = 0;
        }
    }
    for (size_t k = 0; k < (size_t)pn[0] * pn[1]; k++) out[k] = 0.0f;  /* ARRSETCO */
    for (int i2 = 1; i2 <= ny; i2++) {
        const int j2 = i2 + ls[1];
        for (int i1 = 1; i1 <= nx; i1++) {
            const int j1 = i1 + ls[0];
            out[(size_t)(j2 - 1) * pn[0] + (j1 - 1)] = in[(size_t)(i2 - 1) * nx + (i1 - 1)];
        }
    }
    *px = pn[0];
    *py = pn[1];
    *rpix_x_out = rpix_x + (float)ls[0];
    *rpix_y_out = rpix_y + (float)ls[1];
}

/* img/imgtovis.f:55-84: IMGDOUBL (the model padded to P = FFTPWR2(2N), its reference pixel
 * moved to P/2), the grid of the padded image (FFTCONJA: NU = P/2+1, NV = P, uv cells half
 * the size of the image's own grid), then IMGGRIDC CORRECT, IMGFFT and VISDEGRI on it.  The
 * image's reference pixel is (N+1)/2, uvmap's; the padded one is then P/2 = (P+1)/2, the
 * centre the padded geometry below assumes. */
int orc_imgtovis(const orc_uvmap_params *p, int nvis, const float *u, const float *v,
                 const float *w, float *vis, float *wt, const float *image) {
    const int n = p->imsize;
    const float rp = (float)((n + 1) / 2);
    int px, py;
    float rpx, rpy;
    const int pn = orc_fftpwr2(2 * n);
    float *pad = (float *)malloc(sizeof(float) * (size_t)pn * pn);
    orc_imgdoubl(image, n, n, rp, rp, pad, &px, &py, &rpx, &rpy);
    orc_uvmap_params q = *p;
    q.imsize = px;
    int rc = orc_vismodel(&q, nvis, u, v, w, vis, wt, pad);
    free(pad);
    return rc;
}
