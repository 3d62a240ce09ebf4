// geom.cuh -- per-visibility cell geometry of GRDH2D and GRDDEH2D, shared by the plan
// build (device) and a host-side check of its FP32 shortcut against the DOUBLE arithmetic.
//
// GRDH2D places a visibility with DOUBLE cell coordinates (grd/grdh2d.f:114-166),
// GRDDEH2D with a REAL cell from DOUBLE coordinates (grd/grddeh2d.f:92-118).  GB300 runs
// DOUBLE at a small fraction of its FP32 rate, so geom_vis first tries an FP32 evaluation
// with a rigorous error bound (geom_near_identity) and keeps the DOUBLE path for the inputs
// the bound cannot decide.
//
// Every floating-point operation is an explicit round-to-nearest call (no contraction):
// on the device the __*_rn intrinsics, on the host plain operators, which the host build
// of the check compiles with -ffp-contract=off.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define GEOM_HD __host__ __device__ __forceinline__
#else
#define GEOM_HD inline
#endif

namespace sde_geom {

GEOM_HD double dmul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
GEOM_HD double dadd(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
GEOM_HD double dsub(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
GEOM_HD float fmul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
GEOM_HD float fadd(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
GEOM_HD float fsub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
GEOM_HD float ffma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}
GEOM_HD float d2f(double x) {
#ifdef __CUDA_ARCH__
    return __double2float_rn(x);
#else
    return (float)x;
#endif
}
GEOM_HD int d2i_rd(double x) {
#ifdef __CUDA_ARCH__
    return __double2int_rd(x);
#else
    return (int)floor(x);
#endif
}
GEOM_HD int f_bits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_int(x);
#else
    int i;
    memcpy(&i, &x, 4);
    return i;
#endif
}
GEOM_HD float bits_f(int i) {
#ifdef __CUDA_ARCH__
    return __int_as_float(i);
#else
    float x;
    memcpy(&x, &i, 4);
    return x;
#endif
}
GEOM_HD void dsincos(double x, double *s, double *c) {
#ifdef __CUDA_ARCH__
    sincos(x, s, c);
#else
    *s = sin(x);
    *c = cos(x);
#endif
}

// Fortran NINT of a REAL (half away from zero).
GEOM_HD int nint_r(float x) { return (int)roundf(x); }

// Fortran NINT of a DOUBLE: floor(x + 0.5), the negative side mirrored.  x + 0.5 cannot
// round up to the next integer for the values it is given (cells >= 1/2 or offsets that
// are multiples of 2^-45); callers keep |x| far below 2^31.
GEOM_HD int nint_dd(double x) {
    return x >= 0.0 ? d2i_rd(dadd(x, 0.5)) : -d2i_rd(dadd(-x, 0.5));
}

struct GParams {
    float uscale, uoffset, vscale, voffset;
    int uorigin, vorigin, nu, nv, supp, osamp;
    double s[9];
    int doshift, ntu;
    int identity;   // SHIFT is exactly the identity matrix
    int diagonal;   // SHIFT's off-diagonal entries are all zero
    int fast;       // identity SHIFT and UOFFSET = VOFFSET = 0
    int near_id;    // diagonal SHIFT with |S11 - 1|, |S22 - 1| <= 2^-50, no offsets
    double twopi;
};

struct DGeo {
    int nud, nvd, dui, dvi;
    bool valid, conj;
    float rc, rs;
};

// COS and SIN of GRDH2D/GRDDEH2D's phase in DOUBLE.  Below 2^-27 in magnitude the correctly
// rounded values are exactly 1 and the phase itself (|sin x - x| <= |x|^3/6 and x^2/2 are
// below half an ulp there), which is what a phase-centre rotation that differs from the
// identity only by rounding (CRDSHIFT's sin^2 + cos^2 on the diagonal) produces for every
// visibility: no library call is made for it.
GEOM_HD void phase_cos_sin(double ph, double &c, double &s) {
    if (fabs(ph) < 0x1p-27) {
        c = 1.0;
        s = ph;
    } else {
        dsincos(ph, &s, &c);
    }
}

// GRDDEH2D's REAL cell arithmetic (grd/grddeh2d.f:100-118) from the REAL cells
// SNGL(USCALE*ULOCAL + UOFFSET) and the sign of the DOUBLE product USCALE*ULOCAL.
GEOM_HD DGeo degrid_cell_r(const GParams &p, float ucell, float vcell, bool conj, float rc, float rs) {
    DGeo g;
    g.rc = rc;
    g.rs = rs;
    if (ucell > 0.0f) {
        ucell = fadd(ucell, (float)p.uorigin);
        vcell = fadd(vcell, (float)p.vorigin);
    } else {
        ucell = fadd(-ucell, (float)p.uorigin);
        vcell = fadd(-vcell, (float)p.vorigin);
    }
    g.nud = nint_r(ucell);
    g.nvd = nint_r(vcell);
    g.valid = !(g.nud + p.supp > p.nu) && !(g.nvd + p.supp > p.nv) && !(g.nvd - p.supp < 1);
    g.dui = nint_r(fmul((float)p.osamp, fsub((float)g.nud, ucell)));
    g.dvi = nint_r(fmul((float)p.osamp, fsub((float)g.nvd, vcell)));
    g.conj = conj;
    return g;
}

// GRDDEH2D's per-visibility geometry (grd/grddeh2d.f:92-118) from the rotated coordinates:
// FP32 cell, the REAL rotation (rc, rs).
GEOM_HD DGeo degrid_cell(const GParams &p, double ul, double vl, float rc, float rs) {
    const double pu = dmul((double)p.uscale, ul);
    const float ucell = d2f(dadd(pu, (double)p.uoffset));
    const float vcell = d2f(dadd(dmul((double)p.vscale, vl), (double)p.voffset));
    return degrid_cell_r(p, ucell, vcell, pu > 0.0, rc, rs);
}

// The rotation ULOCAL, VLOCAL, WLOCAL = SHIFT applied to (U, V, W) in DOUBLE (GRDDEH2D
// always applies it; GRDH2D when DOSHIFT).  With SHIFT exactly the identity the products
// and sums are exact for finite coordinates (1*x = x, 0*y = +-0, x + +-0 = x up to the sign
// of a zero, which no later step can see), so they are skipped.
GEOM_HD void rotate_uvw(const GParams &p, double ug, double vg, double wg, double &ul, double &vl,
                        double &wl) {
    if (p.identity) {
        ul = ug;
        vl = vg;
        wl = wg;
    } else if (p.diagonal) {
        // zero off-diagonal terms add +-0: the sums are the diagonal products (up to the sign
        // of a zero result, which no later step can see) -- CRDSHIFT without a shift, whose
        // diagonal sin^2 + cos^2 can miss 1 by an ulp
        ul = dmul(p.s[0], ug);
        vl = dmul(p.s[4], vg);
        wl = dmul(p.s[8], wg);
    } else {
        ul = dadd(dadd(dmul(p.s[0], ug), dmul(p.s[1], vg)), dmul(p.s[2], wg));
        vl = dadd(dadd(dmul(p.s[3], ug), dmul(p.s[4], vg)), dmul(p.s[5], wg));
        wl = dadd(dadd(dmul(p.s[6], ug), dmul(p.s[7], vg)), dmul(p.s[8], wg));
    }
}

// GRDDEH2D's per-visibility geometry (grd/grddeh2d.f:92-118): always rotated, FP32 cell.
GEOM_HD DGeo degrid_geom(const GParams &p, float u, float v, float w) {
    const double ug = (double)u, vg = (double)v, wg = (double)w;
    double ul, vl, wl, c, s;
    rotate_uvw(p, ug, vg, wg, ul, vl, wl);
    phase_cos_sin(dmul(p.twopi, dsub(wl, wg)), c, s);
    return degrid_cell(p, ul, vl, d2f(c), d2f(s));
}

// The identity SHIFT without offsets (every uvmap/mapper call without a phase-centre
// shift): GRDDEH2D's REAL cell SNGL(USCALE*U) is the once-rounded REAL product (the DOUBLE
// product of two REALs is exact), its phase is 0 (COS 1, SIN 0).
GEOM_HD DGeo degrid_geom_fast(const GParams &p, float u, float v) {
    return degrid_cell_r(p, fmul(p.uscale, u), fmul(p.vscale, v), dmul((double)p.uscale, (double)u) > 0.0,
                         1.0f, 0.0f);
}

// Both routines' geometry of one visibility.
struct GGeo {
    bool sane;            // |UCELL|, |VCELL| < 2^30 (GRDH2D's cell fits an integer)
    bool gc;              // GRDH2D's conjugation (UCELL > 0)
    int nuc, nvc;         // GRDH2D's NINT cell (valid when sane)
    int dug, dvg;         // GRDH2D's oversampled offsets (valid when sane)
    float fr, fi;         // the observed value in GRDH2D's frame (rotated, conjugated)
    float rc, rs;         // the REAL rotation (COS, SIN of the phase) when DOSHIFT, else (1, 0)
    DGeo dg;              // GRDDEH2D's geometry
};

// GRDH2D's cell arithmetic in DOUBLE from its cells UCELL, VCELL before the origin.
GEOM_HD void grid_cells_dd(const GParams &p, double ucell, double vcell, GGeo &g) {
    g.gc = ucell > 0.0;
    if (g.gc) {
        g.fi = -g.fi;
        ucell = dadd(ucell, (double)(float)p.uorigin);
        vcell = dadd(vcell, (double)(float)p.vorigin);
    } else {
        ucell = dadd(-ucell, (double)(float)p.uorigin);
        vcell = dadd(-vcell, (double)(float)p.vorigin);
    }
    g.sane = fabs(ucell) < 1073741824.0 && fabs(vcell) < 1073741824.0;
    g.nuc = g.nvc = g.dug = g.dvg = 0;
    if (g.sane) {
        g.nuc = nint_dd(ucell);
        g.nvc = nint_dd(vcell);
        g.dug = nint_dd(dmul((double)p.osamp, dsub((double)(float)g.nuc, ucell)));
        g.dvg = nint_dd(dmul((double)p.osamp, dsub((double)(float)g.nvc, vcell)));
    }
}

// The reference's arithmetic, operation by operation (DOUBLE where it is DOUBLE).
GEOM_HD GGeo geom_dd(const GParams &p, float uf, float vf, float wf, float vr, float vi) {
    GGeo g;
    g.rc = 1.0f;
    g.rs = 0.0f;
    if (p.fast) {
        // USCALE*U of two REALs is exact in DOUBLE and adding a zero UOFFSET changes nothing
        g.dg = degrid_geom_fast(p, uf, vf);
        g.fr = vr;
        g.fi = vi;
        grid_cells_dd(p, dmul((double)p.uscale, (double)uf), dmul((double)p.vscale, (double)vf), g);
        return g;
    }
    // one rotation and one phase serve GRDDEH2D (always) and GRDH2D (DOSHIFT)
    const double ug = (double)uf, vg = (double)vf, wg = (double)wf;
    double ul, vl, wl, cd, sd;
    rotate_uvw(p, ug, vg, wg, ul, vl, wl);
    phase_cos_sin(dmul(p.twopi, dsub(wl, wg)), cd, sd);
    g.dg = degrid_cell(p, ul, vl, d2f(cd), d2f(sd));
    double ucell, vcell;
    if (p.doshift) {
        const float c = d2f(cd), s = d2f(-sd);
        g.fr = fsub(fmul(vr, c), fmul(vi, s));
        g.fi = fadd(fmul(vr, s), fmul(vi, c));
        ucell = dadd(dmul((double)p.uscale, ul), (double)p.uoffset);
        vcell = dadd(dmul((double)p.vscale, vl), (double)p.voffset);
        g.rc = g.dg.rc;
        g.rs = g.dg.rs;
    } else {
        g.fr = vr;
        g.fi = vi;
        ucell = dadd(dmul((double)p.uscale, ug), (double)p.uoffset);
        vcell = dadd(dmul((double)p.vscale, vg), (double)p.voffset);
    }
    grid_cells_dd(p, ucell, vcell, g);
    return g;
}

// One axis of geom_near_identity.  P = scale*x is exact as ph + pl (REAL product and its
// FMA residual).  With the axis' SHIFT entry within 2^-50 of 1 and no offset, both
// routines' DOUBLE cells A (USCALE*ULOCAL or USCALE*U, rounded) lie within |P|*2^-49 of P,
// and GRDH2D's cell after the origin, U = RN(sgn*A + origin), within
// B = (|ph| + |t| + 1)*2^-48 of V = sgn*P + origin.  The outputs are decided when that
// error cannot move a value across a rounding boundary:
//   cf  = SNGL(A), GRDDEH2D's REAL cell: ph, when |pl| plus the error stays below half the
//         spacing of REALs on pl's side of ph;
//   n   = NINT(U): n0, the integer nearest t = RN(sgn*ph + origin), when r = V - n0 (from
//         t - n0, exact, and TwoSum's error term and pl) keeps 2^-22 + 2B inside +-1/2;
//   d   = NINT(OSAMP*(n - U)): the integer nearest D = -OSAMP*r, when D keeps
//         OSAMP*2^-22 + 2^-14 + 2*OSAMP*B from the half-integers.
// Otherwise (about one visibility in 10^4, and every non-finite or |P| >= 2^20 or tiny
// one) it returns false and the DOUBLE path decides.
GEOM_HD bool axis_near_identity(float x, float scale, float sgn, int origin, float osamp, int &n,
                                int &d, float &cf) {
    const float ph = fmul(scale, x);
    const float pl = ffma(scale, x, -ph);
    const float aph = fabsf(ph);
    // (a product that is tiny or underflows to zero in REAL is left to DOUBLE, whose sign tests see it)
    if (!(aph < 0x1p20f) || (aph < 0x1p-60f && !(x == 0.0f || scale == 0.0f))) return false;
    // spacing of REALs at |ph|; below a power of two (toward zero) it halves
    const float ulp = fmul(bits_f(f_bits(aph) & 0x7F800000), 0x1p-23f);
    const bool pow2 = (f_bits(aph) & 0x007FFFFF) == 0;
    const bool toward_zero = pl != 0.0f && ((pl < 0.0f) != (ph < 0.0f));
    const float half = (pow2 && toward_zero) ? fmul(0.25f, ulp) : fmul(0.5f, ulp);
    if (ph != 0.0f && !(fadd(fabsf(pl), fmul(aph, 0x1p-47f)) < half)) return false;
    cf = ph;
    // V = sgn*P + origin = t + e + sgn*pl exactly (TwoSum of sgn*ph and the origin)
    const float a = sgn * ph, o = (float)origin;
    const float t = fadd(a, o);
    const float bb = fsub(t, a);
    const float aa = fsub(t, bb);
    const float e = fadd(fsub(a, aa), fsub(o, bb));
    if (!(fabsf(t) < 0x1p21f)) return false;
    const float B = fmul(fadd(fadd(aph, fabsf(t)), 1.0f), 0x1p-48f);
    const float n0 = rintf(t);
    const float r = fadd(fsub(t, n0), fadd(e, sgn * pl));
    if (!(fabsf(r) <= 0.5f - 0x1p-22f - 2.0f * B)) return false;
    const float D = fmul(-osamp, r);
    const float m0 = rintf(D);
    const float MD = fadd(fadd(fmul(osamp, 0x1p-22f), 0x1p-14f), fmul(fmul(2.0f, osamp), B));
    if (!(fabsf(fsub(D, m0)) <= fsub(0.5f, MD))) return false;
    n = (int)n0;
    d = (int)m0;
    return true;
}

// geom_dd's results from FP32 arithmetic for a SHIFT within 2^-50 of the identity on the u
// and v axes (the identity, and CRDSHIFT's matrix for a phase centre at the tangent point,
// whose diagonal sin^2 + cos^2 misses 1 by an ulp) and zero offsets; false when some value
// lies too close to a rounding boundary to decide (axis_near_identity) or the phase is not
// tiny.  The phase keeps its two DOUBLE products.
GEOM_HD bool geom_near_identity(const GParams &p, float uf, float vf, float wf, float vr, float vi, GGeo &g) {
    double cd = 1.0, sd = 0.0;
    if (!p.identity) {
        const double wg = (double)wf;
        const double wl = p.diagonal ? dmul(p.s[8], wg) : wg;
        const double ph = dmul(p.twopi, dsub(wl, wg));
        if (!(fabs(ph) < 0x1p-27)) return false;
        sd = ph;
    }
    const bool conj = fmul(p.uscale, uf) > 0.0f;  // sign of USCALE*U, exact
    const float sgn = conj ? 1.0f : -1.0f;
    float cu, cv;
    if (!axis_near_identity(uf, p.uscale, sgn, p.uorigin, (float)p.osamp, g.nuc, g.dug, cu)) return false;
    if (!axis_near_identity(vf, p.vscale, sgn, p.vorigin, (float)p.osamp, g.nvc, g.dvg, cv)) return false;
    g.sane = true;
    g.gc = conj;
    const float rc = d2f(cd), rs = d2f(sd);
    g.dg = degrid_cell_r(p, cu, cv, conj, rc, rs);
    if (p.doshift) {
        const float c = rc, s = d2f(-sd);
        g.fr = fsub(fmul(vr, c), fmul(vi, s));
        g.fi = fadd(fmul(vr, s), fmul(vi, c));
        g.rc = rc;
        g.rs = rs;
    } else {
        g.fr = vr;
        g.fi = vi;
        g.rc = 1.0f;
        g.rs = 0.0f;
    }
    if (conj) g.fi = -g.fi;
    return true;
}

GEOM_HD GGeo geom_vis(const GParams &p, float uf, float vf, float wf, float vr, float vi) {
    GGeo g;
    if (p.near_id && geom_near_identity(p, uf, vf, wf, vr, vi, g)) return g;
    return geom_dd(p, uf, vf, wf, vr, vi);
}

}  // namespace sde_geom
