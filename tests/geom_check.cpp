// Host check of the plan's FP32 geometry shortcut (sde_geom::geom_near_identity) against
// the operation-by-operation DOUBLE arithmetic (sde_geom::geom_dd): wherever the shortcut
// claims a result, every output both routines read must be identical.  Built by
// tests/test_geom_host.py with -ffp-contract=off, so that the host's operators round each
// operation once, as the device intrinsics do.
//
// Inputs: grids of 256..16384 cells, random cell sizes and signs, SHIFT diagonals that
// differ from 1 by 0, 1 or 2 ulps (CRDSHIFT's output for a phase centre at the tangent
// point, and the identity), and points drawn uniformly over the uv plane plus points placed
// on the rounding boundaries of both routines' cells (NINT half-integers of the gridding
// cell, of its oversampled offsets, of the REAL degridding cell, exact REAL ties of the
// product USCALE*U) and their neighbours.
//
// Usage: geom_check <cases> <seed>; prints "cases shortcut mismatches" and exits 1 on a
// mismatch.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "geom.cuh"

using namespace sde_geom;

static uint64_t rng_state;
static uint64_t next_u64() {
    // splitmix64
    uint64_t z = (rng_state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double uni() { return (double)(next_u64() >> 11) * 0x1p-53; }
static int rint_range(int lo, int hi) { return lo + (int)(next_u64() % (uint64_t)(hi - lo + 1)); }

static GParams make_params() {
    GParams p;
    memset(&p, 0, sizeof p);
    const int n = 1 << rint_range(8, 14);
    const float cell_arcsec = (float)(0.05 + 20.0 * uni());
    const float d2r = 3.141592654f / 180.0f;
    const float cdu = 1.0f / (d2r * ((float)n * (-cell_arcsec / 3600.0f)));
    const float cdv = 1.0f / (d2r * ((float)n * (cell_arcsec / 3600.0f)));
    p.uscale = 1.0f / cdu;
    p.vscale = 1.0f / cdv;
    if (next_u64() & 1) p.uscale = -p.uscale;
    if (next_u64() & 1) p.vscale = -p.vscale;
    p.uoffset = p.voffset = 0.0f;
    p.nu = n / 2 + 1;
    p.nv = n;
    p.uorigin = 1;
    p.vorigin = (n + 1) / 2;
    if ((next_u64() & 7) == 0) p.uorigin = rint_range(1, 64);
    p.supp = 3;
    const int osamps[] = {128, 128, 128, 64, 100, 1, 3};
    p.osamp = osamps[rint_range(0, 6)];
    const double diag[] = {1.0, 1.0 - 0x1p-53, 1.0 - 0x1p-52, 1.0 + 0x1p-52, 1.0 + 0x1p-51};
    for (int k = 0; k < 9; k++) p.s[k] = 0.0;
    p.s[0] = diag[rint_range(0, 4)];
    p.s[4] = diag[rint_range(0, 4)];
    p.s[8] = diag[rint_range(0, 4)];
    p.identity = p.s[0] == 1.0 && p.s[4] == 1.0 && p.s[8] == 1.0;
    p.diagonal = 1;
    p.doshift = !p.identity;
    p.fast = p.identity;
    p.near_id = 1;
    p.ntu = 1;
    p.twopi = (double)(8.0f * atanf(1.0f));
    return p;
}

static bool gvalid_of(const GParams &p, const GGeo &g) {
    return g.sane && !(g.nuc + 2 * p.supp > p.nu) && !(g.nvc + p.supp > p.nv) && !(g.nvc - p.supp < 1);
}

static bool same_f(float a, float b) { return memcmp(&a, &b, 4) == 0; }

// the coordinate x (REAL) whose cell scale*x + origin lands near `target`, and a neighbour
static float place(double target, double origin, float scale, int nb) {
    float x = (float)((target - origin) / (double)scale);
    for (int k = 0; k < abs(nb); k++) x = nextafterf(x, nb > 0 ? INFINITY : -INFINITY);
    return x;
}

int main(int argc, char **argv) {
    const long long cases = argc > 1 ? atoll(argv[1]) : 1000000;
    rng_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
    long long taken = 0, bad = 0;
    GParams p = make_params();
    for (long long c = 0; c < cases; c++) {
        if ((c & 4095) == 0) p = make_params();
        const double umax = 0.55 * p.nv / fabs((double)p.uscale), vmax = 0.55 * p.nv / fabs((double)p.vscale);
        float u = (float)((2.0 * uni() - 1.0) * umax), v = (float)((2.0 * uni() - 1.0) * vmax);
        const int mode = (int)(c % 8);
        const int nb = rint_range(-3, 3);
        if (mode == 1 || mode == 2) {
            // GRDH2D's NINT boundary (k + 1/2) or an oversampled-offset boundary of the u or v cell
            const int k = rint_range(4, p.nu - 4);
            const double tgt = mode == 1 ? k + 0.5 : k - (rint_range(-64, 63) + 0.5) / p.osamp;
            if (next_u64() & 1) u = place(tgt, p.uorigin, (float)fabs(p.uscale), nb) * (p.uscale < 0 ? -1.0f : 1.0f);
            else v = place(tgt, p.vorigin, p.vscale, nb);
        } else if (mode == 3) {
            // a REAL midpoint of the degridding cell: P = scale*x halfway between two REALs
            const float base = (float)((2.0 * uni() - 1.0) * 0.5 * p.nv);
            const float mid = base + 0.5f * (nextafterf(base, INFINITY) - base);
            u = place((double)mid, 0.0, p.uscale, nb);
        } else if (mode == 4) {
            u = (float)rint_range(-3, 3);  // zeros and small integers
        } else if (mode == 5) {
            // exact REAL ties: scale*(k*2^j) for small odd k is a 25-bit product -- halfway
            // between two REALs -- for many scales; the only case where SNGL of the DOUBLE
            // cell can differ from the REAL product (the DOUBLE cell moves it off the tie)
            const int k = 2 * rint_range(1, 15) + 1;
            const int j = rint_range(-8, 12);
            const float x = ldexpf((float)k, j) * ((next_u64() & 1) ? 1.0f : -1.0f);
            if (next_u64() & 1) u = x; else v = x;
        }
        const float w = (float)((2.0 * uni() - 1.0) * 1.0e5);
        const float vr = (float)(2.0 * uni() - 1.0), vi = (float)(2.0 * uni() - 1.0);
        GGeo gs;
        if (!geom_near_identity(p, u, v, w, vr, vi, gs)) continue;
        taken++;
        const GGeo gd = geom_dd(p, u, v, w, vr, vi);
        const bool vs = gvalid_of(p, gs), vd = gvalid_of(p, gd);
        bool ok = vs == vd && gs.gc == gd.gc && same_f(gs.fr, gd.fr) && same_f(gs.fi, gd.fi) &&
                  same_f(gs.rc, gd.rc) && same_f(gs.rs, gd.rs) && gs.dg.nud == gd.dg.nud &&
                  gs.dg.nvd == gd.dg.nvd && gs.dg.dui == gd.dg.dui && gs.dg.dvi == gd.dg.dvi &&
                  gs.dg.valid == gd.dg.valid && gs.dg.conj == gd.dg.conj && same_f(gs.dg.rc, gd.dg.rc) &&
                  same_f(gs.dg.rs, gd.dg.rs);
        if (vd) ok = ok && gs.nuc == gd.nuc && gs.nvc == gd.nvc && gs.dug == gd.dug && gs.dvg == gd.dvg;
        if (!ok) {
            if (bad < 10)
                fprintf(stderr,
                        "mismatch: u=%a v=%a w=%a uscale=%a vscale=%a osamp=%d s=(%a,%a,%a) | "
                        "nuc %d/%d nvc %d/%d dug %d/%d dvg %d/%d gc %d/%d nud %d/%d nvd %d/%d dui %d/%d dvi %d/%d\n",
                        u, v, w, p.uscale, p.vscale, p.osamp, p.s[0], p.s[4], p.s[8], gs.nuc, gd.nuc, gs.nvc,
                        gd.nvc, gs.dug, gd.dug, gs.dvg, gd.dvg, gs.gc, gd.gc, gs.dg.nud, gd.dg.nud, gs.dg.nvd,
                        gd.dg.nvd, gs.dg.dui, gd.dg.dui, gs.dg.dvi, gd.dg.dvi);
            bad++;
        }
    }
    printf("%lld %lld %lld\n", cases, taken, bad);
    return bad ? 1 : 0;
}
