/*
 * sde_oracle.h -- CPU restatement of the SDE imaging hot path (test infrastructure).
 *
 * This library is the ORACLE used by the tests, by __graft_entry__.smoke() and by
 * bench.py's cpu_baseline / --impl reference legs.  It is never linked into, loaded by
 * or called from the product library (libsdegpu).  Each routine restates one Fortran-77
 * routine of timcornwell/sde with the same arithmetic types and evaluation order
 * (REAL -> float, DOUBLE PRECISION -> double, NINT -> round-half-away, no FMA
 * contraction: build with -ffp-contract=off).  Arrays are passed 0-based but index
 * arithmetic follows the Fortran 1-based formulas; 2-D arrays are column-major
 * (Fortran GVIS(NU,NV) == C row-major [NV][NU]).  Complex arrays are interleaved
 * float pairs (re, im).
 *
 * Documented deviations from the reference source:
 *   - FFTX's bit-reverse table is sized to M (reference IBITRV(4096) overflows at
 *     M = 8192, fft/fftx.f:112), and FFTX/FFTR tables are recomputed on every call
 *     (the reference keeps them in non-SAVEd locals, fft/fftx.f:112-115, fft/fftr.f:87).
 */
#ifndef SDE_ORACLE_H
#define SDE_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* error codes returned where the reference calls ERRREPOR */
#define ORC_OK 0
#define ORC_ENOWEIGHT 1   /* grd/grdh2d.f:195-197 'No weight!'          */
#define ORC_EBADMODE 2    /* grd/grdruw2d.f:191 'Unrecognized RMODE'      */
#define ORC_EBADARG 3

double orc_grdsf(double nu);                                   /* grd/grdsf.f:7-76      */
int    orc_fftpwr2(int i);                                     /* fft/fftpwr2.f:7-42    */
int    orc_nint_f(float x);                                    /* Fortran NINT(REAL)    */
int    orc_nint_d(double x);                                   /* Fortran NINT(DOUBLE)  */
void   orc_grdcf(int code_sf, float *cf, int *cfsupp, int *cfosamp); /* grd/grdcf.f:7-95    */
void   orc_grdccf(int code_sf, float *ccf, int ccflen);        /* grd/grdccf.f:7-68     */
void   orc_crdshift(double vra_deg, double vdec_deg, double ira_deg, double idec_deg,
                    float vrota3_deg, double *shift);          /* crd/crdshift.f:7-169  */

void orc_grduwt2d(const float *wt, const float *u, const float *v, const float *w, int nvis,
                  float uscale, float uoffset, float vscale, float voffset, int uorigin,
                  int vorigin, float *newwt, float *gwt, int nu, int nv, const double *shift,
                  int *ndrop);                                 /* grd/grduwt2d.f:7-170  */
int orc_grdruw2d(const float *wt, const float *u, const float *v, const float *w, int nvis,
                 float uscale, float uoffset, float vscale, float voffset, int uorigin,
                 int vorigin, float *newwt, float *gwt, int nu, int nv, const double *shift,
                 const char *rmode, const float *robust, float ds, int *ndrop,
                 double *sumwt_out, double *sumlocwt_out, float *f2_out); /* grd/grdruw2d.f:7-252 */

int orc_grdh2d(const float *vis, const float *wt, const float *u, const float *v, const float *w,
               int nvis, float uscale, float uoffset, float vscale, float voffset, int uorigin,
               int vorigin, float *gvis, int psf, int nu, int nv, const float *gridfnu, int suppu,
               int osampu, const float *gridfnv, int suppv, int osampv, const double *shift,
               float *sumwt, double *lsumwt_out);
/* GRDH2D in parts: accumulate visibilities i0..nvis-1 into a zeroed grid (sums carried in
 * *sumwt_acc / *lsumwt_acc), then finalize with the total LSUMWT */
void orc_grdh2d_acc(const float *vis, const float *wt, const float *u, const float *v,
                    const float *w, int i0, int nvis, float uscale, float uoffset, float vscale,
                    float voffset, int uorigin, int vorigin, float *gvis, int psf, int nu, int nv,
                    const float *gridfnu, int suppu, int osampu, const float *gridfnv, int suppv,
                    int osampv, const double *shift, float *sumwt_acc, double *lsumwt_acc);
int  orc_grdh2d_end(float *gvis, int nu, int nv, int uorigin, int vorigin, int suppu,
                    double lsumwt);              /* grd/grdh2d.f:7-229    */
void orc_grddeh2d(float *vis, float *wt, const float *u, const float *v, const float *w, int nvis,
                  float uscale, float uoffset, float vscale, float voffset, int uorigin,
                  int vorigin, const float *gvis, int nu, int nv, const float *intfnu, int suppu,
                  int osampu, const float *intfnv, int suppv, int osampv, const double *shift,
                  int *nbad);                                  /* grd/grddeh2d.f:7-204  */

void orc_fftx(float *x, float *w, int m, int isig);            /* fft/fftx.f:84-275     */
void orc_fftx1d(float *xarray, float *xwork, float *xwork2, int nx, int dir); /* fft/fftx1d.f */
void orc_fftr(float *r, float *c, float *work, int n, int f);  /* fft/fftr.f:60-176     */
void orc_fftr1d(float *rarray, float *xarray, float *rwork, float *xwork, int nx, int dir);
void orc_fftr1d2(float *rarray, float *xarray, float *xwork, float *xwork2, float *rwork,
                 int nx, int fnu, int dir);
void orc_fftr2d(float *rarray, float *xarray, int nx, int ny, int fnu, int nv, int dir); /* fft/fftr2d.f */

void orc_pixcor2d(const float *in, int nx, int ny, const float *cf, int cflen, int correct,
                  float *out, float cenx, float ceny);         /* pix/pixcor2d.f:7-71   */
int  orc_pixisama(int n, const float *a, int i);               /* pix/pixisama.f:7-64 */
void orc_pix2drcl(const float *drt, const float *psf, const float *box, int nx, int ny, int pnx,
                  int pny, float gain, int nsub, int bsub, float flux, float *cln, float *res,
                  int *ansub, float *maxres, float *tflux, float *cflux, int *cx, int *cy);
void orc_pixrscal(const float *in, float scale, float offset, float *out, int64_t n); /* pix/pixrscal.f */

/* ---- task-level drivers (task/uvmap.f, task/vismodel.f) ---------------------------- */
typedef struct {
    int imsize;          /* Imsize (square)                         */
    float cellsize;      /* arcsec                                  */
    float fov;           /* FOV for weighting (0 = natural)          */
    int rmode;           /* 0 NONE(uniform) 1 NORM 2 ABS 3 AZ-NORM  */
    float robust[3];
    float ds;
    double vra, vdec;    /* visibility phase centre (deg)           */
    float shift_ra, shift_dec; /* image shift (arcsec), task/uvmap.f Shift */
} orc_uvmap_params;

/* Image/grid geometry of IMGMAKE + FFTCONJA (img/imgmake.f, fft/fftconja.f, fft/fftconj.f). */
typedef struct {
    int nx, ny, fnu, nu, nv;
    float uscale, vscale;       /* 1/CDELT of the XFR axes                 */
    int uorigin, vorigin;
    float cenx, ceny;           /* image reference pixel (N+1)/2            */
    double shift[9];
} orc_geom;
void orc_make_geom(const orc_uvmap_params *p, orc_geom *g);

/* uvmap: weighting -> PSF -> dirty, both normalised by the PSF peak.  wt is updated
 * in place to the reweighted values (as the reference does).  Returns an error code. */
int orc_uvmap(const orc_uvmap_params *p, int nvis, const float *u, const float *v,
              const float *w, const float *vis, float *wt, float *dirty, float *psf,
              float *maxpsf, float *sumwt_psf);
/* vismodel: grid-correct -> r2c FFT -> degrid (task/vismodel.f:70-74). */
int orc_vismodel(const orc_uvmap_params *p, int nvis, const float *u, const float *v,
                 const float *w, float *vis, float *wt, const float *image);

/* Clark CLEAN of an N x N dirty image with its N x N PSF (the CLARK branch of task/clean.f
 * and img/imgcclea.f): window = CRDHALF's inner half (w = N/2 pixels from N/4+1), beam patch
 * bpatch, list size numcl.  comp (w x w) is the initial component image and is updated;
 * resid (w x w) receives the final residual; cl/cx/cy (niter entries) the component list.
 * Returns 0, -1 'Zero range in values', -2 'Too many points', -3 negative limit, -10 bad
 * arguments. */
typedef struct {
    int niter;
    float gain, flux;
    int numcl, bpatch;
} orc_clark_params;
#define ORC_CLARK_TRACE 64
typedef struct {
    int aniter, ncycles, window, blc, last_anl;
    float maxres, tflux, extside, last_slim;
    /* IMGCCLEA's per-cycle message (img/imgcclea.f:276-278): ANL, ANITER, MAXRES, TFLUX */
    int t_anl[ORC_CLARK_TRACE], t_aniter[ORC_CLARK_TRACE];
    float t_maxres[ORC_CLARK_TRACE], t_tflux[ORC_CLARK_TRACE];
} orc_clark_result;
int orc_clark(const float *dirty, const float *psf, int n, const float *box, const orc_clark_params *p,
              float *comp, float *resid, float *cl, int *cx, int *cy, orc_clark_result *r);

/* Direct Fourier transforms (uvmap's and vismodel's DFT options), FP32 as the reference
 * computes them (rotation recurrences) and FP64 with exact phases.  Images [ny][nx], vis
 * complex pairs, refx/refy 1-based reference pixel, deltx/delty degrees. */
int  orc_visdft2d(const float *vis, int nvis, const float *wt, const float *u, const float *v, float *image,
                  float *psf, int nx, int ny, float refx, float deltx, float refy, float delty);
void orc_imgdft2d(const float *image, int nx, int ny, float refx, float deltx, float refy, float delty,
                  float *vis, int nvis, const float *wt, const float *u, const float *v);
int  orc64_visdft2d(const float *vis, int nvis, const float *wt, const float *u, const float *v,
                    double *image, double *psf, int nx, int ny, double refx, double deltx, double refy,
                    double delty);
void orc64_imgdft2d(const float *image, int nx, int ny, double refx, double deltx, double refy,
                    double delty, double *vis, int nvis, const float *wt, const float *u, const float *v);

/* GRDURUWT + GRDURUW2 (grd/grduruwt.f, grd/grduruw2.f): ungridded robust weighting.
 * rmode 1 NORM, 2 ABS, 3 NONE; stats (7 doubles): nbu, nbv, ndrop, nsel, uradius, vradius, f2. */
int orc_grduruwt(const float *u, const float *v, const float *w, const float *wt_in, int nvis, float idelt_u,
                 float idelt_v, float wtfov, int rmode, float robust, float ds, const double *shift, int nbu,
                 int nbv, float *newwt, double *stats);

/* GRDH23D / GRDDEH23 (grd/grdh23d.f, grd/grddeh23.f): slow-Z gridding and degridding,
 * gvis [nz][nv][nu] complex, tables of 2*(supp+1)*osamp+1 floats. */
int orc_grdh23d(const float *vis, const float *wt, const float *u, const float *v, const float *w, int nvis,
                float uscale, float uoffset, float vscale, float voffset, int uorigin, int vorigin, float *gvis,
                int psf, int nu, int nv, const float *fnu, int suppu, int osampu, const float *fnv, int suppv,
                int osampv, int nz, float cellz, float refz, const double *shift, float *sumwt);
int orc_grddeh23(float *vis, float *wt, const float *u, const float *v, const float *w, int nvis, float uscale,
                 float uoffset, float vscale, float voffset, int uorigin, int vorigin, const float *gvis, int nu,
                 int nv, const float *fnu, int suppu, int osampu, const float *fnv, int suppv, int osampv, int nz,
                 float cellz, float refz, const double *shift);

/* GRDQH2D (grd/grdqh2d.f): 'BOX' gridding into gvis [nv][nu] complex. */
int orc_grdqh2d(const float *vis, const float *wt, const float *u, const float *v, const float *w, int nvis,
                float uscale, float uoffset, float vscale, float voffset, int uorigin, int vorigin, float *gvis,
                int psf, int nu, int nv, const double *shift, float *sumwt);

/* MODIMG2D (mod/modimg2d.f): components added into image [ny][nx]; type 0 POIN, 1 GAUS,
 * 2 DISK, 3 RECT, 4 SPHE, 5 SHEL, 6 PLOR; offsets and increments in arcsec. */
int orc_modimg2d(int ncomp, const int *type, const float *flux, const float *ra, const float *dec,
                 const float *bmaj, const float *bmin, const float *bpa, float *image, int nx, int ny,
                 float refx, float deltx, float refy, float delty);

/* ---- FP64 oracle: same algorithms in double, plus a direct DFT --------------------- */
int  orc64_grdh2d(const float *vis, const float *wt, const float *u, const float *v,
                  const float *w, int nvis, const orc_geom *g, int psf, double *gvis);
void orc64_fftr2d_inv(const double *xarray, double *image, int nx, int ny, int fnu, int nv);
/* orc64_uvmap_image on nthreads host threads (identical grid; independent FFT lines) */
/* point-source visibilities in double -> complex64 on nthreads threads (benchmark data) */
void orc_point_vis_mt(int64_t n, const float *u, const float *v, int nsrc, const double *flux,
                      const double *l, const double *m, float *out, int nthreads);
/* img/imgdoubl.f + pix/pixrpad.f (2-D) and img/imgtovis.f (the padded degrid) */
void orc_imgdoubl(const float *in, int nx, int ny, float rpix_x, float rpix_y, float *out, int *px,
                  int *py, float *rpix_x_out, float *rpix_y_out);
int  orc_imgtovis(const orc_uvmap_params *p, int nvis, const float *u, const float *v,
                  const float *w, float *vis, float *wt, const float *image);
void orc64_uvmap_image_mt(const orc_geom *g, int nvis, const float *u, const float *v,
                          const float *w, const float *vis, const float *wt, int psf,
                          double *image, int nthreads);
void orc64_uvmap_image(const orc_geom *g, int nvis, const float *u, const float *v,
                       const float *w, const float *vis, const float *wt, int psf,
                       double *image);
void orc64_dft_image(const orc_geom *g, int nvis, const float *u, const float *v,
                     const float *vis, const float *wt, int psf, double *image);

#ifdef __cplusplus
}
#endif
#endif
