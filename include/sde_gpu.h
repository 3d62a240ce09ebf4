/*
 * sde_gpu.h -- C ABI of libsdegpu, the GB300 (sm_103a) implementation of SDE's imaging
 * hot path: uniform/robust weight-density counts, convolutional gridding with the
 * 128x-oversampled prolate-spheroidal kernel, the half-plane 2-D FFT with grid
 * correction, degridding, and the Hogbom CLEAN minor cycle.
 *
 * Two layers:
 *
 *  1. Drop-in entry points with the reference's Fortran-77 calling convention (every
 *     argument by reference, column-major arrays, hidden trailing CHARACTER lengths).
 *     Each replaces one pixel-level routine of timcornwell/sde, cited beside it; they
 *     take HOST arrays, run on the GPU and write the results back in place, honouring
 *     the reference's global ERROR flag (COMMON /SYSI/, include/stdinc.h:66): they return
 *     at once when ERROR is set and set it (through errrepor_) on failure.
 *
 *  2. A handle API (sde_*) that keeps visibilities, grids and images resident in HBM
 *     and runs asynchronously on the context's stream; this is what the batched and
 *     served paths, the Python host layer and the benchmark use.
 *
 * All functions return SDE_OK (0) or an SDE_E* code; sde_last_error() gives the text.
 * Nothing here falls back to the CPU: without a usable GPU every call fails with
 * SDE_ENODEV.
 */
#ifndef SDE_GPU_H
#define SDE_GPU_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------ */
#define SDE_OK 0
#define SDE_EINVAL 1      /* bad argument (size, mode, pointer)                        */
#define SDE_ENOMEM 2      /* device allocation failed / admission refused                */
#define SDE_ECUDA 3       /* CUDA runtime error                                          */
#define SDE_ENOWEIGHT 4   /* gridder found no weight (grd/grdh2d.f:195-197 'No weight!') */
#define SDE_ETIMEDOUT 5   /* a bounded device wait gave up                                */
#define SDE_EBADMODE 6    /* unrecognised RMODE (grd/grdruw2d.f:190-192)                      */
#define SDE_ENODEV 7      /* no CUDA device                                               */
#define SDE_ECANCELLED 8  /* stopped by the interrupt flag (SYSINTRP analogue)            */

const char *sde_last_error(void);
int sde_version(void);

/* ======================================================================================
 * Layer 1: Fortran-77 drop-in entry points (gfortran symbol names).
 * ====================================================================================== */

/* The drop-ins run on one library context, created by the first drop-in call on the device
 * named by the environment variable SDE_DEVICE, or else on the calling thread's current CUDA
 * device (device 0 unless the program selected another).
 *
 * The drop-ins keep the plan of their last GRDH2D/GRDDEH2D call together with a device copy
 * of the U, V, W, WT it was built from; a call whose U, V, W, WT (compared bitwise on the
 * device after the upload), grid geometry and gridding function match reuses it and only
 * loads the new VIS.  No counterpart in the reference.  Statistics, and a call that frees
 * the cached plan and inputs: */
int sde_shim_cache_stats(int64_t *hits, int64_t *misses);
int sde_shim_cache_clear(void);

/* Replaces GRDH2D (source/grd/grdh2d.f:7-9), called by VISGRID (vis/visgrid.f:160-164). */
void grdh2d_(float *vis, float *wt, float *u, float *v, float *w, int *nvis, float *uscale,
             float *uoffset, float *vscale, float *voffset, int *uorigin, int *vorigin,
             float *gvis, int *psf, int *nu, int *nv, float *gridfnu, int *suppu, int *osampu,
             float *gridfnv, int *suppv, int *osampv, double *shift, float *sumwt);

/* Replaces GRDDEH2D (source/grd/grddeh2d.f:7-9), called by VISDEGRI (vis/visdegri.f:135-139). */
void grddeh2d_(float *vis, float *wt, float *u, float *v, float *w, int *nvis, float *uscale,
               float *uoffset, float *vscale, float *voffset, int *uorigin, int *vorigin,
               float *gvis, int *nu, int *nv, float *intfnu, int *suppu, int *osampu,
               float *intfnv, int *suppv, int *osampv, double *shift);

/* Replaces GRDQH2D (source/grd/grdqh2d.f:7-9), called by VISGRID for the 'BOX' gridding
 * function (vis/visgrid.f:154-158): nearest-cell gridding with the shift matrix's phase
 * rotation, u = 0 column folded, shift one column left and (NU-1)*NV/LSUMWT. */
void grdqh2d_(float *vis, float *wt, float *u, float *v, float *w, int *nvis, float *uscale,
              float *uoffset, float *vscale, float *voffset, int *uorigin, int *vorigin, float *gvis,
              int *psf, int *nu, int *nv, double *shift, float *sumwt);

/* Replace GRDH23D (source/grd/grdh23d.f:7-10) and GRDDEH23 (source/grd/grddeh23.f:7-10), the
 * slow-Z gridder and degridder VISGRID (vis/visgrid.f:220-226) and VISDEGRI
 * (vis/visdegri.f:154-159) call for N----SIN third axes: the 2-D window on NZ planes, plane iz
 * rotated by exp(-/+i TWOPI WLOCAL DTOR CELLZ (iz-REFZ)); GVIS [NZ][NV][NU] complex; tables
 * of 2*(SUPP+1)*OSAMP+1 floats (any support and oversampling). */
void grdh23d_(float *vis, float *wt, float *u, float *v, float *w, int *nvis, float *uscale,
              float *uoffset, float *vscale, float *voffset, int *uorigin, int *vorigin, float *gvis,
              int *psf, int *nu, int *nv, float *gridfnu, int *suppu, int *osampu, float *gridfnv,
              int *suppv, int *osampv, int *nz, float *cellz, float *refz, double *shift,
              float *sumwt);
void grddeh23_(float *vis, float *wt, float *u, float *v, float *w, int *nvis, float *uscale,
               float *uoffset, float *vscale, float *voffset, int *uorigin, int *vorigin,
               float *gvis, int *nu, int *nv, float *intfnu, int *suppu, int *osampu,
               float *intfnv, int *suppv, int *osampv, int *nz, float *cellz, float *refz,
               double *shift);

/* Replaces GRDUWT2D (source/grd/grduwt2d.f:7-8), called by GRDUWT (grd/grduwt.f:122-126). */
void grduwt2d_(float *wt, float *u, float *v, float *w, int *nvis, float *uscale,
               float *uoffset, float *vscale, float *voffset, int *uorigin, int *vorigin,
               float *newwt, float *gwt, int *nu, int *nv, double *shift);

/* Replaces GRDRUW2D (source/grd/grdruw2d.f:7-9), called by GRDRUWT (grd/grdruwt.f:172-176). */
void grdruw2d_(float *wt, float *u, float *v, float *w, int *nvis, float *uscale,
               float *uoffset, float *vscale, float *voffset, int *uorigin, int *vorigin,
               float *newwt, float *gwt, int *nu, int *nv, double *shift, char *rmode,
               float *robust, float *ds, size_t rmode_len);

/* Replaces FFTR2D (source/fft/fftr2d.f:7-8), called by ARRFFTR (arr/arrfftr.f:139-140).
 * WORK, WORK2 and RWORK are accepted for signature compatibility and not touched. */
void fftr2d_(float *rarray, float *xarray, float *work, float *work2, float *rwork, int *nx,
             int *ny, int *fnu, int *nv, int *dir);

/* Replaces PIXCOR2D (source/pix/pixcor2d.f:7-8), called by IMGGRIDC (img/imggridc.f:96-97). */
void pixcor2d_(float *in, int *nx, int *ny, float *cf, int *cflen, char *mode, float *out,
               float *cenx, float *ceny, size_t mode_len);

/* Replaces PIX2DRCL (source/pix/pix2drcl.f:7-9), called by IMGCLEAN (img/imgclean.f:186). */
void pix2drcl_(float *drt, float *psf, float *box, int *nx, int *ny, int *pnx, int *pny,
               float *gain, int *nsub, int *bsub, float *flux, float *cln, float *res,
               int *ansub, float *maxres, float *tflux, float *cflux, int *cx, int *cy);

/* Replaces PIXISAMA (source/pix/pixisama.f:7), called by PIX2DRCL (pix/pix2drcl.f:75,87,135). */
int pixisama_(int *n, float *a, int *i);

/* Host-side tables the gridder's callers build (no GPU work):
 * GRDSF (source/grd/grdsf.f:7), GRDCF (source/grd/grdcf.f:7, called by VISGRID,
 * vis/visgrid.f:100) and GRDCCF (source/grd/grdccf.f:7, called by IMGGRIDC,
 * img/imggridc.f:75); codes 'SF' and 'BOX'. */
double grdsf_(double *nu);
void grdcf_(char *cfcode, float *cf, int *cfsupp, int *cfosamp, size_t cfcode_len);
void grdccf_(char *ccfcode, float *ccf, int *ccflen, size_t ccfcode_len);

/* The reference's error channel: COMMON /SYSI/ (include/stdinc.h:64-66).  libsdegpu
 * defines it; a Fortran program's own definition interposes at link time.  errrepor_ and
 * msgput_ are weak defaults (main/err.f:532, main/msg.f:7) that a host program overrides. */
typedef struct {
    int error, msgwidth, sysdebug, sysmon, sysintrp, sysmsg, syspar;
} sde_sysi_common;
extern sde_sysi_common sysi_;
void errrepor_(const char *reason, const char *routine, const char *text, size_t lreason,
               size_t lroutine, size_t ltext);
void msgput_(const char *msg, const char *type, size_t lmsg, size_t ltype);

/* ======================================================================================
 * Layer 2: resident handle API.
 * ====================================================================================== */
typedef struct sde_ctx sde_ctx;     /* one device + one stream + scratch pools          */
typedef struct sde_plan sde_plan;   /* a tile-sorted, device-resident visibility set     */

int sde_ctx_create(sde_ctx **out, int device);
int sde_ctx_destroy(sde_ctx *ctx);
int sde_ctx_sync(sde_ctx *ctx);
void *sde_ctx_stream(sde_ctx *ctx);            /* the cudaStream_t all calls run on       */
int sde_ctx_set_stream(sde_ctx *ctx, void *stream); /* run on a caller's stream instead   */
/* Device memory owned by the context's pools (bytes), for admission control. */
int64_t sde_ctx_bytes_in_use(sde_ctx *ctx);
/* Tracing: with profiling on, every kernel launch is bracketed by CUDA events on the
 * context's stream; sde_ctx_kernel_stats synchronises and returns the summed device time
 * (ms) and launch count of one kernel ("grid", "grid_psf", "degrid", "degrid_exc",
 * "finalize", "col_fft", "row_c2r", "row_r2c", "hogbom", ...).  sde_ctx_launches counts
 * every kernel the library has launched on this context. */
int sde_ctx_profile(sde_ctx *ctx, int enable);
int sde_ctx_kernel_stats(sde_ctx *ctx, const char *kernel, double *total_ms, int64_t *count);
int sde_ctx_reset_stats(sde_ctx *ctx);
int64_t sde_ctx_launches(sde_ctx *ctx);
/* Compensated accumulation of the gridding sums across work items (default on): each work
 * item's shared-memory tile is added into the raw grid with an atomic that returns the
 * previous value, the rounding error of that FP32 add (TwoSum) goes to a second plane, and
 * the finalize pass adds the planes.  Off: plain FP32 sums (half the raw-grid memory).
 * Takes effect for passes started afterwards; batches fix it at sde_batch_create.
 * No counterpart in the reference (GRDH2D sums every visibility into its cell in REAL). */
int sde_ctx_set_compensated(sde_ctx *ctx, int on);

/* Geometry of one gridding/degridding job (the scalar arguments of GRDH2D/GRDDEH2D). */
typedef struct {
    int nu, nv;                 /* half-plane grid: NU = FNU/2+1 columns, NV rows        */
    float uscale, uoffset, vscale, voffset;
    int uorigin, vorigin;
    int supp, osamp;            /* 3, 128 for the 'SF' kernel                           */
    double shift[9];            /* SHIFT(3,3) column-major (crd/crdshift.f)              */
} sde_gridspec;

/* Weighting (GRDUWT2D / GRDRUW2D).  rmode: 0 uniform (GRDUWT2D), 1 NORM, 2 ABS,
 * 3 AZ-NORM, 4 NONE (GRDRUW2D).  Pointers are device pointers (async on the stream).
 * newwt may alias wt.  gwt (nu*nv floats, [nv][nu]) may be NULL.  stats may be NULL;
 * when given, the call synchronises and fills it. */
typedef struct {
    int64_t ndrop;              /* points dropped off the reweighting grid                */
    double sumwt, sumlocwt;     /* GRDRUW2D's SUMWT and SUMLOCWT                          */
    float f2, d2;               /* robust parameters actually used                        */
} sde_wstats;
int sde_weights(sde_ctx *ctx, int rmode, const float robust[3], float ds, const float *wt,
                const float *u, const float *v, const float *w, int64_t nvis, float uscale,
                float uoffset, float vscale, float voffset, int uorigin, int vorigin,
                int nu, int nv, const double shift[9], float *newwt, float *gwt,
                sde_wstats *stats);

/* Plans.  where: SDE_HOST or SDE_DEVICE for the input arrays (vis is complex64 pairs).
 * The plan copies what it needs; inputs may be freed afterwards.  Visibilities with
 * WT <= 0 or outside the gridding bounds are excluded from gridding exactly as GRDH2D
 * excludes them. */
#define SDE_HOST 0
#define SDE_DEVICE 1
int sde_plan_create(sde_ctx *ctx, const sde_gridspec *spec, int64_t nvis, const float *u,
                    const float *v, const float *w, const float *vis, const float *wt,
                    int where, sde_plan **out);
/* The same with the plan's sort-bucket sizes chosen by the caller (an autotuner): the
 * visibilities of one uv tile are cut into work items of at most item_max visibilities
 * (one CTA each), and the visibilities of one cell pair inside a work item into chunks of
 * at most chunk_max (one 4-lane group each).  0 selects the default (16384 / 64).  Limits:
 * chunk_max <= item_max <= 65536, chunk_max <= 4096.  No counterpart in the reference
 * (GRDH2D walks visibilities in input order). */
typedef struct {
    int item_max;
    int chunk_max;
} sde_plan_opts;
int sde_plan_create_opts(sde_ctx *ctx, const sde_gridspec *spec, int64_t nvis, const float *u,
                         const float *v, const float *w, const float *vis, const float *wt,
                         int where, const sde_plan_opts *opts, sde_plan **out);
int sde_plan_destroy(sde_plan *plan);
int64_t sde_plan_nvis(const sde_plan *plan);       /* visibilities that grid              */
int64_t sde_plan_bytes(const sde_plan *plan);
/* work items, chunks and degridding exceptions (GRDDEH2D's reflection branch, FP32/FP64
 * cell mismatches, degrid-only points) of a plan */
int sde_plan_stats(const sde_plan *plan, int64_t *nitems, int64_t *nchunks, int64_t *nexc);
/* Replace the plan's visibilities (same order/length as at creation). */
int sde_plan_set_vis(sde_plan *plan, const float *vis, int where);

/* Grid the plan's residual visibilities (or the PSF) onto a device grid in the final
 * GRDH2D layout: [nv][pitch] complex64, pitch >= nu (use sde_grid_pitch), already
 * symmetrised, shifted by SUPPU and normalised by (NU-1)*NV/sum(UVWT).  sumwt (host,
 * may be NULL) receives GRDH2D's SUMWT; passing it synchronises the stream. */
#define SDE_GRID_VIS 0
#define SDE_GRID_PSF 1
int sde_grid_pitch(int nu);
int sde_plan_grid(sde_plan *plan, int what, float *grid, int pitch, float *sumwt);
/* Dirty image (SDE_GRID_VIS) or PSF (SDE_GRID_PSF) of the plan into image (device, ny x nx,
 * row-major): GRDH2D's grid then FFTR2D's inverse (fft/fftr2d.f:64-90), with PIXCOR2D's
 * correction when correct != 0 and divided by *scale_dev when scale_dev != NULL -- what
 * sde_plan_grid followed by sde_image_from_grid gives, with GRDH2D's finalize applied inside
 * the column pass instead of as a pass of its own.  The column-transformed grid is left in
 * grid ([nv][pitch] complex64) when grid != NULL.  Asynchronous; sumwt as in sde_plan_grid.
 * No counterpart entry point in the reference (uvmap calls GRDH2D, then FFTR2D). */
int sde_plan_image(sde_plan *plan, int what, int nx, int ny, int correct, const float *scale_dev,
                   float *image, float *grid, int pitch, float *sumwt);

/* Degrid a device grid ([nv][pitch] complex64, GRDDEH2D layout) at the plan's
 * visibilities and update the residual: residual = observed - model.  Asynchronous. */
int sde_plan_degrid_residual(sde_plan *plan, const float *grid, int pitch);
/* Reset the residual to the observed visibilities. */
int sde_plan_reset_residual(sde_plan *plan);
/* Degrid a device grid into user-ordered visibilities exactly as GRDDEH2D does
 * (normalised interpolation, reflection, conjugation, phase rotation, WT sign flags).
 * vis_out/wt_out are device or host pointers per `where` (length = nvis at creation);
 * like GRDDEH2D's VIS and WT they are in/out: wt_out holds the WT the plan was made from,
 * and entries GRDDEH2D would not touch (WT <= 0) are left unchanged.  Host arrays are
 * uploaded only when the plan has such entries, and WT is copied back only when a point
 * was not degridded (its WT negated). */
int sde_plan_degrid(sde_plan *plan, const float *grid, int pitch, float *vis_out,
                    float *wt_out, int where, int64_t *nbad);
/* Copy the residual visibilities back in the caller's original order (complex64). */
int sde_plan_get_residual(sde_plan *plan, float *vis_out, int where);

/* 2-D transforms (FFTR2D conventions) on device arrays, with the grid correction
 * (PIXCOR2D 'CORRECT' by the GRDCCF 'SF' table) fused.
 *   grid -> image: column c2c along v (FFTX1D, DIR -1), row c2r along u (FFTR1D2), then
 *     image /= CCF(|x-cx|) CCF(|y-cy|), then image *= *scale_dev when scale_dev != NULL.
 *   image -> grid: image / CCF, row r2c, column c2c (DIR +1).
 * grid is [nv][pitch] complex64 (NU = fnu/2+1 columns used); image is [ny][nx] float32.
 * correct: 1 applies the correction, 0 skips it (plain FFTR2D). */
int sde_image_from_grid(sde_ctx *ctx, float *grid, int pitch, int nx, int ny, int fnu, int nv,
                        int correct, const float *scale_dev, float *image);
int sde_grid_from_image(sde_ctx *ctx, const float *image, int nx, int ny, int fnu, int nv,
                        int correct, float *grid, int pitch);

/* max over an image (ARRSTAT ARRMAX) into a device float, and OUT = scale*IN + offset
 * with scale = 1/(*max_dev) (task/uvmap.f:434-440, 480-482 with pix/pixrscal.f). */
int sde_image_max(sde_ctx *ctx, const float *image, int64_t n, float *max_dev);
int sde_image_scale_by_inverse(sde_ctx *ctx, float *image, int64_t n, const float *max_dev);

/* Hogbom CLEAN (PIX2DRCL) on device arrays: drt, box, cln, res [ny][nx]; psf [pny][pnx];
 * cflux/cx/cy device arrays of |nsub| entries.  One persistent launch runs every
 * iteration; scalars come back in *out (host) after an internal synchronisation.
 * cancel_flag (host pinned or NULL) is polled like SYSINTRP (pix/pix2drcl.f:94-99). */
typedef struct {
    int ansub;
    float maxres, tflux;
} sde_clean_result;
int sde_hogbom(sde_ctx *ctx, const float *drt, const float *psf, const float *box, int nx,
               int ny, int pnx, int pny, float gain, int nsub, int bsub, float flux,
               float tflux_in, float *cln, float *res, float *cflux, int *cx, int *cy,
               volatile int *cancel_flag, sde_clean_result *out);

/* Direct Fourier transforms (the DFT options of uvmap and vismodel) on device arrays:
 *   sde_dft_image  VISDFT3D for a 2-D image (vis/visdft3d.f; task/uvmap.f:416-418):
 *                  dirty(ix,iy) = RNORM sum_k WT_k Re(V_k E), psf = RNORM sum_k WT_k Re(E),
 *                  E = exp(-i CF (u DX (ix-RX) + v DY (iy-RY))), CF = 2 pi^2/180, RNORM =
 *                  1/sum WT over WT > 0 ('No valid data' when that sum is 0); dirty or psf
 *                  may be NULL.
 *   sde_dft_vis    IMGDFT2D (img/imgdft2d.f; task/vismodel.f:75): V_k = sum I(ix,iy) conj(E)
 *                  for WT_k > 0; other points keep their VIS.
 * images [ny][nx] float32, vis complex64 pairs, refx/refy the 1-based reference pixel (a
 * multiple of 1/2), deltx/delty degrees per pixel; nx, ny, |refx|, |refy| <= 8192.  Phases
 * are exact to FP32 rounding (no rotation recurrence) and sums over visibilities are
 * compensated, so both are accurate to ~1e-7 of the peak. */
int sde_dft_image(sde_ctx *ctx, int64_t nvis, const float *u, const float *v, const float *vis,
                  const float *wt, int nx, int ny, double refx, double deltx, double refy,
                  double delty, float *dirty, float *psf);
int sde_dft_vis(sde_ctx *ctx, const float *image, int nx, int ny, double refx, double deltx,
                double refy, double delty, int64_t nvis, const float *u, const float *v,
                const float *wt, float *vis);

/* GRDQH2D on device arrays (the 'BOX' gridder): vis complex64 pairs (ignored for psf), grid
 * [nv][pitch] complex64 (NU columns written), shift the host 3x3 DOUBLE matrix (column-major,
 * as CRDSHIFT makes it).  SDE_ENOWEIGHT ('No weight!') leaves the folded, unnormalised grid. */
int sde_grid_box(sde_ctx *ctx, int64_t nvis, const float *vis, const float *wt, const float *u,
                 const float *v, const float *w, float uscale, float uoffset, float vscale,
                 float voffset, int uorigin, int vorigin, int psf, int nu, int nv,
                 const double *shift, float *grid, int pitch, float *sumwt);

/* Ungridded robust weighting: uvmap's slow weighting (GridWeights = F, task/uvmap.f:283-290),
 * GRDURUWT (grd/grduruwt.f) with GRDURUW2 (grd/grduruw2.f).  Host arrays; the neighbour
 * search runs on the GPU.  Each point's local weight is the summed WT of the points (either
 * conjugation) inside the ellipse of radii |IDELT/(WTFOV SQRT(PI))| around it, found through
 * GRDURUW2's bin plane of linked lists (built in the reference's order, so the sums are its
 * REAL sums); newwt = WT / (sum F2 + D2) with rmode 1 NORM (F2 = (5*10^-R)^2 / mean sum,
 * D2 = 1), 2 ABS (F2 = R^2, D2 = 2 DS^2), 3 NONE (F2 = 1, D2 = 0).  Points with WT <= 0, and
 * points off the bin plane, keep their WT.  nbu/nbv: bin plane size (<= 0: GRDEUSZ0's
 * estimate).  shift: the 3x3 DOUBLE matrix from CRDSHIFT.  Messages: 'Unrecognized RMODE',
 * 'Bad size for binning array', 'Problems with binsize calcs', 'Zero WTSUM'.  Saving or
 * reading summed weights (SAVEWEIGHTS/READWEIGHTS) is not provided. */
typedef struct {
    int nbu, nbv;
    int64_t ndrop, nsel;
    float uradius, vradius, f2, d2;
    double sumlocwt;
} sde_uruwt_stats;
int sde_weights_ungridded(sde_ctx *ctx, int64_t nvis, const float *u, const float *v, const float *w,
                          const float *wt, float idelt_u, float idelt_v, float wtfov, int rmode,
                          const float *robust, float ds, const double *shift, int nbu, int nbv,
                          float *newwt, sde_uruwt_stats *stats);

/* MODIMG2D (mod/modimg2d.f, via MODIMG, mod/modimg.f): ncomp model components added into the
 * device image [ny][nx].  types: 4 characters per component (POIN, GAUS, DISK, RECT, SPHE,
 * SHEL, PLOR); flux, ra, dec (offsets from the reference pixel), bmaj, bmin (arcsec), bpa
 * (degrees): host arrays; refx/refy 1-based, deltx/delty arcsec per pixel (3600 * CDELT).
 * Messages: 'Zero increment in X/Y', 'Major axis zero', 'Minor axis zero', 'Unknown model
 * type XXXX for component N' (all components are checked before any is added).
 * Synchronises. */
int sde_model_image(sde_ctx *ctx, int ncomp, const char *types, const float *flux, const float *ra,
                    const float *dec, const float *bmaj, const float *bmin, const float *bpa, int nx,
                    int ny, float refx, float deltx, float refy, float delty, float *image);

/* IMGDOUBL (source/img/imgdoubl.f:7, with PIXRPAD, source/pix/pixrpad.f:7) for a 2-D image,
 * called by IMGTOVIS (img/imgtovis.f:55) before it transforms and degrids a model: in
 * (device, ny x nx, reference pixel rpix_x, rpix_y, 1-based) is placed in out (device,
 * py x px, zero elsewhere), px = FFTPWR2(2 nx) and py = FFTPWR2(2 ny) (1 for a one-pixel
 * axis; any other px, py is refused), with left margin NINT(px/2 - RPIX) per axis, so the
 * reference pixel moves to about the centre; rpix_out (host, 2 floats, may be NULL)
 * receives the new reference pixel.  Asynchronous on the context's stream. */
int sde_image_double(sde_ctx *ctx, const float *in, int nx, int ny, float rpix_x, float rpix_y,
                     float *out, int px, int py, float *rpix_out);

/* Clark CLEAN, the default algorithm of SDE's clean task: the CLARK branch of
 * task/clean.f:147-205 and IMGCCLEA (img/imgcclea.f) on device arrays.
 *   dirty, psf  N x N images from uvmap (N a power of two, 64..8192; CRPIX = (N+1)/2, so
 *               IMGMAKEX's phase shift is zero).
 *   window      CRDHALF with BLC/TRC unset: w = N/2 pixels from N/4+1 on both axes;
 *               comp (initial components, updated), resid (final residual) and box (NULL
 *               = 1.0 everywhere) are w x w.
 *   transfer    XFR = FFTR2D(PSF) on the N x N grid; IMGRESID's residual
 *               DIRTY - FFTR2D^-1(FFTR2D(comp) * XFR) runs on it after each minor cycle.
 *   minor cycle PIX2DRCC on the list of the Numcl largest |residual| (PIXRABSH histogram,
 *               PIXFLIM limit, at least EXTSIDE * max |residual|, PIX2DRLI order), with
 *               the Bpatch x Bpatch beam patch (IMGSUBPS) and EXTSIDE the largest |PSF|
 *               outside it (PIXREXTS).
 *   cl/cx/cy    device arrays of niter entries for the component list (NULL: scratch).
 * numcl <= 32768 (the task's default); niter > 0; biter = first iteration number (1, or
 * NITER+1 of a restarted run).  An empty list ends the loop (the reference would read an
 * unwritten list entry).  Messages: 'Zero range in values', 'Too many points', 'Limit in
 * absolute value < 0.0'.  Synchronises once per major cycle. */
typedef struct {
    int niter;
    float gain, flux;
    int numcl, bpatch, biter;
} sde_clark_params;
#define SDE_CLARK_TRACE 64
typedef struct {
    int aniter, ncycles, window, blc, last_anl;
    float maxres, tflux, extside, last_slim;
    /* IMGCCLEA's message per major cycle (img/imgcclea.f:276-278), first 64 cycles:
     * list length, components so far, PIX2DRCC's MAXRES, total flux */
    int t_anl[SDE_CLARK_TRACE], t_aniter[SDE_CLARK_TRACE];
    float t_maxres[SDE_CLARK_TRACE], t_tflux[SDE_CLARK_TRACE];
} sde_clark_result;
int sde_clark(sde_ctx *ctx, const float *dirty, const float *psf, int n, const float *box,
              const sde_clark_params *p, float *comp, float *resid, float *cl, int *cx, int *cy,
              sde_clark_result *out);

/* Hogbom CLEAN that allocates nothing.  This entry point has no counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc -- hosts whose device memory
 * all comes from their own allocator or fixed arena, real-time or embedded loops that forbid
 * allocation once running, and serving loops that must never block on the allocator.  It
 * takes the same device arrays and returns the same results as sde_hogbom, on the caller's
 * stream (a cudaStream_t, 0 for the legacy stream, on the current device).  Its scratch --
 * partial maxima of at most 1024 CTAs per search, the grid barrier, status words and result
 * scalars, about 12 KB -- lives in one static device array that comes with the library's
 * device code: a GPU gets it when the library's module is loaded there (with CUDA's lazy
 * module loading, at the first call on that GPU) and keeps it until the process exits, so
 * make the first call at start-up, before an arena has taken all device memory.  The first
 * call on a device, and the first after the caller resets it, also takes that array's
 * address (cudaGetSymbolAddress).  Every call shares
 * the array and the call clears what must start at zero; calls that overlap on the GPU (two
 * streams, two host threads) race on it and must be serialised by the caller.  Windows or
 * PSFs over 2^31-1 pixels are rejected with SDE_EINVAL. */
int sde_hogbom_noalloc(void *stream, const float *drt, const float *psf, const float *box, int nx,
                       int ny, int pnx, int pny, float gain, int nsub, int bsub, float flux,
                       float tflux_in, float *cln, float *res, float *cflux, int *cx, int *cy,
                       volatile int *cancel_flag, sde_clean_result *out);

/* Index (1-based) of the first strictly largest |a| (PIXISAMA) of a device array. */

/* ---- One uvmap job in one call ----------------------------------------------------------
 * The device work of task/uvmap.f for one job: optional weighting (rmode -1: keep WT, the
 * natural weights; 0..4 as sde_weights, with the weighting scales wuscale/wvscale =
 * FOV/CDELT), plan, PSF, PSF peak, dirty image divided by the peak (task/uvmap.f:212-491),
 * from host (where = SDE_HOST) or device arrays to host or device images (out_where).  WT
 * is not modified (the weighting works on a copy).  psf may be NULL; if given it receives
 * the PSF divided by its peak.  Synchronises the context's stream before returning.
 * No counterpart entry point in the reference (uvmap is a task, not a routine). */
typedef struct {
    sde_gridspec spec;
    int nx, ny;
    int rmode;
    float robust[3];
    float ds;
    float wuscale, wvscale;
    int out_where;
} sde_uvmap_args;
typedef struct {
    float psf_peak;
    float sumwt;
    int64_t ngrid;  /* visibilities that gridded */
    int64_t ndrop;  /* dropped by the weighting (off the weighting grid) */
} sde_uvmap_result;
int sde_uvmap(sde_ctx *ctx, const sde_uvmap_args *a, int64_t nvis, const float *u, const float *v,
              const float *w, const float *vis, const float *wt, int where, float *dirty,
              float *psf, sde_uvmap_result *res);

/* ---- Batches of plans: a mosaic's pointings or a group of served jobs ------------------
 * No counterpart entry point in the reference: task/mosclean.f images its pointings one
 * after another and forms the linear mosaic (task/mosclean.f:413-432); a batch images all
 * of them together.  At most 65535 plans; every plan must come from ctx and hold a
 * power-of-two grid large enough for its nx[i] x ny[i] image.  The batch owns per plan a grid, a PSF image and a
 * dirty image (device, row-major nx x ny).
 *   sde_batch_psf      grid and transform every PSF; records each PSF peak.
 *   sde_batch_dirty    dirty image of every plan, divided by its PSF peak (uvmap's
 *                      normalisation, task/uvmap.f:473-483): one persistent gridding launch
 *                      over all plans' work items, one batched finalize, per shape one
 *                      batched column FFT and one batched row c2r with grid correction,
 *                      then the mosaic if one is set.  use_graph != 0: the launch sequence
 *                      is captured in a CUDA graph on the second call and replayed after.
 *   sde_batch_dirty_loop  the same images through sde_plan_grid + sde_image_from_grid,
 *                      one plan at a time (the per-pointing baseline).
 *   sde_batch_set_mosaic  linear mosaic mnx x mny: pointing i's image centre ((n+1)/2,
 *                      1-based) lands on mosaic pixel (cx[i], cy[i]); its primary beam is a
 *                      Gaussian of FWHM fwhm_px[i] pixels; mosaic = sum wt PB I / sum wt PB^2
 *                      where sum wt PB^2 > clip * its maximum, else 0 (the denominator
 *                      and its clip are formed here, once per layout).
 *   sde_batch_image    device pointer: i = -1 the mosaic; which 0 the dirty image of plan
 *                      i, 1 its PSF, 2 its PSF peak (one float). */
typedef struct sde_batch sde_batch;
int sde_batch_create(sde_ctx *ctx, int n, sde_plan *const *plans, const int *nx, const int *ny,
                     sde_batch **out);
int sde_batch_destroy(sde_batch *b);
int64_t sde_batch_bytes(const sde_batch *b);
int sde_batch_psf(sde_batch *b);
int sde_batch_set_mosaic(sde_batch *b, int mnx, int mny, const int *cx, const int *cy,
                         const float *fwhm_px, const float *wt, float clip);
int sde_batch_dirty(sde_batch *b, int use_graph);
int sde_batch_dirty_loop(sde_batch *b);
int sde_batch_graph_nodes(const sde_batch *b);
int sde_batch_image(const sde_batch *b, int i, int which, float **dev);
/* copy n floats of what sde_batch_image names into dst (host or device); synchronises */
int sde_batch_read(const sde_batch *b, int i, int which, float *dst, int64_t n);

int sde_isamax(sde_ctx *ctx, const float *a, int64_t n, int64_t *index_out);

/* Visibilities from a FITS random-groups file: the FTS branch of
 * VISGET(NAME, FILENAME, STOKES, ...) (vis/visget.f:7, 60-68 -> FILGRPGE, VISSTD), for one
 * Stokes parameter, into the arrays sde_plan_create takes.
 *   sde_uvfits_open     parses the header (host only, no CUDA call) and checks what
 *                       fts/ftsgrpre.f and vis/visstd.f check, with their messages
 *                       ('Not a groups file', 'No groups!', 'Cannot read N-bit files',
 *                       'First axis not COMPLEX', 'No stokes axes', 'No frequency',
 *                       'PTYPE=UU not in header', 'Unable to read such data'); groups that
 *                       hold more than one COMPLEX x STOKES block (several channels or IFs)
 *                       are refused.
 *   sde_uvfits_read     reads every group: u, v, w (nread floats each, wavelengths: PTYPE
 *                       UU/VV/WW in seconds are scaled by SNGL(FREQ)), vis (nread complex64
 *                       pairs), wt (nread floats) of Stokes stokes ('I', 'V', 'Q' or 'U';
 *                       after RR/LL/RL/LR -> I/V/Q/U conversion, vis/visconvs.f,
 *                       visconv2.f, visconvp.f), to host or device arrays of ngroups
 *                       entries per where.  A file shorter than GCOUNT groups gives
 *                       nread < ngroups and the reference's warning through msgput_
 *                       (fts/ftsgrpre.f:254-258).  Synchronises. */
typedef struct sde_uvfits sde_uvfits;
typedef struct sde_uvfits_desc {
    int64_t ngroups;         /* GCOUNT */
    int64_t ngroups_in_file; /* whole groups the file holds (<= ngroups) */
    int npar;                /* PCOUNT */
    int bitpix;              /* 16, 32 or -32 */
    int ncomplex;            /* 3: (re, im, wt); 2: (re, im) with a WEIGHT parameter */
    int nstokes;
    int iquv;                /* Stokes axis CRVAL > 0: no conversion, planes by position */
    int uvw_scaled;          /* 1: u, v, w scaled by SNGL(FREQ); 0: already in wavelengths */
    double freq;             /* CRVAL + (1 - CRPIX) * CDELT of the FREQ axis */
    double ra, dec;          /* CRVAL of the RA and DEC axes (0 when absent) */
} sde_uvfits_desc;
int sde_uvfits_open(const char *path, sde_uvfits **out);
int sde_uvfits_describe(const sde_uvfits *f, sde_uvfits_desc *d);
int sde_uvfits_read(sde_ctx *ctx, const sde_uvfits *f, int stokes, float *u, float *v, float *w,
                    float *vis, float *wt, int where, int64_t *nread);
int sde_uvfits_close(sde_uvfits *f);

#ifdef __cplusplus
}
#endif
#endif
