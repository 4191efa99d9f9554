/*
 * qlpix.h -- C ABI of the GB300 pixel-image likelihood library (libqlpix.so).
 *
 * The library evaluates QLens's pixel-level log-evidence for a Cartesian
 * pixellated source: it ray-shoots the masked, split image pixels through the
 * lens model, builds the lensing matrix L on the source grid, convolves L with
 * the PSF, assembles F = L^T C^-1 L + lambda R, solves for the source
 * amplitudes and returns chi^2 plus the regularised log-evidence terms.
 *
 * Drop-in boundary: one call of qlp_eval() replaces one call of
 *   double QLens::invert_image_surface_brightness_map(double &chisq0,
 *                                                     bool verbal, int ranchisq_i)
 *   (qlens.h:944, lens.cpp:12293-13195; Cartesian branch lens.cpp:12431-12624,
 *    chi^2 loop lens.cpp:12950-13016)
 * for source_fit_mode=cartesian, ray_tracing_method=interpolate,
 * inversion_method=dense, regularization curvature (or none).  The return
 * value m2logev of qlp_result is that function's return value, chisq0 is what
 * it writes into its reference argument.
 *
 * Conventions
 *  - Plain C types only; caller-owned input and output buffers; every call
 *    returns an int status (QLP_OK = 0).  No exceptions cross the ABI.
 *  - Image arrays are indexed [i*npixels_y + j] with i along x and j along y,
 *    the layout of QLens's ImagePixelData::surface_brightness[i][j].
 *  - Lens parameters follow the QLens 'lens' command order (see qlp_lens).
 *  - One context per host thread; a context owns one CUDA stream on one GPU.
 *  - Failures the reference reports with sentinels keep those sentinels in
 *    qlp_result.m2logev (2e30 for an unusable source grid, -1e30 for missing
 *    data) and also set a distinct status code.
 */
#ifndef QLPIX_H
#define QLPIX_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define QLP_OK                   0
#define QLP_ERR_ARG              1  /* bad argument or size */
#define QLP_ERR_CUDA             2  /* CUDA runtime error (message in qlp_last_error) */
#define QLP_ERR_NOT_SPD          3  /* F or R not positive definite (reference: die) */
#define QLP_ERR_NO_SOURCE_PIXELS 4  /* no active source cell (reference: return 2e30) */
#define QLP_ERR_GRID_TOO_SMALL   5  /* source grid < 2 cells a side (reference: return 2e30) */
#define QLP_ERR_NO_DATA          6  /* no image data (reference: return -1e30) */
#define QLP_ERR_NOMEM            7  /* device allocation failed */
#define QLP_ERR_TIMEOUT          8  /* a bounded device wait ran out */
#define QLP_ERR_NO_DEVICE        9  /* no CUDA device / library built without GPU support */

/* ---- lens models ---- */
#define QLP_LENS_SPLE  0  /* p = b, alpha, s, q, theta_deg, xc, yc        (models.cpp SPLE_Lens) */
#define QLP_LENS_SHEAR 1  /* p = shear, theta_deg, xc, yc                 (models.cpp Shear) */
#define QLP_LENS_NFW   2  /* p = ks, rs, q, theta_deg, xc, yc             (models.cpp NFW) */
/* The NFW lens in QLens's mass parameterisations ('lens nfw ... pmode=1|2',
 * NFW::initialize_parameters, models.cpp:771-794): ks and rs follow from the
 * mass by NFW::set_ks_rs_from_m200_c200 / set_ks_c200_from_m200_rs
 * (models.cpp:959-976) with the lens's cosmology (qlp_lens.sigma_cr,
 * .kpc_to_arcsec, .critical_density). */
#define QLP_LENS_NFW_M200_C  3  /* p = m200 (M_sun), c200, q, theta_deg, xc, yc        (pmode=1) */
#define QLP_LENS_NFW_M200_RS 4  /* p = m200 (M_sun), rs_kpc, q, theta_deg, xc, yc      (pmode=2) */
#define QLP_MAX_LENSES 8
#define QLP_MAX_PLANES 4
#define QLP_MAX_PARAMS 8

/* ---- precision modes ---- */
#define QLP_NFW_QUADRATURE 0  /* NFW deflection by QLens's adaptive Gauss-Patterson quadrature */
#define QLP_NFW_SURROGATE  1  /* the trained MLP, quadrature where its error bound is exceeded */

#define QLP_FP64  0  /* plain FP64 everywhere */
#define QLP_MIXED 1  /* FP32-class tensor-core SYRK + Cholesky, FP64 refinement/logdet/sums */

typedef struct qlp_ctx qlp_ctx;

typedef struct {
    int type;                    /* QLP_LENS_* */
    int plane;                   /* index into qlp_planes (0 for single-plane lensing) */
    double p[QLP_MAX_PARAMS];    /* default parameters, QLens order */
    /* The cosmology at this lens's redshift, read only by the mass
     * parameterisations QLP_LENS_NFW_M200_C / _RS: the lens's
     * LensProfile::sigma_cr (M_sun/arcsec^2, for the reference source
     * redshift) and LensProfile::kpc_to_arcsec (LensProfile::setup_cosmology,
     * profile.cpp:83-91), and Cosmology::critical_density(zlens) (M_sun/Mpc^3,
     * cosmo.cpp:515). */
    double sigma_cr, kpc_to_arcsec, critical_density;
} qlp_lens;

/* Multi-plane redshift factors (QLens::deflection, lenscalc.cpp:41-80):
 * zfac[i] scales plane i's deflection; beta[i-1][j] couples plane j into
 * plane i.  n_planes = 1 with zfac[0] = 1 is ordinary single-plane lensing. */
typedef struct {
    int n_planes;
    double zfac[QLP_MAX_PLANES];
    double beta[QLP_MAX_PLANES][QLP_MAX_PLANES];
} qlp_planes;

typedef struct {
    int npixels_x, npixels_y;
    const double* xvals;               /* npixels_x+1 pixel-corner x (ImagePixelData::xvals) */
    const double* yvals;               /* npixels_y+1 pixel-corner y */
    const double* surface_brightness;  /* data, [i*npixels_y + j] */
    const double* covinv_map;          /* 1/sigma^2 per pixel, or NULL for a uniform noise */
    double background_pixel_noise;     /* used when covinv_map == NULL */
    const unsigned char* in_mask;      /* 1 = pixel is fitted */
} qlp_image;

typedef struct {
    int nx, ny;                        /* odd sizes; psf[i*ny + j] like QLens psf_matrix[i][j] */
    const double* matrix;
} qlp_psf;

typedef struct {
    int nsplit;                        /* default_imgpixel_nsplit (split_imgpixels on) */
    int npixels_x, npixels_y;          /* source-grid cells (src_npixels) */
    int auto_sourcegrid;               /* 1: bounds from ray-traced sub-pixels (find_optimal_sourcegrid) */
    double xmin, xmax, ymin, ymax;     /* fixed bounds when auto_sourcegrid == 0 */
    double limit_xmin, limit_xmax, limit_ymin, limit_ymax;  /* sourcegrid_limit_* (default +-1e30) */
    double noise_threshold;            /* QLens noise_threshold (default 0 = off) */
    double size_scale;                 /* srcgrid_size_scale (default 0 = off) */
    int regularization;                /* 0 none, 1 curvature */
    double regparam;                   /* lambda */
} qlp_srcgrid_opts;

typedef struct {
    double m2logev;       /* -2 log(evidence) (no priors): chisq0 + regterms + logdet_F */
    double chisq0;
    double logdet_F;
    double logdet_R;
    double Es_times_two;  /* s^T R s */
    double regterms;      /* lambda*Es_times_two - M*ln(lambda) - logdet_R */
    int n_active_pixels;  /* image_npixels */
    int n_active_src;     /* source_npixels (M) */
    long long L_nnz;      /* nonzeros of the pre-PSF L */
    int status;
    int refine_iters;     /* FP64 refinement sweeps used (mixed precision) */
    int nfw_fallbacks;    /* rays that took the NFW quadrature instead of the surrogate */
    double regparam;      /* the regularisation parameter used (the optimised one with
                             qlp_set_regparam_optimization on) */
    int regopt_evals;     /* -2 log(evidence) evaluations of the lambda optimisation (0 = off) */
    double outside_sb_penalty;  /* the outside-surface-brightness prior's penalty, included in
                                   m2logev (0 when the prior is off or not triggered) */
    int nfw_exact_rays;   /* surrogate rays traced again by the quadrature because their error bound
                             reached a cell edge, a cell's centre line or the grid's extremes */
} qlp_result;

/* Training of the NFW deflection surrogate (qlp_nfw_surrogate_train). */
typedef struct {
    int n_train;                 /* quadrature samples to train on (default 1 << 20) */
    int batch;                   /* samples per Adam step (default 16384) */
    int steps;                   /* Adam steps (default 30000) */
    double lr;                   /* peak learning rate: 2 % warm-up, cosine decay to 0.1 % (default 3e-3) */
    unsigned long long seed;     /* samples and initial weights (default 1) */
} qlp_surrogate_opts;

typedef struct {
    double final_loss;           /* weighted mean squared error of the last training batch */
    double val_max_rel;          /* largest relative error of G_0, G_1 on the validation grid */
    double val_mean_rel;         /* mean over the grid cells of their largest relative error */
    double cells_below_1e5;      /* fraction of cells whose bound is <= 1e-5 */
    double train_ms;             /* wall time of sample generation, training and validation */
    int n_params, n_train, steps;
} qlp_surrogate_report;

/* Per-instance description for batched evaluation (uneven masks / grids). */
typedef struct {
    int mask_id;          /* index into the masks given to qlp_set_instance_masks, or -1 = image mask */
    int src_npixels_x;    /* source-grid size for this instance */
    int src_npixels_y;
} qlp_instance;

/* Defaults for a qlp_srcgrid_opts (QLens constructor defaults, lens.cpp:185-560). */
void qlp_srcgrid_defaults(qlp_srcgrid_opts* opts);

/* Create a context: uploads the image, mask, noise and PSF to `device`.
 * Replaces QLens's ImagePixelData/ImagePixelGrid set-up
 * (pixelgrid.cpp:9622-9700, 9940-10099, set_nsplits 10898-10938). */
qlp_ctx* qlp_create(const qlp_image* image, const qlp_psf* psf,
                    const qlp_srcgrid_opts* opts, int device, int* status);

/* Lens list (QLens lens_list + lens redshift planes).  The p[] of each lens
 * are the defaults used by qlp_eval when lens_params is NULL. */
int qlp_set_lens_model(qlp_ctx* ctx, const qlp_lens* lenses, int nlens, const qlp_planes* planes);

/* QLP_FP64 or QLP_MIXED. */
int qlp_set_precision(qlp_ctx* ctx, int mode);

/* Attach the context to an existing CUDA stream (cudaStream_t as void*);
 * NULL restores the context's own stream. */
int qlp_set_stream(qlp_ctx* ctx, void* stream);

/* One likelihood evaluation.  lens_params: the concatenated p[] of every lens
 * (count given by qlp_n_params), or NULL for the model defaults.
 * regparam <= 0 uses opts->regparam.  Replaces
 * QLens::invert_image_surface_brightness_map (lens.cpp:12293). */
int qlp_eval(qlp_ctx* ctx, const double* lens_params, double regparam, qlp_result* out);

/* Maximum number of evaluations of one qlp_eval_batch that run concurrently,
 * each on its own stream with its own workspace (default 16, at most 64).
 * More slots hide the sequential parts of each evaluation behind the others
 * at the cost of one workspace per slot (about 0.5 GB for a 200x200 image,
 * 4x4 split and a 64x64 source grid in QLP_MIXED). */
int qlp_set_batch_slots(qlp_ctx* ctx, int slots);

/* on = 1 (default): qlp_eval_batch captures each slot's launch sequence once
 * as a CUDA graph, sized for the slot's capacity, and replays it for every
 * evaluation (every mask and source-grid size that fits: the kernels read the
 * actual sizes from the evaluation's parameters in device memory), so one
 * evaluation costs the host a parameter upload and one graph launch instead
 * of ~400 kernel launches.  on = 0: kernels are launched one by one and
 * qlp_stage_times reports the batch's stages.  No counterpart in the
 * reference (it has no device launches). */
int qlp_set_graphs(qlp_ctx* ctx, int on);

/* ---- launch schedule and its autotuner (no counterpart in the reference) ----
 * The knobs of the batched path's launches.  None of them changes a result:
 * every kernel sums in a fixed order whatever its CTA size or split, so all
 * schedules give the same bits; they change only the time. */
typedef struct {
    int slots;          /* evaluations in flight in qlp_eval_batch, 1..64 (default 16) */
    int ray_threads;    /* threads per CTA of the FP64 ray shooting: 64, 128 or 256 (default 256) */
    int psfx_threads;   /* threads per CTA of the mixed path's PSF-to-X build: 128, 256 or 512 (default 256) */
    int psfx_split;     /* row chunks (mode 0) or image-row bands (mode 1) per source cell: 1, 2 or 4 (default 1) */
    int psfx_mode;      /* PSF-to-X build: 0 scatters into active-row accumulators through a pixel table,
                           1 into a dense window of image rows (default: 1 for PSFs of 500 taps or more) */
} qlp_schedule;

#define QLP_TUNE_MAX_TRIALS 32
typedef struct {
    qlp_schedule best;                          /* the schedule the context now uses */
    double best_ms;                             /* device ms of the sample batch with it */
    double start_ms;                            /* ... with the schedule the context had before */
    int n_trials;
    qlp_schedule trial[QLP_TUNE_MAX_TRIALS];    /* every schedule timed, in order */
    double trial_ms[QLP_TUNE_MAX_TRIALS];
} qlp_tune_report;

int qlp_get_schedule(const qlp_ctx* ctx, qlp_schedule* out);
int qlp_set_schedule(qlp_ctx* ctx, const qlp_schedule* sched);

/* Time the sample batch (arguments as qlp_eval_batch; inst and lambdas may
 * be NULL) under candidate schedules -- coordinate descent over the knobs
 * above, each trial one warm-up batch (which also captures the graphs) and
 * `reps` timed batches, the best device time kept -- and keep the fastest
 * schedule in the context.  Fails with QLP_ERR_ARG if two schedules give
 * different results for the sample (they must not).  rep may be NULL. */
int qlp_autotune(qlp_ctx* ctx, const double* params, const double* lambdas, const qlp_instance* inst, int n,
                 int reps, qlp_tune_report* rep);

/* ---- regularisation-parameter optimisation ----
 * QLens's 'optimize_regparam on' (QLens::optimize_regularization_parameter,
 * pixelgrid.cpp:15865-15890): qlp_eval and qlp_eval_batch choose lambda per
 * evaluation by Brent's method over log10(lambda) in [minlog, maxlog]
 * (tolerance tol on log10(lambda), at most max_iter iterations; QLens's
 * defaults -3, 5, 0.01, 20), minimising chi^2 over the active pixels + the
 * regularisation terms + log det F (QLens::chisq_regparam_dense,
 * pixelgrid.cpp:16526-16700), and return the evaluation at the best lambda
 * (qlp_result.regparam, .regopt_evals).  L, L^T C^-1 L and R are built once
 * per evaluation; each trial factors F = L^T C^-1 L + lambda R.  Batched
 * evaluations advance their minimisations in lockstep, one trial per slot per
 * round.  on = 0 restores the fixed lambda.  Ignored without regularisation. */
int qlp_set_regparam_optimization(qlp_ctx* ctx, int on, double minlog, double maxlog, double tol, int max_iter);

/* Brent's minimiser that the optimisation uses (the steps of
 * QLens::brents_min_method, pixelgrid.cpp:16849-16932) on a host function:
 * *xmin = the point with the least value, *evals = evaluations.  Exposed to
 * test it against the reference's algorithm. */
int qlp_brent_min(double (*f)(double x, void* user), void* user, double ax, double bx, double tol, int max_iter,
                  double* xmin, int* evals);

/* FP64 refinement sweeps of the mixed path's source amplitudes (0..4,
 * default 1): r = D - F s in FP64 with the sparse operators, s += F32^-1 r.
 * -2 log(evidence) is stationary in s at the solution, so its error is second
 * order in the amplitude error; chisq0 alone is first order.  No counterpart
 * in the reference (it solves in FP64). */
int qlp_set_refinement(qlp_ctx* ctx, int sweeps);

/* QLens 'include_noise_term_in_loglike on' (commands.cpp:13597-13603,
 * lens.cpp:13033-13043; default off, lens.cpp:303): -2 log(evidence) gains minus the log of C^-1 summed over the
 * active pixels (noise map) or the masked-pixel count times log(1/sigma^2)
 * (uniform noise), plus the masked-pixel count times log(2 pi).  Replaces the
 * reference's QLens::include_noise_term_in_loglike flag (qlens.h:402). */
int qlp_set_noise_term(qlp_ctx* ctx, int on);

/* ---- sampler-side batching (no counterpart in the reference's serial
 * loops; its MPI groups do the same one candidate per group,
 * mcmchdr.cpp:3076-3090) ----
 * The speculative first-accept search: candidates are proposed in index order
 * (0, 1, 2, ... within one search), K at a time, evaluated in one batch, and
 * examined in index order; the search stops at the first accepted one.  It
 * gives the candidate a one-at-a-time rejection loop (UCMC::MonoSample's
 * "draw until the likelihood beats the worst live point",
 * mcmchdr.cpp:3063-3098, 3192-3248; a Metropolis step's "propose until
 * accepted", mcmchdr.cpp:439-483) would accept, provided that:
 *   - propose(i) draws everything random about candidate i (its point and any
 *     acceptance variate) and nothing else;
 *   - accept(i) only decides from what propose drew and the result;
 *   - rewind(next) puts the caller's random state back to where it was just
 *     after propose(next - 1); it is called once, when candidates at or past
 *     `next` were proposed but are discarded.
 * K is the smallest batch holding an accepted candidate with 90% chance at
 * the acceptance rate in *st (0: unknown, use k_max), clamped to
 * [k_min, k_max]; *st accumulates over searches.  accepted = -1 when none of
 * max_candidates was accepted.  A callback returning nonzero (propose) or
 * negative (accept) ends the search with QLP_ERR_ARG. */
typedef int (*qlp_propose_fn)(void* user, long index, double* lens_params, double* regparam);
typedef int (*qlp_accept_fn)(void* user, long index, const qlp_result* result);
typedef void (*qlp_rewind_fn)(void* user, long next_index);
typedef struct {
    double accept_rate;            /* accepted / examined so far (in/out) */
    long proposed, evaluated, examined, accepted, discarded, batches;
} qlp_search_state;
int qlp_speculative_search(qlp_ctx* ctx, qlp_propose_fn propose, qlp_accept_fn accept, qlp_rewind_fn rewind,
                           void* user, int k_min, int k_max, long max_candidates, qlp_search_state* st,
                           long* accepted);

/* The same search over a caller-supplied batched likelihood (n results for n
 * candidates of n_params doubles each); no device is needed. */
typedef int (*qlp_batch_eval_fn)(void* user, const double* params, const double* regparams, int n,
                                 qlp_result* out);
int qlp_speculative_search_fn(qlp_batch_eval_fn eval, void* eval_user, int n_params, qlp_propose_fn propose,
                              qlp_accept_fn accept, qlp_rewind_fn rewind, void* user, int k_min, int k_max,
                              long max_candidates, qlp_search_state* st, long* accepted);

/* ---- FITS input (the reference reads these through CFITSIO; this library
 * carries its own reader of FITS image HDUs: BITPIX 8/16/32/64/-32/-64,
 * BSCALE/BZERO).  Pixel (i, j), i along FITS axis 1 and j along axis 2, goes
 * to [i * ny + j].  No device is needed. ---- */
typedef struct {
    int bitpix, naxis;
    int has_pxsize, has_pxnoise, has_psfsig, has_zsrc, has_zlens;
    double pxsize;   /* PXSIZE: square pixel size (arcsec) */
    double pxnoise;  /* PXNOISE: uniform pixel noise */
    double psfsig;   /* PSFSIG: Gaussian PSF width */
    double zsrc, zlens;
} qlp_fits_info;

/* The 2-D image of HDU `hdu` (1 = primary) and the header keywords QLens
 * reads from data images (pixelgrid.cpp:6059-6116).  pix == NULL: sizes and
 * keywords only. */
int qlp_fits_read_image(const char* path, int hdu, double* pix, long cap, int* nx, int* ny, qlp_fits_info* info);

/* 'sbmap loadimg <file.fits>': ImagePixelData::load_data_fits
 * (pixelgrid.cpp:6016-6283).  The pixel grid: square pixels of the file's
 * PXSIZE, else of pixel_size (> 0; QLens 'data_pixel_size'), centred on the
 * origin; else the bounds [xmin, xmax] x [ymin, ymax] (QLens 'grid').  xvals
 * and yvals get nx + 1 and ny + 1 pixel edges.  All three outputs NULL: sizes
 * and keywords only. */
int qlp_load_data_fits(const char* path, int hdu, double pixel_size, double xmin, double xmax, double ymin,
                       double ymax, double* xvals, double* yvals, double* data, long cap, int* nx, int* ny,
                       qlp_fits_info* info);

/* 'sbmap loadmask <file.fits> [-add]': ImagePixelData::load_mask_fits
 * (pixelgrid.cpp:6512-6650) on the current mask (in/out, nx * ny): zero
 * pixels leave the mask (unless add), others join it; a smaller file is
 * centred on the image, a larger one is an error. */
int qlp_load_mask_fits(const char* path, int nx, int ny, int add, unsigned char* mask, int* n_in_mask);

/* 'sbmap loadnoisemap': ImagePixelData::load_noise_map_fits
 * (pixelgrid.cpp:6344-6430): covinv = 1/sigma^2 per pixel; noise_min gets
 * the smallest sigma. */
int qlp_load_noise_map_fits(const char* path, int hdu, int nx, int ny, double* covinv, double* noise_min);

/* 'sbmap loadpsf <file.fits>': QLens::load_psf_fits (pixelgrid.cpp:6737-6870):
 * the symmetric box about the central pixel holding every pixel above
 * threshold x peak (QLens 'psf_threshold', default 0.01), normalised to unit
 * sum.  psf == NULL: sizes only. */
int qlp_load_psf_fits(const char* path, double threshold, double* psf, long cap, int* pnx, int* pny);

/* QLens 'outside_sb_prior on' (lens.cpp:13063-13158; settings
 * 'outside_sb_frac_threshold' (default 0.3), 'outside_sb_noise_threshold'
 * (default -1e30: unused), 'emask_nsplit' (default 1), lens.cpp:294-296, 498).
 * After the inversion the model is re-made over the extended mask `emask`
 * (uint8 [nx*ny], ImagePixelData::extended_mask; NULL: every pixel), whose
 * pixels outside the mask split emask_nsplit ways, and PSF-convolved; the
 * largest |sb| outside the mask at or above t = max(noise_frac sigma_bg,
 * frac_threshold x the in-mask peak) adds (1 + |(sb - t)/t|)^60 - 1 to
 * m2logev (qlp_result.outside_sb_penalty).  Uses the context's own mask: a
 * batch with per-instance masks (qlp_instance.mask_id >= 0) is refused while
 * it is on. */
int qlp_set_outside_sb_prior(qlp_ctx* ctx, int on, double frac_threshold, double noise_frac,
                             const unsigned char* emask, int emask_nsplit);

/* Number of doubles in one lens-parameter vector for the current model. */
int qlp_n_params(const qlp_ctx* ctx);

/* Extra masks for batched evaluation ([n_masks][npixels_x*npixels_y]). */
int qlp_set_instance_masks(qlp_ctx* ctx, const unsigned char* masks, int n_masks);

/* Batched evaluation of n parameter vectors (nested-sampling live points,
 * T-Walk proposals): params is [n][qlp_n_params], regparams [n] (or NULL),
 * inst [n] (or NULL = image mask and opts grid for all).  Results in out[n].
 * Generalises the per-group evaluation of UCMC::MonoSample / TWalk
 * (mcmchdr.cpp:2901-3087, 820) to one device launch sequence. */
int qlp_eval_batch(qlp_ctx* ctx, const double* params, const double* regparams,
                   const qlp_instance* inst, int n, qlp_result* out);

/* Parity hooks: copy intermediates of the last qlp_eval to host buffers
 * (any pointer may be NULL; sizes are in elements and must be large enough,
 * query them with the matching n_* fields of qlp_result).
 *  srcpt_xy   [2*N_sub]  sub-pixel source points, masked pixels in j-outer /
 *                        i-inner order, sub-cells in QLens order
 *  L_rowptr   [N_pix+1], L_index [nnz], L_value [nnz]  pre-PSF L (CSR)
 *  active_index [src_nx*src_ny]  active index per cell ([j*src_nx+i]) or -1
 *  D [M], s [M], model [N_pix] */
int qlp_dump(qlp_ctx* ctx, double* srcpt_xy, int* L_rowptr, int* L_index, double* L_value,
             int* active_index, double* D, double* s, double* model);

/* Copy the first `rows` rows of the PSF-convolved dense L (row-major, M
 * columns) of the last qlp_eval. */
int qlp_dump_Lpsf(qlp_ctx* ctx, int rows, double* out);

/* Milliseconds of device time per stage of the last qlp_eval, or of the
 * last qlp_eval_batch run with graphs off (CUDA events on each evaluation's
 * stream, summed over the batch; zeros after a graph-replayed batch):
 * [0] ray shooting, [1] grid + mapping + L, [2] PSF convolution and D,
 * [3] F = L'^T C^-1 L' (the SYRK), [4] regularisation, factorisations and
 * solve, [5] model image, chi^2 and evidence.  n >= 6. */
int qlp_stage_times(qlp_ctx* ctx, float* ms, int n);

/* Device time in milliseconds from the first to the last kernel of the last
 * qlp_eval / qlp_eval_batch. */
int qlp_last_device_time(qlp_ctx* ctx, float* ms);

/* ---- learned NFW deflection (no counterpart in the reference: QLens
 * always integrates, LensProfile::deflection_numerical, profile.cpp:2359) ----
 * Defaults for qlp_nfw_surrogate_train. */
void qlp_surrogate_defaults(qlp_surrogate_opts* opts);

/* Train the NFW deflection surrogate on `device` (once per process and device;
 * every context on that device shares it): samples from the GPU quadrature,
 * Adam on the project's own forward/backward kernels, then the per-cell error
 * bounds from the tensor-core inference path.  rep may be NULL. */
int qlp_nfw_surrogate_train(int device, const qlp_surrogate_opts* opts, qlp_surrogate_report* rep);

/* QLP_NFW_QUADRATURE (default) or QLP_NFW_SURROGATE (needs a trained
 * surrogate on the context's device).  threshold_arcsec: a ray whose bound on
 * the surrogate's deflection error exceeds it takes the quadrature (<= 0
 * gives 2e-5; at 1e-4 the NFW golden case moves |log L| by up to 0.11).
 * Applies to NFW lenses with q < 1. */
int qlp_set_nfw_mode(qlp_ctx* ctx, int mode, double threshold_arcsec);

/* QLens 'integral_tolerance' (default 1e-3, LensProfile::integral_tolerance,
 * profile.cpp:1484): the relative tolerance at which the adaptive
 * Gauss-Patterson quadrature of the NFW deflection stops
 * (LensIntegral::PattersonIntegrate, profile.cpp:3830-3876).  tol <= 0
 * restores the default. */
int qlp_set_nfw_tolerance(qlp_ctx* ctx, double tol);

/* Test hooks of the surrogate.  qlp_surrogate_grad_check: one forward and
 * backward pass of the training kernels (params [50306], x [batch][3],
 * t [batch][2], both as the network sees them) -> loss and grad [50306].
 * qlp_surrogate_eval: the network through the inference path at n points
 * (log R, phi, q) [n][3] -> t [n][2] = log(G/B), with the quadrature's G [n][2],
 * the baselines B [n] and the relative error bound of each point's cell [n]
 * (infinite outside the trained domain) for the same points (G, B, bound may
 * be NULL). */
int qlp_surrogate_grad_check(int device, const float* params, const float* x, const float* t, int batch,
                             double* loss, float* grad);
int qlp_surrogate_eval(int device, const double* rho_phi_q, int n, double* t, double* G, double* B,
                       double* bound);

/* Number of kernels run by the last qlp_eval / qlp_eval_batch (launched
 * directly or replayed from a graph). */
long long qlp_last_launch_count(const qlp_ctx* ctx);

/* Bytes the last qlp_eval / qlp_eval_batch copied host -> device (the
 * per-evaluation lens model and regularisation parameter) and device -> host
 * (the per-evaluation results). */
int qlp_last_transfer_bytes(const qlp_ctx* ctx, long long* h2d, long long* d2h);

/* No counterpart in the reference (QLens allocates its matrices on every
 * call).  For callers that cannot call cudaMalloc -- a host application that
 * owns the GPU memory budget and only hands this library buffers it already
 * allocated, or a latency-critical loop that cannot afford the implicit
 * synchronisation of cudaMalloc/cudaFree -- this factors an SPD matrix
 * without allocating anything: F (n x n, row-major, leading dimension ld,
 * lower triangle read), D (n) and the outputs s (n) = F^-1 D and logdet
 * (1 double, = log det F) are caller-owned DEVICE buffers on the current
 * device.  The only scratch is a static device array sized for
 * n <= 512 (about 2.1 MB per GPU, held until the process exits); larger n
 * returns QLP_ERR_ARG.  The first call on each device looks up that array's
 * address and keeps it, so the entry point is not for use after the caller
 * resets the device (cudaDeviceReset).  The call runs on `stream`
 * (cudaStream_t as void*, NULL = default stream) and waits for it, so no
 * call may be made while any stream is being captured into a CUDA graph.
 * Every call shares the one array, so calls that overlap on the GPU (other
 * host threads, other streams) race -- serialise them.  Returns
 * QLP_ERR_NOT_SPD, with the pivot's index in qlp_last_error, if a pivot is
 * zero or negative (the reference's Cholesky_dcmp_packed,
 * pixelgrid.cpp:17071-17105, flags only negative ones); s and logdet are then
 * not meaningful. */
int qlp_spd_solve_logdet_noalloc(const double* F, int n, int ld, const double* D, double* s, double* logdet,
                                 void* stream);

/* ---- the fit drivers' likelihood (QLens::fitmodel_loglike_extended_source,
 * lens.cpp:10657-10748) ----
 * A fit parameter vector, as QLens's simplex, Powell, T-Walk and nested
 * samplers move it, mapped to the lens parameters by QLens's ParamSettings
 * (params.h): inverse transform (params.h:722-743), penalty limits (-log L =
 * 1e30 outside them, lens.cpp:10671-10680), then the evaluation, then
 *   -log L = m2logev / 2 + prior terms (params.h:810-840, of the fit
 *            parameters) + Jacobian terms (params.h:884-893, of the
 *            transformed ones).
 * QLens's Gaussian transform is not offered (QLP_ERR_ARG). */
#define QLP_TRANSFORM_NONE   0
#define QLP_TRANSFORM_LOG    1   /* x = log10(value) */
#define QLP_TRANSFORM_LINEAR 2   /* x = a value + b */
#define QLP_TRANSFORM_RATIO  3   /* x = value / value[ratio_param] */
#define QLP_PRIOR_UNIFORM 0
#define QLP_PRIOR_LOG     1
#define QLP_PRIOR_GAUSS   2
#define QLP_FIT_REGPARAM (-1)    /* qlp_fit_param.target: the regularisation parameter lambda */
typedef struct {
    int target;                  /* index into the lens-parameter vector (qlp_n_params), or QLP_FIT_REGPARAM */
    int transform;               /* QLP_TRANSFORM_* (ParamTransform::transform) */
    double a, b;                 /* linear transform */
    int ratio_param;             /* ratio transform: the fit parameter it divides by (not itself a ratio) */
    int include_jacobian;        /* add the transform's Jacobian term (ParamTransform::include_jacobian) */
    int prior;                   /* QLP_PRIOR_* (ParamPrior::prior) */
    double prior_pos, prior_sig; /* Gaussian prior */
    double prior_norm;           /* ParamSettings::prior_norms[i] (set_prior_norms, params.h:862-878), > 0
                                    for non-uniform priors */
    int use_penalty_limits;      /* ParamSettings::use_penalty_limits[i] */
    double penalty_lo, penalty_hi;
} qlp_fit_param;

/* The fit parameters of the context (n in order); the lens parameters and
 * lambda not named keep the lens model's defaults (qlp_lens.p) and
 * opts->regparam. */
int qlp_set_fit_params(qlp_ctx* ctx, const qlp_fit_param* params, int n);

/* -log L of n fit vectors ([n][n_fit]) in one batch (penalised vectors are
 * not evaluated: loglike 1e30, a zeroed result).  out may be NULL. */
int qlp_fit_loglike_batch(qlp_ctx* ctx, const double* fit_params, int n, double* loglike, qlp_result* out);

/* The host side of one fit vector, no device needed: the transformed values
 * (transformed[n]), whether the penalty limits reject it, and the prior plus
 * Jacobian terms that qlp_fit_loglike_batch adds to m2logev / 2. */
int qlp_fit_terms(const qlp_fit_param* params, int n, const double* fit_params, double* transformed, int* penalised,
                  double* terms);

/* Message of the last error on this thread ("" if none). */
const char* qlp_last_error(void);

void qlp_destroy(qlp_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* QLPIX_H */
