/*
 * ps_gb300.h -- C ABI of the GB300 period-search engine.
 *
 * The engine replaces the hot path of the Asteroids@home period_search
 * application (IanSteveC/PeriodSearch): for every trial period of a scan and
 * each of the 10 fixed initial poles, a Levenberg-Marquardt fit of a convex
 * Gaussian-image shape, spin axis, phase function and Lambert weight to the
 * photometry, then the best pole per period.
 *
 * The reference has no plugin API; its in-process seam is the CUDA port's
 * host interface (period_search_cuda/period_search/start_CUDA.h:2-14), and its
 * process-level seam is the BOINC app contract (period_search_in ->
 * period_search_out, period_search_state).  This header covers both:
 *
 *   ps_prepare       <- CUDAPrepare   (start_CUDA.cu:119-238)
 *   ps_precalc_conw  <- CUDAPrecalc   (start_CUDA.cu:248-521)
 *   ps_scan          <- CUDAStart     (start_CUDA.cu:523-801)
 *   ps_destroy       <- CUDAUnprepare (start_CUDA.cu:240-246)
 *   ps_run_files     <- main() of period_search/period_search_BOINC.cpp:147-954
 *
 * Differences from the CUDA port's seam, all deliberate:
 *   - inputs are passed explicitly (ps_problem) instead of through extern
 *     globals; every array is 0-based, caller-owned and only read during the
 *     call that receives it;
 *   - errors come back as ps_status, never through exit();
 *   - rows are returned to the caller (ps_row) instead of being printed into
 *     an MFILE; ps_format_row prints the reference's exact row format;
 *   - a context is used by one host thread at a time; different contexts are
 *     independent.
 *
 * All floating-point quantities are double.  Periods are in hours, epochs in
 * Julian days, angles in degrees unless stated otherwise.
 */
#ifndef PS_GB300_H
#define PS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PS_ABI_VERSION 2
#define PS_N_POLES 10          /* period_search/constants.h:11 */
#define PS_POINTS_MAX 1000     /* points per lightcurve, period_search/constants.h:1 */
#define PS_MAX_N_OBS 20000     /* points per object, period_search/constants.h:2 */
#define PS_MAX_LC 200          /* lightcurves per object, period_search/constants.h:3 */
#define PS_MAX_N_FAC 1000      /* facets, period_search/constants.h:5 */
#define PS_MAX_N_PAR 200       /* parameters, period_search/constants.h:7 */
#define PS_MAX_LM 10           /* Laplace-series degree, period_search/constants.h:8 */

typedef enum ps_status {
    PS_OK = 0,
    PS_ERR_ARG = 1,        /* NULL pointer, inconsistent sizes, bad index range */
    PS_ERR_LIMIT = 2,      /* a reference size limit is exceeded (reference exit code 2) */
    PS_ERR_SINGULAR = 4,   /* singular ellipsoid fit (reference ludcmp exit code 4) */
    PS_ERR_IO = 5,         /* input file missing or malformed, output not writable */
    PS_ERR_CUDA = 10,      /* a CUDA runtime call failed; see ps_last_error */
    PS_ERR_NO_DEVICE = 11, /* no usable sm_103 device */
    PS_ERR_TIMEOUT = 12    /* a device-side bounded wait expired; the context stays usable */
} ps_status;

/* Arithmetic form of the fit kernels. */
typedef enum ps_form {
    PS_FORM_FP64 = 0,  /* plain FP64: the drop-in for the reference fit */
    PS_FORM_MIXED = 1  /* FP32 facet stage and contractions, FP64 phase/chi^2/solve */
} ps_form;

/* The 14-line header of period_search_in (period_search_BOINC.cpp:277-303). */
typedef struct ps_header {
    double per_start;       /* shortest trial period [h] */
    double per_step_coef;   /* period step coefficient */
    double per_end;         /* longest trial period [h] */
    int32_t ia_prd;         /* 1: period free in the fit */
    double jd00;            /* epoch of zero time; <= 0 selects floor(min JD) */
    double phi0_deg;        /* initial rotation angle [deg] */
    double conw;            /* convexity regularisation weight */
    int32_t lmax, mmax;     /* degree and order of the Laplace series */
    int32_t nrows;          /* triangulation rows per octant (8*nrows^2 facets) */
    double par[3];          /* phase function a, d, k */
    int32_t ia_par[3];      /* 1: free */
    double cl;              /* Lambert weight (Lommel-Seeliger weight is 1) */
    int32_t ia_cl;          /* 1: free */
    double stop_condition;  /* > 1: iteration count; < 1: minimum rms improvement */
    int32_t n_iter_min;     /* minimum iterations when stop_condition < 1 */
    double alamda_incr;     /* LM lambda factor */
    double alamda_start;    /* LM lambda start */
} ps_header;

/* One object's photometry, as read from period_search_in
 * (period_search_BOINC.cpp:322-456).  Points are stored lightcurve after
 * lightcurve. */
typedef struct ps_problem {
    ps_header hdr;
    int32_t n_lc;                  /* lightcurves (without the convexity rows) */
    const int32_t *lc_points;      /* [n_lc] points per lightcurve (1..PS_POINTS_MAX) */
    const int32_t *lc_calibrated;  /* [n_lc] file flag: 1 calibrated, 0 relative */
    const double *lc_weight;       /* [n_lc] weights, or NULL; -1 means "not given" */
    int32_t ndata;                 /* sum of lc_points */
    const double *jd;              /* [ndata] epochs [JD] */
    const double *brightness;      /* [ndata] reduced intensities */
    const double *sun;             /* [ndata*3] asteroid->Sun vectors [AU] */
    const double *earth;           /* [ndata*3] asteroid->Earth vectors [AU] */
} ps_problem;

/* ps_options.flags: run the mixed form's shape contraction on the SIMT
 * pipes even where the tensor-core (tcgen05) contraction applies. */
#define PS_FLAG_NO_TENSOR 1

typedef struct ps_options {
    int32_t device;        /* CUDA device ordinal */
    int32_t form;          /* ps_form */
    int32_t ctas_per_sm;   /* resident fit slots per SM; 0 = tuned default */
    int32_t flags;         /* PS_FLAG_* bits, 0 for the defaults */
} ps_options;

/* One output row (period_search_BOINC.cpp:927-931). */
typedef struct ps_row {
    double period_h;       /* best period [h] */
    double rms;            /* best rms deviation */
    double chi2;           /* rms^2 * ndata */
    double dark_or_conw;   /* dark-facet %; row of period index 1: conw_r*escl^2 */
    double lambda_deg;     /* pole longitude [deg], 0..360 */
    double beta_deg;       /* pole latitude [deg] */
} ps_row;

/* One LM fit (one period index, one initial pole). */
typedef struct ps_fit {
    double dev;            /* final rms deviation */
    double dark;           /* |sum Area*normal| of the last accepted shape */
    double totarea;        /* sum of facet areas of the last evaluated shape */
    double period_h;       /* fitted period [h] */
    double lambda_deg;     /* fitted pole longitude [deg] (not wrapped) */
    double beta_deg;       /* fitted pole latitude [deg] */
    double chisq;          /* final chi^2 (with the convexity rows) */
    int32_t niter;         /* LM iterations run */
    int32_t err_code;      /* last gauss_errc code: 0, 1 or 2 */
    double pred_dev;       /* learned prediction of the final rms (screened fits), else 0 */
    int32_t screened;      /* 1: stopped after the screening iterations */
    int32_t reserved;
} ps_fit;

/* Sizes of a prepared object. */
typedef struct ps_info {
    int32_t ndata, n_lc, ncoef, ma, mfit, nfac;
    int64_t n_max;         /* trial periods in the scan */
    double escl;           /* initial size scale */
    double conw_r0;        /* conw / escl^2 */
    double freq_start, freq_step;   /* [1/h] */
    int32_t sm_count, slots;        /* device SMs and resident fit slots */
    int64_t h2d_bytes;              /* bytes ps_prepare copied host -> device */
    int32_t tensor_cores;           /* 1 when the context's form contracts on the tensor cores */
    int32_t tile_points;            /* observations per tile of the context's form */
} ps_info;

/* Device timing of the last ps_scan / ps_fit_batch call, measured with CUDA
 * events on the context's stream around the fit kernel launches. */
typedef struct ps_timing {
    double kernel_ms;      /* fit kernel(s) */
    double total_ms;       /* kernels + result copy */
    int64_t fits;          /* fits computed */
    int64_t evals;         /* model evaluations (mrqcof calls) */
    int32_t launches;      /* kernel launches */
    int32_t cluster_size;  /* CTAs per fit of the last launch: 1, or 2..4 when FP64 fits were each spread over a
                              thread-block cluster (fewer fits than fit slots; bit-identical results) */
    int64_t lit_facets;    /* FP64 form: (point, facet) pairs on the lit side over all evaluations, the work of
                              the facet law and of the shape contraction (bright.c runs both on lit facets
                              only); 0 for the mixed form, whose tensor-core contraction is dense */
} ps_timing;

typedef struct ps_ctx ps_ctx;
typedef struct ps_input ps_input;

const char *ps_status_string(ps_status st);
int32_t ps_abi_version(void);

/* ---- period_search_in parsing (host only) ---- */
/* Parses a period_search_in file with the reference's reading rules
 * (period_search_BOINC.cpp:277-427).  *out stays owned by the library. */
ps_status ps_input_read(const char *path, ps_input **out);
/* A view of the parsed data; valid until ps_input_free. */
ps_status ps_input_problem(const ps_input *in, ps_problem *view);
void ps_input_free(ps_input *in);

/* ---- engine ---- */
/* Prepares an object on a device: input preparation, shape tables,
 * initial ellipsoid and the device-resident copies.  Replaces CUDAPrepare. */
ps_status ps_prepare(const ps_problem *prob, const ps_options *opt, ps_ctx **out);
ps_status ps_get_info(const ps_ctx *ctx, ps_info *out);
/* Convexity-weight optimisation (period_search_BOINC.cpp:487-715).  On entry
 * *conw_r is ignored; on exit it holds the final conw_r and *new_conw tells
 * whether the loop accepted it.  Its fits run in the FP64 form whatever the
 * context's form, so that every form scans at the reference's conw_r (the
 * loop compares a mean over 100 fits with a threshold).  Replaces
 * CUDAPrecalc. */
ps_status ps_precalc_conw(ps_ctx *ctx, double *conw_r, int32_t *new_conw);
/* Rows for period indices n_lo..n_hi (1-based, inclusive) at convexity weight
 * conw_r.  out has n_hi-n_lo+1 rows.  Replaces CUDAStart. */
ps_status ps_scan(ps_ctx *ctx, double conw_r, int64_t n_lo, int64_t n_hi, ps_row *out);
/* Individual fits: period index period_index[i] (1-based), pole pole[i]
 * (1..10).  out has n_fits entries. */
ps_status ps_fit_batch(ps_ctx *ctx, double conw_r, int64_t n_fits, const int64_t *period_index,
                       const int32_t *pole, ps_fit *out);
/* Allocation-free variant of ps_fit_batch.  No counterpart in the reference.
 * For callers that cannot let a library allocate device memory when it is
 * called: applications that give all device memory to their own pool
 * allocator, processes under a fixed device-memory budget, and pipelines that
 * cannot take the device-wide synchronisation of cudaMalloc/cudaFree.  The
 * call allocates nothing (no cudaMalloc, cudaFree or allocating library
 * routine): d_period_index[n_fits] (1-based period indices),
 * d_pole[n_fits] (1..10) and d_out[n_fits] are caller-owned DEVICE memory,
 * the object's tables are those ps_prepare placed on the device, and the work
 * counter and per-slot scratch come from a file-scope device array of 4 MiB
 * that every GPU loading the library reserves until the process exits.
 * The fits are enqueued on `stream` (a cudaStream_t, NULL for the default
 * stream); the call returns without waiting, and d_out is valid once the
 * stream has reached it.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress); make that first call before any
 * stream capture.  Every call shares the one array, so calls whose work
 * overlaps on the GPU (other streams, other contexts, other threads) race;
 * serialise them.  Fit slots: where ps_prepare parked the rows of the
 * relative lightcurves in shared memory (e.g. 60-point lightcurves), every
 * slot of the device runs and the array holds only the work counter.  Else
 * each slot takes a scratch block of S = (longest relative lightcurve's
 * points) * (ma + 3) doubles, rounded up to a multiple of 32, and the launch
 * runs min(device slots, floor((4 MiB - 256 B) / (8 S))) slots: 17 for a
 * 500-point relative lightcurve with ma = 57, i.e. about a ninth of a
 * GB300's 152 slots.  An object whose S exceeds the array is rejected with
 * PS_ERR_LIMIT; within the input limits (PS_POINTS_MAX points per
 * lightcurve, at most 121 coefficients) S stays below 1.1 MB, so that check
 * is a guard.  FP64 form only (a mixed-form context returns PS_ERR_ARG).
 * Entries of the device lists must be valid (period index >= 1, pole
 * 1..10); they are not checked.  ps_last_timing is not updated. */
ps_status ps_fit_batch_noalloc(ps_ctx *ctx, double conw_r, int64_t n_fits, const int64_t *d_period_index,
                               const int32_t *d_pole, ps_fit *d_out, void *stream);
/* One model evaluation (the reference's mrqcof) at parameters cg[ma]
 * (0-based, reference layout): alpha[mfit*mfit] row-major, beta[mfit],
 * area[nfac] (may be NULL); returns chi^2 through *chisq. */
ps_status ps_eval(ps_ctx *ctx, double conw_r, const double *cg, double *alpha, double *beta,
                  double *chisq, double *area);
ps_status ps_last_timing(const ps_ctx *ctx, ps_timing *out);
const char *ps_last_error(const ps_ctx *ctx);
void ps_destroy(ps_ctx *ctx);

/* Measured FMA throughput of a device (TFLOP/s, 2 flops per FMA) for FP64
 * and FP32 SIMT: the compute ceilings that bound the fit kernels. */
ps_status ps_device_fma_peaks(int32_t device, double *fp64_tflops, double *fp32_tflops);

/* ---- learned early stop ----
 * A 10-64-64-1 GELU perceptron (FP32) predicts, from the first K LM
 * iterations of a fit (K = the screening depth, a multiple of 4: log ratios
 * of the accepted chi^2 after iterations K/4, K/2, 3K/4 and K to the
 * starting chi^2, log10 lambda after the same iterations, log Ndata, log
 * trial period [h]), log(final rms / rms after K iterations).  Weights:
 * PS_MLP_FLOATS floats (input mean/std, W1[64][10], b1, W2[64][64], b2,
 * W3[64], b3, target mean/std); a network is trained for one K.  No
 * counterpart in the reference. */
#define PS_MLP_FEATURES 10
#define PS_MLP_FLOATS 4951
#define PS_TRAJ_FLOATS 16   /* features[10] after K iterations, rms after K iterations, final rms,
                               iterations, rms after 8, 16 and 32 iterations (0 if the fit stopped
                               before) */

typedef struct ps_learned_stats {
    int64_t fits_total;        /* fits of the scan (periods x 10 poles) */
    int64_t fits_screened_out; /* never run beyond the screening iterations */
    int64_t fits_completed;    /* run to the end in the mixed form, resumed from their screening
                                  state (stages 2 and 3) */
    int64_t fits_refit;        /* refitted in full in the FP64 form (stage 4) */
    int64_t evals;             /* model evaluations of all stages */
    double screen_ms, complete_ms, refit_ms;   /* kernel time of the stages */
    int64_t best_index;        /* period index of the best row */
    int64_t region_periods;    /* periods whose fits were completed (stages 2 and 3) */
    int64_t evals_screen, evals_complete, evals_refit;   /* model evaluations of each stage */
    int32_t refit_rounds;      /* FP64 refit launches */
    int32_t launches;          /* fit-kernel launches of the call */
} ps_learned_stats;

/* Full fits of periods n_lo..n_hi (10 poles each) in the context's form,
 * recording for every fit PS_TRAJ_FLOATS floats into traj (host), the
 * features after feat_iters iterations (a multiple of 4, 4..48). */
ps_status ps_trajectories(ps_ctx *ctx, double conw_r, int64_t n_lo, int64_t n_hi, int32_t feat_iters,
                          float *traj);
/* Trains the predictor on n samples (features x[n][10], targets y[n]) with
 * the engine's own CUDA kernels (mini-batch Adam on mean squared error).
 * weights: in = initial parameters with the standardisation constants set,
 * out = trained.  loss_history[epochs] may be NULL. */
ps_status ps_mlp_train(int32_t device, float *weights, const float *x, const float *y, int64_t n, int32_t epochs,
                       int32_t batch, float lr, uint64_t seed, float *loss_history);
ps_status ps_mlp_predict(int32_t device, const float *weights, const float *x, int64_t n, float *y);
/* Full-batch loss and gradient (for gradient checks); grad[PS_MLP_FLOATS]
 * holds d loss / d W1..b3 at their offsets, zero elsewhere. */
ps_status ps_mlp_grad(int32_t device, const float *weights, const float *x, const float *y, int64_t n, float *loss,
                      float *grad);
/* The screening pass alone: every fit of periods n_lo..n_hi runs
 * screen_iters LM iterations (a multiple of 4, 4..48) in the mixed form;
 * out[fit] holds the rms after them (dev), the predicted final rms
 * (pred_dev) and screened = 1.  Fit f is period n_lo + f / 10, pole
 * f % 10 + 1. */
ps_status ps_screen(ps_ctx *ctx, double conw_r, int64_t n_lo, int64_t n_hi, int32_t screen_iters,
                    const float *weights, ps_fit *out);
/* Period scan in the context's form followed by a full FP64 refit of the
 * minimum region: every period whose row lies within refit_rel (relative)
 * of the best row, or within refit_halfwidth periods of it, is refitted by
 * the plain FP64 form, repeated with the new rows until no further period
 * qualifies; each refit launch is topped up with the next-lowest rows until
 * its last wave of fit slots is full.  With the mixed form this gives the FP64 form's best period
 * and FP64 values there at close to the mixed form's cost.  Statistics in
 * the ps_learned_stats fields fits_total, fits_completed (the scan),
 * fits_refit, complete_ms (scan), refit_ms, evals, best_index.  stats may
 * be NULL. */
ps_status ps_scan_refined(ps_ctx *ctx, double conw_r, int64_t n_lo, int64_t n_hi, double refit_rel,
                          int32_t refit_halfwidth, ps_row *out, ps_learned_stats *stats);

/* Options of the learned scan (ps_scan_learned). */
typedef struct ps_learned_opts {
    int32_t screen_iters;     /* LM iterations of the screening pass (a multiple of 4, 4..48); the
                                 predictor's weights must have been trained for it */
    double margin;            /* stopping rule of the completion: periods are completed in the order of
                                 their predicted rows until the next one's predicted row times
                                 exp(-margin) lies above the best completed row */
    int32_t batch_periods;    /* periods completed per launch (0: as many as the device's fit slots hold) */
    int32_t region_halfwidth; /* the periods within region_halfwidth of the best completed row are
                                 completed too */
    double refit_rel;         /* refit in full with the FP64 form the periods within refit_rel of the
                                 best row after the completion, */
    int32_t refit_halfwidth;  /* and refit_halfwidth periods on each side of the best */
    int32_t fill_refit_waves; /* 1: top every FP64 refit launch up with the next-lowest rows (whole
                                 periods) until its last wave of fit slots is full -- no extra time, fewer
                                 refit rounds (ps_scan_refined always does); 0: refit exactly the set */
} ps_learned_opts;

/* Period scan with the learned early stop, a cascade in which only the fits
 * that can matter run to the end: (1) every fit runs screen_iters LM
 * iterations in the mixed form, the predictor estimates its final rms and
 * its LM state is kept on the device; (2) periods are completed -- all ten
 * poles resumed from their saved states, continuing exactly as
 * uninterrupted fits -- in the order of their predicted rows (the lowest
 * prediction of their poles), launch by launch, until no remaining period's
 * predicted row, lowered by the margin, can beat the best completed row:
 * the fits that cannot beat the current best are stopped after screening;
 * (3) the periods around the best completed row are completed; (4) the
 * minimum region is refitted in full by the plain FP64 form (as in
 * ps_scan_refined), so that the reported minimum carries FP64 values.  Rows
 * of periods that stopped at screening carry their screened fits' rms
 * (above what full fits reach).  opts NULL selects the defaults
 * (screen_iters 8, margin 0.02, batch from the slots, region +-2 periods,
 * FP64 refit 0.5 % and +-2 periods, refit waves filled).  stats may be
 * NULL. */
ps_status ps_scan_learned(ps_ctx *ctx, double conw_r, int64_t n_lo, int64_t n_hi, const float *weights,
                          const ps_learned_opts *opts, ps_row *out, ps_learned_stats *stats);

/* Self-test of the tensor-core primitives of the mixed form (tcgen05 TF32
 * MMA with A in Tensor Memory and B in shared memory): D = A * B^T for A
 * 128 x K and B 32 x K (row-major FP32, rounded to TF32 on the device),
 * D 128 x 32, K a multiple of 8 up to 480.  PS_ERR_TIMEOUT when the MMA
 * completion was not observed within the wait limit. */
ps_status ps_tc_selftest(int32_t device, const float *A, const float *B, int32_t K, float *D);

/* The same with FP16 operands (tcgen05 kind::f16, two elements per Tensor
 * Memory column, K = 16 per MMA): A and B rounded to FP16 on the device, K a
 * multiple of 16 up to 960. */
ps_status ps_tc_selftest_f16(int32_t device, const float *A, const float *B, int32_t K, float *D);

/* The bounded-wait path of the tensor-core kernels, run on purpose: one CTA
 * holds Tensor Memory and waits on an mbarrier phase that nothing completes
 * (no MMA issued, nothing in flight), gives up after max_polls polls
 * (1 .. 2^22), then frees its Tensor Memory and returns.  PS_ERR_TIMEOUT is
 * the expected result; the context stays usable.  No counterpart in the
 * reference (the CUDA port's kernels have no bounded waits). */
ps_status ps_tc_wait_selftest(int32_t device, int32_t max_polls);

/* ---- the reference's prepared state (CUDA port host calls) ---- */

/* One object as the reference's main() holds it after reading and
 * preparing period_search_in (period_search_BOINC.cpp:343-600): for callers
 * that have done that work themselves, such as the drop-in adaptor of the
 * CUDA port's CUDAPrepare / CUDAPrecalc / CUDAStart.  Arrays are 0-based
 * and read during the call only. */
typedef struct ps_state {
    int32_t lmax, mmax, nrows;        /* Laplace series and facet grid */
    int32_t n_lc;                     /* real lightcurves */
    const int32_t *lc_points;         /* [n_lc] */
    const int32_t *lc_rel;            /* [n_lc] 1 = relative */
    int32_t ndata;                    /* real points */
    const double *tim;                /* [ndata] JD minus the epoch */
    const double *brightness, *sig, *weight;    /* [ndata] */
    const double *ee, *ee0;           /* [ndata * 3] unit vectors asteroid -> Earth / Sun */
    double phi0;                      /* initial rotation angle [rad] */
    double par[3], cl;                /* phase function and Lambert weight start values */
    double alamda_start, alamda_incr;
    double stop_condition;
    int32_t n_iter_min;
    const int32_t *ia;                /* [ncoef + 8] free flags in the reference's parameter order */
    const double *cg_first;           /* [ncoef] initial shape coefficients */
    double escl;                      /* size scale of the initial ellipsoid */
    double freq_start, freq_end, freq_step;     /* [1/h] */
    double conw_r;                    /* initial convexity weight / escl^2 */
} ps_state;

ps_status ps_prepare_state(const ps_state *state, const ps_options *opt, ps_ctx **out);

/* One round of the convexity-weight pre-pass at *conw_r (the CUDA port's
 * CUDAPrecalc, start_CUDA.cu:248-521): fits the first min(10, n_max)
 * periods in the FP64 form, then sets *new_conw = 1 when their mean
 * dark-facet statistic is below 1, else doubles *conw_r.  ps_precalc_conw
 * repeats it. */
ps_status ps_precalc_step(ps_ctx *ctx, double *conw_r, int32_t *new_conw);

/* ---- autotuner ---- */

/* One kernel configuration tried by ps_autotune. */
typedef struct ps_tune_candidate {
    int32_t basis;         /* 0: basis in L2, 1: in shared memory (SIMT contraction), 2: tensor cores */
    int32_t tile_points;   /* observations per tile */
    int32_t ctas_per_sm;   /* fit slots per SM */
    int32_t slots;         /* fit slots on the device */
    double fits_per_s;     /* measured on the sample (fits of sample_iters LM iterations) */
} ps_tune_candidate;

#define PS_TUNE_MAX 16
typedef struct ps_tune_report {
    int32_t n;             /* candidates measured */
    int32_t chosen;        /* index of the fastest, now the context's plan */
    int32_t sample_fits, sample_iters;
    ps_tune_candidate cand[PS_TUNE_MAX];
} ps_tune_report;

/* Times every kernel configuration that the object admits for the
 * context's form -- basis placement (tensor cores, shared memory, L2), tile
 * size and fit slots per SM -- on a sample of fits spread over the scan
 * (sample_fits, 0: two waves of the default plan; each fit stopped after
 * sample_iters LM iterations, 0: 6) and keeps the fastest as the context's
 * plan.  Results of all forms' kernels are valid under every
 * configuration; the mixed form's values differ between configurations
 * within its parity tolerance. */
ps_status ps_autotune(ps_ctx *ctx, double conw_r, int32_t sample_fits, int32_t sample_iters, ps_tune_report *report);

/* ---- multi-object packing ---- */

/* Many small objects (work units of a multi-object run) fitted by one
 * persistent launch with one device work queue.  The contexts must be
 * prepared on the same device with identical shape tables (nrows, Lmax,
 * Mmax) and free-parameter layout; each keeps its own photometry, period
 * grid and convexity weight.  The pack borrows the contexts' device tables:
 * destroy it before them. */
typedef struct ps_pack ps_pack;

ps_status ps_pack_create(ps_ctx *const *ctxs, int32_t n_objects, int32_t form, ps_pack **out);

/* Fits n_fits units (object index into the create-time list, 1-based period
 * index of that object's grid, pole 1..10) with conw_r[object] as each
 * object's convexity weight.  Units are dispatched largest object first
 * (Ndata) for load balance; out[] is in the caller's order. */
ps_status ps_pack_fit(ps_pack *pack, const double *conw_r, int64_t n_fits, const int32_t *object,
                      const int64_t *period_index, const int32_t *pole, ps_fit *out);
/* The learned stop's screening pass over packed units (ps_screen for many
 * objects): every unit runs screen_iters LM iterations, out[] holds the rms
 * after them (dev) and the predictor's estimate of the final rms
 * (pred_dev). */
ps_status ps_pack_screen(ps_pack *pack, const double *conw_r, int64_t n_fits, const int32_t *object,
                         const int64_t *period_index, const int32_t *pole, int32_t screen_iters,
                         const float *weights, ps_fit *out);
/* Full fits of packed units recording PS_TRAJ_FLOATS floats per unit into
 * traj (host, caller's order), as ps_trajectories does for one object. */
ps_status ps_pack_trajectories(ps_pack *pack, const double *conw_r, int64_t n_fits, const int32_t *object,
                               const int64_t *period_index, const int32_t *pole, int32_t feat_iters, float *traj,
                               ps_fit *out);

/* Device timing of the last packed launch. */
ps_status ps_pack_timing(const ps_pack *pack, ps_timing *out);
const char *ps_pack_last_error(const ps_pack *pack);
void ps_pack_destroy(ps_pack *pack);

/* ---- replica validator ---- */

/* Agreement of two replicas of one work unit under the project's validator
 * rule (validator/period_search_validator4.cpp:71-109): same number of
 * entries (at least one) and, on every entry, |(a - b) / (a + b)| / 2
 * within tol = {period 0.1, rms 0.1, chi^2 0.5}. */
typedef struct ps_validate_report {
    int32_t match;            /* 1 when the replicas agree */
    int32_t mismatch_column;  /* column of the first failing entry: 0 period, 1 rms, 2 chi^2; -1 none */
    int64_t entries_a, entries_b;
    int64_t first_mismatch;   /* 0-based entry of the first failure, -1 none */
    double max_dev[3];        /* largest |(a - b) / (a + b)| / 2 per column over all compared entries */
    int64_t argmax_dev[3];    /* entry where it occurs, -1 none */
    int32_t parse_error_a;    /* the reader rejected file a (ps_validate_files) */
    int32_t parse_error_b;
} ps_validate_report;

/* Rows as ps_scan returns them.  tol NULL selects the validator's
 * tolerances. */
ps_status ps_validate_rows(const ps_row *a, int64_t na, const ps_row *b, int64_t nb, const double *tol,
                           ps_validate_report *report);

/* period_search_out files, read the way the validator reads them: fscanf
 * of six numbers until end of file; a partial entry or a NaN period, rms or
 * chi^2 rejects the file (parse_error_*, match 0); the end-of-file read
 * repeats the last entry, so a file ending in a newline has one entry more
 * than rows.  An empty file is rejected.  PS_ERR_IO when a file cannot be
 * opened. */
ps_status ps_validate_files(const char *path_a, const char *path_b, const double *tol,
                            ps_validate_report *report);

/* ---- formats ---- */
/* Writes one row in the reference's format "%.8f  %.6f  %.6f %4.1f %4.0f %4.0f\n"
 * (period_search_BOINC.cpp:928,931).  Returns the number of characters. */
int32_t ps_format_row(const ps_row *row, char *buf, size_t len);
/* Rows of n_periods periods from their fits (PS_N_POLES consecutive fits per
 * period, poles 1..10): the best pole by rms, its period, pole and dark-facet
 * % (period_search_BOINC.cpp:913-931); chi^2 = rms^2 * ndata.  The reduction
 * ps_scan applies, for callers that run the fits with ps_fit_batch. */
ps_status ps_rows_from_fits(const ps_fit *fits, int64_t n_periods, int32_t ndata, ps_row *out);

/* ---- process-level drop-in ---- */
/* Runs the BOINC app's job on files: reads in_path (period_search_in), resumes
 * from state_path (period_search_state, optional) and writes or appends rows
 * to out_path (period_search_out), checkpointing every checkpoint_rows rows
 * (0 = only at the end).  Mirrors period_search_BOINC.cpp:218-954. */
ps_status ps_run_files(const char *in_path, const char *out_path, const char *state_path,
                       const ps_options *opt, int32_t checkpoint_rows);

/* ---- shape tables (host only) ---- */
/* Facet normals nor[nfac*3], facet areas darea[nfac] and the Laplace-series
 * basis dsph[nfac*ncoef] of the trifac grid (trifac.c, areanorm.c,
 * sphfunc.c).  Sizes: nfac = 8*nrows^2, ncoef = sum over m of the (l,m)
 * pairs with cos and sin terms.  Any output may be NULL. */
ps_status ps_shape_tables(int32_t nrows, int32_t lmax, int32_t mmax, int32_t *nfac,
                          int32_t *ncoef, double *nor, double *darea, double *dsph);

#ifdef __cplusplus
}
#endif
#endif
