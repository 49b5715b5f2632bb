/*
 * ps_oracle.h -- CPU restatement of the reference period_search FP64 path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests, the smoke
 * check and the CPU-baseline leg of bench.py call it to produce the values
 * the CUDA engine is compared against.  The product (libps_gb300.so and the
 * periodsearch_gb300 package) never links or calls it.
 *
 * Every routine restates one routine of the reference base CPU build
 * (IanSteveC/PeriodSearch, directory period_search/) and keeps its
 * floating-point operation order, so that on x86-64 with glibc libm and no
 * FMA contraction the results are bit-identical to the reference binary.
 * All state that the reference keeps in globals lives in explicit structs,
 * which makes the library thread-safe (one pso_scan_state per thread).
 *
 * Arrays follow the reference's 1-based convention where they are exposed
 * (index 0 unused) so that golden arrays from the reference's unit tests
 * compare element by element.
 */
#ifndef PS_ORACLE_H
#define PS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define PSO_POINTS_MAX 1000   /* period_search/constants.h:1 */
#define PSO_MAX_N_OBS 20000   /* period_search/constants.h:2 */
#define PSO_MAX_LC 200        /* period_search/constants.h:3 */
#define PSO_MAX_N_FAC 1000    /* period_search/constants.h:5 */
#define PSO_MAX_N_ITER 100    /* period_search/constants.h:6 */
#define PSO_MAX_N_PAR 200     /* period_search/constants.h:7 */
#define PSO_MAX_LM 10         /* period_search/constants.h:8 */
#define PSO_N_POLES 10        /* period_search/constants.h:11 */

/* Per-object geometry and basis tables (L0 setup). */
typedef struct pso_shape {
    int nrows, lmax, mmax;
    int nfac, ndir, ncoef;
    int ifp[PSO_MAX_N_FAC + 1][4];               /* vertex triplets, 1-based */
    double t[PSO_MAX_N_FAC + 1], f[PSO_MAX_N_FAC + 1];   /* vertex angles */
    double at[PSO_MAX_N_FAC + 1], af[PSO_MAX_N_FAC + 1]; /* normal angles */
    double nor[PSO_MAX_N_FAC + 1][4];
    double darea[PSO_MAX_N_FAC + 1];
    double fc[PSO_MAX_N_FAC + 1][PSO_MAX_LM + 1], fs[PSO_MAX_N_FAC + 1][PSO_MAX_LM + 1];
    double pleg[PSO_MAX_N_FAC + 1][PSO_MAX_LM + 1][PSO_MAX_LM + 1];
    double dsph[PSO_MAX_N_FAC + 1][PSO_MAX_N_PAR + 1];
} pso_shape;

/* Parsed period_search_in plus the reference's input preparation. */
typedef struct pso_problem {
    /* header, period_search/period_search_BOINC.cpp:277-303 */
    double per_start, per_step_coef, per_end;
    int ia_prd;
    double jd00, phi0_deg, conw;
    int lmax, mmax, nrows;
    double par[4];
    int ia_par[4];
    double cl;
    int ia_cl;
    double stop_condition;
    int n_iter_min;
    double alamda_incr, alamda_start;
    /* lightcurves (1-based), the convexity pseudo-lightcurve appended last */
    int lcurves;                      /* including the convexity pseudo-LC */
    int lpoints[PSO_MAX_LC + 2];
    int inrel[PSO_MAX_LC + 2];
    int ndata;                        /* real points, without the 3 conv rows */
    double *tim, *brightness, *sig, *weight;  /* [ndata + 4], 1-based */
    double (*ee)[4], (*ee0)[4];               /* [ndata + 4][4], 1-based */
    /* derived */
    int onlyrel;
    double jd_min, jd_max, jd0, phi0;         /* phi0 in radians */
    double escl, a, b, c_axis;                /* ellipsoid after scaling */
    double conw_r;                            /* initial conw / escl^2 */
    double freq_start, freq_end, freq_step;
    int n_max;                                /* number of trial periods */
    int ncoef, ma, nphpar;
    int ia[PSO_MAX_N_PAR + 1];
    double cg_first[PSO_MAX_N_PAR + 1];
    pso_shape *shape;
} pso_problem;

/* Result of one LM fit (one period, one initial pole). */
typedef struct pso_fit_result {
    double dev, dark, totarea, prd, la, be, chisq;
    int niter, err_code;
} pso_fit_result;

/* One output row, period_search/period_search_BOINC.cpp:927-931. */
typedef struct pso_row {
    double period_h, rms, chi2, dark_or_conw, lambda_deg, beta_deg;
} pso_row;

/* The one piece of state the reference carries between fits: the global
 * Chisq, read on the first LM iteration when the first solve fails
 * (period_search/mrqmin.c:61-63 with period_search_BOINC.cpp:873-876). */
typedef struct pso_scan_state {
    double chisq_carry;
} pso_scan_state;

/* ---- L0 setup ---- */
void pso_trifac(int nrows, int ifp[][4]);
void pso_shape_build(pso_shape *s, int nrows, int lmax, int mmax);
void pso_ellfit(const pso_shape *s, double a, double b, double c, double cg[]);
int pso_ludcmp(double **a, int n, int indx[], double *d);
void pso_lubksb(double **a, int n, const int indx[], double b[]);

/* ---- L1 kernels on an explicit evaluation workspace ---- */
typedef struct pso_eval_ws {
    double area[PSO_MAX_N_FAC + 1];
    double dg[PSO_MAX_N_FAC + 1][PSO_MAX_N_PAR + 1];
    double blmat[4][4];
    double dblm[3][4][4];
    double scale;
    /* mrqcof scratch, period_search/mrqcof.c:22-24 */
    double ytemp[PSO_POINTS_MAX + 1];
    double dytemp[PSO_POINTS_MAX + 1][PSO_MAX_N_PAR + 1];
} pso_eval_ws;

void pso_curv(const pso_shape *s, pso_eval_ws *w, const double cg[]);
void pso_blmatrix(pso_eval_ws *w, double bet, double lam);
void pso_phasec(double dcdp[], double alpha, const double p[], double *scale);
void pso_matrix(const pso_eval_ws *w, double omg, double t, double phi0,
                double tmat[][4], double dtm[][4][4]);
double pso_bright(const pso_shape *s, pso_eval_ws *w, const double ee[], const double ee0[],
                  double t, const double cg[], double dyda[], int ma, int nphpar, double phi0);
double pso_conv(const pso_shape *s, const pso_eval_ws *w, int nc, double dres[], int ma);
double pso_mrqcof(const pso_problem *p, pso_eval_ws *w, const double a[],
                  double **alpha, double beta[]);
int pso_gauss_errc(double **a, int n, double b[]);

/* ---- L2 driver ---- */
/* Reads a period_search_in file (period_search_BOINC.cpp:277-456).
 * Returns 0 on success, 2 on a size limit, -1 when the file is missing. */
int pso_problem_read(const char *path, pso_problem **out);
/* Builds the shape tables and the fit set-up for a given convexity weight. */
void pso_problem_setup(pso_problem *p, double conw_r);
void pso_problem_free(pso_problem *p);

void pso_fit(const pso_problem *p, pso_scan_state *st, double freq, int pole,
             pso_fit_result *res);
/* Best-over-poles row for period index n (1-based); is_prepass selects the
 * NaN dark-facet rule of the convexity pre-pass. */
void pso_period(const pso_problem *p, pso_scan_state *st, int n, int is_prepass,
                pso_row *row, pso_fit_result fits[PSO_N_POLES]);
/* The convexity-weight optimisation loop, period_search_BOINC.cpp:487-715. */
double pso_precalc_conw(pso_problem *p, pso_scan_state *st, int *new_conw);
/* Rows for periods n_lo..n_hi (1-based, inclusive) at convexity weight conw_r.
 * Row 1 carries conw_r*escl^2 in its fourth column. */
void pso_scan(pso_problem *p, pso_scan_state *st, double conw_r, int n_lo, int n_hi,
              pso_row *rows);
/* Full run of one input file to an output text (period_search_out format). */
int pso_run_file(const char *in_path, const char *out_path, int n_lo, int n_hi);

/* Accessors for ctypes callers. */
int pso_problem_info(const pso_problem *p, int *ndata, int *ncoef, int *ma, int *mfit,
                     int *nfac, int *n_max, double *conw_r, double *escl);
double pso_eval_alpha(pso_problem *p, const double *cg1, double *alpha_out,
                      double *beta_out, double *area_out);
void pso_fit_one(pso_problem *p, double freq, int pole, double *out7);
int pso_shape_export(int nrows, int lmax, int mmax, int *ifp, double *at, double *af, double *nor,
                     double *darea, double *dsph);
void pso_ellfit_export(int nrows, int lmax, int mmax, double a, double b, double c, double *cg);
double pso_phasec_export(double alpha, const double *p3, double *dcdp3);
double pso_unit_bright(int nrows, int lmax, const double *cg1, const double *ee3, const double *ee03, double t,
                       double phi0, double *dyda_out);
double pso_unit_conv(int nrows, int lmax, const double *cg1, int nc, double *dres_out);
int pso_unit_curv(int nrows, int lmax, const double *cg1, double *area_out, double *dg_out);
void pso_initial_cg(const pso_problem *p, int n, int pole, double *cg0);
double pso_freq(const pso_problem *p, int n);

#ifdef __cplusplus
}
#endif
#endif
