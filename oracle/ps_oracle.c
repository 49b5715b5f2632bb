/*
 * ps_oracle.c -- CPU restatement of the reference period_search FP64 path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker; never linked into the product).
 * Each function names the reference routine it restates, by file:line within
 * the IanSteveC/PeriodSearch project.  The floating-point expressions keep the
 * reference's evaluation order; build with -ffp-contract=off so that no FMA
 * contraction changes the rounding on targets that have FMA.
 *
 * The golden pins for this file are tests/golden/ (period_search_out of the
 * reference and the golden arrays of its unit tests) and, in the development
 * container, outputs of the reference binary built by oracle/Makefile.
 */
#include "ps_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define PI M_PI
#define TINY_MU 1e-8                 /* period_search/constants.h:10 */
#define DEG2RAD (PI / 180)           /* period_search/constants.h:17 */
#define RAD2DEG (180 / PI)           /* period_search/constants.h:18 */

static double **dmatrix(int rows, int cols)
{
    double **m = (double **)malloc(sizeof(double *) * (size_t)(rows + 1));
    double *blk = (double *)calloc((size_t)(rows + 1) * (size_t)(cols + 1), sizeof(double));
    for (int i = 0; i <= rows; i++) m[i] = blk + (size_t)i * (size_t)(cols + 1);
    return m;
}

static void dmatrix_free(double **m)
{
    if (!m) return;
    free(m[0]);
    free(m);
}

/* ------------------------------------------------------------------------ */
/* L0: facet grid, normals, basis, initial ellipsoid                        */
/* ------------------------------------------------------------------------ */

/* Vertex triplets of the standard triangulation, period_search/trifac.c:10-82.
 * nod[row][j] numbers the vertices row by row; facets are emitted octant by
 * octant, upper hemisphere first. */
void pso_trifac(int nrows, int ifp[][4])
{
    int rows = 2 * nrows + 1, cols = 4 * nrows + 1;
    int *nod = (int *)calloc((size_t)rows * (size_t)cols, sizeof(int));
#define NOD(i, j) nod[(i) * cols + (j)]
    int nnod = 1, ntri = 0;
    NOD(0, 0) = nnod;
    for (int i = 1; i <= nrows; i++)
        for (int j = 0; j <= 4 * i - 1; j++) {
            nnod++;
            NOD(i, j) = nnod;
            if (j == 0) NOD(i, 4 * i) = nnod;
        }
    for (int i = nrows - 1; i >= 1; i--)
        for (int j = 0; j <= 4 * i - 1; j++) {
            nnod++;
            NOD(2 * nrows - i, j) = nnod;
            if (j == 0) NOD(2 * nrows - i, 4 * i) = nnod;
        }
    NOD(2 * nrows, 0) = nnod + 1;

    for (int j1 = 1; j1 <= nrows; j1++)
        for (int j3 = 1; j3 <= 4; j3++) {
            int j0 = (j3 - 1) * j1;
            ntri++;
            ifp[ntri][1] = NOD(j1 - 1, j0 - (j3 - 1));
            ifp[ntri][2] = NOD(j1, j0);
            ifp[ntri][3] = NOD(j1, j0 + 1);
            for (int j2 = j0 + 1; j2 <= j0 + j1 - 1; j2++) {
                ntri++;
                ifp[ntri][1] = NOD(j1, j2);
                ifp[ntri][2] = NOD(j1 - 1, j2 - (j3 - 1));
                ifp[ntri][3] = NOD(j1 - 1, j2 - 1 - (j3 - 1));
                ntri++;
                ifp[ntri][1] = NOD(j1 - 1, j2 - (j3 - 1));
                ifp[ntri][2] = NOD(j1, j2);
                ifp[ntri][3] = NOD(j1, j2 + 1);
            }
        }
    for (int j1 = nrows + 1; j1 <= 2 * nrows; j1++)
        for (int j3 = 1; j3 <= 4; j3++) {
            int j0 = (j3 - 1) * (2 * nrows - j1);
            ntri++;
            ifp[ntri][1] = NOD(j1, j0);
            ifp[ntri][2] = NOD(j1 - 1, j0 + 1 + (j3 - 1));
            ifp[ntri][3] = NOD(j1 - 1, j0 + (j3 - 1));
            for (int j2 = j0 + 1; j2 <= j0 + (2 * nrows - j1); j2++) {
                ntri++;
                ifp[ntri][1] = NOD(j1, j2);
                ifp[ntri][2] = NOD(j1 - 1, j2 + (j3 - 1));
                ifp[ntri][3] = NOD(j1, j2 - 1);
                ntri++;
                ifp[ntri][1] = NOD(j1, j2);
                ifp[ntri][2] = NOD(j1 - 1, j2 + 1 + (j3 - 1));
                ifp[ntri][3] = NOD(j1 - 1, j2 + (j3 - 1));
            }
        }
#undef NOD
    free(nod);
}

/* Vertex directions, period_search/period_search_BOINC.cpp:509-540. */
static int vertex_grid(int nrows, double t[], double f[])
{
    double dth = PI / (2 * nrows), dph;
    int k = 1;
    t[1] = 0;
    f[1] = 0;
    for (int i = 1; i <= nrows; i++) {
        dph = PI / (2 * i);
        for (int j = 0; j <= 4 * i - 1; j++) {
            k++;
            t[k] = i * dth;
            f[k] = j * dph;
        }
    }
    for (int i = nrows - 1; i >= 1; i--) {
        dph = PI / (2 * i);
        for (int j = 0; j <= 4 * i - 1; j++) {
            k++;
            t[k] = PI - i * dth;
            f[k] = j * dph;
        }
    }
    int ndir = k + 1;
    t[ndir] = PI;
    f[ndir] = 0;
    return ndir;
}

/* Facet normals and areas, period_search/areanorm.c:10-60. */
static void areanorm(pso_shape *s)
{
    int ndir = s->ndir;
    double *x = (double *)malloc(sizeof(double) * (size_t)(ndir + 1));
    double *y = (double *)malloc(sizeof(double) * (size_t)(ndir + 1));
    double *z = (double *)malloc(sizeof(double) * (size_t)(ndir + 1));
    for (int i = 1; i <= ndir; i++) {
        double st = sin(s->t[i]);
        x[i] = st * cos(s->f[i]);
        y[i] = st * sin(s->f[i]);
        z[i] = cos(s->t[i]);
    }
    for (int i = 1; i <= s->nfac; i++) {
        double vx[4], vy[4], vz[4], c[4];
        for (int j = 2; j <= 3; j++) {
            vx[j] = x[s->ifp[i][j]] - x[s->ifp[i][1]];
            vy[j] = y[s->ifp[i][j]] - y[s->ifp[i][1]];
            vz[j] = z[s->ifp[i][j]] - z[s->ifp[i][1]];
        }
        c[1] = vy[2] * vz[3] - vy[3] * vz[2];
        c[2] = vz[2] * vx[3] - vz[3] * vx[2];
        c[3] = vx[2] * vy[3] - vx[3] * vy[2];
        double clen2 = c[1] * c[1] + c[2] * c[2] + c[3] * c[3];
        double clen = sqrt(clen2);
        s->nor[i][1] = c[1] / clen;
        s->nor[i][2] = c[2] / clen;
        s->nor[i][3] = c[3] / clen;
        s->at[i] = acos(s->nor[i][3]);
        s->af[i] = atan2(s->nor[i][2], s->nor[i][1]);
        s->darea[i] = 0.5 * clen;
    }
    free(x);
    free(y);
    free(z);
}

/* Unnormalised associated Legendre functions and the Laplace-series basis,
 * period_search/sphfunc.c:11-87. */
static void sphfunc(pso_shape *s)
{
    double aleg[PSO_MAX_LM + 1][PSO_MAX_LM + 1][PSO_MAX_LM + 1];
    int lmax = s->lmax, mmax = s->mmax;
    for (int m = 0; m <= lmax; m++)
        for (int l = 0; l <= lmax; l++)
            for (int n = 0; n <= lmax; n++) aleg[n][l][m] = 0;
    aleg[0][0][0] = 1;
    aleg[1][1][0] = 1;
    for (int l = 1; l <= lmax; l++) aleg[0][l][l] = aleg[0][l - 1][l - 1] * (2 * l - 1);
    for (int m = 0; m <= mmax; m++)
        for (int l = m + 1; l <= lmax; l++) {
            int ibot;
            if ((2 * ((l - m) / 2)) == (l - m)) {
                aleg[0][l][m] = -(l + m - 1) * aleg[0][l - 2][m] / (1 * (l - m));
                ibot = 2;
            } else
                ibot = 1;
            if (l != 1)
                for (int n = ibot; n <= l - m; n = n + 2)
                    aleg[n][l][m] = ((2 * l - 1) * aleg[n - 1][l - 1][m] - (l + m - 1) * aleg[n][l - 2][m]) /
                                    (1 * (l - m));
        }
    for (int i = 1; i <= s->nfac; i++) {
        double ts[PSO_MAX_LM + 1], tc[PSO_MAX_LM + 1];
        ts[0] = 1;
        tc[0] = 1;
        ts[1] = sin(s->at[i]);
        tc[1] = cos(s->at[i]);
        for (int j = 2; j <= lmax; j++) {
            ts[j] = ts[1] * ts[j - 1];
            tc[j] = tc[1] * tc[j - 1];
        }
        s->fs[i][0] = 0;
        s->fc[i][0] = 1;
        for (int j = 1; j <= mmax; j++) {
            s->fs[i][j] = sin(j * s->af[i]);
            s->fc[i][j] = cos(j * s->af[i]);
        }
        int k = 0;
        for (int m = 0; m <= mmax; m++)
            for (int l = m; l <= lmax; l++) {
                int ibot = ((2 * ((l - m) / 2)) == (l - m)) ? 0 : 1;
                s->pleg[i][l][m] = 0;
                for (int n = ibot; n <= l - m; n = n + 2)
                    s->pleg[i][l][m] = s->pleg[i][l][m] + aleg[n][l][m] * tc[n] * ts[m];
                k++;
                s->dsph[i][k] = s->fc[i][m] * s->pleg[i][l][m];
                if (m != 0) {
                    k++;
                    s->dsph[i][k] = s->fs[i][m] * s->pleg[i][l][m];
                }
            }
    }
}

void pso_shape_build(pso_shape *s, int nrows, int lmax, int mmax)
{
    s->nrows = nrows;
    s->lmax = lmax;
    s->mmax = mmax;
    s->ncoef = 0;
    for (int m = 0; m <= mmax; m++)
        for (int l = m; l <= lmax; l++) {
            s->ncoef++;
            if (m != 0) s->ncoef++;
        }
    s->ndir = vertex_grid(nrows, s->t, s->f);
    s->nfac = 8 * nrows * nrows;
    pso_trifac(nrows, s->ifp);
    areanorm(s);
    sphfunc(s);
}

/* Numerical-Recipes LU decomposition as used by the reference,
 * period_search/ludcmp.c:9-68.  Returns 4 where the reference exits(4). */
int pso_ludcmp(double **a, int n, int indx[], double *d)
{
    int imax = -999;
    double big, dum, sum, temp;
    double *v = (double *)malloc(sizeof(double) * (size_t)(n + 1));
    *d = 1.0;
    for (int i = 1; i <= n; i++) {
        big = 0.0;
        for (int j = 1; j <= n; j++)
            if ((temp = fabs(a[i][j])) > big) big = temp;
        if (big == 0.0) {
            free(v);
            return 4;
        }
        v[i] = 1.0 / big;
    }
    for (int j = 1; j <= n; j++) {
        for (int i = 1; i < j; i++) {
            sum = a[i][j];
            for (int k = 1; k < i; k++) sum -= a[i][k] * a[k][j];
            a[i][j] = sum;
        }
        big = 0.0;
        for (int i = j; i <= n; i++) {
            sum = a[i][j];
            for (int k = 1; k < j; k++) sum -= a[i][k] * a[k][j];
            a[i][j] = sum;
            if ((dum = v[i] * fabs(sum)) >= big) {
                big = dum;
                imax = i;
            }
        }
        if (j != imax) {
            for (int k = 1; k <= n; k++) {
                dum = a[imax][k];
                a[imax][k] = a[j][k];
                a[j][k] = dum;
            }
            *d = -(*d);
            v[imax] = v[j];
        }
        indx[j] = imax;
        if (a[j][j] == 0.0) a[j][j] = 1.0e-20;
        if (j != n) {
            dum = 1.0 / (a[j][j]);
            for (int i = j + 1; i <= n; i++) a[i][j] *= dum;
        }
    }
    free(v);
    return 0;
}

/* period_search/lubksb.c:3-24 */
void pso_lubksb(double **a, int n, const int indx[], double b[])
{
    int ii = 0;
    for (int i = 1; i <= n; i++) {
        int ip = indx[i];
        double sum = b[ip];
        b[ip] = b[i];
        if (ii)
            for (int j = ii; j <= i - 1; j++) sum -= a[i][j] * b[j];
        else if (sum)
            ii = i;
        b[i] = sum;
    }
    for (int i = n; i >= 1; i--) {
        double sum = b[i];
        for (int j = i + 1; j <= n; j++) sum -= a[i][j] * b[j];
        b[i] = sum / a[i][i];
    }
}

/* Least-squares Laplace series of the log-curvature of an ellipsoid,
 * period_search/ellfit.c:11-88. */
void pso_ellfit(const pso_shape *s, double a, double b, double c, double cg[])
{
    int ndir = s->nfac, ncoef = s->ncoef;
    int *indx = (int *)calloc((size_t)ncoef + 1, sizeof(int));
    double *fitvec = (double *)calloc((size_t)ncoef + 1, sizeof(double));
    double *er = (double *)calloc((size_t)ndir + 1, sizeof(double));
    double **fmat = dmatrix(ndir, ncoef), **fitmat = dmatrix(ncoef, ncoef);
    double d;
    for (int i = 1; i <= ndir; i++) {
        double st = sin(s->at[i]);
        double u = a * st * cos(s->af[i]), v = b * st * sin(s->af[i]), w = c * cos(s->at[i]);
        double sum = u * u + v * v + w * w;
        er[i] = 2 * (log(a * b * c) - log(sum));
    }
    for (int i = 1; i <= ndir; i++) {
        int n = 0;
        for (int m = 0; m <= s->mmax; m++)
            for (int l = m; l <= s->lmax; l++) {
                n++;
                if (m != 0) {
                    fmat[i][n] = s->pleg[i][l][m] * cos(m * s->af[i]);
                    n++;
                    fmat[i][n] = s->pleg[i][l][m] * sin(m * s->af[i]);
                } else
                    fmat[i][n] = s->pleg[i][l][m];
            }
    }
    for (int i = 1; i <= ncoef; i++) {
        for (int j = 1; j <= ncoef; j++) {
            fitmat[i][j] = 0;
            for (int k = 1; k <= ndir; k++) fitmat[i][j] = fitmat[i][j] + fmat[k][i] * fmat[k][j];
        }
        fitvec[i] = 0;
        for (int j = 1; j <= ndir; j++) fitvec[i] = fitvec[i] + fmat[j][i] * er[j];
    }
    pso_ludcmp(fitmat, ncoef, indx, &d);
    pso_lubksb(fitmat, ncoef, indx, fitvec);
    for (int i = 1; i <= ncoef; i++) cg[i] = fitvec[i];
    dmatrix_free(fitmat);
    dmatrix_free(fmat);
    free(fitvec);
    free(er);
    free(indx);
}

/* ------------------------------------------------------------------------ */
/* L1: one model evaluation                                                 */
/* ------------------------------------------------------------------------ */

/* Facet areas and area derivatives from the Laplace series, curv.c:10-39. */
void pso_curv(const pso_shape *s, pso_eval_ws *w, const double cg[])
{
    for (int i = 1; i <= s->nfac; i++) {
        double g = 0;
        int n = 0;
        for (int m = 0; m <= s->mmax; m++)
            for (int l = m; l <= s->lmax; l++) {
                n++;
                double fsum = cg[n] * s->fc[i][m];
                if (m != 0) {
                    n++;
                    fsum = fsum + cg[n] * s->fs[i][m];
                }
                g = g + s->pleg[i][l][m] * fsum;
            }
        g = exp(g);
        w->area[i] = s->darea[i] * g;
        for (int k = 1; k <= n; k++) w->dg[i][k] = g * s->dsph[i][k];
    }
}

/* Pole rotation matrix and its beta/lambda derivatives, blmatrix.c:9-46. */
void pso_blmatrix(pso_eval_ws *w, double bet, double lam)
{
    double cb = cos(bet), sb = sin(bet), cl = cos(lam), sl = sin(lam);
    w->blmat[1][1] = cb * cl;
    w->blmat[1][2] = cb * sl;
    w->blmat[1][3] = -sb;
    w->blmat[2][1] = -sl;
    w->blmat[2][2] = cl;
    w->blmat[2][3] = 0;
    w->blmat[3][1] = sb * cl;
    w->blmat[3][2] = sb * sl;
    w->blmat[3][3] = cb;
    w->dblm[1][1][1] = -sb * cl;
    w->dblm[1][1][2] = -sb * sl;
    w->dblm[1][1][3] = -cb;
    w->dblm[1][2][1] = 0;
    w->dblm[1][2][2] = 0;
    w->dblm[1][2][3] = 0;
    w->dblm[1][3][1] = cb * cl;
    w->dblm[1][3][2] = cb * sl;
    w->dblm[1][3][3] = -sb;
    w->dblm[2][1][1] = -cb * sl;
    w->dblm[2][1][2] = cb * cl;
    w->dblm[2][1][3] = 0;
    w->dblm[2][2][1] = -cl;
    w->dblm[2][2][2] = -sl;
    w->dblm[2][2][3] = 0;
    w->dblm[2][3][1] = -sb * sl;
    w->dblm[2][3][2] = sb * cl;
    w->dblm[2][3][3] = 0;
}

/* Exponential-linear phase function and its derivatives, phasec.c:11-24. */
void pso_phasec(double dcdp[], double alpha, const double p[], double *scale)
{
    double e = exp(-alpha / p[2]);
    double c = 1 + p[1] * e + p[3] * alpha;
    dcdp[1] = e;
    dcdp[2] = p[1] * e * alpha / (p[2] * p[2]);
    dcdp[3] = alpha;
    *scale = c;
}

/* Body rotation at time t and its derivatives, matrix.c:11-58. */
void pso_matrix(const pso_eval_ws *w, double omg, double t, double phi0,
                double tmat[][4], double dtm[][4][4])
{
    double fmat[4][4], dfm[4][4];
    double f = omg * t + phi0;
    f = fmod(f, 2 * PI);
    double cf = cos(f), sf = sin(f);
    fmat[1][1] = cf;
    fmat[1][2] = sf;
    fmat[1][3] = 0;
    fmat[2][1] = -sf;
    fmat[2][2] = cf;
    fmat[2][3] = 0;
    fmat[3][1] = 0;
    fmat[3][2] = 0;
    fmat[3][3] = 1;
    dfm[1][1] = -t * sf;
    dfm[1][2] = t * cf;
    dfm[1][3] = 0;
    dfm[2][1] = -t * cf;
    dfm[2][2] = -t * sf;
    dfm[2][3] = 0;
    dfm[3][1] = 0;
    dfm[3][2] = 0;
    dfm[3][3] = 0;
    for (int i = 1; i <= 3; i++)
        for (int j = 1; j <= 3; j++) {
            tmat[i][j] = 0;
            dtm[1][i][j] = 0;
            dtm[2][i][j] = 0;
            dtm[3][i][j] = 0;
            for (int k = 1; k <= 3; k++) {
                tmat[i][j] = tmat[i][j] + fmat[i][k] * w->blmat[k][j];
                dtm[1][i][j] = dtm[1][i][j] + fmat[i][k] * w->dblm[1][k][j];
                dtm[2][i][j] = dtm[2][i][j] + fmat[i][k] * w->dblm[2][k][j];
                dtm[3][i][j] = dtm[3][i][j] + dfm[i][k] * w->blmat[k][j];
            }
        }
}

/* Disk-integrated brightness of one observation and its derivatives with
 * respect to all ma parameters, bright.c:14-126. */
double pso_bright(const pso_shape *s, pso_eval_ws *w, const double ee[], const double ee0[],
                  double t, const double cg[], double dyda[], int ncoef, int nphpar, double phi0)
{
    int nf = s->nfac;
    int ncoef0 = ncoef - 2 - nphpar;
    int incl[PSO_MAX_N_FAC + 1];
    double mu[PSO_MAX_N_FAC + 1], mu0[PSO_MAX_N_FAC + 1], sv[PSO_MAX_N_FAC + 1], dbr[PSO_MAX_N_FAC + 1];
    double dsmu[PSO_MAX_N_FAC + 1], dsmu0[PSO_MAX_N_FAC + 1];
    double php[6], dphp[6], e[4], e0[4], de[4][4], de0[4][4], tmat[4][4], dtm[4][4][4];

    double cl = exp(cg[ncoef - 1]);
    double cls = cg[ncoef];
    double cos_alpha = ee[1] * ee0[1] + ee[2] * ee0[2] + ee[3] * ee0[3];
    double alpha = acos(cos_alpha);
    for (int i = 1; i <= nphpar; i++) php[i] = cg[ncoef0 + i];
    pso_phasec(dphp, alpha, php, &w->scale);
    double scale = w->scale;
    pso_matrix(w, cg[ncoef0], t, phi0, tmat, dtm);

    double br = 0;
    for (int i = 1; i <= 3; i++) {
        e[i] = 0;
        e0[i] = 0;
        for (int j = 1; j <= 3; j++) {
            e[i] = e[i] + tmat[i][j] * ee[j];
            e0[i] = e0[i] + tmat[i][j] * ee0[j];
            de[i][j] = 0;
            de0[i][j] = 0;
            for (int k = 1; k <= 3; k++) {
                de[i][j] = de[i][j] + dtm[j][i][k] * ee[k];
                de0[i][j] = de0[i][j] + dtm[j][i][k] * ee0[k];
            }
        }
    }

    for (int i = 1; i <= nf; i++) {
        incl[i] = 0;
        mu[i] = e[1] * s->nor[i][1] + e[2] * s->nor[i][2] + e[3] * s->nor[i][3];
        mu0[i] = e0[1] * s->nor[i][1] + e0[2] * s->nor[i][2] + e0[3] * s->nor[i][3];
        if ((mu[i] > TINY_MU) && (mu0[i] > TINY_MU)) {
            incl[i] = 1;
            double dnom = mu[i] + mu0[i];
            sv[i] = mu[i] * mu0[i] * (cl + cls / dnom);
            br = br + w->area[i] * sv[i];
            double q0 = mu0[i] / dnom, q = mu[i] / dnom;
            dsmu[i] = cls * (q0 * q0) + cl * mu0[i];
            dsmu0[i] = cls * (q * q) + cl * mu[i];
            dbr[i] = s->darea[i] * sv[i];
        }
    }

    for (int i = 1; i <= ncoef0 - 3; i++) {
        dyda[i] = 0;
        for (int j = 1; j <= nf; j++)
            if (incl[j] == 1) dyda[i] = dyda[i] + dbr[j] * w->dg[j][i];
        dyda[i] = scale * dyda[i];
    }

    for (int k = 1; k <= 3; k++) {
        dyda[ncoef0 - 3 + k] = 0;
        for (int i = 1; i <= nf; i++)
            if (incl[i] == 1) {
                double sum = 0, sum0 = 0;
                for (int j = 1; j <= 3; j++) {
                    sum = sum + s->nor[i][j] * de[j][k];
                    sum0 = sum0 + s->nor[i][j] * de0[j][k];
                }
                dyda[ncoef0 - 3 + k] = dyda[ncoef0 - 3 + k] + w->area[i] * (dsmu[i] * sum + dsmu0[i] * sum0);
            }
        dyda[ncoef0 - 3 + k] = scale * dyda[ncoef0 - 3 + k];
    }

    for (int i = 1; i <= nphpar; i++) dyda[ncoef0 + i] = br * dphp[i];

    dyda[ncoef - 1] = 0;
    dyda[ncoef] = 0;
    for (int i = 1; i <= nf; i++)
        if (incl[i] == 1) {
            dyda[ncoef - 1] = dyda[ncoef - 1] + mu[i] * mu0[i] * w->area[i];
            dyda[ncoef] = dyda[ncoef] + w->area[i] * mu[i] * mu0[i] / (mu[i] + mu0[i]);
        }
    dyda[ncoef - 1] = scale * dyda[ncoef - 1] * cl;
    dyda[ncoef] = scale * dyda[ncoef];

    br *= scale;
    return br;
}

/* Convexity residual row nc (1..3) and its shape derivatives, conv.c:12-29. */
double pso_conv(const pso_shape *s, const pso_eval_ws *w, int nc, double dres[], int ma)
{
    double res = 0;
    for (int j = 1; j <= ma; j++) dres[j] = 0;
    for (int i = 1; i <= s->nfac; i++) {
        res += w->area[i] * s->nor[i][nc];
        for (int j = 1; j <= s->ncoef; j++) dres[j] += s->darea[i] * w->dg[i][j] * s->nor[i][nc];
    }
    return res;
}

/* Normal equations alpha = J^T W J, beta = J^T W r and chi^2 over all
 * lightcurves, with the relative-lightcurve renormalisation,
 * period_search/mrqcof.c:16-148 (Lastcall == 0 path). */
double pso_mrqcof(const pso_problem *p, pso_eval_ws *w, const double a[], double **alpha,
                  double beta[])
{
    const pso_shape *s = p->shape;
    int ma = p->ma, nphpar = p->nphpar;
    double dyda[PSO_MAX_N_PAR + 1], dave[PSO_MAX_N_PAR + 1];
    double ave = 0, trial_chisq, ymod;
    int mfit = 0, np = 0, np1 = 0, np2 = 0;

    pso_curv(s, w, a);
    pso_blmatrix(w, a[ma - 4 - nphpar], a[ma - 3 - nphpar]);

    for (int j = 1; j <= ma; j++)
        if (p->ia[j]) mfit++;
    for (int j = 1; j <= mfit; j++) {
        for (int k = 1; k <= j; k++) alpha[j][k] = 0;
        beta[j] = 0;
    }
    trial_chisq = 0;

    for (int i = 1; i <= p->lcurves; i++) {
        if (p->inrel[i] == 1) {
            ave = 0;
            for (int l = 1; l <= ma; l++) dave[l] = 0;
        }
        for (int jp = 1; jp <= p->lpoints[i]; jp++) {
            np++;
            if (i < p->lcurves)
                ymod = pso_bright(s, w, p->ee[np], p->ee0[np], p->tim[np], a, dyda, ma, nphpar, p->phi0);
            else
                ymod = pso_conv(s, w, jp, dyda, ma);
            w->ytemp[jp] = ymod;
            if (p->inrel[i] == 1) ave = ave + ymod;
            for (int l = 1; l <= ma; l++) {
                w->dytemp[jp][l] = dyda[l];
                if (p->inrel[i] == 1) dave[l] = dave[l] + dyda[l];
            }
        }
        for (int jp = 1; jp <= p->lpoints[i]; jp++) {
            np1++;
            if (p->inrel[i] == 1) {
                double coef = p->sig[np1] * p->lpoints[i] / ave;
                for (int l = 1; l <= ma; l++)
                    w->dytemp[jp][l] = coef * (w->dytemp[jp][l] - w->ytemp[jp] * dave[l] / ave);
                w->ytemp[jp] = coef * w->ytemp[jp];
                w->dytemp[jp][1] = 0;
            }
        }
        for (int jp = 1; jp <= p->lpoints[i]; jp++) {
            ymod = w->ytemp[jp];
            np2++;
            double sig2i = 1 / (p->sig[np2] * p->sig[np2]);
            double wght = p->weight[np2];
            double dy = p->brightness[np2] - ymod;
            int j = 0;
            for (int l = 1; l <= ma; l++) {
                if (p->ia[l]) {
                    j++;
                    double wt = w->dytemp[jp][l] * sig2i * wght;
                    int k = 0;
                    for (int m = 1; m <= l; m++)
                        if (p->ia[m]) {
                            k++;
                            alpha[j][k] = alpha[j][k] + wt * w->dytemp[jp][m];
                        }
                    beta[j] = beta[j] + dy * wt;
                }
            }
            trial_chisq = trial_chisq + dy * dy * sig2i * wght;
        }
    }
    for (int j = 2; j <= mfit; j++)
        for (int k = 1; k <= j - 1; k++) alpha[k][j] = alpha[j][k];
    return trial_chisq;
}

/* Gauss-Jordan elimination with full pivoting, period_search/gauss_errc.c:9-73.
 * Returns 0, or 1 when a column would be pivoted twice, or 2 on a zero pivot. */
int pso_gauss_errc(double **a, int n, double b[])
{
    int *indxc = (int *)calloc((size_t)n + 2, sizeof(int));
    int *indxr = (int *)calloc((size_t)n + 2, sizeof(int));
    int *ipiv = (int *)calloc((size_t)n + 2, sizeof(int));
    int icol = 0, irow = 0, rc = 0;
    double big, dum, pivinv, temp;
    for (int j = 1; j <= n; j++) ipiv[j] = 0;
    for (int i = 1; i <= n && rc == 0; i++) {
        big = 0.0;
        for (int j = 1; j <= n && rc == 0; j++)
            if (ipiv[j] != 1)
                for (int k = 1; k <= n; k++) {
                    if (ipiv[k] == 0) {
                        if (fabs(a[j][k]) >= big) {
                            big = fabs(a[j][k]);
                            irow = j;
                            icol = k;
                        }
                    } else if (ipiv[k] > 1) {
                        rc = 1;
                        break;
                    }
                }
        if (rc) break;
        ++(ipiv[icol]);
        if (irow != icol) {
            for (int l = 1; l <= n; l++) {
                temp = a[irow][l];
                a[irow][l] = a[icol][l];
                a[icol][l] = temp;
            }
            temp = b[irow];
            b[irow] = b[icol];
            b[icol] = temp;
        }
        indxr[i] = irow;
        indxc[i] = icol;
        if (a[icol][icol] == 0.0) {
            rc = 2;
            break;
        }
        pivinv = 1.0 / a[icol][icol];
        a[icol][icol] = 1.0;
        for (int l = 1; l <= n; l++) a[icol][l] *= pivinv;
        b[icol] *= pivinv;
        for (int ll = 1; ll <= n; ll++)
            if (ll != icol) {
                dum = a[ll][icol];
                a[ll][icol] = 0.0;
                for (int l = 1; l <= n; l++) a[ll][l] -= a[icol][l] * dum;
                b[ll] -= b[icol] * dum;
            }
    }
    if (rc == 0)
        for (int l = n; l >= 1; l--)
            if (indxr[l] != indxc[l])
                for (int k = 1; k <= n; k++) {
                    temp = a[k][indxr[l]];
                    a[k][indxr[l]] = a[k][indxc[l]];
                    a[k][indxc[l]] = temp;
                }
    free(ipiv);
    free(indxc);
    free(indxr);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* L2: LM fit, period rows, convexity pre-pass, scan                        */
/* ------------------------------------------------------------------------ */

typedef struct lm_ws {
    pso_eval_ws *w;
    double **covar, **alpha;
    double atry[PSO_MAX_N_PAR + 1], beta[PSO_MAX_N_PAR + 1], da[PSO_MAX_N_PAR + 1];
    int mfit;
    double alamda, ochisq, chisq;
} lm_ws;

/* One LM step, period_search/mrqmin.c:11-110 (Lastcall == 0 path). */
static int mrqmin(const pso_problem *p, lm_ws *L, double a[])
{
    int ma = p->ma;
    if (L->alamda < 0) {
        L->mfit = 0;
        for (int j = 1; j <= ma; j++)
            if (p->ia[j]) L->mfit++;
        L->alamda = p->alamda_start;
        L->ochisq = pso_mrqcof(p, L->w, a, L->alpha, L->beta);
        for (int j = 1; j <= ma; j++) L->atry[j] = a[j];
    }
    for (int j = 1; j <= L->mfit; j++) {
        for (int k = 1; k <= L->mfit; k++) L->covar[j][k] = L->alpha[j][k];
        L->covar[j][j] = L->alpha[j][j] * (1 + L->alamda);
        L->da[j] = L->beta[j];
    }
    int err = pso_gauss_errc(L->covar, L->mfit, L->da);
    if (err != 0) return err;
    int j = 0;
    for (int l = 1; l <= ma; l++)
        if (p->ia[l]) {
            j++;
            L->atry[l] = a[l] + L->da[j];
        }
    double temp = pso_mrqcof(p, L->w, L->atry, L->covar, L->da);
    L->chisq = temp;
    if (temp < L->ochisq) {
        L->alamda = L->alamda / p->alamda_incr;
        for (int jj = 1; jj <= L->mfit; jj++) {
            for (int k = 1; k <= L->mfit; k++) L->alpha[jj][k] = L->covar[jj][k];
            L->beta[jj] = L->da[jj];
        }
        for (int l = 1; l <= ma; l++) a[l] = L->atry[l];
    } else {
        L->alamda = p->alamda_incr * L->alamda;
        L->chisq = L->ochisq;
    }
    return 0;
}

static const double beta_pole[PSO_N_POLES + 1] = {0, 0, 0, 0, 0, 60, 60, 60, -60, -60, -60};
static const double lambda_pole[PSO_N_POLES + 1] = {0, 0, 90, 180, 270, 60, 180, 300, 60, 180, 300};

/* One fit from initial pole `pole` (1..10) at frequency freq [1/h],
 * period_search/period_search_BOINC.cpp:817-920. */
void pso_fit(const pso_problem *p, pso_scan_state *st, double freq, int pole, pso_fit_result *res)
{
    int ncoef = p->ncoef, nphpar = p->nphpar, ma = p->ma;
    double cg[PSO_MAX_N_PAR + 1], chck[4] = {0, 0, 0, 0};
    lm_ws L;
    L.w = (pso_eval_ws *)malloc(sizeof(pso_eval_ws));
    L.covar = dmatrix(ma, ma);
    L.alpha = dmatrix(ma, ma);

    double prd = 1 / freq;
    for (int i = 1; i <= ncoef; i++) cg[i] = p->cg_first[i];
    cg[ncoef + 1] = beta_pole[pole];
    cg[ncoef + 2] = lambda_pole[pole];
    cg[ncoef + 1] = 90 - cg[ncoef + 1];
    cg[ncoef + 1] = DEG2RAD * cg[ncoef + 1];
    cg[ncoef + 2] = DEG2RAD * cg[ncoef + 2];
    cg[ncoef + 3] = 24 * 2 * PI / prd;
    for (int i = 1; i <= nphpar; i++) cg[ncoef + 3 + i] = p->par[i];
    cg[ncoef + 3 + nphpar + 2] = 1;
    cg[ncoef + 3 + nphpar + 1] = log(p->cl);

    int n_iter_max = 0, n_iter_min = p->n_iter_min;
    double iter_diff_max = -1, rchisq = -1;
    if (p->stop_condition > 1) {
        n_iter_max = (int)p->stop_condition;
        iter_diff_max = 0;
        n_iter_min = 0;
    }
    if (p->stop_condition < 1) {
        n_iter_max = PSO_MAX_N_ITER;
        iter_diff_max = p->stop_condition;
    }
    L.alamda = -1;
    L.chisq = st->chisq_carry;
    int niter = 0, last_err = 0;
    double iter_diff = 1e40, dev_old = 1e30, dev_new = 0;

    while (((niter < n_iter_max) && (iter_diff > iter_diff_max)) || (niter < n_iter_min)) {
        int err = mrqmin(p, &L, cg);
        if (err) last_err = err;
        niter++;
        if ((niter == 1) || (L.chisq < L.ochisq)) {
            L.ochisq = L.chisq;
            pso_curv(p->shape, L.w, cg);
            for (int i = 1; i <= 3; i++) {
                chck[i] = 0;
                for (int j = 1; j <= p->shape->nfac; j++) chck[i] = chck[i] + L.w->area[j] * p->shape->nor[j][i];
            }
            rchisq = L.chisq - (chck[1] * chck[1] + chck[2] * chck[2] + chck[3] * chck[3]) * (p->conw_r * p->conw_r);
        }
        dev_new = sqrt(rchisq / (p->ndata));
        if (dev_old - dev_new > 1e-10) {
            iter_diff = dev_old - dev_new;
            dev_old = dev_new;
        }
    }
    st->chisq_carry = L.chisq;

    double totarea = 0;
    for (int i = 1; i <= p->shape->nfac; i++) totarea = totarea + L.w->area[i];
    double sum = chck[1] * chck[1] + chck[2] * chck[2] + chck[3] * chck[3];
    res->dev = dev_new;
    res->dark = sqrt(sum);
    res->totarea = totarea;
    res->prd = 2 * PI / cg[ncoef + 3];
    res->la = RAD2DEG * cg[ncoef + 2];
    res->be = 90 - RAD2DEG * cg[ncoef + 1];
    res->chisq = L.chisq;
    res->niter = niter;
    res->err_code = last_err;

    dmatrix_free(L.covar);
    dmatrix_free(L.alpha);
    free(L.w);
}

/* Best pole for period index n, period_search_BOINC.cpp:583-705 (pre-pass)
 * and :807-925 (scan). */
void pso_period(const pso_problem *p, pso_scan_state *st, int n, int is_prepass, pso_row *row,
                pso_fit_result fits[PSO_N_POLES])
{
    double freq = p->freq_start - (n - 1) * p->freq_step;
    double per_best = 0, dark_best = 0, la_best = 0, be_best = 0, dev_best = 1e40;
    for (int m = 1; m <= PSO_N_POLES; m++) {
        pso_fit_result r;
        pso_fit(p, st, freq, m, &r);
        if (fits) fits[m - 1] = r;
        if (r.dev < dev_best) {
            dev_best = r.dev;
            per_best = r.prd;
            dark_best = r.dark / r.totarea * 100;
            la_best = r.la;
            be_best = r.be;
        }
    }
    if (la_best < 0) la_best += 360;
    if (is_prepass && isnan(dark_best)) dark_best = 1.0;
    row->period_h = 24 * per_best;
    row->rms = dev_best;
    row->chi2 = dev_best * dev_best * (p->ndata);
    row->dark_or_conw = dark_best;
    row->lambda_deg = la_best;
    row->beta_deg = be_best;
}

/* Shape tables, frequency grid, free-parameter mask and initial ellipsoid for
 * convexity weight conw_r, period_search_BOINC.cpp:491-575 / 721-805. */
void pso_problem_setup(pso_problem *p, double conw_r)
{
    int nd = p->ndata;
    for (int j = 1; j <= 3; j++) {
        p->brightness[nd + j] = 0;
        p->sig[nd + j] = 1 / conw_r;
    }
    p->conw_r = conw_r;
    if (!p->shape) p->shape = (pso_shape *)calloc(1, sizeof(pso_shape));
    pso_shape_build(p->shape, p->nrows, p->lmax, p->mmax);
    p->ncoef = p->shape->ncoef;
    pso_ellfit(p->shape, p->a, p->b, p->c_axis, p->cg_first);
    p->freq_start = 1 / p->per_start;
    p->freq_end = 1 / p->per_end;
    p->freq_step = 0.5 / (p->jd_max - p->jd_min) / 24 * p->per_step_coef;
    p->nphpar = 3;
    p->ma = p->ncoef + 5 + p->nphpar;
    int nc = p->ncoef;
    p->ia[nc + 1] = 1;
    p->ia[nc + 2] = 1;
    p->ia[nc + 3] = p->ia_prd;
    for (int i = 1; i <= nc; i++) p->ia[i] = 1;
    if (p->onlyrel == 1) p->ia[1] = 0;
    for (int i = 1; i <= p->nphpar; i++) p->ia[nc + 3 + i] = p->ia_par[i];
    p->ia[nc + 3 + p->nphpar + 1] = p->ia_cl;
    p->ia[nc + 3 + p->nphpar + 2] = 0;
    p->n_max = (int)((p->freq_start - p->freq_end) / p->freq_step) + 1;
}

double pso_precalc_conw(pso_problem *p, pso_scan_state *st, int *new_conw)
{
    double conw_r = p->conw / p->escl / p->escl;
    *new_conw = 0;
    while ((*new_conw != 1) && ((conw_r * p->escl * p->escl) < 10.0)) {
        pso_problem_setup(p, conw_r);
        int max_test_periods = 10;
        if (p->n_max < max_test_periods) max_test_periods = p->n_max;
        double sum_dark_facet = 0.0;
        for (int n = 1; n <= max_test_periods; n++) {
            pso_row row;
            pso_period(p, st, n, 1, &row, NULL);
            sum_dark_facet = sum_dark_facet + row.dark_or_conw;
        }
        double ave_dark_facet = sum_dark_facet / max_test_periods;
        if (ave_dark_facet < 1.0) *new_conw = 1;
        if (ave_dark_facet >= 1.0) conw_r = conw_r * 2;
    }
    return conw_r;
}

void pso_scan(pso_problem *p, pso_scan_state *st, double conw_r, int n_lo, int n_hi, pso_row *rows)
{
    pso_problem_setup(p, conw_r);
    for (int n = n_lo; n <= n_hi; n++) {
        pso_row *r = &rows[n - n_lo];
        pso_period(p, st, n, 0, r, NULL);
        if (n == 1) r->dark_or_conw = conw_r * p->escl * p->escl;
    }
}

/* ------------------------------------------------------------------------ */
/* Input file, period_search_BOINC.cpp:277-485                               */
/* ------------------------------------------------------------------------ */

static void skip_line(FILE *f)
{
    int c;
    while ((c = fgetc(f)) != EOF && c != '\n') {
    }
}

void pso_problem_free(pso_problem *p)
{
    if (!p) return;
    free(p->tim);
    free(p->brightness);
    free(p->sig);
    free(p->weight);
    free(p->ee);
    free(p->ee0);
    free(p->shape);
    free(p);
}

int pso_problem_read(const char *path, pso_problem **out)
{
    FILE *f = fopen(path, "r");
    *out = NULL;
    if (!f) return -1;
    pso_problem *p = (pso_problem *)calloc(1, sizeof(pso_problem));
    int rc = 0;
    if (fscanf(f, "%lf %lf %lf %d", &p->per_start, &p->per_step_coef, &p->per_end, &p->ia_prd) != 4) rc = 3;
    skip_line(f);
    if (fscanf(f, "%lf", &p->jd00) != 1) rc = 3;
    skip_line(f);
    if (fscanf(f, "%lf", &p->phi0_deg) != 1) rc = 3;
    skip_line(f);
    if (fscanf(f, "%lf", &p->conw) != 1) rc = 3;
    skip_line(f);
    if (fscanf(f, "%d %d", &p->lmax, &p->mmax) != 2) rc = 3;
    skip_line(f);
    if (fscanf(f, "%d", &p->nrows) != 1) rc = 3;
    skip_line(f);
    for (int i = 1; i <= 3; i++) {
        if (fscanf(f, "%lf %d", &p->par[i], &p->ia_par[i]) != 2) rc = 3;
        skip_line(f);
    }
    if (fscanf(f, "%lf %d", &p->cl, &p->ia_cl) != 2) rc = 3;
    skip_line(f);
    if (fscanf(f, "%lf", &p->stop_condition) != 1) rc = 3;
    skip_line(f);
    if (fscanf(f, "%d", &p->n_iter_min) != 1) rc = 3;
    skip_line(f);
    if (fscanf(f, "%lf", &p->alamda_incr) != 1) rc = 3;
    skip_line(f);
    if (fscanf(f, "%lf", &p->alamda_start) != 1) rc = 3;
    skip_line(f);
    int lcurves = 0;
    if (rc || fscanf(f, "%d", &lcurves) != 1) rc = 3;
    if (!rc && (lcurves > PSO_MAX_LC || lcurves < 1)) rc = 2;
    if (rc) {
        fclose(f);
        free(p);
        return rc;
    }
    p->tim = (double *)calloc(PSO_MAX_N_OBS + 4, sizeof(double));
    p->brightness = (double *)calloc(PSO_MAX_N_OBS + 4, sizeof(double));
    p->sig = (double *)calloc(PSO_MAX_N_OBS + 4, sizeof(double));
    p->weight = (double *)calloc(PSO_MAX_N_OBS + 4, sizeof(double));
    p->ee = (double(*)[4])calloc(PSO_MAX_N_OBS + 4, sizeof(double[4]));
    p->ee0 = (double(*)[4])calloc(PSO_MAX_N_OBS + 4, sizeof(double[4]));
    double al0 = PI, al0_abs = PI;
    int ial0 = -1, ial0_abs = -1, ndata = 0, k2 = 0;
    double jd_min = 1e20, jd_max = -1e40;
    p->onlyrel = 1;
    for (int i = 1; i <= lcurves && !rc; i++) {
        int i_temp = 0;
        double ave = 0;
        if (fscanf(f, "%d %d", &p->lpoints[i], &i_temp) != 2) {
            rc = 3;
            break;
        }
        skip_line(f);
        p->inrel[i] = 1 - i_temp;
        if (p->inrel[i] == 0) p->onlyrel = 0;
        if (p->lpoints[i] > PSO_POINTS_MAX || p->lpoints[i] < 1) {
            rc = 2;
            break;
        }
        for (int j = 1; j <= p->lpoints[i]; j++) {
            double e[4], e0[4];
            ndata++;
            if (ndata > PSO_MAX_N_OBS) {
                rc = 2;
                break;
            }
            if (fscanf(f, "%lf %lf", &p->tim[ndata], &p->brightness[ndata]) != 2 ||
                fscanf(f, "%lf %lf %lf", &e0[1], &e0[2], &e0[3]) != 3 ||
                fscanf(f, "%lf %lf %lf", &e[1], &e[2], &e[3]) != 3) {
                rc = 3;
                break;
            }
            if (p->tim[ndata] < jd_min) jd_min = p->tim[ndata];
            if (p->tim[ndata] > jd_max) jd_max = p->tim[ndata];
            double e0len = sqrt(e0[1] * e0[1] + e0[2] * e0[2] + e0[3] * e0[3]);
            double elen = sqrt(e[1] * e[1] + e[2] * e[2] + e[3] * e[3]);
            ave += p->brightness[ndata];
            for (int k = 1; k <= 3; k++) {
                p->ee[ndata][k] = e[k] / elen;
                p->ee0[ndata][k] = e0[k] / e0len;
            }
            if (j == 1) {
                double cos_alpha = (e[1] * e0[1] + e[2] * e0[2] + e[3] * e0[3]) / (elen * e0len);
                double al = acos(cos_alpha);
                if (al < al0) {
                    al0 = al;
                    ial0 = ndata;
                }
                if ((al < al0_abs) && (p->inrel[i] == 0)) {
                    al0_abs = al;
                    ial0_abs = ndata;
                }
            }
        }
        if (rc) break;
        ave /= p->lpoints[i];
        for (int j = 1; j <= p->lpoints[i]; j++) {
            k2++;
            p->sig[k2] = ave;
        }
    }
    if (rc) {
        fclose(f);
        pso_problem_free(p);
        return rc;
    }
    /* trailing "lc weight" pairs, period_search_BOINC.cpp:416-427 */
    double weight_lc[PSO_MAX_LC + 2];
    for (int i = 1; i <= lcurves; i++) weight_lc[i] = -1;
    for (;;) {
        int lc_number;
        double wv;
        if (fscanf(f, "%d", &lc_number) != 1) break;
        if (fscanf(f, "%lf", &wv) != 1) break;
        if (lc_number >= 1 && lc_number <= lcurves) weight_lc[lc_number] = wv;
    }
    fclose(f);

    p->jd0 = p->jd00;
    if (p->jd0 <= 0) p->jd0 = (int)jd_min;
    for (int i = 1; i <= ndata; i++) p->tim[i] = p->tim[i] - p->jd0;
    p->phi0 = p->phi0_deg * DEG2RAD;
    int k = 0;
    for (int i = 1; i <= lcurves; i++)
        for (int j = 1; j <= p->lpoints[i]; j++) {
            k++;
            p->weight[k] = (weight_lc[i] == -1) ? 1 : weight_lc[i];
        }
    for (int i = 1; i <= 3; i++) p->weight[k + i] = 1;
    if (p->onlyrel == 0) {
        al0 = al0_abs;
        ial0 = ial0_abs;
    }
    double a = 1.05, b = 1.00, c_axis = 0.95;
    double rfit = sqrt(2 * p->sig[ial0] / (0.5 * PI * (1 + cos(al0))));
    double escl = rfit / sqrt((a * b + b * c_axis + a * c_axis) / 3);
    if (p->onlyrel == 0) escl *= 0.8;
    p->a = a * escl;
    p->b = b * escl;
    p->c_axis = c_axis * escl;
    p->escl = escl;
    p->ndata = ndata;
    p->jd_min = jd_min;
    p->jd_max = jd_max;
    p->lcurves = lcurves + 1;
    p->lpoints[p->lcurves] = 3;
    p->inrel[p->lcurves] = 0;
    p->conw_r = p->conw / escl / escl;
    *out = p;
    return 0;
}

static void write_row(FILE *f, const pso_row *r)
{
    fprintf(f, "%.8f  %.6f  %.6f %4.1f %4.0f %4.0f\n", r->period_h, r->rms, r->chi2, r->dark_or_conw,
            r->lambda_deg, r->beta_deg);
}

int pso_run_file(const char *in_path, const char *out_path, int n_lo, int n_hi)
{
    pso_problem *p;
    int rc = pso_problem_read(in_path, &p);
    if (rc) return rc;
    pso_scan_state st = {0};
    int new_conw;
    double conw_r = pso_precalc_conw(p, &st, &new_conw);
    pso_problem_setup(p, conw_r);
    if (n_hi <= 0 || n_hi > p->n_max) n_hi = p->n_max;
    if (n_lo < 1) n_lo = 1;
    FILE *f = fopen(out_path, "w");
    if (!f) {
        pso_problem_free(p);
        return 1;
    }
    for (int n = n_lo; n <= n_hi; n++) {
        pso_row r;
        pso_period(p, &st, n, 0, &r, NULL);
        if (n == 1) r.dark_or_conw = conw_r * p->escl * p->escl;
        write_row(f, &r);
    }
    fclose(f);
    pso_problem_free(p);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Flat accessors for ctypes callers (tests, smoke, CPU baseline)          */
/* ------------------------------------------------------------------------ */

int pso_problem_info(const pso_problem *p, int *ndata, int *ncoef, int *ma, int *mfit, int *nfac,
                     int *n_max, double *conw_r, double *escl)
{
    int mf = 0;
    for (int j = 1; j <= p->ma; j++)
        if (p->ia[j]) mf++;
    *ndata = p->ndata;
    *ncoef = p->ncoef;
    *ma = p->ma;
    *mfit = mf;
    *nfac = p->shape ? p->shape->nfac : 0;
    *n_max = p->n_max;
    *conw_r = p->conw_r;
    *escl = p->escl;
    return 0;
}

/* mrqcof at parameters cg1 (0-based, ma values): writes alpha (mfit*mfit,
 * row-major), beta (mfit) and the facet areas (nfac); returns chi^2. */
double pso_eval_alpha(pso_problem *p, const double *cg1, double *alpha_out, double *beta_out,
                      double *area_out)
{
    int ma = p->ma, mf = 0;
    for (int j = 1; j <= ma; j++)
        if (p->ia[j]) mf++;
    double a[PSO_MAX_N_PAR + 1], beta[PSO_MAX_N_PAR + 1];
    for (int j = 1; j <= ma; j++) a[j] = cg1[j - 1];
    double **alpha = dmatrix(ma, ma);
    pso_eval_ws *w = (pso_eval_ws *)malloc(sizeof(pso_eval_ws));
    double chisq = pso_mrqcof(p, w, a, alpha, beta);
    for (int j = 1; j <= mf; j++) {
        for (int k = 1; k <= mf; k++) alpha_out[(j - 1) * mf + (k - 1)] = alpha[j][k];
        beta_out[j - 1] = beta[j];
    }
    if (area_out)
        for (int i = 1; i <= p->shape->nfac; i++) area_out[i - 1] = w->area[i];
    free(w);
    dmatrix_free(alpha);
    return chisq;
}

/* One fit; out7 = {dev, dark, totarea, prd, la, be, chisq}. */
void pso_fit_one(pso_problem *p, double freq, int pole, double *out7)
{
    pso_scan_state st = {0};
    pso_fit_result r;
    pso_fit(p, &st, freq, pole, &r);
    out7[0] = r.dev;
    out7[1] = r.dark;
    out7[2] = r.totarea;
    out7[3] = r.prd;
    out7[4] = r.la;
    out7[5] = r.be;
    out7[6] = r.chisq;
}

/* Flat export of the L0 tables for unit pins: ifp[nfac*3] (1-based vertex
 * numbers), at/af/darea[nfac], nor[nfac*3], dsph[nfac*ncoef]; 0-based. */
int pso_shape_export(int nrows, int lmax, int mmax, int *ifp, double *at, double *af, double *nor,
                     double *darea, double *dsph)
{
    pso_shape *s = (pso_shape *)calloc(1, sizeof(pso_shape));
    pso_shape_build(s, nrows, lmax, mmax);
    for (int i = 1; i <= s->nfac; i++) {
        for (int j = 1; j <= 3; j++) {
            if (ifp) ifp[(i - 1) * 3 + j - 1] = s->ifp[i][j];
            if (nor) nor[(i - 1) * 3 + j - 1] = s->nor[i][j];
        }
        if (at) at[i - 1] = s->at[i];
        if (af) af[i - 1] = s->af[i];
        if (darea) darea[i - 1] = s->darea[i];
        if (dsph)
            for (int k = 1; k <= s->ncoef; k++) dsph[(size_t)(i - 1) * s->ncoef + k - 1] = s->dsph[i][k];
    }
    int nc = s->ncoef;
    free(s);
    return nc;
}

/* Initial ellipsoid coefficients cg[ncoef] (0-based) for axes a, b, c. */
void pso_ellfit_export(int nrows, int lmax, int mmax, double a, double b, double c, double *cg)
{
    pso_shape *s = (pso_shape *)calloc(1, sizeof(pso_shape));
    pso_shape_build(s, nrows, lmax, mmax);
    double tmp[PSO_MAX_N_PAR + 1];
    pso_ellfit(s, a, b, c, tmp);
    for (int k = 1; k <= s->ncoef; k++) cg[k - 1] = tmp[k];
    free(s);
}

/* Phase function at phase angle alpha with parameters p3[3]: returns Scale,
 * derivatives in dcdp3[3]. */
double pso_phasec_export(double alpha, const double *p3, double *dcdp3)
{
    double p[4] = {0, p3[0], p3[1], p3[2]}, d[4], scale;
    pso_phasec(d, alpha, p, &scale);
    dcdp3[0] = d[1];
    dcdp3[1] = d[2];
    dcdp3[2] = d[3];
    return scale;
}

/* One observation's brightness and derivatives (bright.c:14-126) on the
 * nrows-row grid with the Laplace series of degree and order lmax, at
 * parameters cg1[ma] (0-based; ma = (lmax+1)^2 + 8, three phase parameters),
 * facet areas by curv and pole matrices by blmatrix from cg1: the
 * quantities the reference's unit test of bright() pins.  ee, ee0: unit
 * vectors [3]; dyda_out[ma] (0-based).  Test infrastructure. */
double pso_unit_bright(int nrows, int lmax, const double *cg1, const double *ee3, const double *ee03, double t,
                       double phi0, double *dyda_out)
{
    pso_shape *s = (pso_shape *)calloc(1, sizeof(pso_shape));
    pso_eval_ws *w = (pso_eval_ws *)calloc(1, sizeof(pso_eval_ws));
    pso_shape_build(s, nrows, lmax, lmax);
    const int nphpar = 3, ma = s->ncoef + 5 + nphpar;
    double cg[PSO_MAX_N_PAR + 1], dyda[PSO_MAX_N_PAR + 1], ee[4], ee0[4];
    cg[0] = 0;
    for (int k = 1; k <= ma; k++) cg[k] = cg1[k - 1];
    ee[0] = ee0[0] = 0;
    for (int k = 1; k <= 3; k++) {
        ee[k] = ee3[k - 1];
        ee0[k] = ee03[k - 1];
    }
    pso_curv(s, w, cg);
    pso_blmatrix(w, cg[ma - 4 - nphpar], cg[ma - 3 - nphpar]);
    double y = pso_bright(s, w, ee, ee0, t, cg, dyda, ma, nphpar, phi0);
    for (int k = 1; k <= ma; k++) dyda_out[k - 1] = dyda[k];
    free(w);
    free(s);
    return y;
}

/* Facet areas and g Dsph (curv.c:10-39) on the nrows-row grid with the
 * Laplace series of degree and order lmax, at shape coefficients
 * cg1[ncoef] (0-based): area_out[nfac], dg_out[nfac][ncoef] (row-major).
 * Returns nfac.  Test infrastructure. */
int pso_unit_curv(int nrows, int lmax, const double *cg1, double *area_out, double *dg_out)
{
    pso_shape *s = (pso_shape *)calloc(1, sizeof(pso_shape));
    pso_eval_ws *w = (pso_eval_ws *)calloc(1, sizeof(pso_eval_ws));
    pso_shape_build(s, nrows, lmax, lmax);
    double cg[PSO_MAX_N_PAR + 1];
    cg[0] = 0;
    for (int k = 1; k <= s->ncoef; k++) cg[k] = cg1[k - 1];
    pso_curv(s, w, cg);
    for (int i = 1; i <= s->nfac; i++) {
        area_out[i - 1] = w->area[i];
        for (int k = 1; k <= s->ncoef; k++) dg_out[(size_t)(i - 1) * s->ncoef + k - 1] = w->dg[i][k];
    }
    const int nf = s->nfac;
    free(w);
    free(s);
    return nf;
}

/* Convexity row nc (conv.c:12-29) on the same grid at parameters cg1[ma]:
 * returns the residual, derivatives in dres_out[ma] (0-based).  Test
 * infrastructure. */
double pso_unit_conv(int nrows, int lmax, const double *cg1, int nc, double *dres_out)
{
    pso_shape *s = (pso_shape *)calloc(1, sizeof(pso_shape));
    pso_eval_ws *w = (pso_eval_ws *)calloc(1, sizeof(pso_eval_ws));
    pso_shape_build(s, nrows, lmax, lmax);
    const int ma = s->ncoef + 8;
    double cg[PSO_MAX_N_PAR + 1], dres[PSO_MAX_N_PAR + 1];
    cg[0] = 0;
    for (int k = 1; k <= ma; k++) cg[k] = cg1[k - 1];
    pso_curv(s, w, cg);
    double r = pso_conv(s, w, nc, dres, ma);
    for (int k = 1; k <= ma; k++) dres_out[k - 1] = dres[k];
    free(w);
    free(s);
    return r;
}

/* Starting parameter vector (0-based, ma values) of the fit of period index
 * n from pole m, period_search_BOINC.cpp:819-844. */
void pso_initial_cg(const pso_problem *p, int n, int pole, double *cg0)
{
    int nc = p->ncoef, nph = p->nphpar;
    double freq = p->freq_start - (n - 1) * p->freq_step;
    double prd = 1 / freq;
    double cg[PSO_MAX_N_PAR + 1];
    for (int i = 1; i <= nc; i++) cg[i] = p->cg_first[i];
    cg[nc + 1] = DEG2RAD * (90 - beta_pole[pole]);
    cg[nc + 2] = DEG2RAD * lambda_pole[pole];
    cg[nc + 3] = 24 * 2 * PI / prd;
    for (int i = 1; i <= nph; i++) cg[nc + 3 + i] = p->par[i];
    cg[nc + 3 + nph + 2] = 1;
    cg[nc + 3 + nph + 1] = log(p->cl);
    for (int i = 1; i <= p->ma; i++) cg0[i - 1] = cg[i];
}

double pso_freq(const pso_problem *p, int n) { return p->freq_start - (n - 1) * p->freq_step; }
