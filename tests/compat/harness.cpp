// Test program standing in for the CUDA port's main()
// (period_search_cuda/period_search/period_search_BOINC.cpp:583-834): the
// reference's input preparation comes from the oracle (pinned to the
// reference binary), the globals are filled as the port fills them, and the
// port's call sequence -- CUDAPrepare, the convexity-weight loop around
// CUDAPrecalc, CUDAStart, CUDAUnprepare -- runs against the drop-in adaptor.
//
//     harness period_search_in period_search_out period_search_state
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "boinc_api.h"
#include "mfile.h"
#include "ps_oracle.h"
#include "start_CUDA.h"

// the port's globals (globals.h), defined here as its main program does
int l_max, m_max, n_coef, num_fac, l_curves, n_ph_par, l_points[PSO_MAX_LC + 2], in_rel[PSO_MAX_LC + 2], max_l_points;
double weight[PSO_MAX_N_OBS + 4];

static const char *g_state_path = "period_search_state";

// the port's checkpoint: the number of rows written (period_search_BOINC.cpp:96-125)
int DoCheckpoint(MFILE &mf, int nlines, int newConw, double conwr)
{
    mf.flush();
    std::FILE *f = std::fopen(g_state_path, "w");
    if (!f) return 1;
    std::fprintf(f, "%d %d %.17g", nlines, newConw, conwr);
    std::fclose(f);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc < 4) return 64;
    g_state_path = argv[3];
    pso_problem *p = nullptr;
    if (pso_problem_read(argv[1], &p) != 0 || !p) return 65;
    pso_problem_setup(p, p->conw_r);     // shape tables, ellipsoid start, frequency grid, flags
    l_max = p->lmax;
    m_max = p->mmax;
    n_coef = p->ncoef;
    num_fac = p->shape->nfac;
    l_curves = p->lcurves;
    n_ph_par = p->nphpar;
    max_l_points = 0;
    for (int i = 1; i <= l_curves; i++) {
        l_points[i] = p->lpoints[i];
        in_rel[i] = p->inrel[i];
        if (i < l_curves && l_points[i] > max_l_points) max_l_points = l_points[i];
    }
    int ndata = p->ndata;
    for (int q = 1; q <= ndata + 3; q++) weight[q] = p->weight[q];
    std::vector<double> tim(ndata + 4), br(ndata + 4), sig(ndata + 4), cg(PSO_MAX_N_PAR + 1);
    std::vector<double> ee((ndata + 4) * 3), ee0((ndata + 4) * 3);
    for (int q = 1; q <= ndata; q++) {
        tim[q] = p->tim[q];
        br[q] = p->brightness[q];
        sig[q] = p->sig[q];
        for (int k = 0; k < 3; k++) {
            ee[3 * q + k] = p->ee[q][k + 1];
            ee0[3 * q + k] = p->ee0[q][k + 1];
        }
    }
    for (int i = 1; i <= n_coef; i++) cg[i] = p->cg_first[i];
    int ia[PSO_MAX_N_PAR + 1], ia_par[4];
    for (int l = 1; l <= PSO_MAX_N_PAR; l++) ia[l] = p->ia[l];
    for (int i = 1; i <= 3; i++) ia_par[i] = p->ia_par[i];
    double beta_pole[11] = {0}, lambda_pole[11] = {0}, par[4] = {0, p->par[1], p->par[2], p->par[3]};
    if (!CUDAPrepare(0, beta_pole, lambda_pole, par, p->cl, p->alamda_start, p->alamda_incr,
                     reinterpret_cast<double(*)[3]>(ee.data()), reinterpret_cast<double(*)[3]>(ee0.data()), tim.data(),
                     p->phi0, 0, ndata))
        return 66;
    double conw_r = p->conw_r;
    int new_conw = 0;
    while (new_conw != 1 && conw_r * p->escl * p->escl < 10.0) {
        for (int j = 1; j <= 3; j++) {
            br[ndata + j] = 0;
            sig[ndata + j] = 1 / conw_r;
        }
        CUDAPrecalc(0, p->freq_start, p->freq_end, p->freq_step, p->stop_condition, p->n_iter_min, &conw_r, ndata + 3,
                    ia, ia_par, &new_conw, cg.data(), sig.data(), num_fac, br.data());
    }
    for (int j = 1; j <= 3; j++) {
        br[ndata + j] = 0;
        sig[ndata + j] = 1 / conw_r;
    }
    MFILE out;
    if (out.open(argv[2], "w")) return 67;
    CUDAStart(0, 1, p->freq_start, p->freq_end, p->freq_step, p->stop_condition, p->n_iter_min, conw_r, ndata + 3, ia,
              ia_par, cg.data(), out, p->escl, sig.data(), num_fac, br.data());
    out.close();
    CUDAUnprepare();
    pso_problem_free(p);
    return 0;
}
