// start_CUDA_gb300.cpp -- source-level drop-in for the CUDA port's host
// calls (period_search_cuda/period_search/start_CUDA.h:2-14) on top of the
// GB300 engine's C ABI.
//
// A maintainer builds the CUDA port's period_search_BOINC.cpp with this file
// in place of start_CUDA.cu and the port's .cu kernels, links
// libps_gb300.so, and changes nothing else: CUDAPrepare, CUDAPrecalc,
// CUDAStart, CUDAUnprepare and GetCUDAOccupancy keep their signatures, read
// the same globals (globals.h) and write the same rows and checkpoints into
// the MFILE.  The object is prepared on the device at the first CUDAPrecalc
// or CUDAStart, from the state the port's main() has built
// (ps_prepare_state); each CUDAPrecalc runs one convexity-weight round
// (ps_precalc_step); CUDAStart scans the remaining periods in chunks
// (ps_scan) and checkpoints after each chunk.
//
// The environment variable PS_GB300_FORM=mixed selects the mixed-precision
// form (default: the plain FP64 form, the drop-in).  Fatal errors print to
// stderr and exit with the reference's codes (2: size limits, 4: singular
// ellipsoid fit, 1: device or other failure), as the port does.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "boinc_api.h"
#include "mfile.h"
#include "ps_gb300.h"
#include "start_CUDA.h"

// The port's globals (period_search_cuda/period_search/globals.h), defined
// by its main program.  Arrays are 1-based; l_curves counts the convexity
// pseudo-lightcurve appended last.
extern int l_max, m_max, n_coef, num_fac, l_curves, n_ph_par, l_points[], in_rel[], max_l_points;
extern double weight[];

namespace {

struct Adaptor {
    int device = 0;
    bool have_prepare = false;
    double par[3] = {0, 0, 0}, cl = 0, alamda_start = 0, alamda_incr = 0, phi0 = 0;
    int ndata = 0;                        // real points, as passed to CUDAPrepare
    std::vector<double> tim, ee, ee0;     // 0-based copies
    ps_ctx *ctx = nullptr;
};

Adaptor g_ad;

[[noreturn]] void fatal(ps_status st, const char *where, const ps_ctx *ctx)
{
    std::fprintf(stderr, "%s: %s%s%s\n", where, ps_status_string(st), ctx ? ": " : "", ctx ? ps_last_error(ctx) : "");
    std::fflush(stderr);
    std::exit(st == PS_ERR_LIMIT ? 2 : st == PS_ERR_SINGULAR ? 4 : 1);
}

int form_from_env()
{
    const char *f = std::getenv("PS_GB300_FORM");
    return (f && std::strcmp(f, "mixed") == 0) ? PS_FORM_MIXED : PS_FORM_FP64;
}

// Prepares the device context from the port's state at the first call that
// has all of it (CUDAPrecalc or CUDAStart).  ndata_all includes the three
// convexity rows; ia, cg_first, sig and brightness are 1-based.
void ensure_context(double freq_start, double freq_end, double freq_step, double stop_condition, int n_iter_min,
                    double conw_r, int ndata_all, int *ia, int *ia_par, double *cg_first, double *sig,
                    int Numfac, double *brightness, double escl)
{
    if (g_ad.ctx) return;
    if (!g_ad.have_prepare) fatal(PS_ERR_ARG, "CUDAPrecalc/CUDAStart before CUDAPrepare", nullptr);
    const int nd = ndata_all - 3;
    if (nd != g_ad.ndata) fatal(PS_ERR_ARG, "ndata differs from CUDAPrepare's", nullptr);
    // phase-function flags, as the port's CUDAPrecalc/CUDAStart set them
    for (int i = 1; i <= n_ph_par; i++) ia[n_coef + 3 + i] = ia_par[i];
    const int n_lc = l_curves - 1;
    std::vector<int32_t> lc_points(static_cast<size_t>(n_lc)), lc_rel(static_cast<size_t>(n_lc));
    for (int i = 0; i < n_lc; i++) {
        lc_points[static_cast<size_t>(i)] = l_points[i + 1];
        lc_rel[static_cast<size_t>(i)] = in_rel[i + 1];
    }
    const int ma = n_coef + 5 + n_ph_par;
    std::vector<int32_t> ia0(static_cast<size_t>(ma));
    for (int l = 0; l < ma; l++) ia0[static_cast<size_t>(l)] = ia[l + 1];
    std::vector<double> br(brightness + 1, brightness + 1 + nd), sg(sig + 1, sig + 1 + nd),
        wt(weight + 1, weight + 1 + nd), cg(cg_first + 1, cg_first + 1 + n_coef);
    int nrows = 0;
    while (8 * (nrows + 1) * (nrows + 1) <= Numfac) nrows++;
    if (8 * nrows * nrows != Numfac) fatal(PS_ERR_ARG, "Numfac is not 8 * nrows^2", nullptr);
    ps_state st{};
    st.lmax = l_max;
    st.mmax = m_max;
    st.nrows = nrows;
    st.n_lc = n_lc;
    st.lc_points = lc_points.data();
    st.lc_rel = lc_rel.data();
    st.ndata = nd;
    st.tim = g_ad.tim.data();
    st.brightness = br.data();
    st.sig = sg.data();
    st.weight = wt.data();
    st.ee = g_ad.ee.data();
    st.ee0 = g_ad.ee0.data();
    st.phi0 = g_ad.phi0;
    for (int k = 0; k < 3; k++) st.par[k] = g_ad.par[k];
    st.cl = g_ad.cl;
    st.alamda_start = g_ad.alamda_start;
    st.alamda_incr = g_ad.alamda_incr;
    st.stop_condition = stop_condition;
    st.n_iter_min = n_iter_min;
    st.ia = ia0.data();
    st.cg_first = cg.data();
    st.escl = escl;
    st.freq_start = freq_start;
    st.freq_end = freq_end;
    st.freq_step = freq_step;
    st.conw_r = conw_r;
    ps_options opt{};
    opt.device = g_ad.device;
    opt.form = form_from_env();
    const ps_status s = ps_prepare_state(&st, &opt, &g_ad.ctx);
    if (s != PS_OK) fatal(s, "ps_prepare_state", nullptr);
}

}  // namespace

int CUDAPrepare(int cudadev, double *beta_pole, double *lambda_pole, double *par, double cl, double Alamda_start,
                double Alamda_incr, double ee[][3], double ee0[][3], double *tim, double Phi_0, int checkex, int ndata)
{
    (void)beta_pole;     // the 10 initial poles are the engine's own (period_search_BOINC.cpp:197-206)
    (void)lambda_pole;
    (void)checkex;
    if (g_ad.ctx) {
        ps_destroy(g_ad.ctx);
        g_ad.ctx = nullptr;
    }
    g_ad.device = cudadev;
    for (int k = 0; k < 3; k++) g_ad.par[k] = par[k + 1];
    g_ad.cl = cl;
    g_ad.alamda_start = Alamda_start;
    g_ad.alamda_incr = Alamda_incr;
    g_ad.phi0 = Phi_0;
    g_ad.ndata = ndata;
    g_ad.tim.assign(tim + 1, tim + 1 + ndata);
    g_ad.ee.resize(3 * static_cast<size_t>(ndata));
    g_ad.ee0.resize(3 * static_cast<size_t>(ndata));
    for (int q = 0; q < ndata; q++)
        for (int k = 0; k < 3; k++) {
            g_ad.ee[3 * static_cast<size_t>(q) + k] = ee[q + 1][k];
            g_ad.ee0[3 * static_cast<size_t>(q) + k] = ee0[q + 1][k];
        }
    g_ad.have_prepare = true;
    return 1;
}

int CUDAPrecalc(int cudadev, double freq_start, double freq_end, double freq_step, double stop_condition,
                int n_iter_min, double *conw_r, int ndata, int *ia, int *ia_par, int *new_conw, double *cg_first,
                double *sig, int Numfac, double *brightness)
{
    (void)cudadev;
    // escl is not an argument here; it only scales the first printed row
    ensure_context(freq_start, freq_end, freq_step, stop_condition, n_iter_min, *conw_r, ndata, ia, ia_par, cg_first,
                   sig, Numfac, brightness, 1.0);
    int32_t nc = *new_conw;
    const ps_status st = ps_precalc_step(g_ad.ctx, conw_r, &nc);
    if (st != PS_OK) fatal(st, "ps_precalc_step", g_ad.ctx);
    *new_conw = nc;
    return 1;
}

int CUDAStart(int cudadev, int n_start_from, double freq_start, double freq_end, double freq_step,
              double stop_condition, int n_iter_min, double conw_r, int ndata, int *ia, int *ia_par,
              double *cg_first, MFILE &mf, double escl, double *sig, int Numfac, double *brightness)
{
    (void)cudadev;
    ensure_context(freq_start, freq_end, freq_step, stop_condition, n_iter_min, conw_r, ndata, ia, ia_par, cg_first,
                   sig, Numfac, brightness, escl);
    ps_info info{};
    ps_get_info(g_ad.ctx, &info);
    const int64_t n_max = info.n_max;
    // chunks of whole waves of the device's fit slots (10 poles per period)
    const int64_t chunk = std::max<int64_t>(1, 4 * static_cast<int64_t>(info.slots) / 10);
    std::vector<ps_row> rows(static_cast<size_t>(chunk));
    char buf[256];
    for (int64_t n0 = n_start_from; n0 <= n_max; n0 += chunk) {
        const int64_t n1 = std::min(n_max, n0 + chunk - 1);
        const ps_status st = ps_scan(g_ad.ctx, conw_r, n0, n1, rows.data());
        if (st != PS_OK) fatal(st, "ps_scan", g_ad.ctx);
        for (int64_t n = n0; n <= n1; n++) {
            const ps_row &r = rows[static_cast<size_t>(n - n0)];
            // start_CUDA.cu:763-767: the first row carries conw_r * escl^2; poles rounded
            const double col4 = n == 1 ? conw_r * escl * escl : r.dark_or_conw;
            mf.printf("%.8f  %.6f  %.6f %4.1f %4.0f %4.0f\n", r.period_h, r.rms, r.chi2, col4, std::round(r.lambda_deg),
                      std::round(r.beta_deg));
        }
        boinc_fraction_done(static_cast<double>(n1) / static_cast<double>(n_max));
        if (boinc_time_to_checkpoint() || boinc_is_standalone()) {
            const int retval = DoCheckpoint(mf, static_cast<int>(n1), 1, conw_r);
            if (retval) {
                std::fprintf(stderr, "%s APP: period_search checkpoint failed %d\n",
                             boinc_msg_prefix(buf, sizeof buf), retval);
                std::exit(retval);
            }
            boinc_checkpoint_completed();
        }
    }
    return 1;
}

void CUDAUnprepare(void)
{
    if (g_ad.ctx) ps_destroy(g_ad.ctx);
    g_ad.ctx = nullptr;
    g_ad.have_prepare = false;
}

void GetCUDAOccupancy(const int cudaDevice)
{
    std::fprintf(stderr, "GB300 engine on device %d: one persistent fit kernel, slots set per object at prepare\n",
                 cudaDevice);
}
