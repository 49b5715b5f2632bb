// ps_engine.h -- device-side data of the fit kernels and their launchers.
#pragma once

#include <cstddef>
#include <cstdint>

#include "ps_gb300.h"

namespace psg {

// One object's tables in device memory (all arrays device pointers, 0-based).
struct DevObject {
    int nfac, ncoef, ma, mfit, npairs, mmax;
    int n_lc;           // lightcurves including the convexity rows (last)
    int ndata;          // real points
    int max_rel_points; // longest relative lightcurve (scratch rows per slot)
    const double *nx, *ny, *nz, *darea;  // [nfac]
    const double *dsph;                  // [nfac][ncoef]
    const double *pleg;                  // [npairs][nfac]
    const double *fc, *fs;               // [mmax+1][nfac]
    const int *pair_m, *pair_n;          // [npairs]
    const double *tim, *bright, *sig, *weight;  // [ndata+3]; sig of the last 3 rows unused
    const double *eex, *eey, *eez, *e0x, *e0y, *e0z;  // [ndata]
    const int *lc_start, *lc_npts, *lc_rel;  // [n_lc]
    const int *free_list;                // [mfit]
    const double *cg_first;              // [ncoef]
    const float *dsph_f;                 // [nfac][ncoef] FP32 copy for the mixed form
};

// Constants of one scan (period_search_BOINC.cpp:817-868).
struct FitConfig {
    double phi0, alamda_start, alamda_incr, iter_diff_max, conw_r;
    double freq_start, freq_step, log_cl, par0, par1, par2;
    int n_iter_max, n_iter_min;
};

// Work description of one launch: fit f is (period n_lo + f/10, pole f%10+1)
// unless explicit lists are given.
struct FitWork {
    int64_t n_lo, nfits;
    const int64_t *period_index;  // optional [nfits], 1-based
    const int *pole;              // optional [nfits], 1..10
    unsigned long long *queue;    // device work counter, zero before launch
    double *scratch;              // per-slot scratch for relative lightcurves
    size_t scratch_stride;        // doubles per slot
    ps_fit *out;                  // [nfits]
};

// Shared-memory plan of a fit slot; identical on host and device.
struct SlotLayout {
    int ma, mfit, nfac, P;
    size_t o_cg, o_atry, o_beta, o_da, o_alpha, o_covar, o_area, o_gv, o_W, o_J, o_ym, o_pt, o_red,
        o_dave, o_col, o_misc, o_end;  // offsets in doubles
    size_t o_ipiv;                     // offset in bytes of the int area
    size_t bytes;
};

constexpr int kThreads = 256;
constexpr int kPointStride = 32;   // doubles of per-point set-up
constexpr int kRedStride = 8;      // doubles of per-point facet sums
constexpr int kMisc = 32;

#if defined(__CUDACC__)
#define PSG_HD __host__ __device__
#else
#define PSG_HD
#endif

PSG_HD inline SlotLayout make_layout(int ma, int mfit, int nfac, int P)
{
    SlotLayout L{};
    L.ma = ma;
    L.mfit = mfit;
    L.nfac = nfac;
    L.P = P;
    size_t o = 0;
    auto take = [&o](size_t n) {
        size_t r = o;
        o += (n + 1) & ~size_t(1);  // keep 16-byte alignment of every block
        return r;
    };
    int wcols = nfac > mfit ? nfac : mfit;
    L.o_cg = take(ma);
    L.o_atry = take(ma);
    L.o_beta = take(mfit);
    L.o_da = take(mfit);
    L.o_alpha = take(static_cast<size_t>(mfit) * mfit);
    L.o_covar = take(static_cast<size_t>(mfit) * mfit);
    L.o_area = take(nfac);
    L.o_gv = take(nfac);
    L.o_W = take(static_cast<size_t>(P) * wcols);
    L.o_J = take(static_cast<size_t>(P) * ma);
    L.o_ym = take(P);
    L.o_pt = take(static_cast<size_t>(P) * kPointStride);
    L.o_red = take(static_cast<size_t>(P) * kRedStride);
    L.o_dave = take(ma);
    L.o_col = take(mfit + 1);
    L.o_misc = take(kMisc);
    L.o_end = o;
    L.o_ipiv = o * sizeof(double);
    L.bytes = L.o_ipiv + sizeof(int) * static_cast<size_t>(mfit + 2 + 8);
    L.bytes = (L.bytes + 15) & ~size_t(15);
    return L;
}

// Launchers (ps_engine.cu).  All enqueue on `stream`; return cudaError_t as int.
int launch_fits(int form, const DevObject &ob, const FitConfig &cfg, const FitWork &w, int grid,
                int P, size_t smem, void *stream);
int launch_eval(int form, const DevObject &ob, const FitConfig &cfg, const double *cg, double *alpha,
                double *beta, double *chisq, double *area, double *scratch, int P, size_t smem,
                void *stream);
int set_kernel_smem(int form, size_t smem);
int occupancy_slots(int form, size_t smem, int *per_sm);
int measure_fma_peaks(double *fp64_tflops, double *fp32_tflops, void *stream);

// Allocation-free launch of the FP64 fit kernel: the work counter and the
// per-slot scratch come from a file-scope device array of
// kStaticScratchDoubles doubles (ps_engine.cu).  Returns -1 when one slot's
// scratch (w.scratch_stride doubles) does not fit, else a cudaError_t.
constexpr size_t kStaticScratchDoubles = size_t(1) << 19;  // 4 MiB
int launch_fits_noalloc(int form, const DevObject &ob, const FitConfig &cfg, FitWork w, int max_grid, int P,
                        size_t smem, void *stream, int *grid_used);

}  // namespace psg
