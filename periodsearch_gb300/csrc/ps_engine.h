// ps_engine.h -- device-side data of the fit kernels and their launchers.
#pragma once

#include <cstddef>
#include <cstdint>

#include "ps_gb300.h"

namespace psg {

#if defined(__CUDACC__)
#define PSG_HD __host__ __device__
#else
#define PSG_HD
#endif

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
    const double *alpha_pt;              // [ndata] solar phase angle acos(ee . ee0), host libm
    const double *sig2i;                 // [ndata] 1 / sig^2 of every point (mrqcof.c:112)
    const float *nx_f, *ny_f, *nz_f, *darea_f;  // [nfac] FP32 copies for the mixed form
    const int *lc_start, *lc_npts, *lc_rel;  // [n_lc]
    const int *free_list;                // [mfit]
    const double *cg_first;              // [ncoef]
    const float *dsph_f;                 // [nfac][ncoef] FP32 copy for the mixed form
    const float4 *geo_f;                 // [ndata][2] FP32 (ee, alpha), (ee0, 0) for the mixed form
};

// Constants of one scan (period_search_BOINC.cpp:817-868).
struct FitConfig {
    double phi0, alamda_start, alamda_incr, iter_diff_max, conw_r;
    double conv_sig;              // 1 / conw_r, the sigma of the convexity rows
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
    int rel_rows;                 // > 0: relative-lightcurve rows in shared memory (make_layout)
    // multi-object packed launch (launch_pack): fit f belongs to object
    // object[f], described by objs[object[f]] and cfgs[object[f]]
    const struct DevObject *objs;
    const struct FitConfig *cfgs;
    const int *object;
    // learned early stop (all optional)
    int iter_limit;               // > 0: stop every fit after this many LM iterations (screening)
    int screen_iters;             // iterations after which the predictor's features are taken (a
                                  // multiple of 4; 0: kScreenIters)
    float *traj;                  // [nfits][kTrajFloats] trajectory records, or nullptr
    const float *mlp;             // stop-predictor weights (layout of kMlp*), or nullptr
    // kBasisTensorWide: every slot keeps its normal matrix (mfit x mfit
    // doubles) at alpha_g + blockIdx.x * alpha_stride
    double *alpha_g;
    size_t alpha_stride;
    // resumable fits: the LM state of fit f lives in state[slot][state_stride(ma)]
    // with slot = state_slot ? state_slot[f] : f; a fit stopped by iter_limit
    // saves its state there, and with resume != 0 every fit continues from it
    double *state;
    const int64_t *state_slot;
    int resume;
    // FP64 form, optional: every CTA adds its count of lit facet-point pairs
    // (the facet law's and the shape contraction's work) when it ends
    unsigned long long *lit;
};

// Learned early stop: features of a fit after kScreenIters LM iterations,
// the record written per fit, and the layout of the predictor's weights
// (a 10-64-64-1 GELU MLP with input and output standardisation).
constexpr int kScreenIters = 4;
constexpr int kFeat = 10;
constexpr int kHidden = 64;
constexpr int kTrajFloats = 16;   // features[10], dev_k, dev_final, niter, dev after 8/16/32 iterations
constexpr int kMlpMu = 0, kMlpSd = kFeat, kMlpW1 = 2 * kFeat, kMlpB1 = kMlpW1 + kHidden * kFeat,
              kMlpW2 = kMlpB1 + kHidden, kMlpB2 = kMlpW2 + kHidden * kHidden, kMlpW3 = kMlpB2 + kHidden,
              kMlpB3 = kMlpW3 + kHidden, kMlpYMu = kMlpB3 + 1, kMlpYSd = kMlpYMu + 1, kMlpFloats = kMlpYSd + 1;

// Shared-memory plan of a fit slot; identical on host and device.  Offsets
// are in bytes; every block starts on a 16-byte boundary.  Blocks of type
// "real" hold doubles in the FP64 form and floats in the mixed form.
// Where the mixed form's shape contraction takes the basis Dsph from
// (SlotLayout::dsph_smem): global memory, shared memory (both with the SIMT
// contraction), or Tensor Memory with the tcgen05 contraction.
// kBasisTensorWide: the tcgen05 contraction for Laplace series of 65 to 96
// coefficients (L = 8: 81), whose split basis does not fit the 128 Tensor
// Memory lanes of one region (see tensor_wide_ok), with the alpha/beta
// accumulation on the SIMT pipes and the kept normal matrix in global memory.
enum BasisMode : int { kBasisGlobal = 0, kBasisSmem = 1, kBasisTensor = 2, kBasisTensorWide = 3 };
PSG_HD inline bool basis_on_tensor(int mode) { return mode == kBasisTensor || mode == kBasisTensorWide; }

struct SlotLayout {
    int form, ma, mfit, nfac, ncoef, P, wcols, dsph_smem;
    size_t cg, atry, beta, da, alpha, covar, area, gv, areaR, gvR, W, J, pt, ym, red, dave, col, misc, ipiv, dsph;
    size_t bhi, blo, tcm;   // tensor-core operand tiles (TF32 high/low parts) and barrier/TMEM slot
    size_t pt2;             // second point set-up buffer (tensor-core path: next tile's set-up)
    size_t fac, fpart;      // tensor-core path: facet normals and per-evaluation areas, facet-sum partials
    size_t aop;             // tensor-core path: alpha/beta MMA operands
    size_t accs;            // per-point weights and residuals of the accumulation (mixed form)
    size_t davef;           // FP32 copy of a relative lightcurve's derivative sums (mixed form)
    size_t bmat;            // rotation matrices and phase/scattering parameters of an evaluation
    size_t rels;            // relative-lightcurve rows in shared memory, or 0 (global scratch)
    size_t pref;            // tensor-core path: per-point data prefetched for the contraction window
    size_t flist;           // tensor-core path: the free parameters' columns
    size_t lit;             // FP64 form: per point of a tile, its lit-facet count, then its lit facets
    size_t bytes;
};


constexpr int kThreads = 384;   // threads of an FP64-form fit slot
// Threads of a fit slot: the FP64 form runs 384 (12 warps at up to 170
// registers: more warps to hide its FP64 latency than 256, 512 would spill);
// the mixed form runs 512 (16 warps) to hide FP32/shared-memory latency.
template <int FORM>
PSG_HD constexpr int threads_of()
{
    return FORM == PS_FORM_MIXED ? 512 : 384;
}
constexpr int kPointStride = 33;   // reals of per-point set-up (odd: a warp with one point per lane hits 32 banks)
constexpr int kRedStride = 8;      // doubles of per-point facet sums
constexpr int kMisc = 40;
// Prefetch area of the tensor-core path, for a 32-point tile: times (32
// doubles), two copies of the FP32 geometry (32 x 2 float4 each) and sig^-2,
// weight, brightness (32 x 3 doubles).
constexpr size_t kPrefTim = 0, kPrefGeo = 256, kPrefAcc = 1280, kPrefGeo2 = 2048, kPrefBytes = 3072;
constexpr size_t kTcAlphaOperands = 32768;   // tensor-core alpha/beta operands: two 128 x 32 TF32 tiles


// Saved LM state of a stopped fit: the parameters cg[ma], then lambda,
// chi^2 of the accepted point, the last trial chi^2, the regularised
// chi^2, iter_diff, the previous and current rms, the three convexity
// residuals of the accepted shape, its facet-area sum, the iteration count,
// the last solver code and the learned prediction.
PSG_HD constexpr int state_stride(int ma) { return ma + 16; }

// Parked row of a relative lightcurve's point (scratch): the ma model-row
// entries, the model value, and two values the second pass prepares.
PSG_HD constexpr int rel_row_stride(int ma) { return ma + 3; }

// Facets of the tensor-core contraction, padded with empty facets to a
// multiple of 32 (four facet quarters of whole 8-facet core matrices; a
// multiple of the 16 facets of one FP16 MMA).
PSG_HD constexpr int tc_kpad(int nfac) { return (nfac + 31) & ~31; }


// dsph_smem: the mixed form keeps the FP32 basis Dsph[F][C] in shared memory
// for the whole launch (it is read once per point tile by every warp).
// rel_rows > 0: the rows of relative lightcurves (up to rel_rows points)
// are parked in shared memory instead of the per-slot global scratch.
PSG_HD inline SlotLayout make_layout(int form, int ma, int mfit, int nfac, int ncoef, int P, int dsph_smem,
                                     int rel_rows = 0)
{
    SlotLayout L{};
    L.form = form;
    L.ma = ma;
    L.mfit = mfit;
    L.nfac = nfac;
    L.ncoef = ncoef;
    L.P = P;
    L.dsph_smem = dsph_smem;
    L.wcols = ((nfac > mfit ? nfac : mfit) + 3) & ~3;
    const size_t rs = form == PS_FORM_MIXED ? sizeof(float) : sizeof(double);
    size_t o = 0;
    auto take = [&o](size_t bytes) {
        size_t r = o;
        o += (bytes + 15) & ~size_t(15);
        return r;
    };
    const size_t d = sizeof(double);
    L.cg = take(ma * d);
    L.atry = take(ma * d);
    L.beta = take(mfit * d);
    L.da = take(mfit * d);
    L.alpha = take(dsph_smem == kBasisTensorWide ? 0 : static_cast<size_t>(mfit) * mfit * d);
    L.covar = take(static_cast<size_t>(mfit) * mfit * d);
    L.area = take(nfac * d);
    L.gv = take(nfac * d);
    L.areaR = form == PS_FORM_MIXED ? take(nfac * rs) : L.area;
    L.gvR = form == PS_FORM_MIXED ? take(nfac * rs) : L.gv;
    // the tensor-core path writes W straight into the MMA operand
    // (FP64 form: room for the accumulation weights of a tile, [P][mfit],
    // and a staged tile of rows and model values, [P][ma] + [P], behind them)
    const int wrow = form == PS_FORM_FP64 && mfit + ma + 1 > L.wcols ? mfit + ma + 1 : L.wcols;
    L.W = take(basis_on_tensor(dsph_smem) ? 0 : static_cast<size_t>(P) * wrow * rs);
    L.J = take(static_cast<size_t>(P) * ma * rs);
    L.pt = take(static_cast<size_t>(P) * kPointStride * rs);
    L.ym = take(P * d);
    L.red = take(static_cast<size_t>(P) * kRedStride * d);
    L.dave = take(ma * d);
    L.col = take((mfit + 1) * d);
    L.misc = take(kMisc * d);
    L.ipiv = take(sizeof(int) * static_cast<size_t>(mfit + 2 + 16));
    L.dsph = dsph_smem == kBasisSmem ? take(static_cast<size_t>(nfac) * ncoef * sizeof(float)) : 0;
    if (basis_on_tensor(dsph_smem)) {
        const bool wide = dsph_smem == kBasisTensorWide;
        // B = [W_hi; W_lo]: 2P rows, the low parts right after the high parts
        // (8-row groups stride-byte-offset apart); the accumulator rows are
        // staged over it for the epilogue
        // The same region then stages the alpha accumulator; the alpha/beta
        // operands (two 128 x 32 TF32 tiles) have their own region, so that
        // their MMAs overlap the next tile's facet stage.
        // (FP16 elements, facets padded to tc_kpad)
        // (wide: the region also stages the second readback and the SIMT
        // accumulation's weighted rows)
        const size_t tile = static_cast<size_t>(P) * tc_kpad(nfac) * 2;
        size_t readback = 128 * 65 * sizeof(float);
        if (wide) {
            const size_t wt = static_cast<size_t>(P) * mfit * sizeof(float);
            readback = 2 * 128 * 33 * sizeof(float);
            if (wt > readback) readback = wt;
        }
        L.bhi = take(2 * tile > readback ? 2 * tile : readback);
        L.blo = L.bhi + tile;
        L.aop = take(wide ? 0 : kTcAlphaOperands);
        L.tcm = take(32);
        L.pt2 = take(static_cast<size_t>(P) * kPointStride * rs);
        L.fac = take(static_cast<size_t>(tc_kpad(nfac)) * 4 * sizeof(float));
        L.fpart = take(4 * static_cast<size_t>(P) * 9 * sizeof(float));
        L.pref = take(kPrefBytes);
        L.flist = take(static_cast<size_t>(mfit + 1) * sizeof(int));
    } else {
        L.bhi = L.blo = L.tcm = 0;
        L.pt2 = L.pt;
        L.fac = L.fpart = L.aop = L.pref = L.flist = 0;
    }
    // 32 residuals then 32 weights, whatever the tile size
    L.accs = form == PS_FORM_MIXED ? take(64 * sizeof(float)) : 0;
    L.davef = form == PS_FORM_MIXED ? take(static_cast<size_t>(ma) * sizeof(float)) : 0;
    L.bmat = take(32 * rs);
    L.rels = rel_rows > 0 ? take(static_cast<size_t>(rel_rows) * rel_row_stride(ma) * rs) : 0;
    // FP64 form: P counts (int) and P x wcols facet indices (uint16_t)
    L.lit = form == PS_FORM_FP64 ? take(static_cast<size_t>(P) * (4 + 2 * L.wcols)) : 0;
    L.bytes = o;
    return L;
}

// Launchers (ps_engine.cu).  All enqueue on `stream`; return cudaError_t as int.
int launch_fits(int form, const DevObject &ob, const FitConfig &cfg, const FitWork &w, int grid,
                int P, size_t smem, int dsph_smem, void *stream);
// FP64 fits each spread over a thread-block cluster of cs CTAs (2..8),
// bit-identical to launch_fits' FP64 kernel; w without trajectories, saved
// states or an iteration limit.
int launch_fits_split(const DevObject &ob, const FitConfig &cfg, const FitWork &w, int clusters, int cs, int P,
                      size_t smem, void *stream);
int split_max_clusters(int cs, size_t smem, int *clusters);
int launch_eval(int form, const DevObject &ob, const FitConfig &cfg, const double *cg, double *alpha,
                double *beta, double *chisq, double *area, double *scratch, int P, size_t smem,
                int dsph_smem, int rel_rows, void *stream);
int set_kernel_smem(int form, size_t smem, int ncoef, int dsph_smem);
// Multi-object packed launch (ps_pack.cu): objects with identical shape
// tables (facet grid, Laplace series, free parameters) share one persistent
// launch; w.objs / w.cfgs / w.object / w.period_index / w.pole describe the
// fits.  The basis and facet constants are taken from w.objs[0].
int launch_pack(int form, const FitWork &w, int ncoef, int grid, int P, size_t smem, int dsph_smem, void *stream);
int set_pack_smem(int form, size_t smem, int ncoef, int dsph_smem);
int occupancy_slots(int form, size_t smem, int ncoef, int dsph_smem, int *per_sm);
// Whether the tensor-core path supports an object: at most 64 coefficients
// (the high and low FP16 parts of the basis fill 128 Tensor Memory lanes),
// at most 63 free parameters (alpha and the beta column in 64 rows), a
// padded facet count whose basis columns (two facets each) leave the 64
// contraction and 128 alpha accumulator columns within 512, and 32-point
// tiles.
PSG_HD inline bool tensor_basis_ok(int nfac, int ncoef, int mfit, int P)
{
    return ncoef <= 64 && mfit <= 63 && (((tc_kpad(nfac) >> 1) + 31) & ~31) + 64 + 128 <= 512 && P == 32;
}
// The wide tensor-core path (kBasisTensorWide) for 64 < C <= 96
// coefficients: region R1 holds the FP16 high parts of all C coefficients
// (lanes 0..C-1) and the low parts of the first 128 - C (lanes C..127);
// region R2 holds the low parts of the other n2 = 2C - 128 <= 64, the first
// half of the facets in lanes 0..n2-1 and the second half in lanes
// 64..64+n2-1 (Fp/4 columns).  With the two accumulators (64 columns each)
// the Tensor Memory holds 3 Fp / 4 + 128 <= 512 columns, i.e. up to 512
// facets (nrows = 8).  The alpha/beta accumulation runs on the SIMT pipes
// (FP32 partial sums, up to 90 free parameters).
PSG_HD inline bool tensor_wide_ok(int nfac, int ncoef, int mfit, int P)
{
    return ncoef > 64 && ncoef <= 96 && mfit <= 90 && ((3 * (tc_kpad(nfac) >> 2) + 31) & ~31) + 128 <= 512 &&
           P == 32;
}
int measure_fma_peaks(double *fp64_tflops, double *fp32_tflops, void *stream);
// Learned early stop (ps_mlp.cu).
int mlp_train(float *h_P, const float *h_x, const float *h_y, int n, int epochs, int batch, float lr, uint64_t seed,
              float *h_loss_hist);
int mlp_predict(const float *h_P, const float *h_x, int n, float *h_out);
int mlp_grad(const float *h_P, const float *h_x, const float *h_y, int n, float *h_loss, float *h_G);

// Allocation-free launch of the FP64 fit kernel: the work counter and the
// per-slot scratch come from a file-scope device array of
// kStaticScratchDoubles doubles (ps_engine.cu).  Returns -1 when one slot's
// scratch (w.scratch_stride doubles) does not fit, else a cudaError_t.
constexpr size_t kStaticScratchDoubles = size_t(1) << 19;  // 4 MiB
int launch_fits_noalloc(int form, const DevObject &ob, const FitConfig &cfg, FitWork w, int max_grid, int P,
                        size_t smem, void *stream, int *grid_used);

}  // namespace psg
