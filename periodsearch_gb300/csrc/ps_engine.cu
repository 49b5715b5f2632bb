// ps_engine.cu -- fit kernels of the GB300 period-search engine (sm_103a).
//
// One CTA is one fit slot.  A slot pulls fits (period index, initial pole)
// from a device work counter and runs the whole Levenberg-Marquardt fit on
// the device: model evaluation (the reference's mrqcof with curv, blmatrix,
// bright and conv), the damped normal-equation solve (gauss_errc), the
// accept/reject and lambda update (mrqmin) and the stop rule of the driver
// loop (period_search_BOINC.cpp:868-893).  Nothing returns to the host until
// every fit of the launch is done.
//
// Evaluation of one parameter vector, per tile of P observations:
//   1. point set-up (one thread per point, FP64): solar phase angle, phase
//      function, body rotation f = fmod(omega*t + phi0, 2*pi) and the rotated
//      Earth/Sun directions with their beta/lambda/omega derivatives;
//   2. facet stage (one warp per point, lanes over facets): mu, mu0, the
//      Lommel-Seeliger + Lambert law, brightness, rotation and scattering
//      derivatives; lit facets write W[p][i] = Darea_i * s_pi * g_i;
//   3. shape contraction J[p][k] = Scale_p * sum_i W[p][i] * Dsph[i][k]
//      (the reference's sum over lit facets of dbr * Dg);
//   4. relative lightcurves: per-lightcurve sums, then the renormalisation of
//      mrqcof.c:90-104 from a per-slot scratch copy of the lightcurve's rows;
//   5. normal-matrix accumulation alpha = J^T W J, beta, chi^2 over the free
//      parameters, each alpha element summed over points in data order.
// The three convexity rows (conv.c) are three more rows of the same
// contraction with W[c][i] = Darea_i * g_i * n_i[c].
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "ps_engine.h"

namespace psg {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoPi = 2 * kPi;
constexpr double kRad2Deg = 180 / kPi;
constexpr double kDeg2Rad = kPi / 180;
constexpr double kTinyMu = 1e-8;

__constant__ double c_beta_pole[PS_N_POLES] = {0, 0, 0, 0, 60, 60, 60, -60, -60, -60};
__constant__ double c_lambda_pole[PS_N_POLES] = {0, 90, 180, 270, 60, 180, 300, 60, 180, 300};

struct Smem {
    double *cg, *atry, *beta, *da, *alpha, *covar, *area, *gv, *W, *J, *ym, *pt, *red, *dave, *col, *misc;
    int *ipiv;
};

__device__ inline Smem carve(double *base, const SlotLayout &L)
{
    Smem s;
    s.cg = base + L.o_cg;
    s.atry = base + L.o_atry;
    s.beta = base + L.o_beta;
    s.da = base + L.o_da;
    s.alpha = base + L.o_alpha;
    s.covar = base + L.o_covar;
    s.area = base + L.o_area;
    s.gv = base + L.o_gv;
    s.W = base + L.o_W;
    s.J = base + L.o_J;
    s.ym = base + L.o_ym;
    s.pt = base + L.o_pt;
    s.red = base + L.o_red;
    s.dave = base + L.o_dave;
    s.col = base + L.o_col;
    s.misc = base + L.o_misc;
    s.ipiv = reinterpret_cast<int *>(reinterpret_cast<char *>(base) + L.o_ipiv);
    return s;
}

// misc slots
enum : int {
    M_CHISQ = 0,   // chi^2 accumulator of the current evaluation
    M_AVE = 1,     // relative-lightcurve model sum
    M_AREA = 2,    // sum of facet areas of the current evaluation
    M_CHK = 3,     // 3 convexity residuals (sum Area*n) of the current evaluation
    M_CL = 7,      // exp(log cl)
    M_RED = 16     // 16 doubles of block-reduction scratch
};

// Row j of packed lower-triangle element e (j*(j+1)/2 <= e < (j+1)*(j+2)/2),
// from an FP32 square root corrected in integers.
__device__ inline int tri_row(int e)
{
    int j = static_cast<int>((sqrtf(8.0f * static_cast<float>(e) + 1.0f) - 1.0f) * 0.5f);
    while (j * (j + 1) / 2 > e) j--;
    while ((j + 1) * (j + 2) / 2 <= e) j++;
    return j;
}

// Thread that sets up point p of a tile: points are spread over the warps
// (p % 8 -> warp, p / 8 -> lane) so that all four SM sub-partitions work.
__device__ inline int setup_thread(int p) { return (p % (kThreads / 32)) * 32 + p / (kThreads / 32); }

__device__ inline double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block; every thread gets the result.  red holds >= 8 doubles.
__device__ inline double block_sum(double v, double *red)
{
    v = warp_sum(v);
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double t = 0;
#pragma unroll
    for (int i = 0; i < kThreads / 32; i++) t += red[i];
    __syncthreads();
    return t;
}

// ---------------------------------------------------------------------------
// Model evaluation (mrqcof) at parameters a[] into matrix M (mfit x mfit,
// lower triangle accumulated then mirrored) and vector bv.  Leaves chi^2,
// the facet-area sum and the convexity residuals in misc.
// ---------------------------------------------------------------------------
template <int FORM>
__device__ void evaluate(const DevObject &ob, const FitConfig &cfg, const SlotLayout &L, Smem &s,
                         const double *a, double *M, double *bv, double *scratch)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int F = ob.nfac, C = ob.ncoef, ma = ob.ma, mf = ob.mfit, P = L.P;
    const int wcols = L.nfac > L.mfit ? L.nfac : L.mfit;

    // curv.c:10-39 -- g_i = exp(sum over (m,l) of P_l^m (c cos + c' sin)).
    double asum = 0;
    for (int i = tid; i < F; i += kThreads) {
        double g = 0;
        for (int q = 0; q < ob.npairs; q++) {
            int m = ob.pair_m[q], n = ob.pair_n[q];
            double fsum = a[n] * ob.fc[m * F + i];
            if (m != 0) fsum = fsum + a[n + 1] * ob.fs[m * F + i];
            g = g + ob.pleg[q * F + i] * fsum;
        }
        g = exp(g);
        double ar = ob.darea[i] * g;
        s.area[i] = ar;
        s.gv[i] = g;
        asum += ar;
    }
    double tot = block_sum(asum, s.misc + M_RED);
    if (tid == 0) {
        s.misc[M_AREA] = tot;
        s.misc[M_CHISQ] = 0;
        s.misc[M_CL] = exp(a[ma - 2]);
    }
    for (int e = tid; e < mf * mf; e += kThreads) M[e] = 0;
    for (int j = tid; j < mf; j += kThreads) bv[j] = 0;

    const double bet = a[C], lam = a[C + 1];
    const double cb = cos(bet), sb = sin(bet), clm = cos(lam), slm = sin(lam);
    // Blmat and its derivatives (row-major 3x3 each), registers of every thread.
    const double B[9] = {cb * clm, cb * slm, -sb, -slm, clm, 0, sb * clm, sb * slm, cb};
    const double DB0[9] = {-sb * clm, -sb * slm, -cb, 0, 0, 0, cb * clm, cb * slm, -sb};
    const double DB1[9] = {-cb * slm, cb * clm, 0, -clm, -slm, 0, -sb * slm, sb * clm, 0};
    const double omg = a[C + 2];
    const double php0 = a[C + 3], php1 = a[C + 4], php2 = a[C + 5];
    const double cls = a[C + 7];
    __syncthreads();
    const double cl = s.misc[M_CL];

    const double conv_sig = 1 / cfg.conw_r;
    const double conv_sig2i = 1 / (conv_sig * conv_sig);

    for (int lc = 0; lc < ob.n_lc; lc++) {
        const int start = ob.lc_start[lc], npts = ob.lc_npts[lc];
        const bool rel = ob.lc_rel[lc] != 0;
        const bool conv = (lc == ob.n_lc - 1);
        if (rel) {
            for (int l = tid; l < ma; l += kThreads) s.dave[l] = 0;
            if (tid == 0) s.misc[M_AVE] = 0;
        }
        // ---- pass 1: model rows of this lightcurve, tile by tile ----
        for (int t0 = 0; t0 < npts; t0 += P) {
            const int np = min(P, npts - t0);
            if (!conv) {
                // 1. point set-up (bright.c:27-57, phasec.c, matrix.c)
                // point sp is set up by thread setup_thread(sp) == tid
                const int sp = (tid % 32) * (kThreads / 32) + tid / 32;
                if (sp < np) {
                    const int q = start + t0 + sp;
                    const double ee[3] = {ob.eex[q], ob.eey[q], ob.eez[q]};
                    const double e0v[3] = {ob.e0x[q], ob.e0y[q], ob.e0z[q]};
                    const double t = ob.tim[q];
                    double cos_alpha = ee[0] * e0v[0] + ee[1] * e0v[1] + ee[2] * e0v[2];
                    double alpha = acos(cos_alpha);
                    double ex = exp(-alpha / php1);
                    double scale = 1 + php0 * ex + php2 * alpha;
                    double f = omg * t + cfg.phi0;
                    f = fmod(f, kTwoPi);
                    double cf = cos(f), sf = sin(f);
                    const double fm[9] = {cf, sf, 0, -sf, cf, 0, 0, 0, 1};
                    const double dfm[9] = {-t * sf, t * cf, 0, -t * cf, -t * sf, 0, 0, 0, 0};
                    double tm[9], d0[9], d1[9], d2[9];
#pragma unroll
                    for (int i = 0; i < 3; i++)
#pragma unroll
                        for (int j = 0; j < 3; j++) {
                            double x = 0, y0 = 0, y1 = 0, y2 = 0;
#pragma unroll
                            for (int k = 0; k < 3; k++) {
                                x = x + fm[i * 3 + k] * B[k * 3 + j];
                                y0 = y0 + fm[i * 3 + k] * DB0[k * 3 + j];
                                y1 = y1 + fm[i * 3 + k] * DB1[k * 3 + j];
                                y2 = y2 + dfm[i * 3 + k] * B[k * 3 + j];
                            }
                            tm[i * 3 + j] = x;
                            d0[i * 3 + j] = y0;
                            d1[i * 3 + j] = y1;
                            d2[i * 3 + j] = y2;
                        }
                    double *pt = s.pt + sp * kPointStride;
#pragma unroll
                    for (int i = 0; i < 3; i++) {
                        double x = 0, y = 0;
#pragma unroll
                        for (int j = 0; j < 3; j++) {
                            x = x + tm[i * 3 + j] * ee[j];
                            y = y + tm[i * 3 + j] * e0v[j];
                        }
                        pt[i] = x;
                        pt[3 + i] = y;
                    }
                    // de[i][j] = sum_k dtm[j][i][k] ee[k]; stored de[i*3+j] (j = derivative)
                    const double *dd[3] = {d0, d1, d2};
#pragma unroll
                    for (int i = 0; i < 3; i++)
#pragma unroll
                        for (int j = 0; j < 3; j++) {
                            double x = 0, y = 0;
#pragma unroll
                            for (int k = 0; k < 3; k++) {
                                x = x + dd[j][i * 3 + k] * ee[k];
                                y = y + dd[j][i * 3 + k] * e0v[k];
                            }
                            pt[6 + i * 3 + j] = x;
                            pt[15 + i * 3 + j] = y;
                        }
                    pt[24] = scale;
                    pt[25] = ex;
                    pt[26] = php0 * ex * alpha / (php1 * php1);
                    pt[27] = alpha;
                }
                __syncthreads();
                // 2. facet stage (bright.c:59-120), one warp per point
                for (int p = warp; p < np; p += kThreads / 32) {
                    const double *pt = s.pt + p * kPointStride;
                    const double e1 = pt[0], e2 = pt[1], e3 = pt[2];
                    const double f1 = pt[3], f2 = pt[4], f3 = pt[5];
                    double de[9], de0[9];
#pragma unroll
                    for (int k = 0; k < 9; k++) {
                        de[k] = pt[6 + k];
                        de0[k] = pt[15 + k];
                    }
                    double br = 0, r0 = 0, r1 = 0, r2 = 0, dcl = 0, dcls = 0;
                    double *Wp = s.W + static_cast<size_t>(p) * wcols;
                    for (int i = lane; i < F; i += 32) {
                        const double nx = ob.nx[i], ny = ob.ny[i], nz = ob.nz[i];
                        const double mu = e1 * nx + e2 * ny + e3 * nz;
                        const double mu0 = f1 * nx + f2 * ny + f3 * nz;
                        double w = 0;
                        if (mu > kTinyMu && mu0 > kTinyMu) {
                            const double ar = s.area[i];
                            const double dnom = mu + mu0;
                            const double sv = mu * mu0 * (cl + cls / dnom);
                            br = br + ar * sv;
                            const double q0 = mu0 / dnom, q1 = mu / dnom;
                            const double dsmu = cls * (q0 * q0) + cl * mu0;
                            const double dsmu0 = cls * (q1 * q1) + cl * mu;
                            w = ob.darea[i] * sv * s.gv[i];
                            const double s0 = nx * de[0] + ny * de[3] + nz * de[6];
                            const double s1 = nx * de[1] + ny * de[4] + nz * de[7];
                            const double s2 = nx * de[2] + ny * de[5] + nz * de[8];
                            const double t0v = nx * de0[0] + ny * de0[3] + nz * de0[6];
                            const double t1v = nx * de0[1] + ny * de0[4] + nz * de0[7];
                            const double t2v = nx * de0[2] + ny * de0[5] + nz * de0[8];
                            r0 = r0 + ar * (dsmu * s0 + dsmu0 * t0v);
                            r1 = r1 + ar * (dsmu * s1 + dsmu0 * t1v);
                            r2 = r2 + ar * (dsmu * s2 + dsmu0 * t2v);
                            dcl = dcl + mu * mu0 * ar;
                            dcls = dcls + ar * mu * mu0 / dnom;
                        }
                        Wp[i] = w;
                    }
                    br = warp_sum(br);
                    r0 = warp_sum(r0);
                    r1 = warp_sum(r1);
                    r2 = warp_sum(r2);
                    dcl = warp_sum(dcl);
                    dcls = warp_sum(dcls);
                    if (lane == 0) {
                        double *rd = s.red + p * kRedStride;
                        rd[0] = br;
                        rd[1] = r0;
                        rd[2] = r1;
                        rd[3] = r2;
                        rd[4] = dcl;
                        rd[5] = dcls;
                    }
                }
            } else {
                // convexity rows (conv.c:12-29): W = Darea g n_c, residual = sum Area n_c
                for (int p = warp; p < np; p += kThreads / 32) {
                    const double *nc = (p == 0) ? ob.nx : (p == 1) ? ob.ny : ob.nz;
                    double res = 0;
                    double *Wp = s.W + static_cast<size_t>(p) * wcols;
                    for (int i = lane; i < F; i += 32) {
                        res = res + s.area[i] * nc[i];
                        Wp[i] = ob.darea[i] * s.gv[i] * nc[i];
                    }
                    res = warp_sum(res);
                    if (lane == 0) s.red[p * kRedStride] = res;
                }
            }
            __syncthreads();
            // 3. shape contraction and the remaining columns of J
            for (int o = tid; o < np * C; o += kThreads) {
                const int p = o / C, k = o - p * C;
                const double *Wp = s.W + static_cast<size_t>(p) * wcols;
                const double *ds = ob.dsph + k;
                double acc = 0;
                for (int i = 0; i < F; i++) acc = acc + Wp[i] * ds[static_cast<size_t>(i) * C];
                s.J[p * ma + k] = conv ? acc : s.pt[p * kPointStride + 24] * acc;
            }
            if (tid < np) {
                const int p = tid;
                double *Jp = s.J + p * ma;
                const double *rd = s.red + p * kRedStride;
                if (!conv) {
                    const double *pt = s.pt + p * kPointStride;
                    const double scale = pt[24];
                    Jp[C] = scale * rd[1];
                    Jp[C + 1] = scale * rd[2];
                    Jp[C + 2] = scale * rd[3];
                    Jp[C + 3] = rd[0] * pt[25];
                    Jp[C + 4] = rd[0] * pt[26];
                    Jp[C + 5] = rd[0] * pt[27];
                    Jp[C + 6] = scale * rd[4] * cl;
                    Jp[C + 7] = scale * rd[5];
                    s.ym[p] = rd[0] * scale;
                } else {
                    for (int k = C; k < ma; k++) Jp[k] = 0;
                    s.ym[p] = rd[0];
                    s.misc[M_CHK + p] = rd[0];
                }
            }
            __syncthreads();
            if (rel) {
                // 4a. lightcurve sums and a copy of the rows (mrqcof.c:51-88)
                double *dst = scratch + static_cast<size_t>(t0) * (ma + 1);
                for (int e = tid; e < np * ma; e += kThreads) {
                    int p = e / ma, l = e - p * ma;
                    dst[static_cast<size_t>(p) * (ma + 1) + l] = s.J[e];
                }
                if (tid < np) dst[static_cast<size_t>(tid) * (ma + 1) + ma] = s.ym[tid];
                for (int l = tid; l < ma; l += kThreads) {
                    double d = s.dave[l];
                    for (int p = 0; p < np; p++) d = d + s.J[p * ma + l];
                    s.dave[l] = d;
                }
                if (tid == 0) {
                    double av = s.misc[M_AVE];
                    for (int p = 0; p < np; p++) av = av + s.ym[p];
                    s.misc[M_AVE] = av;
                }
                __syncthreads();
                continue;
            }
            // 5. accumulate (mrqcof.c:106-136)
            {
                double *wt = s.W;  // reuse: [P][mfit]
                for (int e = tid; e < np * mf; e += kThreads) {
                    const int p = e / mf, j = e - p * mf;
                    const int q = start + t0 + p;
                    const double sg = conv ? conv_sig : ob.sig[q];
                    const double sig2i = 1 / (sg * sg);
                    const double wg = ob.weight[q];
                    wt[p * mf + j] = s.J[p * ma + ob.free_list[j]] * sig2i * wg;
                }
                __syncthreads();
                const int ntri = mf * (mf + 1) / 2;
                for (int e = tid; e < ntri; e += kThreads) {
                    const int j = tri_row(e);
                    const int k = e - j * (j + 1) / 2;
                    const int lk = ob.free_list[k];
                    double acc = M[j * mf + k];
                    for (int p = 0; p < np; p++) acc = acc + wt[p * mf + j] * s.J[p * ma + lk];
                    M[j * mf + k] = acc;
                }
                for (int j = tid; j < mf; j += kThreads) {
                    double acc = bv[j];
                    for (int p = 0; p < np; p++) {
                        const int q = start + t0 + p;
                        const double y = conv ? 0.0 : ob.bright[q];
                        const double dy = y - s.ym[p];
                        acc = acc + dy * wt[p * mf + j];
                    }
                    bv[j] = acc;
                }
                if (tid == kThreads - 1) {
                    double c2 = s.misc[M_CHISQ];
                    for (int p = 0; p < np; p++) {
                        const int q = start + t0 + p;
                        const double sg = conv ? conv_sig : ob.sig[q];
                        const double sig2i = conv ? conv_sig2i : 1 / (sg * sg);
                        const double y = conv ? 0.0 : ob.bright[q];
                        const double dy = y - s.ym[p];
                        c2 = c2 + dy * dy * sig2i * ob.weight[q];
                    }
                    s.misc[M_CHISQ] = c2;
                }
                __syncthreads();
            }
        }
        if (!rel) continue;
        // ---- pass 2: renormalise and accumulate (mrqcof.c:90-136) ----
        const double ave = s.misc[M_AVE];
        for (int t0 = 0; t0 < npts; t0 += P) {
            const int np = min(P, npts - t0);
            const double *src = scratch + static_cast<size_t>(t0) * (ma + 1);
            for (int e = tid; e < np * ma; e += kThreads) {
                const int p = e / ma, l = e - p * ma;
                const int q = start + t0 + p;
                const double coef = ob.sig[q] * npts / ave;
                const double yt = src[static_cast<size_t>(p) * (ma + 1) + ma];
                double v = coef * (src[static_cast<size_t>(p) * (ma + 1) + l] - yt * s.dave[l] / ave);
                s.J[e] = (l == 0) ? 0.0 : v;
            }
            if (tid < np) {
                const int q = start + t0 + tid;
                const double coef = ob.sig[q] * npts / ave;
                s.ym[tid] = coef * src[static_cast<size_t>(tid) * (ma + 1) + ma];
            }
            __syncthreads();
            double *wt = s.W;
            for (int e = tid; e < np * mf; e += kThreads) {
                const int p = e / mf, j = e - p * mf;
                const int q = start + t0 + p;
                const double sig2i = 1 / (ob.sig[q] * ob.sig[q]);
                wt[p * mf + j] = s.J[p * ma + ob.free_list[j]] * sig2i * ob.weight[q];
            }
            __syncthreads();
            const int ntri = mf * (mf + 1) / 2;
            for (int e = tid; e < ntri; e += kThreads) {
                const int j = tri_row(e);
                const int k = e - j * (j + 1) / 2;
                const int lk = ob.free_list[k];
                double acc = M[j * mf + k];
                for (int p = 0; p < np; p++) acc = acc + wt[p * mf + j] * s.J[p * ma + lk];
                M[j * mf + k] = acc;
            }
            for (int j = tid; j < mf; j += kThreads) {
                double acc = bv[j];
                for (int p = 0; p < np; p++) {
                    const double dy = ob.bright[start + t0 + p] - s.ym[p];
                    acc = acc + dy * wt[p * mf + j];
                }
                bv[j] = acc;
            }
            if (tid == kThreads - 1) {
                double c2 = s.misc[M_CHISQ];
                for (int p = 0; p < np; p++) {
                    const int q = start + t0 + p;
                    const double sig2i = 1 / (ob.sig[q] * ob.sig[q]);
                    const double dy = ob.bright[q] - s.ym[p];
                    c2 = c2 + dy * dy * sig2i * ob.weight[q];
                }
                s.misc[M_CHISQ] = c2;
            }
            __syncthreads();
        }
    }
    // mirror the lower triangle (mrqcof.c:139-141)
    for (int e = tid; e < mf * mf; e += kThreads) {
        const int j = e / mf, k = e - j * mf;
        if (k > j) M[e] = M[k * mf + j];
    }
    __syncthreads();
}

// Gauss-Jordan elimination with full pivoting on A (n x n, row-major in
// shared memory) and right-hand side b (gauss_errc.c:9-73).  Only the
// solution is needed by the LM step, so the columns that already hold the
// inverse are not updated and the final column unscrambling is skipped; the
// pivot choices and the solution are those of the full algorithm.
// Returns 0, 1 (no usable pivot: NaN entries) or 2 (zero pivot).
__device__ int gauss_jordan(double *A, double *b, int n, double *col, int *ipiv, double *red)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int k = tid; k < n; k += kThreads) ipiv[k] = 0;
    __syncthreads();
    for (int step = 0; step < n; step++) {
        // pivot search: largest |a| over unpivoted rows and columns; ties go
        // to the last element in row-major order (the reference's >=).
        double bv = -1.0;
        int bi = -1;
        for (int e = tid; e < n * n; e += kThreads) {
            const int j = e / n, k = e - j * n;
            if (ipiv[j] != 1 && ipiv[k] == 0) {
                const double v = fabs(A[e]);
                if (v >= 0.0 && (v > bv || (v == bv && e > bi))) {
                    bv = v;
                    bi = e;
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > bv || (ov == bv && oi > bi)) {
                bv = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            red[warp] = bv;
            ipiv[n + 2 + warp] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            double v = red[0];
            int idx = ipiv[n + 2];
            for (int w = 1; w < kThreads / 32; w++) {
                const double ov = red[w];
                const int oi = ipiv[n + 2 + w];
                if (ov > v || (ov == v && oi > idx)) {
                    v = ov;
                    idx = oi;
                }
            }
            ipiv[n] = idx;
            if (idx >= 0) ipiv[idx - (idx / n) * n] += 1;
        }
        __syncthreads();
        const int idx = ipiv[n];
        if (idx < 0) return 1;
        const int irow = idx / n, icol = idx - irow * n;
        if (irow != icol) {
            for (int l = tid; l < n; l += kThreads) {
                const double t = A[irow * n + l];
                A[irow * n + l] = A[icol * n + l];
                A[icol * n + l] = t;
            }
            if (tid == 0) {
                const double t = b[irow];
                b[irow] = b[icol];
                b[icol] = t;
            }
            __syncthreads();
        }
        const double piv = A[icol * n + icol];
        if (piv == 0.0) return 2;
        const double pivinv = 1.0 / piv;
        __syncthreads();
        // scale the pivot row over the columns not yet pivoted
        for (int l = tid; l < n; l += kThreads)
            if (ipiv[l] == 0) A[icol * n + l] *= pivinv;
        if (tid == 0) b[icol] *= pivinv;
        for (int r = tid; r < n; r += kThreads) col[r] = A[r * n + icol];
        __syncthreads();
        for (int e = tid; e < n * n; e += kThreads) {
            const int r = e / n, l = e - r * n;
            if (r != icol && ipiv[l] == 0) A[e] -= A[icol * n + l] * col[r];
        }
        for (int r = tid; r < n; r += kThreads)
            if (r != icol) b[r] -= b[icol] * col[r];
        __syncthreads();
    }
    return 0;
}

// ---------------------------------------------------------------------------
// One fit (period_search_BOINC.cpp:817-921 with mrqmin.c:11-110).
// ---------------------------------------------------------------------------
template <int FORM>
__device__ void run_fit(const DevObject &ob, const FitConfig &cfg, const SlotLayout &L, Smem &s,
                        double *scratch, int64_t n, int pole, ps_fit *out)
{
    const int tid = threadIdx.x;
    const int C = ob.ncoef, ma = ob.ma, mf = ob.mfit;
    const double freq = cfg.freq_start - (n - 1) * cfg.freq_step;
    const double prd = 1 / freq;
    for (int i = tid; i < ma; i += kThreads) {
        double v;
        if (i < C) v = ob.cg_first[i];
        else if (i == C) v = kDeg2Rad * (90 - c_beta_pole[pole - 1]);
        else if (i == C + 1) v = kDeg2Rad * c_lambda_pole[pole - 1];
        else if (i == C + 2) v = 24 * 2 * kPi / prd;
        else if (i == C + 3) v = cfg.par0;
        else if (i == C + 4) v = cfg.par1;
        else if (i == C + 5) v = cfg.par2;
        else if (i == C + 6) v = cfg.log_cl;
        else v = 1;
        s.cg[i] = v;
        s.atry[i] = v;
    }
    __syncthreads();

    double alamda = -1, ochisq = 0, chisq = 0, rchisq = -1;
    double iter_diff = 1e40, dev_old = 1e30, dev_new = 0;
    double chk_acc[3] = {0, 0, 0}, chk_first[3] = {0, 0, 0}, chk_trial[3] = {0, 0, 0};
    double area_first = 0, area_trial = 0, totarea = 0;
    int niter = 0, last_err = 0;
    while (((niter < cfg.n_iter_max) && (iter_diff > cfg.iter_diff_max)) || (niter < cfg.n_iter_min)) {
        bool accepted = false;
        bool evaluated_trial = false;
        if (alamda < 0) {
            alamda = cfg.alamda_start;
            evaluate<FORM>(ob, cfg, L, s, s.cg, s.alpha, s.beta, scratch);
            ochisq = s.misc[M_CHISQ];
            area_first = s.misc[M_AREA];
            for (int c = 0; c < 3; c++) chk_first[c] = s.misc[M_CHK + c];
            totarea = area_first;
        }
        for (int e = tid; e < mf * mf; e += kThreads) {
            const int j = e / mf, k = e - j * mf;
            s.covar[e] = (j == k) ? s.alpha[e] * (1 + alamda) : s.alpha[e];
        }
        for (int j = tid; j < mf; j += kThreads) s.da[j] = s.beta[j];
        __syncthreads();
        const int err = gauss_jordan(s.covar, s.da, mf, s.col, s.ipiv, s.misc + M_RED);
        __syncthreads();
        if (err == 0) {
            for (int j = tid; j < mf; j += kThreads) {
                const int l = ob.free_list[j];
                s.atry[l] = s.cg[l] + s.da[j];
            }
            __syncthreads();
            evaluate<FORM>(ob, cfg, L, s, s.atry, s.covar, s.da, scratch);
            evaluated_trial = true;
            chisq = s.misc[M_CHISQ];
            area_trial = s.misc[M_AREA];
            for (int c = 0; c < 3; c++) chk_trial[c] = s.misc[M_CHK + c];
            totarea = area_trial;
            if (chisq < ochisq) {
                accepted = true;
                alamda = alamda / cfg.alamda_incr;
                for (int e = tid; e < mf * mf; e += kThreads) s.alpha[e] = s.covar[e];
                for (int j = tid; j < mf; j += kThreads) s.beta[j] = s.da[j];
                for (int l = tid; l < ma; l += kThreads) s.cg[l] = s.atry[l];
                __syncthreads();
            } else {
                alamda = cfg.alamda_incr * alamda;
                chisq = ochisq;
            }
        } else {
            last_err = err;
        }
        (void)evaluated_trial;
        niter++;
        if ((niter == 1) || (chisq < ochisq)) {
            ochisq = chisq;
            // curv(cg) of the driver: the accepted shape is the trial one;
            // otherwise (first iteration, rejected or failed solve) cg is
            // still the starting vector of the first evaluation.
            const double *src = accepted ? chk_trial : chk_first;
            for (int c = 0; c < 3; c++) chk_acc[c] = src[c];
            totarea = accepted ? area_trial : area_first;
            rchisq = chisq - (chk_acc[0] * chk_acc[0] + chk_acc[1] * chk_acc[1] + chk_acc[2] * chk_acc[2]) *
                                 (cfg.conw_r * cfg.conw_r);
        }
        dev_new = sqrt(rchisq / ob.ndata);
        if (dev_old - dev_new > 1e-10) {
            iter_diff = dev_old - dev_new;
            dev_old = dev_new;
        }
    }
    if (tid == 0) {
        ps_fit r;
        r.dev = dev_new;
        r.dark = sqrt(chk_acc[0] * chk_acc[0] + chk_acc[1] * chk_acc[1] + chk_acc[2] * chk_acc[2]);
        r.totarea = totarea;
        r.period_h = 24 * (2 * kPi / s.cg[C + 2]);
        r.lambda_deg = kRad2Deg * s.cg[C + 1];
        r.beta_deg = 90 - kRad2Deg * s.cg[C];
        r.chisq = chisq;
        r.niter = niter;
        r.err_code = last_err;
        *out = r;
    }
    __syncthreads();
}

template <int FORM>
__global__ void __launch_bounds__(kThreads) fit_kernel(DevObject ob, FitConfig cfg, FitWork w, int P)
{
    extern __shared__ __align__(16) double smem[];
    const SlotLayout L = make_layout(ob.ma, ob.mfit, ob.nfac, P);
    Smem s = carve(smem, L);
    double *scratch = w.scratch + static_cast<size_t>(blockIdx.x) * w.scratch_stride;
    __shared__ long long next;
    for (;;) {
        if (threadIdx.x == 0) next = static_cast<long long>(atomicAdd(w.queue, 1ULL));
        __syncthreads();
        const long long f = next;
        __syncthreads();
        if (f >= w.nfits) break;
        int64_t n;
        int pole;
        if (w.period_index) {
            n = w.period_index[f];
            pole = w.pole[f];
        } else {
            n = w.n_lo + f / PS_N_POLES;
            pole = static_cast<int>(f % PS_N_POLES) + 1;
        }
        run_fit<FORM>(ob, cfg, L, s, scratch, n, pole, w.out + f);
    }
}

template <int FORM>
__global__ void __launch_bounds__(kThreads) eval_kernel(DevObject ob, FitConfig cfg, const double *cg, double *alpha,
                                                        double *beta, double *chisq, double *area, double *scratch,
                                                        int P)
{
    extern __shared__ __align__(16) double smem[];
    const SlotLayout L = make_layout(ob.ma, ob.mfit, ob.nfac, P);
    Smem s = carve(smem, L);
    for (int i = threadIdx.x; i < ob.ma; i += kThreads) s.cg[i] = cg[i];
    __syncthreads();
    evaluate<FORM>(ob, cfg, L, s, s.cg, s.alpha, s.beta, scratch);
    const int mf = ob.mfit;
    for (int e = threadIdx.x; e < mf * mf; e += kThreads) alpha[e] = s.alpha[e];
    for (int j = threadIdx.x; j < mf; j += kThreads) beta[j] = s.beta[j];
    if (area)
        for (int i = threadIdx.x; i < ob.nfac; i += kThreads) area[i] = s.area[i];
    if (threadIdx.x == 0) *chisq = s.misc[M_CHISQ];
}

// FMA throughput probe: 8 independent FMA chains per thread.
template <class T>
__global__ void __launch_bounds__(256) fma_probe(T *sink, int iters, T x, T y)
{
    T a[8];
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = static_cast<T>(threadIdx.x + k);
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int k = 0; k < 8; k++) a[k] = a[k] * x + y;
    T t = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) t += a[k];
    if (t == static_cast<T>(-1.2345)) sink[threadIdx.x] = t;
}

}  // namespace

// Measured FMA throughput of the current device in TFLOP/s (2 flops per FMA),
// FP64 and FP32, best of a few launches of blocks_per_sm * SMs CTAs.
int measure_fma_peaks(double *fp64_tflops, double *fp32_tflops, void *stream)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double *sink = nullptr;
    if (cudaMalloc(&sink, 256 * sizeof(double)) != cudaSuccess) return static_cast<int>(cudaGetLastError());
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int grid = sms * 4, iters64 = 1 << 12, iters32 = 1 << 15;
    double best64 = 0, best32 = 0;
    for (int rep = 0; rep < 3; rep++) {
        float ms = 0;
        cudaEventRecord(e0, st);
        fma_probe<double><<<grid, 256, 0, st>>>(sink, iters64, 0.999999, 1e-7);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        double fl = 2.0 * 8 * iters64 * static_cast<double>(grid) * 256;
        if (ms > 0) best64 = fl / (ms * 1e-3) / 1e12 > best64 ? fl / (ms * 1e-3) / 1e12 : best64;
        cudaEventRecord(e0, st);
        fma_probe<float><<<grid, 256, 0, st>>>(reinterpret_cast<float *>(sink), iters32, 0.999999f, 1e-7f);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        fl = 2.0 * 8 * iters32 * static_cast<double>(grid) * 256;
        if (ms > 0) best32 = fl / (ms * 1e-3) / 1e12 > best32 ? fl / (ms * 1e-3) / 1e12 : best32;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    *fp64_tflops = best64;
    *fp32_tflops = best32;
    return static_cast<int>(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Scratch for the allocation-free entry point (ps_fit_batch_noalloc).
//
// Some hosts cannot let a library allocate device memory when it is called:
// applications that hand all of the GPU's memory to their own pool allocator
// up front, processes running under a fixed device-memory budget where a
// failed allocation in the middle of a job is not acceptable, and pipelines
// that keep other streams busy and cannot afford the device-wide
// synchronisation that cudaMalloc/cudaFree imply.  For them the fit kernel
// can take its work counter and its per-slot scratch from this file-scope
// array instead.  Every GPU that loads the library reserves it until the
// process exits.  Layout: the first 32 doubles hold the work counter (cleared
// before each launch), then one scratch block per fit slot.
// ---------------------------------------------------------------------------
constexpr size_t kStaticCounterDoubles = 32;
static __device__ __align__(256) double g_noalloc_scratch[kStaticScratchDoubles];

namespace {
std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[64] = {};  // device address of g_noalloc_scratch, per device ordinal
}  // namespace

int launch_fits_noalloc(int form, const DevObject &ob, const FitConfig &cfg, FitWork w, int max_grid, int P,
                        size_t smem, void *stream, int *grid_used)
{
    if (form != PS_FORM_FP64) return static_cast<int>(cudaErrorInvalidValue);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return static_cast<int>(e);
    if (dev < 0 || dev >= 64) return static_cast<int>(cudaErrorInvalidDevice);
    double *base = nullptr;
    {
        // Host code cannot use the array's name as a device address; look the
        // address up once per device, with that device current.
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[dev]) {
            e = cudaGetSymbolAddress(reinterpret_cast<void **>(&g_noalloc_ptr[dev]), g_noalloc_scratch);
            if (e != cudaSuccess) {
                g_noalloc_ptr[dev] = nullptr;
                return static_cast<int>(e);
            }
        }
        base = g_noalloc_ptr[dev];
    }
    const size_t usable = kStaticScratchDoubles - kStaticCounterDoubles;
    const int64_t slots = static_cast<int64_t>(usable / w.scratch_stride);
    if (slots < 1) return -1;  // one slot's scratch exceeds the array
    int64_t grid = slots < max_grid ? slots : max_grid;
    if (grid > w.nfits) grid = w.nfits;
    w.queue = reinterpret_cast<unsigned long long *>(base);
    w.scratch = base + kStaticCounterDoubles;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    e = cudaMemsetAsync(base, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return static_cast<int>(e);
    fit_kernel<0><<<static_cast<int>(grid), kThreads, smem, st>>>(ob, cfg, w, P);
    *grid_used = static_cast<int>(grid);
    return static_cast<int>(cudaGetLastError());
}

int set_kernel_smem(int form, size_t smem)
{
    cudaError_t e;
    if (form == PS_FORM_FP64) {
        e = cudaFuncSetAttribute(fit_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(eval_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    } else {
        return static_cast<int>(cudaErrorInvalidValue);
    }
    return static_cast<int>(e);
}

int occupancy_slots(int form, size_t smem, int *per_sm)
{
    if (form != PS_FORM_FP64) return static_cast<int>(cudaErrorInvalidValue);
    return static_cast<int>(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, fit_kernel<0>, kThreads, smem));
}

int launch_fits(int form, const DevObject &ob, const FitConfig &cfg, const FitWork &w, int grid, int P, size_t smem,
                void *stream)
{
    if (form != PS_FORM_FP64) return static_cast<int>(cudaErrorInvalidValue);
    fit_kernel<0><<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(ob, cfg, w, P);
    return static_cast<int>(cudaGetLastError());
}

int launch_eval(int form, const DevObject &ob, const FitConfig &cfg, const double *cg, double *alpha, double *beta,
                double *chisq, double *area, double *scratch, int P, size_t smem, void *stream)
{
    if (form != PS_FORM_FP64) return static_cast<int>(cudaErrorInvalidValue);
    eval_kernel<0><<<1, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(ob, cfg, cg, alpha, beta, chisq, area,
                                                                               scratch, P);
    return static_cast<int>(cudaGetLastError());
}

}  // namespace psg
