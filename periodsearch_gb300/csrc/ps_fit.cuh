// ps_fit.cuh -- fit kernels of the GB300 period-search engine (sm_103a),
// shared by the single-object launchers (ps_engine.cu) and the multi-object
// packed launch (ps_pack.cu).
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
//
// The mixed form runs the contraction on the tensor cores when the shape
// tables allow it (tensor_basis_ok): tcgen05 FP16 MMAs with the basis split
// into high and low FP16 parts (scaled by a power of two) resident in Tensor
// Memory for the CTA's lifetime (A = [Dsph_hi^T; Dsph_lo^T], 128 lanes, two
// facets per column) and W split the same way in shared memory (B), so that
// the four partial products give the contraction to FP32 accuracy; the
// normal-matrix accumulation runs as TF32 high/low MMAs.  Otherwise both run
// on the SIMT pipes.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <type_traits>

#include "ps_engine.h"
#include "ps_tc.cuh"

namespace psg {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoPi = 2 * kPi;
constexpr double kRad2Deg = 180 / kPi;
constexpr double kDeg2Rad = kPi / 180;
constexpr double kTinyMu = 1e-8;
// 2*pi split for the mixed form's phase reduction: hi = 2*pi rounded to
// double, lo = 2*pi - hi.
constexpr double kTwoPiHi = 6.283185307179586;
constexpr double kTwoPiLo = 2.4492935982947064e-16;
constexpr double kInvTwoPi = 0.15915494309189535;

__constant__ double c_beta_pole[PS_N_POLES] = {0, 0, 0, 0, 60, 60, 60, -60, -60, -60};
// blmatrix.c:9-46 entry by entry: factor a (0 zero, 1 cos beta, 2 sin beta,
// 3 one) | factor b << 2 (0 one, 1 cos lambda, 2 sin lambda) | 16 negated;
// rows of B, then dB/dbeta, then dB/dlambda
__constant__ unsigned char c_bl_code[27] = {5,  9,  18, 27, 7, 0, 6,  10, 1,  22, 26, 17, 0, 0,
                                            0,  5,  9,  18, 25, 5, 0, 23, 27, 0,  26, 6,  0};
__constant__ double c_lambda_pole[PS_N_POLES] = {0, 90, 180, 270, 60, 180, 300, 60, 180, 300};

// Arithmetic type of the facet stage, the contraction and the model rows.
template <int FORM> struct RealOf { using T = double; };
template <> struct RealOf<PS_FORM_MIXED> { using T = float; };

template <int FORM>
struct Smem {
    using R = typename RealOf<FORM>::T;
    double *cg, *atry, *beta, *da, *alpha, *covar, *area, *gv, *ym, *red, *dave, *col, *misc;
    R *areaR, *gvR, *W, *J, *pt;
    R *pt2;       // the other point set-up buffer (== pt unless set-up runs one tile ahead)
    float *accs;  // mixed form: per-point FP32 weights and residuals of a tile
    float *davef; // mixed form: FP32 copy of a relative lightcurve's derivative sums
    R *bmat;      // [27] rotation matrix and its beta/lambda derivatives, [27..29] phase
                  // function a, d, k, [30] Lommel-Seeliger and [31] Lambert weight
    int *ipiv;
    float *dsph;  // FP32 basis in shared memory (mixed form), or nullptr
    // tensor-core contraction: operand tiles, MMA-completion barrier, Tensor
    // Memory address slot and the abort flag set when a wait gives up
    unsigned char *bhi, *blo;
    uint64_t *mbar, *mbar2;   // completion of the contraction MMAs / of the alpha MMAs
    float4 *fac;              // per facet pair (2j, 2j + 1): {nx, nx', ny, ny'}, {nz, nz', Area, Area'} (fac_at)
    float *fpart;             // [4][P][9] facet-sum partials of the four facet quarters
    unsigned char *aop;       // alpha/beta MMA operands
    unsigned char *pref;      // per-point data prefetched for the contraction window
    int *flist;               // the free parameters' columns (tensor-core path)
    // FP64 form: lit-facet count of each point of the tile, and its lit
    // facets in increasing order ([P][wcols], the W row holds their values)
    int *nlit;
    uint16_t *lidx;
    uint32_t *tslot;
    int *abort;
};

template <int FORM>
__device__ inline Smem<FORM> carve(char *base, const SlotLayout &L)
{
    using R = typename RealOf<FORM>::T;
    Smem<FORM> s;
    s.cg = reinterpret_cast<double *>(base + L.cg);
    s.atry = reinterpret_cast<double *>(base + L.atry);
    s.beta = reinterpret_cast<double *>(base + L.beta);
    s.da = reinterpret_cast<double *>(base + L.da);
    s.alpha = reinterpret_cast<double *>(base + L.alpha);
    s.covar = reinterpret_cast<double *>(base + L.covar);
    s.area = reinterpret_cast<double *>(base + L.area);
    s.gv = reinterpret_cast<double *>(base + L.gv);
    s.areaR = reinterpret_cast<R *>(base + L.areaR);
    s.gvR = reinterpret_cast<R *>(base + L.gvR);
    s.W = reinterpret_cast<R *>(base + L.W);
    s.J = reinterpret_cast<R *>(base + L.J);
    s.pt = reinterpret_cast<R *>(base + L.pt);
    s.pt2 = reinterpret_cast<R *>(base + L.pt2);
    s.accs = reinterpret_cast<float *>(base + L.accs);
    s.davef = reinterpret_cast<float *>(base + L.davef);
    s.bmat = reinterpret_cast<R *>(base + L.bmat);
    s.ym = reinterpret_cast<double *>(base + L.ym);
    s.red = reinterpret_cast<double *>(base + L.red);
    s.dave = reinterpret_cast<double *>(base + L.dave);
    s.col = reinterpret_cast<double *>(base + L.col);
    s.misc = reinterpret_cast<double *>(base + L.misc);
    s.ipiv = reinterpret_cast<int *>(base + L.ipiv);
    s.nlit = L.form == PS_FORM_FP64 ? reinterpret_cast<int *>(base + L.lit) : nullptr;
    s.lidx = L.form == PS_FORM_FP64 ? reinterpret_cast<uint16_t *>(base + L.lit + 4 * static_cast<size_t>(L.P))
                                     : nullptr;
    s.dsph = L.dsph_smem == kBasisSmem ? reinterpret_cast<float *>(base + L.dsph) : nullptr;
    if (basis_on_tensor(L.dsph_smem)) {
        s.bhi = reinterpret_cast<unsigned char *>(base + L.bhi);
        s.blo = reinterpret_cast<unsigned char *>(base + L.blo);
        s.mbar = reinterpret_cast<uint64_t *>(base + L.tcm);
        s.tslot = reinterpret_cast<uint32_t *>(base + L.tcm + 8);
        s.abort = reinterpret_cast<int *>(base + L.tcm + 12);
        s.mbar2 = reinterpret_cast<uint64_t *>(base + L.tcm + 16);
        s.fac = reinterpret_cast<float4 *>(base + L.fac);
        s.fpart = reinterpret_cast<float *>(base + L.fpart);
        s.aop = reinterpret_cast<unsigned char *>(base + L.aop);
        s.pref = reinterpret_cast<unsigned char *>(base + L.pref);
        s.flist = reinterpret_cast<int *>(base + L.flist);
        // wide path: the SIMT accumulation's weighted rows are staged in the
        // operand region (free between a tile's readback and the next
        // tile's facet stage)
        if (L.dsph_smem == kBasisTensorWide) s.W = reinterpret_cast<R *>(base + L.bhi);
    } else {
        s.bhi = s.blo = nullptr;
        s.mbar = s.mbar2 = nullptr;
        s.tslot = nullptr;
        s.fac = nullptr;
        s.fpart = nullptr;
        s.aop = nullptr;
        s.pref = nullptr;
        s.flist = nullptr;
        s.abort = nullptr;
    }
    return s;
}

// misc slots
enum : int {
    M_CHISQ = 0,   // chi^2 accumulator of the current evaluation
    M_AVE = 1,     // relative-lightcurve model sum
    M_AREA = 2,    // sum of facet areas of the current evaluation
    M_CHK = 3,     // 3 convexity residuals (sum Area*n) of the current evaluation
    M_INVAVE = 6,  // mixed form: 1 / sum of the current relative lightcurve's model
    M_CL = 7,      // exp(log cl)
    M_TRIG = 8,    // cos/sin of the pole angles beta, lambda (4 doubles)
    M_PIV = 12,    // pivot broadcast of the solvers (2 doubles + status)
    M_RED = 16,    // 16 doubles of block-reduction scratch
    M_LM = 32,     // 4 doubles: lambda, ochisq, dev, iter_diff of the fit, broadcast from thread 0
    M_WEXP = 36,   // tensor-core path: exponent of the evaluation's W scale
    M_LIT = 37     // FP64 form: the CTA's count of lit facet-point pairs (an unsigned 64-bit integer)
};

// FP64 form: the CTA's lit facet-point counter in misc.
__device__ inline unsigned long long *lit_counter(double *misc)
{
    return reinterpret_cast<unsigned long long *>(misc + M_LIT);
}

// Facet table of the tensor-core path, interleaved by facet pairs so that
// the facet stage loads each pair's components as FP32x2 register pairs:
// float4 2j = {nx_2j, nx_2j+1, ny_2j, ny_2j+1}, float4 2j + 1 = {nz_2j,
// nz_2j+1, Area_2j, Area_2j+1}.  Component c (0 nx, 1 ny, 2 nz, 3 Area) of
// facet i:
__device__ inline float &fac_at(float4 *fac, int i, int c)
{
    return reinterpret_cast<float *>(fac)[(i >> 1) * 8 + 2 * c + (i & 1)];
}

// Row j of packed lower-triangle element e (j*(j+1)/2 <= e < (j+1)*(j+2)/2),
// from an FP32 square root corrected in integers.
__device__ inline int tri_row(int e)
{
    int j = static_cast<int>((sqrtf(8.0f * static_cast<float>(e) + 1.0f) - 1.0f) * 0.5f);
    while (j * (j + 1) / 2 > e) j--;
    while ((j + 1) * (j + 2) / 2 <= e) j++;
    return j;
}

template <class T>
__device__ inline T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block; every thread gets the result.  red holds >= NT/32 doubles.
template <int NT>
__device__ inline double block_sum(double v, double *red)
{
    v = warp_sum(v);
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double t = 0;
#pragma unroll
    for (int i = 0; i < NT / 32; i++) t += red[i];
    __syncthreads();
    return t;
}

// Asynchronous global -> shared copies (cp.async, 8 or 16 bytes, both
// addresses aligned to the size), completed by cp_async_wait_all of the
// issuing thread.
__device__ inline void cp_async8(void *dst_smem, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst_smem))),
                 "l"(src)
                 : "memory");
}
__device__ inline void cp_async16(void *dst_smem, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst_smem))),
                 "l"(src)
                 : "memory");
}
__device__ inline void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ inline void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Rotation phase omega*t + phi0 reduced to [0, 2*pi).  The FP64 form rounds
// the product and the sum separately and reduces with fmod, as the
// reference does (matrix.c:21-22).  The mixed form reduces in FP64 with a
// two-part 2*pi (the product rounded once), exact to ~1e-16 rad, and hands
// the phase on in FP32 (its only use is the FP32 cos/sin), so the final
// wrap into [0, 2*pi) runs in FP32.
__device__ inline double rotation_phase_fp64(double omg, double t, double phi0)
{
    return fmod(__dadd_rn(__dmul_rn(omg, t), phi0), kTwoPi);
}

__device__ inline float rotation_phase_mixed(double omg, double t, double phi0)
{
    constexpr float kTwoPiF = 6.28318548f;   // 2*pi rounded to FP32
    const double x = fma(omg, t, phi0);
    const double q = floor(x * kInvTwoPi);
    double f = fma(-q, kTwoPiHi, x);
    f = fma(-q, kTwoPiLo, f);
    float ff = static_cast<float>(f);
    if (ff < 0.f) ff += kTwoPiF;
    if (ff >= kTwoPiF) ff -= kTwoPiF;
    return ff;
}

// FP64 form: sum_i W[p][i] Dsph[i][k] (ds = Dsph + k) for point p of the
// tile.  Model rows sum over the point's lit facets, in increasing order as
// bright.c:79-86 does (a dense sum over all facets adds only exact zeros,
// so the two agree bit for bit); convexity rows sum over every facet.
template <class S>
__device__ inline double contract_fp64(const S &s, const double *ds, int p, int C, int F, int wcols, bool conv)
{
    const double *Wp = s.W + static_cast<size_t>(p) * wcols;
    double acc = 0;
    if (conv) {
        for (int i = 0; i < F; i++) acc = acc + Wp[i] * ds[static_cast<size_t>(i) * C];
    } else {
        const uint16_t *idx = s.lidx + static_cast<size_t>(p) * wcols;
        const int n = s.nlit[p];
        for (int j = 0; j < n; j++) acc = acc + Wp[j] * ds[static_cast<size_t>(idx[j]) * C];
    }
    return acc;
}

// Lit-facet terms of the Lommel-Seeliger + Lambert law (bright.c:65-74,
// 116-117).  The reference divides four times by mu + mu0; both forms
// multiply by one reciprocal instead (the FP64 form's correctly rounded, so
// each quotient is within an ulp of the reference's; the mixed form's
// approximate).
template <class R, int FORM>
struct LitTerms {
    R sv, dsmu, dsmu0, dcls_w;  // s, ds/dmu, ds/dmu0, mu*mu0/(mu+mu0)
    __device__ inline LitTerms(R mu, R mu0, R cl, R cls)
    {
        const R dnom = mu + mu0;
        if constexpr (FORM == PS_FORM_FP64) {
            const R r = 1.0 / dnom;
            sv = mu * mu0 * (cl + cls * r);
            const R q0 = mu0 * r, q1 = mu * r;
            dsmu = cls * (q0 * q0) + cl * mu0;
            dsmu0 = cls * (q1 * q1) + cl * mu;
            dcls_w = mu * mu0 * r;
        } else {
            R r;
            asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(dnom));   // ~1 ulp: the mixed form's budget
            sv = mu * mu0 * (cl + cls * r);
            const R q0 = mu0 * r, q1 = mu * r;
            dsmu = cls * (q0 * q0) + cl * mu0;
            dsmu0 = cls * (q1 * q1) + cl * mu;
            dcls_w = mu * mu0 * r;
        }
    }
};

// One butterfly level over lane bit m: of the pair (a, c) a lane keeps a
// (bit clear) or c (bit set), adding the partner lane's copy of it; one
// shuffle carries the half each lane gives away.  ia, ic: the values' ids.
__device__ inline double fold_pair(double a, double c, int ia, int ic, int m, int lane, int &id)
{
    const bool hi = (lane & m) != 0;
    const double give = hi ? a : c, keep = hi ? c : a;
    id = hi ? ic : ia;
    return keep + __shfl_xor_sync(0xffffffffu, give, m);
}

// Sums nine FP64 values over the warp and stores sum k at out[k]: every
// level pairs the same lanes as warp_sum, so each sum is warp_sum's bit for
// bit, in 12 shuffles and 12 additions instead of 45.  Each sum ends in the
// lanes that kept it; they store it (the same value).
__device__ inline void warp_sum9(const double (&v)[9], double *out, int lane)
{
    double w[5];
    int iw[5];
#pragma unroll
    for (int j = 0; j < 4; j++) w[j] = fold_pair(v[2 * j], v[2 * j + 1], 2 * j, 2 * j + 1, 16, lane, iw[j]);
    w[4] = v[8] + __shfl_xor_sync(0xffffffffu, v[8], 16);
    iw[4] = 8;
    double x[3];
    int ix[3];
    x[0] = fold_pair(w[0], w[1], iw[0], iw[1], 8, lane, ix[0]);
    x[1] = fold_pair(w[2], w[3], iw[2], iw[3], 8, lane, ix[1]);
    x[2] = w[4] + __shfl_xor_sync(0xffffffffu, w[4], 8);
    ix[2] = iw[4];
    double y[2];
    int iy[2];
    y[0] = fold_pair(x[0], x[1], ix[0], ix[1], 4, lane, iy[0]);
    y[1] = x[2] + __shfl_xor_sync(0xffffffffu, x[2], 4);
    iy[1] = ix[2];
    int iz;
    const double z = fold_pair(y[0], y[1], iy[0], iy[1], 2, lane, iz);
    out[iz] = z + __shfl_xor_sync(0xffffffffu, z, 1);
}

// FP64 facet stage of point p of the tile (bright.c:59-120), one warp.  A
// first pass lists the point's lit facets in increasing order (s.lidx,
// s.nlit); the law and the facet sums then run over that list with every
// lane busy (an FP64 instruction holds its sub-partition's FP64 unit for
// the whole warp, however few lanes are active), lane l taking the list's
// entries l, l + 32, ...  W is left in the W row at the list positions.
// The facet sums go to s.red[p * kRedStride + 0..5]: brightness, the three
// rotation derivatives, the Lambert and the scattering-weight derivatives.
__device__ inline void facet_point_fp64(const DevObject &ob, Smem<PS_FORM_FP64> &s, int p, int wcols, double cl,
                                        double cls)
{
    const int lane = threadIdx.x & 31, F = ob.nfac;
    const double *pt = s.pt + p * kPointStride;
    const double e1 = pt[0], e2 = pt[1], e3 = pt[2];
    const double f1 = pt[3], f2 = pt[4], f3 = pt[5];
    uint16_t *idx = s.lidx + static_cast<size_t>(p) * wcols;
    // The lit test in FP32 where it is decided beyond its rounding: the FP32
    // dot products of the FP32-rounded unit vectors are within ~4e-7 of the
    // FP64 ones, so outside a 1e-4 band (scaled by the direction's 1-norm)
    // around kTinyMu the FP64 test gives the same answer; inside it the FP64
    // test runs (on the FP64 unit, which the first pass then leaves alone).
    const float e1f = static_cast<float>(e1), e2f = static_cast<float>(e2), e3f = static_cast<float>(e3);
    const float f1f = static_cast<float>(f1), f2f = static_cast<float>(f2), f3f = static_cast<float>(f3);
    const float band_e = 1e-4f * fmaxf(1.f, fabsf(e1f) + fabsf(e2f) + fabsf(e3f));
    const float band_f = 1e-4f * fmaxf(1.f, fabsf(f1f) + fabsf(f2f) + fabsf(f3f));
    const float tiny = static_cast<float>(kTinyMu);
    int n = 0;
    for (int i0 = 0; i0 < F; i0 += 32) {
        const int i = i0 + lane;
        bool lit = false;
        if (i < F) {
            const float nxf = ob.nx_f[i], nyf = ob.ny_f[i], nzf = ob.nz_f[i];
            const float muf = e1f * nxf + e2f * nyf + e3f * nzf;
            const float mu0f = f1f * nxf + f2f * nyf + f3f * nzf;
            if (muf > tiny + band_e && mu0f > tiny + band_f) {
                lit = true;
            } else if (!(muf < tiny - band_e || mu0f < tiny - band_f)) {
                const double mu = e1 * ob.nx[i] + e2 * ob.ny[i] + e3 * ob.nz[i];
                const double mu0 = f1 * ob.nx[i] + f2 * ob.ny[i] + f3 * ob.nz[i];
                lit = mu > kTinyMu && mu0 > kTinyMu;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, lit);
        if (lit) idx[n + __popc(m & ((1u << lane) - 1u))] = static_cast<uint16_t>(i);
        n += __popc(m);
    }
    __syncwarp();
    // The rotation derivatives sum_i Area_i (dsmu_i (n_i . D_k) + dsmu0_i
    // (n_i . E_k)) (bright.c:87-104; D_k, E_k: the derivative directions of
    // the Earth and Sun vectors) are D_k . U + E_k . V with U = sum Area
    // dsmu n and V = sum Area dsmu0 n: the law accumulates U and V, the six
    // dot products run once per point.
    double br = 0, ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, vz = 0, dcl = 0, dcls = 0;
    double *Wp = s.W + static_cast<size_t>(p) * wcols;
    for (int j = lane; j < n; j += 32) {
        const int i = idx[j];
        const double nx = ob.nx[i], ny = ob.ny[i], nz = ob.nz[i];
        const double mu = e1 * nx + e2 * ny + e3 * nz;
        const double mu0 = f1 * nx + f2 * ny + f3 * nz;
        const double ar = s.area[i];
        const LitTerms<double, PS_FORM_FP64> lt(mu, mu0, cl, cls);
        br = br + ar * lt.sv;
        Wp[j] = ob.darea[i] * lt.sv * s.gv[i];
        const double cu = ar * lt.dsmu, cv = ar * lt.dsmu0;
        ux = ux + cu * nx;
        uy = uy + cu * ny;
        uz = uz + cu * nz;
        vx = vx + cv * nx;
        vy = vy + cv * ny;
        vz = vz + cv * nz;
        dcl = dcl + mu * mu0 * ar;
        dcls = dcls + ar * lt.dcls_w;
    }
    // the nine sums go through the point's J row (written by the
    // contraction only after the stage's barrier)
    double *sums = s.J + static_cast<size_t>(p) * ob.ma;
    const double v9[9] = {br, ux, uy, uz, vx, vy, vz, dcl, dcls};
    warp_sum9(v9, sums, lane);
    __syncwarp();
    if (lane == 0) {
        // D_k = (de[k], de[3 + k], de[6 + k]), E_k likewise from de0
        const double *de = pt + 6, *de0 = pt + 15;
        double *rd = s.red + p * kRedStride;
        rd[0] = sums[0];
#pragma unroll
        for (int k = 0; k < 3; k++)
            rd[1 + k] = de[k] * sums[1] + de[3 + k] * sums[2] + de[6 + k] * sums[3] + de0[k] * sums[4] +
                        de0[3 + k] * sums[5] + de0[6 + k] * sums[6];
        rd[4] = sums[7];
        rd[5] = sums[8];
        s.nlit[p] = n;
        atomicAdd(lit_counter(s.misc), static_cast<unsigned long long>(n));
    }
}

// Accumulates the rows J[0..np) (model values in ym) of one tile into the
// normal matrix M (lower triangle), bv and chi^2 (mrqcof.c:106-136).  The
// FP64 form sums every alpha element over points in data order in FP64; the
// mixed form sums the tile in FP32 and adds the tile sum to the FP64 total.
// Mixed form: every thread keeps its share of the alpha lower triangle
// (elements tid + u*256) and of beta (element tid) as FP32 partial sums in
// registers and adds them to the FP64 totals every few tiles.
constexpr int kAccPerThread = 8;    // with 512 threads: mfit <= 90
constexpr int kTilesPerFlush = 8;
// The tensor-core path's FP32 alpha accumulator in Tensor Memory (products
// of TF32 high/low parts) is added to the FP64 normal matrix every 16 tiles.
constexpr int kTcTilesPerFlush = 16;

template <int FORM>
__device__ inline void flush_partials(double *M, double *bv, int mf, float (&accA)[kAccPerThread], float &accB)
{
    constexpr int NT = threads_of<FORM>();
    const int tid = threadIdx.x;
    const int ntri = mf * (mf + 1) / 2;
#pragma unroll
    for (int u = 0; u < kAccPerThread; u++) {
        const int e = tid + u * NT;
        if (e < ntri) {
            const int j = tri_row(e);
            const int k = e - j * (j + 1) / 2;
            M[j * mf + k] += static_cast<double>(accA[u]);
        }
        accA[u] = 0.f;
    }
    if (tid < mf) bv[tid] += static_cast<double>(accB);
    accB = 0.f;
}

template <int FORM>
__device__ void accumulate_tile(const DevObject &ob, Smem<FORM> &s, double *M, double *bv, int np, int q0pt,
                                bool conv, double conv_sig, float (&accA)[kAccPerThread], float &accB,
                                const double *Jrows = nullptr, const double *ymv = nullptr, int part = 0,
                                int parts = 1)
{
    using R = typename RealOf<FORM>::T;
    constexpr int NT = threads_of<FORM>();
    const int tid = threadIdx.x;
    const int ma = ob.ma, mf = ob.mfit;
    R *wt = s.W;  // [np][mf], reuses the facet-weight tile
    if constexpr (FORM == PS_FORM_FP64) {
        // FP64 form: the tile's rows and model values (Jrows, ymv: another
        // CTA's tile staged here, by default the CTA's own), and of the
        // normal matrix only the elements e = part NT + tid (mod parts NT);
        // chi^2 is summed whole
        if (!Jrows) Jrows = s.J;
        if (!ymv) ymv = s.ym;
        for (int e = tid; e < np * mf; e += NT) {
            const int p = e / mf, j = e - p * mf;
            const int q = q0pt + p;
            const double sig2i = conv ? 1 / (conv_sig * conv_sig) : ob.sig2i[q];
            const double wg = ob.weight[q];
            wt[p * mf + j] = Jrows[p * ma + ob.free_list[j]] * sig2i * wg;
        }
    } else {
        // per point: FP32 weight sig2i*w and residual; chi^2 of the tile
        // summed over one warp in FP64
        float *dyv = s.accs;
        float *wtp = dyv + 32;
        if (tid < 32) {
            double c2 = 0;
            if (tid < np) {
                const int q = q0pt + tid;
                const double sig2i = conv ? 1 / (conv_sig * conv_sig) : ob.sig2i[q];
                const double wg = ob.weight[q];
                const double dy = (conv ? 0.0 : ob.bright[q]) - s.ym[tid];
                dyv[tid] = static_cast<float>(dy);
                wtp[tid] = static_cast<float>(sig2i * wg);
                c2 = dy * dy * sig2i * wg;
            }
            c2 = warp_sum(c2);
            if (tid == 0) s.misc[M_CHISQ] += c2;
        }
        __syncthreads();
        for (int e = tid; e < np * mf; e += NT) {
            const int p = e / mf, j = e - p * mf;
            wt[p * mf + j] = s.J[p * ma + ob.free_list[j]] * wtp[p];
        }
    }
    __syncthreads();
    const int ntri = mf * (mf + 1) / 2;
    if constexpr (FORM == PS_FORM_FP64) {
        for (int e = part * NT + tid; e < ntri; e += parts * NT) {
            const int j = tri_row(e);
            const int k = e - j * (j + 1) / 2;
            const int lk = ob.free_list[k];
            double acc = M[j * mf + k];
            for (int p = 0; p < np; p++) acc = acc + wt[p * mf + j] * Jrows[p * ma + lk];
            M[j * mf + k] = acc;
        }
        for (int j = part * NT + tid; j < mf; j += parts * NT) {
            double acc = bv[j];
            for (int p = 0; p < np; p++) {
                const double y = conv ? 0.0 : ob.bright[q0pt + p];
                acc = acc + (y - ymv[p]) * wt[p * mf + j];
            }
            bv[j] = acc;
        }
    } else {
        const float *dyv = s.accs;
#pragma unroll
        for (int u = 0; u < kAccPerThread; u++) {
            const int e = tid + u * NT;
            if (e < ntri) {
                const int j = tri_row(e);
                const int k = e - j * (j + 1) / 2;
                const int lk = ob.free_list[k];
                float acc = accA[u];
                for (int p = 0; p < np; p++) acc = fmaf(wt[p * mf + j], s.J[p * ma + lk], acc);
                accA[u] = acc;
            }
        }
        if (tid < mf) {
            float acc = accB;
            for (int p = 0; p < np; p++) acc = fmaf(dyv[p], wt[p * mf + tid], acc);
            accB = acc;
        }
    }
    if (FORM == PS_FORM_FP64 && tid == NT - 1) {
        const double *yv = ymv ? ymv : s.ym;
        double c2 = s.misc[M_CHISQ];
        for (int p = 0; p < np; p++) {
            const int q = q0pt + p;
            const double sig2i = conv ? 1 / (conv_sig * conv_sig) : ob.sig2i[q];
            const double y = conv ? 0.0 : ob.bright[q];
            const double dy = y - yv[p];
            c2 = c2 + dy * dy * sig2i * ob.weight[q];
        }
        s.misc[M_CHISQ] = c2;
    }
    __syncthreads();
}

// Basis element Dsph[i][k] of the mixed form: from shared memory with an
// explicit shared-space load, or from global memory through the read-only
// path.
template <bool SMEM_D>
__device__ inline float load_basis(const float *d, int idx)
{
    if constexpr (SMEM_D) {
        float v;
        const unsigned addr = static_cast<unsigned>(__cvta_generic_to_shared(d + idx));
        asm("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
        return v;
    } else {
        return __ldg(d + idx);
    }
}

// Mixed-form shape contraction J[p][k] = Scale_p * sum_i W[p][i] Dsph[i][k]
// of one tile, FP32 on the SIMT pipes.  Register tile: warp w owns points
// (w % 8) + 8 r (r < 4) and coefficients lane + 32 ((w / 8) + 2 u) (u < KU);
// W is read four facets at a time (float4 broadcast), Dsph one coalesced row
// per facet.
template <int NT, int KU, bool SMEM_D>
__device__ void contract_mixed(Smem<PS_FORM_MIXED> &s, const float *dsph, int np, int F, int C, int ma, int wcols,
                               bool conv)
{
    static_assert(NT == 512, "the register tile assumes 16 warps");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = warp & 7, half = warp >> 3;
    constexpr int kPW = 4;
    float acc[kPW][KU];
#pragma unroll
    for (int r = 0; r < kPW; r++)
#pragma unroll
        for (int u = 0; u < KU; u++) acc[r][u] = 0.f;
    int kk[KU];
    bool kv[KU];
#pragma unroll
    for (int u = 0; u < KU; u++) {
        kk[u] = lane + 32 * (half + 2 * u);
        kv[u] = kk[u] < C;
    }
    bool any = false;
#pragma unroll
    for (int u = 0; u < KU; u++) any |= kv[u];
    const float *Wf = s.W;
    if (any) {
        for (int i = 0; i < F; i += 4) {
            float4 w4[kPW];
#pragma unroll
            for (int r = 0; r < kPW; r++) {
                const int p = g + 8 * r;
                w4[r] = (p < np) ? *reinterpret_cast<const float4 *>(Wf + static_cast<size_t>(p) * wcols + i)
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int ii = 0; ii < 4; ii++) {
                float d[KU];
#pragma unroll
                for (int u = 0; u < KU; u++) d[u] = kv[u] ? load_basis<SMEM_D>(dsph, (i + ii) * C + kk[u]) : 0.f;
#pragma unroll
                for (int r = 0; r < kPW; r++) {
                    const float wv = ii == 0 ? w4[r].x : ii == 1 ? w4[r].y : ii == 2 ? w4[r].z : w4[r].w;
#pragma unroll
                    for (int u = 0; u < KU; u++) acc[r][u] = fmaf(wv, d[u], acc[r][u]);
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < kPW; r++) {
        const int p = g + 8 * r;
        if (p < np) {
            const float sc = conv ? 1.f : s.pt[p * kPointStride + 24];
#pragma unroll
            for (int u = 0; u < KU; u++)
                if (kv[u]) s.J[p * ma + kk[u]] = sc * acc[r][u];
        }
    }
}

// Mixed-form point set-up in three parts (bright.c:27-57, phasec.c,
// matrix.c): setup_mixed_phase (the rotation phase and its cos and sin into
// pt[28], pt[29]), setup_mixed_geo (the phase function into pt[24..27], the
// products of the pole matrix and its beta/lambda derivatives with the Earth
// and Sun vectors into pt[0..17], the time into pt[30]) and
// setup_mixed_rotate (the rotation about the spin axis into pt[0..23]).  The
// rotation fm commutes out of the products (matrix.c): with u = B ee,
// e = fm u, de/dbeta = fm (dB/dbeta ee), de/dlambda = fm (dB/dlambda ee) and
// de/domega = (dfm/domega) u = t (e_y, -e_x, 0); the same for the Sun vector.
// The tensor-core path runs the first two on different warps (the FP64
// rotation phase holds its sub-partition's FP64 unit for the whole warp)
// and applies the rotation where it reads the records; the SIMT variants
// run all three (setup_point).
__device__ inline void setup_mixed_phase(double td, double omg, double phi0, float *pt)
{
    const float f = rotation_phase_mixed(omg, td, phi0);
    float sf, cf;
    sincosf(f, &sf, &cf);
    pt[28] = cf;
    pt[29] = sf;
}

// part < 0: all of it; part 0: the phase function and the pole matrix's
// products; part 1: its derivatives' products and the time (two warps of
// the tensor-core path share the work).
__device__ inline void setup_mixed_geo(float4 g0, float4 g1, const float *bm, float *pt, int part = -1)
{
    const float ee[3] = {g0.x, g0.y, g0.z}, e0v[3] = {g1.x, g1.y, g1.z};
    if (part <= 0) {
        const float alpha = g0.w;
        const float php0 = bm[27], php1 = bm[28], php2 = bm[29];
        const float inv_w = 1.f / php1;
        const float ex = expf(-alpha * inv_w);
        pt[24] = 1 + php0 * ex + php2 * alpha;
        pt[25] = ex;
        pt[26] = php0 * ex * alpha * (inv_w * inv_w);
        pt[27] = alpha;
    }
    if (part != 0) pt[30] = g1.w;
#pragma unroll
    for (int m = 0; m < 3; m++) {
        if ((part == 0 && m != 0) || (part == 1 && m == 0)) continue;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float *row = bm + 9 * m + 3 * k;
            pt[6 * m + k] = row[0] * ee[0] + row[1] * ee[1] + row[2] * ee[2];
            pt[6 * m + 3 + k] = row[0] * e0v[0] + row[1] * e0v[1] + row[2] * e0v[2];
        }
    }
}

__device__ inline void setup_mixed_rotate(float *pt)
{
    const float cf = pt[28], sf = pt[29], t = pt[30];
    float u[18];
#pragma unroll
    for (int i = 0; i < 18; i++) u[i] = pt[i];
#pragma unroll
    for (int m = 0; m < 3; m++) {
        const float *ue = u + 6 * m, *us = u + 6 * m + 3;
        const float r0 = cf * ue[0] + sf * ue[1], r1 = cf * ue[1] - sf * ue[0];
        const float s0 = cf * us[0] + sf * us[1], s1 = cf * us[1] - sf * us[0];
        if (m == 0) {
            pt[0] = r0;
            pt[1] = r1;
            pt[2] = ue[2];
            pt[3] = s0;
            pt[4] = s1;
            pt[5] = us[2];
            // d/domega (column 2 of de and de0)
            pt[6 + 2] = t * r1;
            pt[6 + 3 + 2] = -t * r0;
            pt[6 + 6 + 2] = 0.f;
            pt[15 + 2] = t * s1;
            pt[15 + 3 + 2] = -t * s0;
            pt[15 + 6 + 2] = 0.f;
        } else {
            const int j = m - 1;   // column 0: d/dbeta, 1: d/dlambda
            pt[6 + j] = r0;
            pt[6 + 3 + j] = r1;
            pt[6 + 6 + j] = ue[2];
            pt[15 + j] = s0;
            pt[15 + 3 + j] = s1;
            pt[15 + 6 + j] = us[2];
        }
    }
}

// Point set-up of observation q (bright.c:27-57, phasec.c, matrix.c): the
// rotated Earth and Sun directions with their beta/lambda/omega derivatives,
// the phase function and its derivatives, into pt[0..27].
template <int FORM>
__device__ inline void setup_point(const DevObject &ob, const FitConfig &cfg, int q, double omg,
                                   const typename RealOf<FORM>::T *bm, typename RealOf<FORM>::T *pt)
{
    if constexpr (FORM == PS_FORM_MIXED) {
        setup_mixed_phase(ob.tim[q], omg, cfg.phi0, pt);
        setup_mixed_geo(ob.geo_f[2 * q], ob.geo_f[2 * q + 1], bm, pt);
        setup_mixed_rotate(pt);
        return;
    }
    const typename RealOf<FORM>::T *B = bm, *DB0 = bm + 9, *DB1 = bm + 18;
    const typename RealOf<FORM>::T php0 = bm[27], php1 = bm[28], php2 = bm[29];
    using R = typename RealOf<FORM>::T;
    constexpr bool kFP64 = FORM == PS_FORM_FP64;
    R ee[3], e0v[3], alpha;
    if constexpr (kFP64) {
        ee[0] = ob.eex[q];
        ee[1] = ob.eey[q];
        ee[2] = ob.eez[q];
        e0v[0] = ob.e0x[q];
        e0v[1] = ob.e0y[q];
        e0v[2] = ob.e0z[q];
        alpha = ob.alpha_pt[q];
    } else {
        const float4 g0 = ob.geo_f[2 * q], g1 = ob.geo_f[2 * q + 1];
        ee[0] = g0.x;
        ee[1] = g0.y;
        ee[2] = g0.z;
        alpha = g0.w;
        e0v[0] = g1.x;
        e0v[1] = g1.y;
        e0v[2] = g1.z;
    }
    const double td = ob.tim[q];
    const R t = R(td);
    R ex;
    R inv_w = 0;
    if constexpr (kFP64) {
        ex = exp(-alpha / php1);
    } else {
        inv_w = 1.f / php1;
        ex = expf(-alpha * inv_w);
    }
    const R scale = 1 + php0 * ex + php2 * alpha;
    const double f = rotation_phase_fp64(omg, td, cfg.phi0);
    const R cf = cos(f), sf = sin(f);
    const R fm[9] = {cf, sf, R(0), -sf, cf, R(0), R(0), R(0), R(1)};
    const R dfm[9] = {-t * sf, t * cf, R(0), -t * cf, -t * sf, R(0), R(0), R(0), R(0)};
    R tm[9], d0[9], d1[9], d2[9];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            R x = 0, y0 = 0, y1 = 0, y2 = 0;
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
#pragma unroll
    for (int i = 0; i < 3; i++) {
        R x = 0, y = 0;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            x = x + tm[i * 3 + j] * ee[j];
            y = y + tm[i * 3 + j] * e0v[j];
        }
        pt[i] = x;
        pt[3 + i] = y;
    }
    // de[i][j] = sum_k dtm[j][i][k] ee[k]; stored de[i*3+j] (j = derivative)
    const R *dd[3] = {d0, d1, d2};
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            R x = 0, y = 0;
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
    if constexpr (kFP64) pt[26] = php0 * ex * alpha / (php1 * php1);
    else pt[26] = php0 * ex * alpha * (inv_w * inv_w);
    pt[27] = alpha;
}

// ---------------------------------------------------------------------------
// Tensor-core contraction of the mixed form (kBasisTensor).
// ---------------------------------------------------------------------------
constexpr uint32_t kTcWaitTries = 1u << 22;   // mbarrier polls before a wait gives up
constexpr int kErrTcTimeout = 16;             // ps_fit.err_code of a fit cut short by a failed wait

// Tensor Memory columns: the basis [0, Fp/2) (FP16 pairs of facets, Fp =
// tc_kpad(F)), the contraction accumulator [tc_dcol, tc_dcol + 64) (column
// p: A W_hi^T for point p, 32 + p: A W_lo^T) and the alpha accumulator
// [tc_acol, tc_acol + 128).  The wide path (kBasisTensorWide) has the
// second basis region R2 at [Fp/2, 3 Fp/4), the accumulator at tc_dcol and
// R2's accumulator at tc_dcol + 64 (columns 0..31: products with the first
// half of the facets, 32..63: with the second half), and no alpha
// accumulator.
__device__ inline uint32_t tc_r2col(int F) { return static_cast<uint32_t>(tc_kpad(F) >> 1); }
__device__ inline uint32_t tc_dcol(int F, bool wide = false)
{
    return static_cast<uint32_t>(((wide ? 3 * (tc_kpad(F) >> 2) : (tc_kpad(F) >> 1)) + 31) & ~31);
}
__device__ inline uint32_t tc_acol(int F) { return tc_dcol(F) + 64; }

__device__ inline uint32_t tc_cols(int F, bool wide = false)
{
    uint32_t n = 32;
    while (n < (wide ? tc_dcol(F, true) + 128 : tc_acol(F) + 128)) n <<= 1;
    return n;
}

// Per-thread view of the CTA's tensor-core state (every thread keeps the
// same values).
struct TcState {
    uint32_t tbase = 0;     // Tensor Memory base address
    int basis_exp = 0;      // the basis is held scaled by 2^basis_exp
    uint32_t phase = 0;     // parity of the contraction barrier's next phase
    uint32_t aphase = 0;    // parity of the alpha barrier's next phase
    bool apending = false;  // alpha MMAs committed and not waited for
    bool afresh = true;     // the alpha accumulator holds nothing since the last flush
    bool wide = false;      // kBasisTensorWide layout
};

// Waits for the committed alpha MMAs (their operands' shared memory is then
// free); a wait that gives up sets the abort flag.
__device__ inline void tc_alpha_wait(Smem<PS_FORM_MIXED> &s, TcState &t)
{
    if (!t.apending || *s.abort) return;
    const bool ok = __syncthreads_and(tc::mbar_wait(s.mbar2, t.aphase, kTcWaitTries));
    t.apending = false;
    if (!ok) {
        if (threadIdx.x == 0) *s.abort = 1;
        __syncthreads();
        return;
    }
    t.aphase ^= 1u;
    tc::fence_after_sync();
}

// Allocates the CTA's Tensor Memory, initialises the barriers, stages the
// facet constants (zero for the padding facets) and loads the basis into
// Tensor Memory as A = [Dsph_hi^T; Dsph_lo^T]: lane m < 64 holds coefficient
// m, lane 64 + m what remains of it, both FP16 and scaled by 2^basis_exp
// (the largest magnitude just below 2^14, so that the low parts stay normal
// FP16 numbers for elements down to 2^-3 of it); column j holds facets 2j
// and 2j + 1.
template <int NT, bool WIDE = false>
__device__ void tc_setup(const DevObject &ob, Smem<PS_FORM_MIXED> &s, TcState &t)
{
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int F = ob.nfac, C = ob.ncoef, Fp = tc_kpad(F);
    if (warp == 0) tc::tmem_alloc(s.tslot, tc_cols(F, WIDE));
    if (tid == 0) {
        tc::mbar_init(s.mbar, 1);
        tc::mbar_init(s.mbar2, 1);
        *s.abort = 0;
    }
    double mx = 0.0;
    for (int e = tid; e < F * C; e += NT) mx = fmax(mx, fabs(ob.dsph[e]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) s.red[warp] = mx;
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    mx = 0.0;
    for (int w = 0; w < NT / 32; w++) mx = fmax(mx, s.red[w]);
    const int bexp = (mx > 0.0 && mx < 1e300) ? 13 - ilogb(mx) : 0;
    const double bscale = ldexp(1.0, bexp);
    const uint32_t tbase = *s.tslot;
    for (int i = tid; i < Fp; i += NT) {
        fac_at(s.fac, i, 0) = i < F ? ob.nx_f[i] : 0.f;
        fac_at(s.fac, i, 1) = i < F ? ob.ny_f[i] : 0.f;
        fac_at(s.fac, i, 2) = i < F ? ob.nz_f[i] : 0.f;
        fac_at(s.fac, i, 3) = 0.f;
    }
    if constexpr (!WIDE)
        for (int i = tid; i < static_cast<int>(kTcAlphaOperands / 4); i += NT)
            reinterpret_cast<uint32_t *>(s.aop)[i] = 0;
    for (int j = tid; j < ob.mfit; j += NT) s.flist[j] = ob.free_list[j];
    if (warp < 4) {
        // lane m of R1: coefficient c, high part (low = false) or low part;
        // lane m of R2 (wide path): low part of coefficient c2 for the
        // facet half h2 (-1: unused lane)
        const int m = warp * 32 + lane;
        int c, c2 = -1, h2 = 0;
        bool low;
        if constexpr (WIDE) {
            const int L1 = 128 - C, n2 = C - L1;
            low = m >= C;
            c = low ? m - C : m;
            if ((m & 63) < n2) {
                c2 = L1 + (m & 63);
                h2 = m >> 6;
            }
        } else {
            c = m & 63;
            low = m >= 64;
        }
        const uint32_t row = tbase + (static_cast<uint32_t>(warp * 32) << 16);
        auto part = [&](int cc, int i, bool lo) {
            const double d = (cc >= 0 && cc < C && i < F) ? ob.dsph[static_cast<size_t>(i) * C + cc] * bscale : 0.0;
            const float hi = tc::round_f16(static_cast<float>(d));
            return lo ? static_cast<float>(d - static_cast<double>(hi)) : hi;
        };
        for (int j0 = 0; j0 < Fp / 2; j0 += 8) {
            uint32_t v[8];
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] = tc::pack_f16x2(part(c, 2 * (j0 + j), low), part(c, 2 * (j0 + j) + 1, low));
            tc::tmem_st8(row + static_cast<uint32_t>(j0), v);
        }
        if constexpr (WIDE) {
            // R2 column j: facets 2j, 2j + 1 of the lane's facet half
            for (int j0 = 0; j0 < Fp / 4; j0 += 8) {
                uint32_t v[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int i = h2 * (Fp / 2) + 2 * (j0 + j);
                    v[j] = tc::pack_f16x2(part(c2, i, true), part(c2, i + 1, true));
                }
                tc::tmem_st8(row + tc_r2col(F) + static_cast<uint32_t>(j0), v);
            }
        }
        tc::tmem_wait_st();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    t.tbase = tbase;
    t.basis_exp = bexp;
    t.wide = WIDE;
}

// Releases the Tensor Memory.  After an abandoned wait the MMAs in flight
// get one more bounded wait first.
__device__ void tc_teardown(Smem<PS_FORM_MIXED> &s, const TcState &t, int F)
{
    if (*s.abort && threadIdx.x == 0) {
        tc::mbar_wait(s.mbar, t.phase, kTcWaitTries);
        if (t.apending) tc::mbar_wait(s.mbar2, t.aphase, kTcWaitTries);
    }
    tc::fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(t.tbase, tc_cols(F, t.wide));
}

// Issues the alpha/beta MMAs of the operands in s.aop (built and fenced,
// behind a CTA barrier) and commits them to the alpha barrier.  Called by
// every thread; thread 0 issues.  (Issuing them from an idle warp during
// the next contraction window measured no faster: the MMA issue slots of an
// SM are shared by its threads.)
__device__ inline void tc_alpha_issue(Smem<PS_FORM_MIXED> &s, TcState &t, int F)
{
    if (threadIdx.x == 0 && !*s.abort) {
        tc::fence_after_sync();
        const uint32_t idesc = tc::idesc_tf32(128, 128);
        const uint32_t a0 = tc::smem_u32(s.aop), b0 = tc::smem_u32(s.aop + 16384), d = t.tbase + tc_acol(F);
        for (int kk = 0; kk < 4; kk++) {
            const uint32_t off = static_cast<uint32_t>(kk) * 256;
            tc::mma_tf32_ss(d, tc::smem_desc(a0 + off, 128, 1024), tc::smem_desc(b0 + off, 128, 1024), idesc,
                            (t.afresh && kk == 0) ? 0u : 1u);
        }
        tc::mma_commit(s.mbar2);
    }
    t.apending = true;
    t.afresh = false;
}

// Issues D = A [W_hi; W_lo]^T for the tile as Fp/16 FP16 MMAs of 128 x 64 x
// 16 (one MMA costs the issuing thread about the same for N = 32 and N = 64,
// and the same for K = 8 TF32 and K = 16 FP16 elements) and a commit to the
// barrier.  The facet stage has written the operand: FP16 high parts of W
// in rows 0..31, low parts in rows 32..63, canonical K-major layout (8-row x
// 8-facet core matrices, K-adjacent ones 128 bytes apart).
template <int NT, bool WIDE = false>
__device__ void contract_tc_issue(Smem<PS_FORM_MIXED> &s, int F, TcState &t)
{
    const int tid = threadIdx.x;
    const int Fp = tc_kpad(F), kcs = Fp >> 3;
    const uint32_t tbase = t.tbase;
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0 && !*s.abort) {
        tc::fence_after_sync();
        const uint32_t idesc = tc::idesc_f16(128, 64);
        const uint32_t sbo = static_cast<uint32_t>(kcs) * 128;
        const uint32_t bh = tc::smem_u32(s.bhi), d = tbase + tc_dcol(F, WIDE);
        for (int ks = 0; ks < Fp / 16; ks++) {
            const uint32_t a = tbase + static_cast<uint32_t>(ks) * 8, off = static_cast<uint32_t>(ks) * 256;
            tc::mma_f16_ts(d, a, tc::smem_desc(bh + off, 128, sbo), idesc, ks > 0);
        }
        if constexpr (WIDE) {
            // R2 against the W_hi rows (N = 32) of each facet half: the
            // products of lanes 0.. with the first half land in columns
            // 0..31, those of lanes 64.. with the second half in 32..63
            const uint32_t idesc32 = tc::idesc_f16(128, 32), d2 = d + 64, a2 = tbase + tc_r2col(F);
            const int half_steps = Fp / 32;
            for (int h = 0; h < 2; h++)
                for (int ks = 0; ks < half_steps; ks++) {
                    const uint32_t off = static_cast<uint32_t>(h * half_steps + ks) * 256;
                    tc::mma_f16_ts(d2 + 32u * h, a2 + static_cast<uint32_t>(ks) * 8, tc::smem_desc(bh + off, 128, sbo),
                                   idesc32, ks > 0);
                }
        }
        tc::mma_commit(s.mbar);
    }
}

// Facet stage of the tensor-core path (bright.c:59-120).  Warp w takes
// points 8 (w % 4) .. +7 (lane / 4) and the facet quarter w / 4, each lane
// of a point taking two adjacent facets of every 8 (lane % 4), so that one
// warp store covers a whole 8-point x 8-facet core matrix of the MMA
// operand [W_hi; W_lo] (FP16 pairs, W scaled by wscale = 2^k so that the
// evaluation's largest W is just below 2^14).  The per-point sums (brightness, rotation and
// scattering derivatives) are reduced over the four lanes and then over the
// quarters into s.fpart[p * 9 + 0..5] (FP32: the J columns they feed are).  The tile's operand region must be free (previous
// MMAs waited for).
template <int NT>
__device__ void facet_stage_tc(const DevObject &ob, Smem<PS_FORM_MIXED> &s, int np, float cl, float cls,
                               float wscale)
{
    static_assert(NT == 512, "16 warps: 4 point groups x 4 facet quarters");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int kcs = tc_kpad(ob.nfac) >> 3;   // 8-facet core matrices per row group
    const int cq = kcs >> 2;                 // per facet quarter
    const int quarter = warp >> 2, g = warp & 3, p = g * 8 + (lane >> 2), fl = lane & 3;
    // The point records of this path hold the pole products before the
    // rotation about the spin axis (setup_mixed_geo) and its cos/sin
    // (setup_mixed_phase): Earth and Sun directions rotated here.
    float e1 = 0, e2 = 0, e3 = 0, f1 = 0, f2 = 0, f3 = 0;
    if (p < np) {
        const float *pt = s.pt + p * kPointStride;
        const float cf = pt[28], sf = pt[29];
        e1 = cf * pt[0] + sf * pt[1];
        e2 = cf * pt[1] - sf * pt[0];
        e3 = pt[2];
        f1 = cf * pt[3] + sf * pt[4];
        f2 = cf * pt[4] - sf * pt[3];
        f3 = pt[5];
    }
    // The rotation derivatives sum_i Area_i (dsmu (n_i . D_k) + dsmu0 (n_i .
    // E_k)) over the lit facets are D_k . U + E_k . V with U = sum Area dsmu
    // n and V = sum Area dsmu0 n (D_k, E_k: the derivative directions of the
    // Earth and Sun vectors), so the facet loop accumulates U and V.
    // A lane's two facets of each 8 run as the halves of FP32x2 operations
    // (one paired instruction each, on the facet table's interleaved pairs),
    // each half summing its own facets; the halves are added at the end.
    const float2 E1 = make_float2(e1, e1), E2 = make_float2(e2, e2), E3 = make_float2(e3, e3);
    const float2 F1 = make_float2(f1, f1), F2 = make_float2(f2, f2), F3 = make_float2(f3, f3);
    const float2 CL = make_float2(cl, cl), CLS = make_float2(cls, cls), WS = make_float2(wscale, wscale);
    const float2 z2 = make_float2(0.f, 0.f);
    float2 br = z2, dcl = z2, dcls = z2, ux = z2, uy = z2, uz = z2, vx = z2, vy = z2, vz = z2;
    uint32_t *bh = reinterpret_cast<uint32_t *>(s.bhi), *bl = reinterpret_cast<uint32_t *>(s.blo);
    for (int kc = quarter * cq; kc < (quarter + 1) * cq; kc++) {
        const int i = kc * 8 + 2 * fl;
        const int cm = g * kcs + kc;    // core matrix (8-point group, 8-facet group)
        const float4 fa = s.fac[i], fb = s.fac[i + 1];
        const float2 nx = make_float2(fa.x, fa.y), ny = make_float2(fa.z, fa.w), nz = make_float2(fb.x, fb.y);
        float2 mu = __fmul2_rn(E1, nx), mu0 = __fmul2_rn(F1, nx);
        mu = __ffma2_rn(E2, ny, mu);
        mu0 = __ffma2_rn(F2, ny, mu0);
        mu = __ffma2_rn(E3, nz, mu);
        mu0 = __ffma2_rn(F3, nz, mu0);
        // Branch-free: the 8 points of a warp see different lit facets,
        // so a branch would diverge on almost every step (and a
        // warp-uniform skip of groups unlit for all 8 points measured
        // slower, twice); unlit and padding facets get zero area (every
        // term vanishes) and a safe denominator.
        const bool lit0 = mu.x > float(kTinyMu) && mu0.x > float(kTinyMu);
        const bool lit1 = mu.y > float(kTinyMu) && mu0.y > float(kTinyMu);
        // Area (= Darea g, also the weight of W: the Lambert and
        // Lommel-Seeliger terms share it)
        const float2 ax = make_float2(lit0 ? fb.z : 0.f, lit1 ? fb.w : 0.f);
        const float2 m = make_float2(lit0 ? mu.x : 1.f, lit1 ? mu.y : 1.f);
        const float2 m0 = make_float2(lit0 ? mu0.x : 1.f, lit1 ? mu0.y : 1.f);
        // LitTerms<float, PS_FORM_MIXED> on both halves
        const float2 dnom = __fadd2_rn(m, m0);
        float2 r;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r.x) : "f"(dnom.x));
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r.y) : "f"(dnom.y));
        const float2 mm = __fmul2_rn(m, m0);
        const float2 sv = __fmul2_rn(mm, __ffma2_rn(CLS, r, CL));
        const float2 q0 = __fmul2_rn(m0, r), q1 = __fmul2_rn(m, r);
        const float2 dsmu = __ffma2_rn(CLS, __fmul2_rn(q0, q0), __fmul2_rn(CL, m0));
        const float2 dsmu0 = __ffma2_rn(CLS, __fmul2_rn(q1, q1), __fmul2_rn(CL, m));
        const float2 axs = __fmul2_rn(ax, sv);
        br = __fadd2_rn(br, axs);
        const float2 wv = __fmul2_rn(axs, WS);
        const float2 cu = __fmul2_rn(ax, dsmu), cv = __fmul2_rn(ax, dsmu0);
        ux = __ffma2_rn(cu, nx, ux);
        uy = __ffma2_rn(cu, ny, uy);
        uz = __ffma2_rn(cu, nz, uz);
        vx = __ffma2_rn(cv, nx, vx);
        vy = __ffma2_rn(cv, ny, vy);
        vz = __ffma2_rn(cv, nz, vz);
        dcl = __ffma2_rn(mm, ax, dcl);
        dcls = __ffma2_rn(ax, __fmul2_rn(mm, r), dcls);
        const uint32_t hp = tc::pack_f16x2(wv.x, wv.y);
        bh[cm * 32 + lane] = hp;
        bl[cm * 32 + lane] = tc::pack_f16x2(wv.x - tc::f16_lo(hp), wv.y - tc::f16_hi(hp));
    }
    float v[9] = {br.x + br.y, dcl.x + dcl.y, dcls.x + dcls.y, ux.x + ux.y, uy.x + uy.y,
                  uz.x + uz.y, vx.x + vx.y, vy.x + vy.y, vz.x + vz.y};
#pragma unroll
    for (int k = 0; k < 9; k++) {
        v[k] += __shfl_xor_sync(0xffffffffu, v[k], 1);
        v[k] += __shfl_xor_sync(0xffffffffu, v[k], 2);
    }
    if (fl == 0) {
        float *fp = s.fpart + (quarter * 32 + p) * 9;
#pragma unroll
        for (int k = 0; k < 9; k++) fp[k] = v[k];
    }
    __syncthreads();
    if (tid < np) {
        float t[9];
#pragma unroll
        for (int k = 0; k < 9; k++) {
            float a = 0.f;
#pragma unroll
            for (int q = 0; q < 4; q++) a += s.fpart[(q * 32 + tid) * 9 + k];
            t[k] = a;
        }
        // the point's sums in FP32 over its own quarter-0 partials (read
        // above by this thread only): brightness, the three rotation
        // derivatives, the Lambert and the scattering-weight derivatives
        // D_k . U with D_k = fm u_k (k: beta, lambda) is u_k . fm^T U; the
        // omega derivative is D_2 = t (e_y, -e_x, 0), e = fm u_0
        const float *pt = s.pt + tid * kPointStride;
        const float cf = pt[28], sf = pt[29], tt = pt[30];
        const float Ux = cf * t[3] - sf * t[4], Uy = sf * t[3] + cf * t[4], Uz = t[5];
        const float Vx = cf * t[6] - sf * t[7], Vy = sf * t[6] + cf * t[7], Vz = t[8];
        float *rf = s.fpart + tid * 9;
        rf[0] = t[0];
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const float *ue = pt + 6 * (k + 1), *us = ue + 3;
            rf[1 + k] = ue[0] * Ux + ue[1] * Uy + ue[2] * Uz + us[0] * Vx + us[1] * Vy + us[2] * Vz;
        }
        rf[3] = tt * (pt[1] * Ux - pt[0] * Uy + pt[4] * Vx - pt[3] * Vy);
        rf[4] = t[1];
        rf[5] = t[2];
    }
}

// Convexity rows (conv.c:12-29) on the tensor-core path: rows 0..2 of the
// MMA operand hold Darea g n_c (scaled by wscale) split into FP16 high and
// low parts; the residuals sum Area n_c in FP64.
template <int NT>
__device__ void conv_rows_tc(const DevObject &ob, Smem<PS_FORM_MIXED> &s, float wscale)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int F = ob.nfac, half = tc_kpad(F) >> 1;
    uint32_t *bh = reinterpret_cast<uint32_t *>(s.bhi), *bl = reinterpret_cast<uint32_t *>(s.blo);
    for (int e = tid; e < 3 * half; e += NT) {
        const int c = e / half, i = 2 * (e - c * half);
        const double *nc = (c == 0) ? ob.nx : (c == 1) ? ob.ny : ob.nz;
        float w[2], h[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            w[u] = i + u < F ? static_cast<float>(ob.darea[i + u] * s.gv[i + u] * nc[i + u]) * wscale : 0.f;
            h[u] = tc::round_f16(w[u]);
        }
        // row c of the first 8-row group, facets i, i + 1 of core matrix i / 8
        const int off = (i >> 3) * 32 + c * 4 + ((i & 7) >> 1);
        bh[off] = tc::pack_f16x2(h[0], h[1]);
        bl[off] = tc::pack_f16x2(w[0] - h[0], w[1] - h[1]);
    }
    if (warp < 3) {
        const double *nc = (warp == 0) ? ob.nx : (warp == 1) ? ob.ny : ob.nz;
        double res = 0;
        for (int i = lane; i < F; i += 32) res = res + s.area[i] * nc[i];
        res = warp_sum(res);
        if (lane == 0) s.red[warp * kRedStride] = res;
    }
}

// Waits for the tile's MMAs, stages the accumulator (lane m = row m) in
// shared memory and writes J[p][k] = Scale_p jscale (D[k][p] + D[k][32 + p]
// + D[64 + k][p] + D[64 + k][32 + p]): basis high and low parts times W high
// and low parts, jscale undoing the operands' power-of-two scales.  A wait
// that gives up sets the abort flag; the caller ends the fit.
template <int NT, bool WIDE = false>
__device__ void contract_tc_finish(Smem<PS_FORM_MIXED> &s, int np, int F, int C, int ma, bool conv, TcState &t,
                                   float jscale)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t tbase = t.tbase;
    if (*s.abort) return;
    const bool ok = __syncthreads_and(tc::mbar_wait(s.mbar, t.phase, kTcWaitTries));
    if (!ok) {
        if (tid == 0) *s.abort = 1;
        __syncthreads();
        return;
    }
    t.phase ^= 1u;
    tc::fence_after_sync();
    // every warp reads, for 8 points of its lane quadrant's rows (warp w may
    // access Tensor Memory lanes 32 (w % 4) .. + 31), the products with W_hi
    // (column p) and W_lo (column 32 + p) and stages their sum Y[m][p]
    float *Y = reinterpret_cast<float *>(s.bhi);   // [128][33]
    float *Y2 = Y + 128 * 33;                      // wide path: [128][33] from R2's accumulator
    {
        const int quad = warp & 3, pg = warp >> 2;
        const uint32_t taddr = tbase + (static_cast<uint32_t>(quad * 32) << 16) + tc_dcol(F, WIDE) + 8 * pg;
        float *yr = Y + (quad * 32 + lane) * 33 + 8 * pg;
        uint32_t vh[8], vl[8];
        tc::tmem_ld8(taddr, vh);
        tc::tmem_ld8(taddr + 32, vl);
        tc::tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 8; j++) yr[j] = __uint_as_float(vh[j]) + __uint_as_float(vl[j]);
        if constexpr (WIDE) {
            // lanes 0..63 hold the first facet half's products (columns
            // 0..31), lanes 64..127 the second half's (columns 32..63)
            uint32_t v2[8];
            tc::tmem_ld8(taddr + 64 + (quad >= 2 ? 32 : 0), v2);
            tc::tmem_wait_ld();
            float *y2 = Y2 + (quad * 32 + lane) * 33 + 8 * pg;
#pragma unroll
            for (int j = 0; j < 8; j++) y2[j] = __uint_as_float(v2[j]);
        }
    }
    __syncthreads();
    if constexpr (WIDE) {
        // J[p][k] = Scale_p jscale (high part of k times W_hi and W_lo + low
        // part of k times W: from R1's lanes C + k for k < 128 - C, else
        // from R2's two facet halves); thread: k = tid % 128, points
        // tid / 128 + 4 i
        const int k = tid & 127, L1 = 128 - C;
        if (k < C) {
            for (int p = tid >> 7; p < np; p += NT / 128) {
                const float sc = (conv ? 1.f : s.pt[p * kPointStride + 24]) * jscale;
                const float lo = k < L1 ? Y[(C + k) * 33 + p] : Y2[(k - L1) * 33 + p] + Y2[(64 + k - L1) * 33 + p];
                s.J[p * ma + k] = sc * (Y[k * 33 + p] + lo);
            }
        }
        return;
    }
    // J[p][k] = Scale_p jscale (Y[k][p] + Y[64 + k][p]); thread: k = tid % 64,
    // points tid / 64 + 8 i (C <= 64 on this path)
    {
        const int k = tid & 63;
        if (k < C) {
            const float *yh = Y + k * 33, *yl = Y + (64 + k) * 33;
            for (int p = tid >> 6; p < np; p += NT / 64) {
                const float sc = (conv ? 1.f : s.pt[p * kPointStride + 24]) * jscale;
                s.J[p * ma + k] = sc * (yh[p] + yl[p]);
            }
        }
    }
}

// alpha/beta accumulation of one tile on the tensor cores (mrqcof.c:106-136):
// D += A B^T over the tile's points with A = [Wt_hi; Wt_lo] (row j: the
// weighted column J[.][l_j] sig^-2 w of free parameter j, 128 x 32) and B =
// [Jt_hi; Jt_lo] (row k < mfit: column J[.][l_k]; row mfit: the residuals
// dy), both split into TF32 high and low parts, so that the four quadrants
// of the 128 x 128 FP32 accumulator sum to alpha (and beta in column mfit)
// at FP32 accuracy.  The accumulator stays in Tensor Memory across tiles
// until tc_alpha_flush.  chi^2 is summed in FP64 by warp 0, unless the
// caller has prepared the weights, residuals and chi^2 (prepared).  With
// rows (a relative lightcurve's second pass) the operands are built straight
// from the parked rows (stride rw: renormalisation factor in column 0, y/ave
// in ma, residual in ma + 1, weight in ma + 2), renormalising on the way
// (mrqcof.c:90-104).
template <int NT>
__device__ void accumulate_tile_tc(const DevObject &ob, Smem<PS_FORM_MIXED> &s, int np, int q0pt, bool conv,
                                   double conv_sig, TcState &t, bool prepared, const float *rows = nullptr,
                                   int rw = 0)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ma = ob.ma, mf = ob.mfit;
    float *dyv = s.accs;
    float *wtp = dyv + 32;
    if (tid < 32 && !prepared) {
        double c2 = 0;
        if (tid < np) {
            const int q = q0pt + tid;
            const double sig2i = conv ? 1 / (conv_sig * conv_sig) : ob.sig2i[q];
            const double wg = ob.weight[q];
            const double dy = (conv ? 0.0 : ob.bright[q]) - s.ym[tid];
            dyv[tid] = static_cast<float>(dy);
            wtp[tid] = static_cast<float>(sig2i * wg);
            c2 = dy * dy * sig2i * wg;
        }
        c2 = warp_sum(c2);
        if (tid == 0) s.misc[M_CHISQ] += c2;
    }
    tc_alpha_wait(s, t);
    __syncthreads();
    // operands in the canonical K-major layout, K = the tile's 32 points
    // (zero beyond np): 8-row x 4-point core matrices, K-adjacent ones 128
    // bytes apart, 8-row groups 1024 bytes apart; high parts in rows 0..63,
    // low parts in rows 64..127
    unsigned char *Ab = s.aop, *Bb = s.aop + 16384;
    const int rg_end = (mf + 1 + 7) >> 3;   // row groups past it stay zero (cleared at set-up)
    static_assert(NT == 512, "16 warps x 4 core matrices of each operand");
    // warp w: core matrices c = w + 16 i of both operands (row group c / 8,
    // points 4 (c % 8) .. + 3), the same J element feeding A and B
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int c = warp + 16 * i, rg = c >> 3, kc = c & 7;
        if (rg < rg_end) {
            const int row = rg * 8 + (lane >> 2), p = kc * 4 + (lane & 3);
            float va = 0.f, vb = 0.f;
            if (p < np) {
                if (rows) {
                    const float *r = rows + static_cast<size_t>(p) * rw;
                    if (row < mf) {
                        const int l = s.flist[row];
                        vb = l == 0 ? 0.f : r[0] * (r[l] - r[ma] * s.davef[l]);
                        va = vb * r[ma + 2];
                    } else if (row == mf) {
                        vb = r[ma + 1];
                    }
                } else if (row < mf) {
                    vb = s.J[p * ma + s.flist[row]];
                    va = vb * wtp[p];
                } else if (row == mf) {
                    vb = dyv[p];
                }
            }
            const uint32_t ah = tc::to_tf32(va), bh = tc::to_tf32(vb);
            const uint32_t al = tc::to_tf32(va - __uint_as_float(ah)), bl = tc::to_tf32(vb - __uint_as_float(bh));
            reinterpret_cast<uint32_t *>(Ab + (rg * 8 + kc) * 128)[lane] = ah;
            reinterpret_cast<uint32_t *>(Ab + ((rg + 8) * 8 + kc) * 128)[lane] = al;
            reinterpret_cast<uint32_t *>(Bb + (rg * 8 + kc) * 128)[lane] = bh;
            reinterpret_cast<uint32_t *>(Bb + ((rg + 8) * 8 + kc) * 128)[lane] = bl;
        }
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc_alpha_issue(s, t, ob.nfac);
}

// Adds the alpha accumulator to the FP64 normal matrix M (lower triangle)
// and bv, and marks it empty: each quadrant pair is summed on the way out of
// Tensor Memory (rows m and 64 + m, columns k and 64 + k).
template <int NT>
__device__ void tc_alpha_flush(const DevObject &ob, Smem<PS_FORM_MIXED> &s, double *M, double *bv, TcState &t)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int mf = ob.mfit;
    if (t.afresh) return;
    tc_alpha_wait(s, t);
    if (*s.abort) return;
    float *S = reinterpret_cast<float *>(s.bhi);   // [128][65], after the tile's contraction
    {
        // every warp: 16 of the 64 column pairs of its lane quadrant
        const int quad = warp & 3, cgrp = warp >> 2;
        const uint32_t taddr =
            t.tbase + (static_cast<uint32_t>(quad * 32) << 16) + tc_acol(ob.nfac) + 16 * cgrp;
        float *sr = S + (quad * 32 + lane) * 65 + 16 * cgrp;
#pragma unroll
        for (int q = 0; q < 2; q++) {
            uint32_t vh[8], vl[8];
            tc::tmem_ld8(taddr + 8 * q, vh);
            tc::tmem_ld8(taddr + 64 + 8 * q, vl);
            tc::tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 8; j++) sr[8 * q + j] = __uint_as_float(vh[j]) + __uint_as_float(vl[j]);
        }
    }
    __syncthreads();
    const int ntri = mf * (mf + 1) / 2;
    for (int e = tid; e < ntri; e += NT) {
        const int j = tri_row(e);
        const int k = e - j * (j + 1) / 2;
        M[j * mf + k] += static_cast<double>(S[j * 65 + k] + S[(64 + j) * 65 + k]);
    }
    for (int j = tid; j < mf; j += NT) bv[j] += static_cast<double>(S[j * 65 + mf] + S[(64 + j) * 65 + mf]);
    t.afresh = true;
    tc::fence_before_sync();
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Model evaluation (mrqcof) at parameters a[] into matrix M (mfit x mfit,
// lower triangle accumulated then mirrored) and vector bv.  Leaves chi^2,
// the facet-area sum and the convexity residuals in misc.
// ---------------------------------------------------------------------------
template <int FORM, int KU>
__device__ void evaluate(const DevObject &ob, const FitConfig &cfg, const SlotLayout &L, Smem<FORM> &s,
                         const double *a, double *M, double *bv, typename RealOf<FORM>::T *scratch, TcState &tcs)
{
    using R = typename RealOf<FORM>::T;
    constexpr bool kFP64 = FORM == PS_FORM_FP64;
    // tensor-core path: the point set-up of the next tile runs on warps 1..15
    // while thread 0 issues the current tile's MMAs
    constexpr bool kPipe = !kFP64 && (KU == 0 || KU == 3);
    // alpha/beta on the tensor cores (KU 0), or on the SIMT pipes behind the
    // wide tensor-core contraction (KU 3: 65..96 coefficients)
    constexpr bool kTcAlpha = !kFP64 && KU == 0;
    constexpr bool kWide = !kFP64 && KU == 3;
    constexpr int NT = threads_of<FORM>();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int F = ob.nfac, C = ob.ncoef, ma = ob.ma, mf = ob.mfit, P = L.P;
    const int wcols = L.wcols;
    const int RW = rel_row_stride(ma);   // parked row of a relative lightcurve
    const R *nxR, *nyR, *nzR, *dareaR;
    const R *dsphR;
    if constexpr (kFP64) {
        nxR = ob.nx;
        nyR = ob.ny;
        nzR = ob.nz;
        dareaR = ob.darea;
        dsphR = ob.dsph;
    } else {
        nxR = ob.nx_f;
        nyR = ob.ny_f;
        nzR = ob.nz_f;
        dareaR = ob.darea_f;
        dsphR = ob.dsph_f;
    }

    // curv.c:10-39 -- g_i = exp(sum over (m,l) of P_l^m (c cos + c' sin)), FP64.
    double asum = 0;
    for (int i = tid; i < F; i += NT) {
        double g = 0;
        if constexpr (kFP64) {
            for (int q = 0; q < ob.npairs; q++) {
                int m = ob.pair_m[q], n = ob.pair_n[q];
                double fsum = a[n] * ob.fc[m * F + i];
                if (m != 0) fsum = fsum + a[n + 1] * ob.fs[m * F + i];
                g = g + ob.pleg[q * F + i] * fsum;
            }
        } else {
            // the same sum as the dot product of the facet's FP64 basis row
            // (Dsph[i][n] = P_l^m cos(m phi_i), Dsph[i][n + 1] = P_l^m
            // sin(m phi_i)) with the shape coefficients: independent loads
            // instead of a pair-index chain per term; it rounds differently
            // from curv.c's order by about 1e-16
            const double *drow = ob.dsph + static_cast<size_t>(i) * ob.ncoef;
#pragma unroll 7
            for (int k = 0; k < ob.ncoef; k++) g = fma(drow[k], a[k], g);
        }
        g = exp(g);
        double ar = ob.darea[i] * g;
        s.area[i] = ar;
        s.gv[i] = g;
        if constexpr (!kFP64) {
            s.areaR[i] = static_cast<R>(ar);
            s.gvR[i] = static_cast<R>(g);
            if constexpr (kPipe) fac_at(s.fac, i, 3) = static_cast<float>(ar);
        }
        asum += ar;
    }
    double tot = block_sum<NT>(asum, s.misc + M_RED);
    if (tid == 0) {
        s.misc[M_AREA] = tot;
        s.misc[M_CHISQ] = 0;
        s.misc[M_CL] = exp(a[ma - 2]);
        s.misc[M_TRIG] = cos(a[C]);
        s.misc[M_TRIG + 1] = sin(a[C]);
        s.misc[M_TRIG + 2] = cos(a[C + 1]);
        s.misc[M_TRIG + 3] = sin(a[C + 1]);
    }
    for (int e = tid; e < mf * mf; e += NT) M[e] = 0;
    for (int j = tid; j < mf; j += NT) bv[j] = 0;

    // blmatrix.c:9-46 in FP64 from the angles' cos/sin of thread 0, one
    // entry per lane of warp 0 (every FP64 instruction holds the FP64 unit
    // for the whole warp, so each scalar is computed once), stored in the
    // facet-stage type with the phase and scattering parameters.
    __syncthreads();
    if (warp == 0) {
        R v;
        if (lane < 27) {
            const int code = c_bl_code[lane];
            const int fa = code & 3, fb = (code >> 2) & 3;
            const double va = fa == 1 ? s.misc[M_TRIG] : fa == 2 ? s.misc[M_TRIG + 1] : fa == 3 ? 1.0 : 0.0;
            const double vb = fb == 1 ? s.misc[M_TRIG + 2] : fb == 2 ? s.misc[M_TRIG + 3] : 1.0;
            const double p = va * vb;
            v = R((code & 16) ? -p : p);
        } else {
            v = R(lane == 31 ? s.misc[M_CL] : a[lane == 30 ? C + 7 : C + 3 + (lane - 27)]);
        }
        s.bmat[lane] = v;
    } else if (kPipe && warp == 1) {
        // Scale of the contraction operand W = Darea g s: s <= |cl| +
        // |cls| / 2 (mu mu0 <= 1, mu mu0 / (mu + mu0) <= 1/2), and the
        // convexity rows' W <= Darea g, so 2^k puts the evaluation's largest
        // W just below 2^14.
        float mx = 0.f;
        for (int i = lane; i < F; i += 32) mx = fmaxf(mx, fac_at(s.fac, i, 3));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        const float wmax =
            mx * fmaxf(1.f, fabsf(static_cast<float>(s.misc[M_CL])) + 0.5f * fabsf(static_cast<float>(a[C + 7])));
        if (lane == 0) s.misc[M_WEXP] = (wmax > 0.f && wmax < 1e30f) ? static_cast<double>(13 - ilogbf(wmax)) : 0.0;
    }
    const double omg = a[C + 2];
    __syncthreads();
    const R cls = s.bmat[30], cl = s.bmat[31];
    // power-of-two scales of the tensor-core contraction's operands
    const int wexp = kPipe ? static_cast<int>(s.misc[M_WEXP]) : 0;
    const float wscale = ldexpf(1.f, wexp);
    const float jscale = ldexpf(1.f, -(wexp + tcs.basis_exp));

    const double conv_sig = cfg.conv_sig;
    float accA[kAccPerThread];
    float accB = 0.f;
#pragma unroll
    for (int u = 0; u < kAccPerThread; u++) accA[u] = 0.f;
    int tiles_since_flush = 0;
    const float *dsphF = nullptr;
    if constexpr (!kFP64) dsphF = s.dsph ? s.dsph : ob.dsph_f;
    // Point set-up threads.  An FP64 instruction holds its sub-partition's
    // FP64 unit for the whole warp however few lanes are active, so the
    // set-up keeps its points on as few warps as possible: the mixed form
    // (FP64 only for the rotation phase) on one warp, lane = point; the FP64
    // form on warps 0..3, one per sub-partition.  On the tensor-core path
    // warp 1 sets up the evaluation's first tile here; later tiles are set
    // up in the contraction window of the tile before (warps 1..3).
    const int pipe_sp = warp == 1 ? lane : -1;
    if constexpr (kPipe) {
        if (ob.n_lc > 1 && pipe_sp >= 0 && pipe_sp < min(P, ob.lc_npts[0])) {
            const int q = ob.lc_start[0] + pipe_sp;
            float *pt0 = s.pt + pipe_sp * kPointStride;
            setup_mixed_phase(ob.tim[q], omg, cfg.phi0, pt0);
            setup_mixed_geo(ob.geo_f[2 * q], ob.geo_f[2 * q + 1], s.bmat, pt0);
        }
        __syncthreads();   // the first tile's facet stage reads it
    }

    for (int lc = 0; lc < ob.n_lc; lc++) {
        const int start = ob.lc_start[lc], npts = ob.lc_npts[lc];
        const bool rel = ob.lc_rel[lc] != 0;
        const bool conv = (lc == ob.n_lc - 1);
        if (rel) {
            for (int l = tid; l < ma; l += NT) s.dave[l] = 0;
            if (tid == 0) s.misc[M_AVE] = 0;
        }
        // ---- pass 1: model rows of this lightcurve, tile by tile ----
        for (int t0 = 0; t0 < npts; t0 += P) {
            const int np = min(P, npts - t0);
            if (!conv) {
                // 1. point set-up (bright.c:27-57, phasec.c, matrix.c), one
                // thread per point on as few warps as possible; with the
                // tensor cores it was done during the previous tile's MMAs
                if constexpr (!kPipe) {
                    const int ppw = (P + 3) / 4;   // FP64 form: points per warp
                    const int sp = kFP64 ? (lane < ppw && warp < 4 ? warp * ppw + lane : -1) : (warp == 0 ? lane : -1);
                    if (sp >= 0 && sp < np)
                        setup_point<FORM>(ob, cfg, start + t0 + sp, omg, s.bmat,
                                          s.pt + sp * kPointStride);
                }
                // (with the tensor cores the set-up is a tile old: the
                // barrier after the previous tile's contraction ordered it)
                if constexpr (!kPipe) __syncthreads();
                // 2. facet stage (bright.c:59-120), one warp per point
                if constexpr (kPipe) {
                    // prefetch for the contraction window: the next tile's
                    // times (warp 1) and geometry (warps 2 and 3, a copy
                    // each), this tile's accumulation data (warp 14)
                    if (kTcAlpha && warp == 14) {
                        if (!rel && lane < np) {
                            const int q = start + t0 + lane;
                            double *d = reinterpret_cast<double *>(s.pref + kPrefAcc) + 3 * lane;
                            cp_async8(d, ob.sig2i + q);
                            cp_async8(d + 1, ob.weight + q);
                            cp_async8(d + 2, ob.bright + q);
                        }
                        cp_async_commit();
                    } else if (warp >= 1 && warp <= 3) {
                        const int nlc = t0 + P < npts ? lc : lc + 1, nt0 = t0 + P < npts ? t0 + P : 0;
                        if (nlc < ob.n_lc - 1 && lane < min(P, ob.lc_npts[nlc] - nt0)) {
                            const int q = ob.lc_start[nlc] + nt0 + lane;
                            if (warp == 1) {
                                cp_async8(reinterpret_cast<double *>(s.pref + kPrefTim) + lane, ob.tim + q);
                            } else {
                                float4 *g = reinterpret_cast<float4 *>(s.pref + (warp == 2 ? kPrefGeo : kPrefGeo2)) +
                                            2 * lane;
                                cp_async16(g, ob.geo_f + 2 * q);
                                cp_async16(g + 1, ob.geo_f + 2 * q + 1);
                            }
                        }
                        cp_async_commit();
                    }
                    facet_stage_tc<NT>(ob, s, np, cl, cls, wscale);
                }
                else if constexpr (kFP64) {
                    for (int p = warp; p < np; p += NT / 32) facet_point_fp64(ob, s, p, wcols, cl, cls);
                }
                else
                for (int p = warp; p < np; p += NT / 32) {
                    const R *pt = s.pt + p * kPointStride;
                    const R e1 = pt[0], e2 = pt[1], e3 = pt[2];
                    const R f1 = pt[3], f2 = pt[4], f3 = pt[5];
                    R de[9], de0[9];
#pragma unroll
                    for (int k = 0; k < 9; k++) {
                        de[k] = pt[6 + k];
                        de0[k] = pt[15 + k];
                    }
                    R br = 0, r0 = 0, r1 = 0, r2 = 0, dcl = 0, dcls = 0;
                    R *Wp = s.W + static_cast<size_t>(p) * wcols;
                    for (int i = lane; i < F; i += 32) {
                        const R nx = nxR[i], ny = nyR[i], nz = nzR[i];
                        const R mu = e1 * nx + e2 * ny + e3 * nz;
                        const R mu0 = f1 * nx + f2 * ny + f3 * nz;
                        R w = 0;
                        if (mu > R(kTinyMu) && mu0 > R(kTinyMu)) {
                            const R ar = s.areaR[i];
                            const LitTerms<R, FORM> lt(mu, mu0, cl, cls);
                            br = br + ar * lt.sv;
                            w = dareaR[i] * lt.sv * s.gvR[i];
                            const R s0 = nx * de[0] + ny * de[3] + nz * de[6];
                            const R s1 = nx * de[1] + ny * de[4] + nz * de[7];
                            const R s2 = nx * de[2] + ny * de[5] + nz * de[8];
                            const R t0v = nx * de0[0] + ny * de0[3] + nz * de0[6];
                            const R t1v = nx * de0[1] + ny * de0[4] + nz * de0[7];
                            const R t2v = nx * de0[2] + ny * de0[5] + nz * de0[8];
                            r0 = r0 + ar * (lt.dsmu * s0 + lt.dsmu0 * t0v);
                            r1 = r1 + ar * (lt.dsmu * s1 + lt.dsmu0 * t1v);
                            r2 = r2 + ar * (lt.dsmu * s2 + lt.dsmu0 * t2v);
                            dcl = dcl + mu * mu0 * ar;
                            dcls = dcls + ar * lt.dcls_w;
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
            } else if constexpr (kPipe) {
                conv_rows_tc<NT>(ob, s, wscale);
            } else {
                // convexity rows (conv.c:12-29): W = Darea g n_c, residual =
                // sum Area n_c (the residual in FP64 in both forms)
                for (int p = warp; p < np; p += NT / 32) {
                    const double *nc = (p == 0) ? ob.nx : (p == 1) ? ob.ny : ob.nz;
                    double res = 0;
                    R *Wp = s.W + static_cast<size_t>(p) * wcols;
                    for (int i = lane; i < F; i += 32) {
                        res = res + s.area[i] * nc[i];
                        Wp[i] = R(ob.darea[i] * s.gv[i] * nc[i]);
                    }
                    res = warp_sum(res);
                    if (lane == 0) s.red[p * kRedStride] = res;
                }
            }
            // (the tensor-core issue below begins with a barrier of its own)
            if constexpr (!kPipe) __syncthreads();
            // 3. shape contraction and the remaining columns of J
            if constexpr (kFP64) {
                for (int o = tid; o < np * C; o += NT) {
                    const int p = o / C, k = o - p * C;
                    const double acc = contract_fp64(s, dsphR + k, p, C, F, wcols, conv);
                    s.J[p * ma + k] = conv ? acc : s.pt[p * kPointStride + 24] * acc;
                }
            } else if constexpr (kPipe) {
                contract_tc_issue<NT, kWide>(s, F, tcs);   // the work below overlaps the MMAs
            } else {
                if (s.dsph)
                    contract_mixed<NT, KU, true>(s, dsphF, np, F, C, ma, wcols, conv);
                else
                    contract_mixed<NT, KU, false>(s, dsphF, np, F, C, ma, wcols, conv);
            }
            // remaining columns of J: one thread per point (not thread 0 on the
            // tensor-core path: it issues the MMAs)
            const int jp = kPipe ? (tid + 32) % NT : tid;
            if (jp < np) {
                const int p = jp;
                R *Jp = s.J + p * ma;
                const double *rd = s.red + p * kRedStride;
                if (!conv) {
                    R v[6];
                    if constexpr (kPipe) {
#pragma unroll
                        for (int k = 0; k < 6; k++) v[k] = s.fpart[p * 9 + k];
                    } else {
#pragma unroll
                        for (int k = 0; k < 6; k++) v[k] = R(rd[k]);
                    }
                    const R *pt = s.pt + p * kPointStride;
                    const R scale = pt[24];
                    const R br = v[0];
                    Jp[C] = scale * v[1];
                    Jp[C + 1] = scale * v[2];
                    Jp[C + 2] = scale * v[3];
                    Jp[C + 3] = br * pt[25];
                    Jp[C + 4] = br * pt[26];
                    Jp[C + 5] = br * pt[27];
                    Jp[C + 6] = scale * v[4] * cl;
                    Jp[C + 7] = scale * v[5];
                    s.ym[p] = static_cast<double>(br * scale);
                } else {
                    for (int k = C; k < ma; k++) Jp[k] = 0;
                    s.ym[p] = rd[0];
                    s.misc[M_CHK + p] = rd[0];
                }
            }
            if constexpr (kPipe) {
                // the accumulation's per-point FP64 work (weights, residuals,
                // chi^2) of an absolute lightcurve or of the convexity rows,
                // here on warp 14 (its own copy of the model value) while
                // thread 0 issues the contraction and warp 15 writes the J
                // columns (same per-point values and reduction as in the
                // accumulation itself)
                if (rel && warp == NT / 32 - 1) {
                    // relative lightcurve: park the model value with the
                    // row and add the tile to the lightcurve sum
                    double y = 0;
                    if (jp < np) {
                        y = s.ym[jp];
                        scratch[static_cast<size_t>(t0 + jp) * RW + ma] = R(y);
                    }
                    y = warp_sum(y);
                    if (lane == 0) s.misc[M_AVE] += y;
                }
                if (kTcAlpha && !rel && warp == NT / 32 - 2) {
                    double c2 = 0;
                    cp_async_wait_all();
                    if (lane < np) {
                        const int q = start + t0 + lane;
                        const double *pa = reinterpret_cast<const double *>(s.pref + kPrefAcc) + 3 * lane;
                        const double ymv = conv ? s.red[lane * kRedStride]
                                                : static_cast<double>(s.fpart[lane * 9] *
                                                                      s.pt[lane * kPointStride + 24]);
                        const double sig2i = conv ? 1 / (conv_sig * conv_sig) : pa[0];
                        const double wg = conv ? ob.weight[q] : pa[1];
                        const double dy = (conv ? 0.0 : pa[2]) - ymv;
                        s.accs[lane] = static_cast<float>(dy);
                        s.accs[32 + lane] = static_cast<float>(sig2i * wg);
                        c2 = dy * dy * sig2i * wg;
                    }
                    c2 = warp_sum(c2);
                    if (lane == 0) s.misc[M_CHISQ] += c2;
                }
            }
            bool next_setup = false;
            if constexpr (kPipe) {
                // point set-up of the next tile into the other buffer, one
                // point per lane: the rotation phase on warp 1, the phase
                // function and pole products on warps 2 and 3 (the facet
                // stage applies the rotation)
                const int nlc = t0 + P < npts ? lc : lc + 1, nt0 = t0 + P < npts ? t0 + P : 0;
                next_setup = nlc < ob.n_lc - 1;   // the last lightcurve is the convexity rows
                if (next_setup && warp >= 1 && warp <= 3) {
                    const bool have = lane < min(P, ob.lc_npts[nlc] - nt0);
                    float *ptn = s.pt2 + lane * kPointStride;
                    cp_async_wait_all();
                    if (warp == 1) {
                        if (have) setup_mixed_phase(reinterpret_cast<const double *>(s.pref + kPrefTim)[lane], omg,
                                                    cfg.phi0, ptn);
                    } else {
                        const float4 *g =
                            reinterpret_cast<const float4 *>(s.pref + (warp == 2 ? kPrefGeo : kPrefGeo2)) + 2 * lane;
                        if (have) setup_mixed_geo(g[0], g[1], s.bmat, ptn, warp - 2);
                    }
                }
                contract_tc_finish<NT, kWide>(s, np, F, C, ma, conv, tcs, jscale);
            }
            __syncthreads();
            if (next_setup) {
                R *t = s.pt;
                s.pt = s.pt2;
                s.pt2 = t;
            }
            if (rel) {
                // 4a. lightcurve sums and a copy of the rows (mrqcof.c:51-88)
                // (on the tensor-core path warp 15 has parked the model
                // values and summed them during the contraction; the FP64
                // column sums run on sub-partitions 2 and 3)
                R *dst = scratch + static_cast<size_t>(t0) * RW;
                for (int e = tid; e < np * ma; e += NT) {
                    int p = e / ma, l = e - p * ma;
                    dst[static_cast<size_t>(p) * RW + l] = s.J[e];
                }
                if (!kPipe && tid < np) dst[static_cast<size_t>(tid) * RW + ma] = R(s.ym[tid]);
                for (int l = kPipe ? tid - 64 : tid; l < ma; l += NT) {
                    if (l < 0) break;
                    if constexpr (kFP64) {
                        double d = s.dave[l];
                        for (int p = 0; p < np; p++) d = d + s.J[p * ma + l];
                        s.dave[l] = d;
                    } else {
                        float d = 0.f;
                        for (int p = 0; p < np; p++) d += s.J[p * ma + l];
                        s.dave[l] += static_cast<double>(d);
                    }
                }
                if constexpr (kFP64) {
                    // the reference's order
                    if (tid == 0) {
                        double av = s.misc[M_AVE];
                        for (int p = 0; p < np; p++) av = av + s.ym[p];
                        s.misc[M_AVE] = av;
                    }
                } else if (!kPipe && warp == 0) {
                    const double v = warp_sum(lane < np ? s.ym[lane] : 0.0);
                    if (lane == 0) s.misc[M_AVE] += v;
                }
                __syncthreads();
                continue;
            }
            // 5. accumulate (mrqcof.c:106-136)
            if constexpr (kTcAlpha) {
                accumulate_tile_tc<NT>(ob, s, np, start + t0, conv, conv_sig, tcs, true);
                if (++tiles_since_flush == kTcTilesPerFlush) {
                    tc_alpha_flush<NT>(ob, s, M, bv, tcs);
                    tiles_since_flush = 0;
                }
            } else {
                accumulate_tile<FORM>(ob, s, M, bv, np, start + t0, conv, conv_sig, accA, accB);
                if constexpr (!kFP64) {
                    if (++tiles_since_flush == kTilesPerFlush) {
                        flush_partials<FORM>(M, bv, mf, accA, accB);
                        tiles_since_flush = 0;
                    }
                }
            }
        }
        if (!rel) continue;
        // ---- pass 2: renormalise and accumulate (mrqcof.c:90-136) ----
        const double ave = s.misc[M_AVE];
        // the mixed form multiplies by one reciprocal of the lightcurve sum;
        // the FP64 form divides as the reference does
        // the mixed form's renormalisation runs in FP32 on FP32 copies, with
        // one reciprocal of the lightcurve sum (computed once, not per warp)
        if constexpr (!kFP64) {
            for (int l = tid; l < ma; l += NT) s.davef[l] = static_cast<float>(s.dave[l]);
            if (tid == 0) s.misc[M_INVAVE] = 1.0 / ave;
            __syncthreads();
        }
        const double inv_ave = kFP64 ? 0.0 : s.misc[M_INVAVE];
        if constexpr (kTcAlpha) {
            // The per-point FP64 work of the whole lightcurve at once, one
            // tile per warp (the tiles' FP64 chains on different
            // sub-partitions): renormalisation factor coef and y/ave into
            // the row's columns 0 (unused by the renormalised row) and ma,
            // residual and weight into ma + 1 and ma + 2; the tiles' chi^2
            // sums are added in tile order (16 tiles a round).
            for (int r0 = 0; r0 * P < npts; r0 += NT / 32) {
                const int tt = r0 + warp;
                const int p = tt * P + lane;
                double c2 = 0;
                if (lane < P && p < npts) {
                    const int q = start + p;
                    R *row = scratch + static_cast<size_t>(p) * RW;
                    const double yt = static_cast<double>(row[ma]);
                    const double coef = ob.sig[q] * npts * inv_ave;
                    const double ym = coef * yt;
                    const double sig2i = ob.sig2i[q];
                    const double wg = ob.weight[q];
                    const double dy = ob.bright[q] - ym;
                    row[0] = static_cast<float>(coef);
                    row[ma] = static_cast<float>(yt * inv_ave);
                    row[ma + 1] = static_cast<float>(dy);
                    row[ma + 2] = static_cast<float>(sig2i * wg);
                    c2 = dy * dy * sig2i * wg;
                }
                c2 = warp_sum(c2);
                if (lane == 0) s.red[warp] = c2;
                __syncthreads();
                if (tid == 0)
                    for (int w = 0; w < NT / 32 && (r0 + w) * P < npts; w++) s.misc[M_CHISQ] += s.red[w];
                if ((r0 + NT / 32) * P < npts) __syncthreads();
            }
        }
        for (int t0 = 0; t0 < npts; t0 += P) {
            const int np = min(P, npts - t0);
            const R *src = scratch + static_cast<size_t>(t0) * RW;
            // model values of the tile in FP64 (the FP64 form keeps its own
            // values; the mixed form parks them as FP32); on the tensor-core
            // path they were prepared above, and the tile's residuals and
            // weights go where the accumulation reads them
            if constexpr (kTcAlpha) {
                // operands built from the parked rows (renormalised on the way)
                accumulate_tile_tc<NT>(ob, s, np, start + t0, false, conv_sig, tcs, true, src, RW);
                if (++tiles_since_flush == kTcTilesPerFlush) {
                    tc_alpha_flush<NT>(ob, s, M, bv, tcs);
                    tiles_since_flush = 0;
                }
                continue;
            }
            if (tid < np) {
                const int q = start + t0 + tid;
                const double yt = static_cast<double>(src[static_cast<size_t>(tid) * RW + ma]);
                double coef, ytr;
                if constexpr (kFP64) {
                    coef = ob.sig[q] * npts / ave;
                    ytr = yt / ave;
                } else {
                    coef = ob.sig[q] * npts * inv_ave;
                    ytr = yt * inv_ave;
                }
                s.ym[tid] = coef * yt;
                if constexpr (!kFP64) {
                    s.accs[tid] = static_cast<float>(coef);        // consumed before the
                    s.accs[32 + tid] = static_cast<float>(ytr);    // accumulation reuses it
                }
            }
            __syncthreads();
            for (int e = tid; e < np * ma; e += NT) {
                const int p = e / ma, l = e - p * ma;
                const R v = src[static_cast<size_t>(p) * RW + l];
                R out;
                if constexpr (kFP64) {
                    const int q = start + t0 + p;
                    const double coef = ob.sig[q] * npts / ave;
                    const double yt = src[static_cast<size_t>(p) * RW + ma];
                    out = coef * (v - yt * s.dave[l] / ave);
                } else {
                    out = s.accs[p] * (v - s.accs[32 + p] * s.davef[l]);
                }
                s.J[e] = (l == 0) ? R(0) : out;
            }
            __syncthreads();
            accumulate_tile<FORM>(ob, s, M, bv, np, start + t0, false, conv_sig, accA, accB);
            if constexpr (!kFP64) {
                if (++tiles_since_flush == kTilesPerFlush) {
                    flush_partials<FORM>(M, bv, mf, accA, accB);
                    tiles_since_flush = 0;
                }
            }
        }
    }
    if constexpr (kTcAlpha) tc_alpha_flush<NT>(ob, s, M, bv, tcs);
    else if constexpr (!kFP64) flush_partials<FORM>(M, bv, mf, accA, accB);
    __syncthreads();
    // mirror the lower triangle (mrqcof.c:139-141)
    for (int e = tid; e < mf * mf; e += NT) {
        const int j = e / mf, k = e - j * mf;
        if (k > j) M[e] = M[k * mf + j];
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// FP64 evaluation split over a thread-block cluster (kMaxSplit CTAs at most).
//
// One fit's point tiles are dealt round-robin to the cluster's CTAs, which
// compute their tiles' model rows (point set-up, facet stage, shape
// contraction, the remaining columns) at the same time; after each round
// every CTA takes the round's tiles in data order -- its own from its shared
// memory, the others' through distributed shared memory -- and runs what
// sums over points: the relative lightcurves' sums, parked rows and second
// pass, and chi^2 in full, the normal matrix and beta for its share of the
// elements only.  Every sum therefore runs in the same order as in the
// single-CTA FP64 form, and the split fit is bit-identical to it.  Every
// CTA computes the convexity rows; then each copies its share of the matrix
// into the others, so that all of them take the same LM decisions and keep
// the same control flow (and the same sequence of cluster barriers).
// ---------------------------------------------------------------------------
constexpr int kMaxSplit = 8;

__device__ void evaluate_split(const DevObject &ob, const FitConfig &cfg, const SlotLayout &L, Smem<PS_FORM_FP64> &s,
                               const double *a, double *M, double *bv, double *scratch)
{
    namespace cgr = cooperative_groups;
    constexpr int NT = threads_of<PS_FORM_FP64>();
    cgr::cluster_group cl = cgr::this_cluster();
    const int rank = static_cast<int>(cl.block_rank()), cs = static_cast<int>(cl.num_blocks());
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int F = ob.nfac, C = ob.ncoef, ma = ob.ma, mf = ob.mfit, P = L.P;
    const int wcols = L.wcols;
    const int RW = rel_row_stride(ma);

    // curv.c:10-39 and blmatrix.c:9-46 on every CTA (as in evaluate)
    double asum = 0;
    for (int i = tid; i < F; i += NT) {
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
    double tot = block_sum<NT>(asum, s.misc + M_RED);
    if (tid == 0) {
        s.misc[M_AREA] = tot;
        s.misc[M_CHISQ] = 0;
        s.misc[M_CL] = exp(a[ma - 2]);
        s.misc[M_TRIG] = cos(a[C]);
        s.misc[M_TRIG + 1] = sin(a[C]);
        s.misc[M_TRIG + 2] = cos(a[C + 1]);
        s.misc[M_TRIG + 3] = sin(a[C + 1]);
    }
    for (int e = tid; e < mf * mf; e += NT) M[e] = 0;
    for (int j = tid; j < mf; j += NT) bv[j] = 0;
    __syncthreads();
    if (warp == 0) {
        double v;
        if (lane < 27) {
            const int code = c_bl_code[lane];
            const int fa = code & 3, fb = (code >> 2) & 3;
            const double va = fa == 1 ? s.misc[M_TRIG] : fa == 2 ? s.misc[M_TRIG + 1] : fa == 3 ? 1.0 : 0.0;
            const double vb = fb == 1 ? s.misc[M_TRIG + 2] : fb == 2 ? s.misc[M_TRIG + 3] : 1.0;
            const double p = va * vb;
            v = (code & 16) ? -p : p;
        } else {
            v = lane == 31 ? s.misc[M_CL] : a[lane == 30 ? C + 7 : C + 3 + (lane - 27)];
        }
        s.bmat[lane] = v;
    }
    const double omg = a[C + 2];
    __syncthreads();
    const double cls = s.bmat[30], cl_w = s.bmat[31];
    const double conv_sig = cfg.conv_sig;
    float accA[kAccPerThread];
    float accB = 0.f;

    // model rows of one tile into s.J / s.ym (bright.c:14-126, as in evaluate)
    auto compute_tile = [&](int lc, int t0, int np, bool conv) {
        const int start = ob.lc_start[lc];
        if (!conv) {
            const int ppw = (P + 3) / 4;
            const int sp = (lane < ppw && warp < 4) ? warp * ppw + lane : -1;
            if (sp >= 0 && sp < np)
                setup_point<PS_FORM_FP64>(ob, cfg, start + t0 + sp, omg, s.bmat, s.pt + sp * kPointStride);
            __syncthreads();
            for (int p = warp; p < np; p += NT / 32) facet_point_fp64(ob, s, p, wcols, cl_w, cls);
        } else {
            for (int p = warp; p < np; p += NT / 32) {
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
        for (int o = tid; o < np * C; o += NT) {
            const int p = o / C, k = o - p * C;
            const double acc = contract_fp64(s, ob.dsph + k, p, C, F, wcols, conv);
            s.J[p * ma + k] = conv ? acc : s.pt[p * kPointStride + 24] * acc;
        }
        if (tid < np) {
            const int p = tid;
            double *Jp = s.J + p * ma;
            const double *rd = s.red + p * kRedStride;
            if (!conv) {
                const double *pt = s.pt + p * kPointStride;
                const double scale = pt[24];
                const double br = rd[0];
                Jp[C] = scale * rd[1];
                Jp[C + 1] = scale * rd[2];
                Jp[C + 2] = scale * rd[3];
                Jp[C + 3] = br * pt[25];
                Jp[C + 4] = br * pt[26];
                Jp[C + 5] = br * pt[27];
                Jp[C + 6] = scale * rd[4] * cl_w;
                Jp[C + 7] = scale * rd[5];
                s.ym[p] = br * scale;
            } else {
                for (int k = C; k < ma; k++) Jp[k] = 0;
                s.ym[p] = rd[0];
                s.misc[M_CHK + p] = rd[0];
            }
        }
        __syncthreads();
    };

    // A tile's sums (mrqcof.c:51-136), over points in data order, on every
    // CTA: the relative lightcurves' sums and rows and chi^2 in full, of the
    // normal matrix only the CTA's share of the elements (accumulate_tile's
    // part).  Jt, yt: the tile's rows and model values (the CTA's own tile,
    // or another CTA's staged in Jst/ymst); the second pass stages its
    // renormalised rows there too, so that s.J, which the other CTAs read
    // during the round, stays as computed.
    double *Jst = s.W + static_cast<size_t>(P) * mf, *ymst = Jst + static_cast<size_t>(P) * ma;
    auto consume_tile = [&](int lc, int t0, int np, const double *Jt, const double *yt) {
        const int start = ob.lc_start[lc], npts = ob.lc_npts[lc];
        if (!ob.lc_rel[lc]) {
            accumulate_tile<PS_FORM_FP64>(ob, s, M, bv, np, start + t0, false, conv_sig, accA, accB, Jt, yt, rank,
                                          cs);
            return;
        }
        if (t0 == 0) {
            for (int l = tid; l < ma; l += NT) s.dave[l] = 0;
            if (tid == 0) s.misc[M_AVE] = 0;
            __syncthreads();
        }
        double *dst = scratch + static_cast<size_t>(t0) * RW;
        for (int e = tid; e < np * ma; e += NT) {
            int p = e / ma, l = e - p * ma;
            dst[static_cast<size_t>(p) * RW + l] = Jt[e];
        }
        if (tid < np) dst[static_cast<size_t>(tid) * RW + ma] = yt[tid];
        for (int l = tid; l < ma; l += NT) {
            double d = s.dave[l];
            for (int p = 0; p < np; p++) d = d + Jt[p * ma + l];
            s.dave[l] = d;
        }
        if (tid == 0) {
            double av = s.misc[M_AVE];
            for (int p = 0; p < np; p++) av = av + yt[p];
            s.misc[M_AVE] = av;
        }
        __syncthreads();
        if (t0 + P < npts) return;
        // second pass of the lightcurve (mrqcof.c:90-136)
        const double ave = s.misc[M_AVE];
        for (int u0 = 0; u0 < npts; u0 += P) {
            const int nq = min(P, npts - u0);
            const double *src = scratch + static_cast<size_t>(u0) * RW;
            if (tid < nq) {
                const int q = start + u0 + tid;
                const double ytv = src[static_cast<size_t>(tid) * RW + ma];
                const double coef = ob.sig[q] * npts / ave;
                ymst[tid] = coef * ytv;
            }
            for (int e = tid; e < nq * ma; e += NT) {
                const int p = e / ma, l = e - p * ma;
                const double v = src[static_cast<size_t>(p) * RW + l];
                const int q = start + u0 + p;
                const double coef = ob.sig[q] * npts / ave;
                const double ytv = src[static_cast<size_t>(p) * RW + ma];
                const double out = coef * (v - ytv * s.dave[l] / ave);
                Jst[e] = (l == 0) ? 0.0 : out;
            }
            __syncthreads();
            accumulate_tile<PS_FORM_FP64>(ob, s, M, bv, nq, start + u0, false, conv_sig, accA, accB, Jst, ymst, rank,
                                          cs);
        }
    };

    // rounds of cs tiles over the real lightcurves, in data order
    int rlc[kMaxSplit], rt0[kMaxSplit], rnp[kMaxSplit];
    int nround = 0;
    auto flush_round = [&]() {
        cl.sync();   // every CTA's tile of the round is in its shared memory
        for (int k = 0; k < nround; k++) {
            const double *Jt = s.J, *yt = s.ym;
            if (k != rank) {
                // rank k's tile, read through distributed shared memory
                const double *rJ = cl.map_shared_rank(s.J, k);
                const double *rY = cl.map_shared_rank(s.ym, k);
                for (int e = tid; e < rnp[k] * ma; e += NT) Jst[e] = rJ[e];
                if (tid < rnp[k]) ymst[tid] = rY[tid];
                __syncthreads();
                Jt = Jst;
                yt = ymst;
            }
            consume_tile(rlc[k], rt0[k], rnp[k], Jt, yt);
        }
        cl.sync();   // the round's tile buffers are free again
        nround = 0;
    };
    const int nreal = ob.n_lc - 1;
    for (int lc = 0; lc < nreal; lc++) {
        const int npts = ob.lc_npts[lc];
        for (int t0 = 0; t0 < npts; t0 += P) {
            const int np = min(P, npts - t0);
            rlc[nround] = lc;
            rt0[nround] = t0;
            rnp[nround] = np;
            if (nround == rank) compute_tile(lc, t0, np, false);
            if (++nround == cs) flush_round();
        }
    }
    if (nround > 0) flush_round();
    // convexity rows (conv.c:12-29) on every CTA, each accumulating its share
    {
        const int lc = ob.n_lc - 1, start = ob.lc_start[lc], npts = ob.lc_npts[lc];
        for (int t0 = 0; t0 < npts; t0 += P) {
            const int np = min(P, npts - t0);
            compute_tile(lc, t0, np, true);
            accumulate_tile<PS_FORM_FP64>(ob, s, M, bv, np, start + t0, true, conv_sig, accA, accB, s.J, s.ym, rank,
                                          cs);
        }
    }
    // every CTA copies its share of the lower triangle and of bv into the
    // others, then mirrors (mrqcof.c:139-141): the same matrix, solve and
    // decisions everywhere
    {
        const int ntri = mf * (mf + 1) / 2;
        for (int r = 0; r < cs; r++) {
            if (r == rank) continue;
            double *rM = cl.map_shared_rank(M, r), *rb = cl.map_shared_rank(bv, r);
            for (int e = rank * NT + tid; e < ntri; e += cs * NT) {
                const int j = tri_row(e), k = e - j * (j + 1) / 2;
                rM[j * mf + k] = M[j * mf + k];
            }
            for (int j = rank * NT + tid; j < mf; j += cs * NT) rb[j] = bv[j];
        }
    }
    cl.sync();
    for (int e = tid; e < mf * mf; e += NT) {
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
template <int NT>
__device__ int gauss_jordan(double *A, double *b, int n, double *col, int *ipiv, double *red)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int k = tid; k < n; k += NT) ipiv[k] = 0;
    __syncthreads();
    for (int step = 0; step < n; step++) {
        // pivot search: largest |a| over unpivoted rows and columns; ties go
        // to the last element in row-major order (the reference's >=).  The
        // bits of |a| order as its values do (NaN patterns, above +inf's,
        // skipped as v >= 0 skips them), so the search compares 64-bit
        // integers, off the FP64 unit, and picks the same pivots.
        constexpr long long kInfBits = 0x7ff0000000000000LL;
        long long bv = -1;
        int bi = -1;
        for (int e = tid; e < n * n; e += NT) {
            const int j = e / n, k = e - j * n;
            if (ipiv[j] != 1 && ipiv[k] == 0) {
                const long long v = __double_as_longlong(A[e]) & 0x7fffffffffffffffLL;
                if (v <= kInfBits && (v > bv || (v == bv && e > bi))) {
                    bv = v;
                    bi = e;
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > bv || (ov == bv && oi > bi)) {
                bv = ov;
                bi = oi;
            }
        }
        long long *redk = reinterpret_cast<long long *>(red);
        if (lane == 0) {
            redk[warp] = bv;
            ipiv[n + 2 + warp] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            long long v = redk[0];
            int idx = ipiv[n + 2];
            for (int w = 1; w < NT / 32; w++) {
                const long long ov = redk[w];
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
            for (int l = tid; l < n; l += NT) {
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
        if (tid == 0) red[0] = 1.0 / piv;
        __syncthreads();
        const double pivinv = red[0];
        // scale the pivot row over the columns not yet pivoted
        for (int l = tid; l < n; l += NT)
            if (ipiv[l] == 0) A[icol * n + l] *= pivinv;
        if (tid == 0) b[icol] *= pivinv;
        for (int r = tid; r < n; r += NT) col[r] = A[r * n + icol];
        __syncthreads();
        for (int e = tid; e < n * n; e += NT) {
            const int r = e / n, l = e - r * n;
            if (r != icol && ipiv[l] == 0) A[e] -= A[icol * n + l] * col[r];
        }
        for (int r = tid; r < n; r += NT)
            if (r != icol) b[r] -= b[icol] * col[r];
        __syncthreads();
    }
    return 0;
}

// Cholesky factorisation A = L L^T of the damped normal matrix (symmetric
// positive definite; lower triangle used, overwritten by L) and the solve of
// L L^T x = b, in FP64.  The forward substitution runs inside the
// factorisation (b is the bordering column: y_j = b_j / L_jj, then b_i -=
// L_ij y_j with the trailing update).
//
// Columns are taken two at a time, with one pair of look-ahead.  Every FP64
// instruction holds its sub-partition's FP64 unit for the whole warp, so the
// serial chain of a pivot and the bulk of the trailing update run on
// different sub-partitions at the same time.  While pair j is applied to
// the columns beyond pair j + 2 (the workers: warps of sub-partitions 1..3
// but warp 1), warp 0 applies it to the 2 x 2 block of pair j + 2 and to
// its two rows of b and factors the block, and warp 1 applies it to the
// rest of pair j + 2's columns and scales them once warp 0 has published
// the pivot (a named barrier of the two warps) -- one CTA barrier per pair.
// The 2 x 2 pivot takes its two reciprocal square roots (of the leading
// element and of the block's determinant) in one lane-parallel sequence.
// The back substitution runs on warp 0 with b in registers and the rows of
// L pre-scaled by their reciprocal diagonal.  Returns 2 when a pivot is not
// positive.
__device__ inline void chol_pivot_pair(double *A, double *b, int n, int j, double *col, double *flag, int lane)
{
    const bool two = j + 1 < n;
    const double a = A[j * n + j];
    const double bq = two ? A[(j + 1) * n + j] : 0.0;
    const double c = two ? A[(j + 1) * n + j + 1] : 1.0;
    // lane 0: the leading element, lane 1: the determinant a c - bq^2
    // (L11 = sqrt(det / a), so 1 / L11 = a rsqrt(a) rsqrt(det))
    const double x = lane == 1 ? fma(a, c, -(bq * bq)) : a;
    const bool okx = x > 0.0;
    const double r = okx ? rsqrt(x) : 0.0;
    const unsigned okm = __ballot_sync(0xffffffffu, okx);
    const double i0 = __shfl_sync(0xffffffffu, r, 0);
    const double rd = __shfl_sync(0xffffffffu, r, 1);
    // lane 1: l10 = bq / L00, lane 2: y0 = b_j / L00, lane 3: 1 / L11
    const double u = lane == 1 ? bq : lane == 2 ? b[j] : a;
    double v = u * i0;
    if (lane == 3) v *= rd;
    const double l10 = __shfl_sync(0xffffffffu, v, 1);
    const double y0 = __shfl_sync(0xffffffffu, v, 2);
    const double i1 = __shfl_sync(0xffffffffu, v, 3);
    const bool ok = (okm & 1u) && (!two || (okm & 2u));
    if (lane == 0) {
        *flag = ok ? 1.0 : 0.0;
        col[j] = i0;
        b[j] = y0;
        if (two) {
            col[j + 1] = i1;
            b[j + 1] = (b[j + 1] - l10 * y0) * i1;
        }
    }
    if (two && lane == 1) A[(j + 1) * n + j] = l10;
    for (int i = j + (two ? 2 : 1) + lane; i < n; i += 32) {
        const double a0 = A[i * n + j] * i0;
        A[i * n + j] = a0;
        if (two) A[i * n + j + 1] = (A[i * n + j + 1] - a0 * l10) * i1;
    }
}

// The 2 x 2 block [a bq; bq c] of pair (j, j + 1) and its rows bj, bj1 of
// b, already updated, in registers of every lane of warp 0: stores 1/L_jj,
// 1/L_j+1,j+1 (col) and L_j+1,j, arrives on the helper warp's named barrier
// (the helper scales the columns below), then stores y (b).
__device__ inline void chol_pivot_block(double a, double bq, double c, double bj, double bj1, double *A, double *b,
                                        int n, int j, bool two, double *col, double *flag, int lane)
{
    const double x = lane == 1 ? fma(a, c, -(bq * bq)) : a;
    const bool okx = x > 0.0;
    const double r = okx ? rsqrt(x) : 0.0;
    const unsigned okm = __ballot_sync(0xffffffffu, okx);
    const double i0 = __shfl_sync(0xffffffffu, r, 0);
    const double rd = __shfl_sync(0xffffffffu, r, 1);
    const double u = lane == 1 ? bq : lane == 2 ? bj : a;
    double v = u * i0;
    if (lane == 3) v *= rd;
    const double l10 = __shfl_sync(0xffffffffu, v, 1);
    const double y0 = __shfl_sync(0xffffffffu, v, 2);
    const double i1 = __shfl_sync(0xffffffffu, v, 3);
    const bool ok = (okm & 1u) && (!two || (okm & 2u));
    if (lane == 0) {
        *flag = ok ? 1.0 : 0.0;
        col[j] = i0;
        b[j] = y0;
        if (two) {
            col[j + 1] = i1;
            A[(j + 1) * n + j] = l10;
        }
    }
    // the helper warp may scale the columns now
    asm volatile("bar.arrive 1, 64;" ::: "memory");
    if (lane == 0 && two) b[j + 1] = (bj1 - l10 * y0) * i1;
}

template <int NT>
__device__ int cholesky_solve(double *A, double *b, int n, double *col, double *flag)
{
    static_assert(NT % 128 == 0 && NT >= 256, "whole warps on every sub-partition");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // trailing-update workers: the warps of sub-partitions 1..3 but warp 1
    constexpr int kWorkers = (NT / 128 * 3 - 1) * 32;
    const bool worker = (warp & 3) != 0 && warp != 1;
    const int wtid = ((warp >> 2) * 3 + (warp & 3) - 2) * 32 + lane;
    __syncthreads();
    if (warp == 0) chol_pivot_pair(A, b, n, 0, col, flag, lane);
    __syncthreads();
    if (*flag == 0.0) return 2;
    for (int j = 0; j + 2 < n; j += 2) {
        // pair (j, j + 1) is factored; b[j], b[j + 1] hold its y
        const bool two = j + 1 < n;
        const int jn = j + 2;
        const bool twon = jn + 1 < n;
        // pair j's L in rows jn, jn + 1 and its y
        const double p0 = A[jn * n + j], p1 = two ? A[jn * n + j + 1] : 0.0;
        const double q0 = twon ? A[(jn + 1) * n + j] : 0.0, q1 = (twon && two) ? A[(jn + 1) * n + j + 1] : 0.0;
        if (warp == 0) {
            // the next pair's 2 x 2 block and rows of b, one value per lane
            // (lane 0: a, 1: bq, 2: c, 3: b_jn, 4: b_jn+1), then its pivot
            const double y0 = b[j], y1 = two ? b[j + 1] : 0.0;
            double xv = 0.0, u1 = 0.0, v1 = 0.0, u2 = 0.0, v2 = 0.0;
            if (lane == 0) { xv = A[jn * n + jn]; u1 = p0; v1 = p0; u2 = p1; v2 = p1; }
            if (lane == 1 && twon) { xv = A[(jn + 1) * n + jn]; u1 = q0; v1 = p0; u2 = q1; v2 = p1; }
            if (lane == 2) { xv = twon ? A[(jn + 1) * n + jn + 1] : 1.0; u1 = q0; v1 = q0; u2 = q1; v2 = q1; }
            if (lane == 3) { xv = b[jn]; u1 = p0; v1 = y0; u2 = p1; v2 = y1; }
            if (lane == 4 && twon) { xv = b[jn + 1]; u1 = q0; v1 = y0; u2 = q1; v2 = y1; }
            const double xu = xv - u1 * v1 - u2 * v2;
            const double a = __shfl_sync(0xffffffffu, xu, 0);
            const double bq = __shfl_sync(0xffffffffu, xu, 1);
            const double cc = __shfl_sync(0xffffffffu, xu, 2);
            const double bj = __shfl_sync(0xffffffffu, xu, 3);
            const double bj1 = __shfl_sync(0xffffffffu, xu, 4);
            chol_pivot_block(a, bq, cc, bj, bj1, A, b, n, jn, twon, col, flag, lane);
        } else if (warp == 1) {
            // the rest of the next pair's columns: update now, scale once
            // warp 0 has published the pivot
            const int i = jn + 2 + lane, i2 = i + 32;
            double c0 = 0, c1 = 0, d0 = 0, d1 = 0;
            if (i < n) {
                const double li0 = A[i * n + j], li1 = two ? A[i * n + j + 1] : 0.0;
                c0 = A[i * n + jn] - li0 * p0 - li1 * p1;
                if (twon) c1 = A[i * n + jn + 1] - li0 * q0 - li1 * q1;
            }
            if (i2 < n) {
                const double li0 = A[i2 * n + j], li1 = two ? A[i2 * n + j + 1] : 0.0;
                d0 = A[i2 * n + jn] - li0 * p0 - li1 * p1;
                if (twon) d1 = A[i2 * n + jn + 1] - li0 * q0 - li1 * q1;
            }
            asm volatile("bar.sync 1, 64;" ::: "memory");
            const double i0 = col[jn];
            const double i1 = twon ? col[jn + 1] : 0.0, l10 = twon ? A[(jn + 1) * n + jn] : 0.0;
            if (i < n) {
                const double a0 = c0 * i0;
                A[i * n + jn] = a0;
                if (twon) A[i * n + jn + 1] = (c1 - a0 * l10) * i1;
            }
            if (i2 < n) {
                const double a0 = d0 * i0;
                A[i2 * n + jn] = a0;
                if (twon) A[i2 * n + jn + 1] = (d1 - a0 * l10) * i1;
            }
            for (int r = i2 + 32; r < n; r += 32) {   // n > 66: the remaining rows, unpipelined
                const double li0 = A[r * n + j], li1 = two ? A[r * n + j + 1] : 0.0;
                const double e0 = A[r * n + jn] - li0 * p0 - li1 * p1;
                const double a0 = e0 * i0;
                A[r * n + jn] = a0;
                if (twon) A[r * n + jn + 1] = (A[r * n + jn + 1] - li0 * q0 - li1 * q1 - a0 * l10) * i1;
            }
        } else if (worker) {
            // apply pair j to the columns beyond the next pair
            const int j2 = j + 4;
            if (j2 < n) {
                const int m = n - j2;
                const int ntri = m * (m + 1) / 2;
                const double y0 = b[j], y1 = two ? b[j + 1] : 0.0;
                for (int e = wtid; e < ntri + m; e += kWorkers) {
                    if (e < ntri) {
                        const int r = tri_row(e);
                        const int cc = e - r * (r + 1) / 2;
                        const int i = j2 + r, k = j2 + cc;
                        double v = A[i * n + k] - A[i * n + j] * A[k * n + j];
                        if (two) v -= A[i * n + j + 1] * A[k * n + j + 1];
                        A[i * n + k] = v;
                    } else {
                        const int i = j2 + (e - ntri);
                        double v = b[i] - A[i * n + j] * y0;
                        if (two) v -= A[i * n + j + 1] * y1;
                        b[i] = v;
                    }
                }
            }
        }
        __syncthreads();
        if (*flag == 0.0) return 2;
    }
    // L^T x = y: with the rows of L scaled, L'_jk = L_jk / L_jj (k < j),
    // x = col .* z where z_j = y_j - sum_{i > j} L'_ij z_i
    const int nstrict = n * (n - 1) / 2;
    for (int e = tid; e < nstrict; e += NT) {
        const int r = tri_row(e) + 1;
        const int cc = e - r * (r - 1) / 2;
        A[r * n + cc] *= col[r];
    }
    __syncthreads();
    if (warp == 0) {
        if (n <= 96) {
            double z0 = lane < n ? b[lane] : 0.0, z1 = lane + 32 < n ? b[lane + 32] : 0.0,
                   z2 = lane + 64 < n ? b[lane + 64] : 0.0;
            for (int jj = n - 1; jj >= 1; jj--) {
                const int slot = jj >> 5;
                const double own = slot == 0 ? z0 : slot == 1 ? z1 : z2;
                const double zj = __shfl_sync(0xffffffffu, own, jj & 31);
                const double *row = A + jj * n;
                if (lane < jj) z0 -= row[lane] * zj;
                if (lane + 32 < jj) z1 -= row[lane + 32] * zj;
                if (lane + 64 < jj) z2 -= row[lane + 64] * zj;
            }
            if (lane < n) b[lane] = z0 * col[lane];
            if (lane + 32 < n) b[lane + 32] = z1 * col[lane + 32];
            if (lane + 64 < n) b[lane + 64] = z2 * col[lane + 64];
        } else {
            for (int jj = n - 1; jj >= 1; jj--) {
                const double zj = b[jj];
                for (int i = lane; i < jj; i += 32) b[i] -= A[jj * n + i] * zj;
                __syncwarp();
            }
            for (int i = lane; i < n; i += 32) b[i] *= col[i];
        }
    }
    __syncthreads();
    return 0;
}

// Learned stop predictor, evaluated by warp 0: standardised features f[10]
// -> 64 GELU -> 64 GELU -> 1, output de-standardised.  Predicts
// log(final rms / rms after kScreenIters iterations).  sh: 64 floats.
__device__ inline float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }

__device__ float mlp_predict_warp(const float *W, const float *f, float *sh)
{
    const int lane = threadIdx.x & 31;
    float x[kFeat];
#pragma unroll
    for (int i = 0; i < kFeat; i++) x[i] = (f[i] - W[kMlpMu + i]) / W[kMlpSd + i];
    float h1[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int u = lane + 32 * h;
        float z = W[kMlpB1 + u];
#pragma unroll
        for (int i = 0; i < kFeat; i++) z = fmaf(W[kMlpW1 + u * kFeat + i], x[i], z);
        h1[h] = gelu(z);
    }
    sh[lane] = h1[0];
    sh[lane + 32] = h1[1];
    __syncwarp();
    float y = 0.f;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int u = lane + 32 * h;
        float z = W[kMlpB2 + u];
        for (int j = 0; j < kHidden; j++) z = fmaf(W[kMlpW2 + u * kHidden + j], sh[j], z);
        y = fmaf(W[kMlpW3 + u], gelu(z), y);
    }
    y = warp_sum(y) + W[kMlpB3];
    __syncwarp();
    return y * W[kMlpYSd] + W[kMlpYMu];
}

// ---------------------------------------------------------------------------
// One fit (period_search_BOINC.cpp:817-921 with mrqmin.c:11-110).
// ---------------------------------------------------------------------------
template <int FORM, int KU>
__device__ void run_fit(const DevObject &ob, const FitConfig &cfg, const SlotLayout &L, Smem<FORM> &s,
                        typename RealOf<FORM>::T *scratch, int64_t n, int pole, ps_fit *out, const FitWork &w,
                        long long fidx, TcState &tcs, bool split = false)
{
    constexpr bool kTensor = FORM == PS_FORM_MIXED && (KU == 0 || KU == 3);
    // one model evaluation; with split (FP64 form, cluster launch) spread
    // over the cluster's CTAs (evaluate_split)
    auto eval = [&](const double *a, double *M, double *bv) {
        if constexpr (FORM == PS_FORM_FP64) {
            if (split) {
                evaluate_split(ob, cfg, L, s, a, M, bv, scratch);
                return;
            }
        }
        evaluate<FORM, KU>(ob, cfg, L, s, a, M, bv, scratch, tcs);
    };
    constexpr int NT = threads_of<FORM>();
    const int tid = threadIdx.x;
    const int C = ob.ncoef, ma = ob.ma, mf = ob.mfit;
    const double freq = cfg.freq_start - (n - 1) * cfg.freq_step;
    const double prd = 1 / freq;
    // learned early stop: features after K iterations (accepted chi^2 and
    // lambda every K/4 iterations); the saved state of a resumable fit
    const int K = w.screen_iters > 0 ? w.screen_iters : kScreenIters;
    const int K4 = K >> 2;
    double *st = w.state ? w.state + (w.state_slot ? w.state_slot[fidx] : fidx) * state_stride(ma) : nullptr;
    const bool resume = w.resume && st;
    for (int i = tid; i < ma; i += NT) {
        double v;
        if (resume) v = st[i];
        else if (i < C) v = ob.cg_first[i];
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
    // learned early stop: accepted chi^2 and lambda of the first iterations
    double hist[5], lam_hist[4];
    double pred_dev = 0;
    bool screened = false;
    if (resume) {
        // continue where the fit stopped: alpha and beta are those of the
        // accepted parameters, recomputed by one evaluation (the same
        // deterministic evaluation the uninterrupted fit would hold)
        alamda = st[ma];
        ochisq = st[ma + 1];
        chisq = st[ma + 2];
        rchisq = st[ma + 3];
        iter_diff = st[ma + 4];
        dev_old = st[ma + 5];
        dev_new = st[ma + 6];
        for (int c = 0; c < 3; c++) chk_acc[c] = st[ma + 7 + c];
        totarea = st[ma + 10];
        niter = static_cast<int>(st[ma + 11]);
        last_err = static_cast<int>(st[ma + 12]);
        pred_dev = st[ma + 13];
        eval(s.cg, s.alpha, s.beta);
        if constexpr (kTensor) {
            if (*s.abort) last_err = kErrTcTimeout;
        }
    }
    while (last_err != kErrTcTimeout &&
           (((niter < cfg.n_iter_max) && (iter_diff > cfg.iter_diff_max)) || (niter < cfg.n_iter_min))) {
        bool accepted = false;
        if (alamda < 0) {
            alamda = cfg.alamda_start;
            eval(s.cg, s.alpha, s.beta);
            if constexpr (kTensor) {
                if (*s.abort) {
                    last_err = kErrTcTimeout;
                    break;
                }
            }
            ochisq = s.misc[M_CHISQ];
            hist[0] = ochisq;
            area_first = s.misc[M_AREA];
            for (int c = 0; c < 3; c++) chk_first[c] = s.misc[M_CHK + c];
            totarea = area_first;
        }
        for (int e = tid; e < mf * mf; e += NT) {
            const int j = e / mf, k = e - j * mf;
            s.covar[e] = (j == k) ? s.alpha[e] * (1 + alamda) : s.alpha[e];
        }
        for (int j = tid; j < mf; j += NT) s.da[j] = s.beta[j];
        __syncthreads();
        int err;
        if constexpr (FORM == PS_FORM_FP64) {
            err = gauss_jordan<NT>(s.covar, s.da, mf, s.col, s.ipiv, s.misc + M_RED);
        } else {
            // The damped normal matrix is symmetric positive definite: solve
            // it by Cholesky in FP64; if a pivot is not positive (rounding on
            // a nearly singular alpha), redo the step with Gauss-Jordan.
            err = cholesky_solve<NT>(s.covar, s.da, mf, s.col, s.misc + M_PIV);
            if (err) {
                for (int e = tid; e < mf * mf; e += NT) {
                    const int j = e / mf, k = e - j * mf;
                    s.covar[e] = (j == k) ? s.alpha[e] * (1 + alamda) : s.alpha[e];
                }
                for (int j = tid; j < mf; j += NT) s.da[j] = s.beta[j];
                __syncthreads();
                err = gauss_jordan<NT>(s.covar, s.da, mf, s.col, s.ipiv, s.misc + M_RED);
            }
        }
        __syncthreads();
        if (err == 0) {
            for (int j = tid; j < mf; j += NT) {
                const int l = ob.free_list[j];
                s.atry[l] = s.cg[l] + s.da[j];
            }
            __syncthreads();
            eval(s.atry, s.covar, s.da);
            if constexpr (kTensor) {
                if (*s.abort) {
                    last_err = kErrTcTimeout;
                    break;
                }
            }
            chisq = s.misc[M_CHISQ];
            area_trial = s.misc[M_AREA];
            for (int c = 0; c < 3; c++) chk_trial[c] = s.misc[M_CHK + c];
            totarea = area_trial;
            if (chisq < ochisq) {
                accepted = true;
                for (int e = tid; e < mf * mf; e += NT) s.alpha[e] = s.covar[e];
                for (int j = tid; j < mf; j += NT) s.beta[j] = s.da[j];
                for (int l = tid; l < ma; l += NT) s.cg[l] = s.atry[l];
            } else {
                chisq = ochisq;
            }
        } else {
            last_err = err;
        }
        niter++;
        // The scalar bookkeeping of the step (mrqmin.c:91-107 and
        // period_search_BOINC.cpp:873-892) runs on thread 0 and is broadcast:
        // an FP64 instruction holds the FP64 unit for the whole warp, so
        // every warp computing it would cost 16 times the FP64 time.
        if (tid == 0) {
            if (err == 0) alamda = accepted ? alamda / cfg.alamda_incr : cfg.alamda_incr * alamda;
            if ((niter == 1) || accepted) {
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
            s.misc[M_LM] = alamda;
            s.misc[M_LM + 1] = ochisq;
            s.misc[M_LM + 2] = dev_new;
            s.misc[M_LM + 3] = iter_diff;
        }
        __syncthreads();
        alamda = s.misc[M_LM];
        ochisq = s.misc[M_LM + 1];
        dev_new = s.misc[M_LM + 2];
        iter_diff = s.misc[M_LM + 3];
        if (!resume && niter <= K && niter % K4 == 0) {
            hist[niter / K4] = ochisq;
            lam_hist[niter / K4 - 1] = alamda;
        }
        // trajectory records: the rms after 8, 16 and 32 iterations as well
        if (w.traj && tid == 0 && (niter == 8 || niter == 16 || niter == 32))
            w.traj[static_cast<size_t>(fidx) * kTrajFloats + (niter == 8 ? 13 : niter == 16 ? 14 : 15)] =
                static_cast<float>(dev_new);
        if (!resume && niter == K && (w.traj || w.mlp)) {
            // features and prediction on warp 0 only (FP64 logarithms)
            if (tid < 32) {
                float f[kFeat];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    f[i] = static_cast<float>(log(hist[i + 1] / hist[0]));
                    f[4 + i] = static_cast<float>(log10(lam_hist[i]));
                }
                f[8] = static_cast<float>(log(static_cast<double>(ob.ndata)));
                f[9] = static_cast<float>(log(prd));
                if (w.traj && tid == 0) {
                    float *rec = w.traj + static_cast<size_t>(fidx) * kTrajFloats;
                    for (int i = 0; i < kFeat; i++) rec[i] = f[i];
                    rec[10] = static_cast<float>(dev_new);
                }
                if (w.mlp && w.iter_limit == K) {
                    const float y = mlp_predict_warp(w.mlp, f, reinterpret_cast<float *>(s.pt));
                    if (tid == 0) pred_dev = dev_new * exp(static_cast<double>(y));
                }
            }
            __syncthreads();
        }
        if (w.iter_limit > 0 && niter >= w.iter_limit) {
            screened = true;
            if (st) {
                // save the state for a later resume (thread 0 holds the
                // prediction; every thread holds the broadcast scalars)
                for (int i = tid; i < ma; i += NT) st[i] = s.cg[i];
                if (tid == 0) {
                    st[ma] = alamda;
                    st[ma + 1] = ochisq;
                    st[ma + 2] = chisq;
                    st[ma + 3] = rchisq;
                    st[ma + 4] = iter_diff;
                    st[ma + 5] = dev_old;
                    st[ma + 6] = dev_new;
                    for (int c = 0; c < 3; c++) st[ma + 7 + c] = chk_acc[c];
                    st[ma + 10] = totarea;
                    st[ma + 11] = niter;
                    st[ma + 12] = last_err;
                    st[ma + 13] = pred_dev;
                }
            }
            break;
        }
    }
    if (w.traj && tid == 0) {
        float *rec = w.traj + static_cast<size_t>(fidx) * kTrajFloats;
        rec[11] = static_cast<float>(dev_new);
        rec[12] = static_cast<float>(niter);
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
        r.pred_dev = pred_dev;
        r.screened = screened ? 1 : 0;
        r.reserved = 0;
        if (out) *out = r;
    }
    __syncthreads();
}

template <int FORM, int KU>
__global__ void __launch_bounds__(threads_of<FORM>(), 1)
    fit_kernel(DevObject ob, FitConfig cfg, FitWork w, int P, int dsph_smem)
{
    using R = typename RealOf<FORM>::T;
    constexpr int NT = threads_of<FORM>();
    extern __shared__ __align__(16) char smem[];
    const SlotLayout L = make_layout(FORM, ob.ma, ob.mfit, ob.nfac, ob.ncoef, P, dsph_smem, w.rel_rows);
    Smem<FORM> s = carve<FORM>(smem, L);
    constexpr bool kTensor = FORM == PS_FORM_MIXED && (KU == 0 || KU == 3);
    if (s.dsph)
        for (int e = threadIdx.x; e < ob.nfac * ob.ncoef; e += NT) s.dsph[e] = ob.dsph_f[e];
    TcState tcs;
    if constexpr (kTensor) tc_setup<NT, KU == 3>(ob, s, tcs);
    // the wide tensor-core path keeps the slot's normal matrix in global memory
    if (L.dsph_smem == kBasisTensorWide) s.alpha = w.alpha_g + static_cast<size_t>(blockIdx.x) * w.alpha_stride;
    R *scratch = L.rels ? reinterpret_cast<R *>(smem + L.rels)
                        : reinterpret_cast<R *>(w.scratch + static_cast<size_t>(blockIdx.x) * w.scratch_stride);
    if (FORM == PS_FORM_FP64 && threadIdx.x == 0) *lit_counter(s.misc) = 0;
    __shared__ long long next;
    for (;;) {
        if (threadIdx.x == 0) next = static_cast<long long>(atomicAdd(w.queue, 1ULL));
        __syncthreads();
        const long long f = next;
        __syncthreads();
        if (f >= w.nfits) break;
        if constexpr (kTensor) {
            if (*s.abort) break;
        }
        int64_t n;
        int pole;
        if (w.period_index) {
            n = w.period_index[f];
            pole = w.pole[f];
        } else {
            n = w.n_lo + f / PS_N_POLES;
            pole = static_cast<int>(f % PS_N_POLES) + 1;
        }
        run_fit<FORM, KU>(ob, cfg, L, s, scratch, n, pole, w.out + f, w, f, tcs);
    }
    if constexpr (kTensor) tc_teardown(s, tcs, ob.nfac);
    if (FORM == PS_FORM_FP64 && threadIdx.x == 0 && w.lit) atomicAdd(w.lit, *lit_counter(s.misc));
}

// FP64 fits, each spread over a thread-block cluster (evaluate_split): the
// cluster's leader takes fits from the work counter and hands every fit to
// all of the cluster's CTAs, which run the same LM loop together; the
// leader writes the result.  Bit-identical to fit_kernel<FP64>.
__global__ void __launch_bounds__(threads_of<PS_FORM_FP64>(), 1)
    fit_kernel_split(DevObject ob, FitConfig cfg, FitWork w, int P)
{
    namespace cgr = cooperative_groups;
    cgr::cluster_group cl = cgr::this_cluster();
    const int rank = static_cast<int>(cl.block_rank()), cs = static_cast<int>(cl.num_blocks());
    extern __shared__ __align__(16) char smem[];
    const SlotLayout L = make_layout(PS_FORM_FP64, ob.ma, ob.mfit, ob.nfac, ob.ncoef, P, 0, w.rel_rows);
    Smem<PS_FORM_FP64> s = carve<PS_FORM_FP64>(smem, L);
    TcState tcs;
    double *scratch = L.rels ? reinterpret_cast<double *>(smem + L.rels)
                             : w.scratch + static_cast<size_t>(blockIdx.x) * w.scratch_stride;
    if (threadIdx.x == 0) *lit_counter(s.misc) = 0;
    __shared__ long long next;
    for (;;) {
        if (rank == 0 && threadIdx.x == 0) {
            const long long f = static_cast<long long>(atomicAdd(w.queue, 1ULL));
            for (int r = 0; r < cs; r++) *cl.map_shared_rank(&next, r) = f;
        }
        cl.sync();
        const long long f = next;
        cl.sync();
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
        run_fit<PS_FORM_FP64, 1>(ob, cfg, L, s, scratch, n, pole, rank == 0 ? w.out + f : nullptr, w, f, tcs, true);
    }
    if (threadIdx.x == 0 && w.lit) atomicAdd(w.lit, *lit_counter(s.misc));
}

template <int FORM, int KU>
__global__ void __launch_bounds__(threads_of<FORM>(), 1) eval_kernel(DevObject ob, FitConfig cfg, const double *cg, double *alpha,
                                                        double *beta, double *chisq, double *area, double *scratch,
                                                        int P, int dsph_smem, int rel_rows)
{
    using R = typename RealOf<FORM>::T;
    constexpr int NT = threads_of<FORM>();
    extern __shared__ __align__(16) char smem[];
    const SlotLayout L = make_layout(FORM, ob.ma, ob.mfit, ob.nfac, ob.ncoef, P, dsph_smem, rel_rows);
    Smem<FORM> s = carve<FORM>(smem, L);
    constexpr bool kTensor = FORM == PS_FORM_MIXED && (KU == 0 || KU == 3);
    if (s.dsph)
        for (int e = threadIdx.x; e < ob.nfac * ob.ncoef; e += NT) s.dsph[e] = ob.dsph_f[e];
    TcState tcs;
    if constexpr (kTensor) tc_setup<NT, KU == 3>(ob, s, tcs);
    for (int i = threadIdx.x; i < ob.ma; i += NT) s.cg[i] = cg[i];
    if (FORM == PS_FORM_FP64 && threadIdx.x == 0) *lit_counter(s.misc) = 0;
    // the wide tensor-core path accumulates straight into the output matrix
    if (L.dsph_smem == kBasisTensorWide) s.alpha = alpha;
    __syncthreads();
    R *rows = L.rels ? reinterpret_cast<R *>(smem + L.rels) : reinterpret_cast<R *>(scratch);
    evaluate<FORM, KU>(ob, cfg, L, s, s.cg, s.alpha, s.beta, rows, tcs);
    if constexpr (kTensor) {
        const bool aborted = *s.abort != 0;
        tc_teardown(s, tcs, ob.nfac);
        if (aborted) {
            if (threadIdx.x == 0) *chisq = NAN;
            return;
        }
    }
    const int mf = ob.mfit;
    if (L.dsph_smem != kBasisTensorWide)
        for (int e = threadIdx.x; e < mf * mf; e += NT) alpha[e] = s.alpha[e];
    for (int j = threadIdx.x; j < mf; j += NT) beta[j] = s.beta[j];
    if (area)
        for (int i = threadIdx.x; i < ob.nfac; i += NT) area[i] = s.area[i];
    if (threadIdx.x == 0) *chisq = s.misc[M_CHISQ];
}

}  // namespace
}  // namespace psg
