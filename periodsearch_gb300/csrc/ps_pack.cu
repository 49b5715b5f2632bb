// ps_pack.cu -- multi-object packed launch of the fit kernels: many objects
// (work units of a multi-object run, each with its own photometry, period
// grid and convexity weight) share one persistent launch and one device work
// queue, so that small objects fill the GPU together and the tail of one
// object overlaps the next.  The objects must share the shape tables (facet
// grid and Laplace series, hence the basis held in Tensor Memory and the
// facet constants) and the free-parameter layout; each fit reads its
// object's description into shared memory before it starts.
#include "ps_fit.cuh"

namespace psg {
namespace {

template <int FORM, int KU>
__global__ void __launch_bounds__(threads_of<FORM>(), 1) pack_kernel(FitWork w, int P, int dsph_smem)
{
    using R = typename RealOf<FORM>::T;
    constexpr int NT = threads_of<FORM>();
    constexpr bool kTensor = FORM == PS_FORM_MIXED && (KU == 0 || KU == 3);
    extern __shared__ __align__(16) char smem[];
    __shared__ DevObject s_ob;
    __shared__ FitConfig s_cfg;
    __shared__ long long next;
    if (threadIdx.x == 0) s_ob = w.objs[0];
    __syncthreads();
    const SlotLayout L = make_layout(FORM, s_ob.ma, s_ob.mfit, s_ob.nfac, s_ob.ncoef, P, dsph_smem);
    Smem<FORM> s = carve<FORM>(smem, L);
    if (s.dsph)
        for (int e = threadIdx.x; e < s_ob.nfac * s_ob.ncoef; e += NT) s.dsph[e] = s_ob.dsph_f[e];
    TcState tcs;
    if constexpr (kTensor) tc_setup<NT, KU == 3>(s_ob, s, tcs);
    if (dsph_smem == kBasisTensorWide) s.alpha = w.alpha_g + static_cast<size_t>(blockIdx.x) * w.alpha_stride;
    R *scratch = reinterpret_cast<R *>(w.scratch + static_cast<size_t>(blockIdx.x) * w.scratch_stride);
    if (FORM == PS_FORM_FP64 && threadIdx.x == 0) *lit_counter(s.misc) = 0;
    for (;;) {
        if (threadIdx.x == 0) next = static_cast<long long>(atomicAdd(w.queue, 1ULL));
        __syncthreads();
        const long long f = next;
        __syncthreads();
        if (f >= w.nfits) break;
        if constexpr (kTensor) {
            if (*s.abort) break;
        }
        if (threadIdx.x == 0) {
            const int o = w.object[f];
            s_ob = w.objs[o];
            s_cfg = w.cfgs[o];
        }
        __syncthreads();
        run_fit<FORM, KU>(s_ob, s_cfg, L, s, scratch, w.period_index[f], w.pole[f], w.out + f, w, f, tcs);
    }
    if constexpr (kTensor) tc_teardown(s, tcs, s_ob.nfac);
    if (FORM == PS_FORM_FP64 && threadIdx.x == 0 && w.lit) atomicAdd(w.lit, *lit_counter(s.misc));
}

template <class Fn>
cudaError_t for_pack(int form, int ncoef, int dsph_smem, Fn fn)
{
    if (form == PS_FORM_FP64) return fn(std::integral_constant<int, PS_FORM_FP64>{}, std::integral_constant<int, 1>{});
    if (dsph_smem == kBasisTensor)
        return fn(std::integral_constant<int, PS_FORM_MIXED>{}, std::integral_constant<int, 0>{});
    if (dsph_smem == kBasisTensorWide)
        return fn(std::integral_constant<int, PS_FORM_MIXED>{}, std::integral_constant<int, 3>{});
    if (ncoef <= 64) return fn(std::integral_constant<int, PS_FORM_MIXED>{}, std::integral_constant<int, 1>{});
    return fn(std::integral_constant<int, PS_FORM_MIXED>{}, std::integral_constant<int, 2>{});
}

}  // namespace

// Raises (never lowers) the kernel's dynamic shared-memory limit on the
// current device, as set_kernel_smem does.
int set_pack_smem(int form, size_t smem, int ncoef, int dsph_smem)
{
    if (form != PS_FORM_FP64 && form != PS_FORM_MIXED) return static_cast<int>(cudaErrorInvalidValue);
    static std::mutex mu;
    static int raised[64][2][4] = {};
    int dev = 0;
    const cudaError_t de = cudaGetDevice(&dev);
    if (de != cudaSuccess) return static_cast<int>(de);
    const int ku = form == PS_FORM_FP64 ? 1
                   : dsph_smem == kBasisTensor ? 0
                   : dsph_smem == kBasisTensorWide ? 3
                   : (ncoef <= 64 ? 1 : 2);
    std::lock_guard<std::mutex> lock(mu);
    int *cur = (dev >= 0 && dev < 64) ? &raised[dev][form][ku] : nullptr;
    if (cur && *cur >= static_cast<int>(smem)) return 0;
    const cudaError_t e = for_pack(form, ncoef, dsph_smem, [&](auto f, auto kk) {
        constexpr int FORM = decltype(f)::value, KU = decltype(kk)::value;
        return cudaFuncSetAttribute(pack_kernel<FORM, KU>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(smem));
    });
    if (e == cudaSuccess && cur) *cur = static_cast<int>(smem);
    return static_cast<int>(e);
}

int launch_pack(int form, const FitWork &w, int ncoef, int grid, int P, size_t smem, int dsph_smem, void *stream)
{
    if (form != PS_FORM_FP64 && form != PS_FORM_MIXED) return static_cast<int>(cudaErrorInvalidValue);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for_pack(form, ncoef, dsph_smem, [&](auto f, auto ku) {
        constexpr int FORM = decltype(f)::value, KU = decltype(ku)::value;
        pack_kernel<FORM, KU><<<grid, threads_of<FORM>(), smem, st>>>(w, P, dsph_smem);
        return cudaSuccess;
    });
    return static_cast<int>(cudaGetLastError());
}

}  // namespace psg
