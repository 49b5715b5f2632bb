// ps_engine.cu -- single-object launchers of the fit kernels (ps_fit.cuh),
// the FMA peak probe and the allocation-free launch.
#include "ps_fit.cuh"

namespace psg {
namespace {

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
// Device address of g_noalloc_scratch, per device ordinal, looked up once.
// The cache assumes that the device's primary context outlives every call:
// after cudaDeviceReset (or a reset of the primary context) the address is
// stale, so a process that resets a device must not call the entry point on
// it again.
double *g_noalloc_ptr[64] = {};
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
    // Rows parked in shared memory (w.rel_rows > 0): the kernel reads no
    // global scratch, only the counter, and every slot of the plan runs.
    // Otherwise each slot takes a scratch block of the array.
    const size_t usable = kStaticScratchDoubles - kStaticCounterDoubles;
    const int64_t slots = w.rel_rows > 0 ? max_grid : static_cast<int64_t>(usable / w.scratch_stride);
    if (slots < 1) return -1;  // one slot's scratch exceeds the array
    int64_t grid = slots < max_grid ? slots : max_grid;
    if (grid > w.nfits) grid = w.nfits;
    w.queue = reinterpret_cast<unsigned long long *>(base);
    w.scratch = base + kStaticCounterDoubles;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    e = cudaMemsetAsync(base, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return static_cast<int>(e);
    fit_kernel<PS_FORM_FP64, 1><<<static_cast<int>(grid), kThreads, smem, st>>>(ob, cfg, w, P, 0);
    *grid_used = static_cast<int>(grid);
    return static_cast<int>(cudaGetLastError());
}

namespace {

// Mixed-form kernel variant: 0 = tensor-core contraction and alpha; 3 = the
// wide tensor-core contraction (65..96 coefficients) with the SIMT alpha;
// otherwise the SIMT contraction's coefficient slots per lane, 1 for C <= 64
// and 2 up to 128 (the largest Laplace series, L = 10, has 121
// coefficients).
inline int ku_of(int ncoef, int dsph_smem)
{
    if (dsph_smem == kBasisTensor) return 0;
    if (dsph_smem == kBasisTensorWide) return 3;
    return ncoef <= 64 ? 1 : 2;
}

template <class Fn>
cudaError_t for_mixed(int ncoef, int dsph_smem, Fn fn)
{
    switch (ku_of(ncoef, dsph_smem)) {
    case 0: return fn(std::integral_constant<int, 0>{});
    case 1: return fn(std::integral_constant<int, 1>{});
    case 3: return fn(std::integral_constant<int, 3>{});
    default: return fn(std::integral_constant<int, 2>{});
    }
}

}  // namespace

// The dynamic shared-memory limit is a property of the kernel function (per
// device), shared by every context of the process: it is only ever raised,
// so that a context whose slots need less shared memory does not lower it
// under another context's launches.
int set_kernel_smem(int form, size_t smem, int ncoef, int dsph_smem)
{
    static std::mutex mu;
    static int raised[64][2][4] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return static_cast<int>(e);
    const int ku = form == PS_FORM_FP64 ? 1 : ku_of(ncoef, dsph_smem);
    std::lock_guard<std::mutex> lock(mu);
    int *cur = (dev >= 0 && dev < 64 && (form == PS_FORM_FP64 || form == PS_FORM_MIXED)) ? &raised[dev][form][ku] : nullptr;
    if (cur && *cur >= static_cast<int>(smem)) return 0;
    const int bytes = static_cast<int>(smem);
    if (form == PS_FORM_FP64) {
        e = cudaFuncSetAttribute(fit_kernel<PS_FORM_FP64, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(eval_kernel<PS_FORM_FP64, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(fit_kernel_split, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    } else if (form == PS_FORM_MIXED) {
        e = for_mixed(ncoef, dsph_smem, [&](auto ku) {
            constexpr int KU = decltype(ku)::value;
            cudaError_t r = cudaFuncSetAttribute(fit_kernel<PS_FORM_MIXED, KU>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
            if (r == cudaSuccess)
                r = cudaFuncSetAttribute(eval_kernel<PS_FORM_MIXED, KU>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         bytes);
            return r;
        });
    } else {
        return static_cast<int>(cudaErrorInvalidValue);
    }
    if (e == cudaSuccess && cur) *cur = bytes;
    return static_cast<int>(e);
}

int occupancy_slots(int form, size_t smem, int ncoef, int dsph_smem, int *per_sm)
{
    if (form == PS_FORM_FP64)
        return static_cast<int>(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            per_sm, fit_kernel<PS_FORM_FP64, 1>, threads_of<PS_FORM_FP64>(), smem));
    if (form == PS_FORM_MIXED)
        return static_cast<int>(for_mixed(ncoef, dsph_smem, [&](auto ku) {
            constexpr int KU = decltype(ku)::value;
            return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, fit_kernel<PS_FORM_MIXED, KU>,
                                                                 threads_of<PS_FORM_MIXED>(), smem);
        }));
    return static_cast<int>(cudaErrorInvalidValue);
}

int launch_fits(int form, const DevObject &ob, const FitConfig &cfg, const FitWork &w, int grid, int P, size_t smem,
                int dsph_smem, void *stream)
{
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (form == PS_FORM_FP64) {
        fit_kernel<PS_FORM_FP64, 1><<<grid, threads_of<PS_FORM_FP64>(), smem, st>>>(ob, cfg, w, P, 0);
    } else if (form == PS_FORM_MIXED) {
        for_mixed(ob.ncoef, dsph_smem, [&](auto ku) {
            constexpr int KU = decltype(ku)::value;
            fit_kernel<PS_FORM_MIXED, KU><<<grid, threads_of<PS_FORM_MIXED>(), smem, st>>>(ob, cfg, w, P, dsph_smem);
            return cudaSuccess;
        });
    } else {
        return static_cast<int>(cudaErrorInvalidValue);
    }
    return static_cast<int>(cudaGetLastError());
}

namespace {
cudaLaunchConfig_t split_config(int clusters, int cs, size_t smem, cudaStream_t st, cudaLaunchAttribute *attr)
{
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(static_cast<unsigned>(clusters * cs));
    lc.blockDim = dim3(static_cast<unsigned>(threads_of<PS_FORM_FP64>()));
    lc.dynamicSmemBytes = smem;
    lc.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = static_cast<unsigned>(cs);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    return lc;
}
}  // namespace

// Clusters of cs CTAs of the split FP64 kernel that the device runs at once
// (its shared memory attribute must have been raised by set_kernel_smem).
int split_max_clusters(int cs, size_t smem, int *clusters)
{
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t lc = split_config(1, cs, smem, nullptr, attr);
    return static_cast<int>(cudaOccupancyMaxActiveClusters(clusters, fit_kernel_split, &lc));
}

int launch_fits_split(const DevObject &ob, const FitConfig &cfg, const FitWork &w, int clusters, int cs, int P,
                      size_t smem, void *stream)
{
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t lc = split_config(clusters, cs, smem, static_cast<cudaStream_t>(stream), attr);
    return static_cast<int>(cudaLaunchKernelEx(&lc, fit_kernel_split, ob, cfg, w, P));
}

int launch_eval(int form, const DevObject &ob, const FitConfig &cfg, const double *cg, double *alpha, double *beta,
                double *chisq, double *area, double *scratch, int P, size_t smem, int dsph_smem, int rel_rows,
                void *stream)
{
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (form == PS_FORM_FP64) {
        eval_kernel<PS_FORM_FP64, 1><<<1, threads_of<PS_FORM_FP64>(), smem, st>>>(ob, cfg, cg, alpha, beta, chisq,
                                                                                   area, scratch, P, 0, rel_rows);
    } else if (form == PS_FORM_MIXED) {
        for_mixed(ob.ncoef, dsph_smem, [&](auto ku) {
            constexpr int KU = decltype(ku)::value;
            eval_kernel<PS_FORM_MIXED, KU><<<1, threads_of<PS_FORM_MIXED>(), smem, st>>>(
                ob, cfg, cg, alpha, beta, chisq, area, scratch, P, dsph_smem, rel_rows);
            return cudaSuccess;
        });
    } else {
        return static_cast<int>(cudaErrorInvalidValue);
    }
    return static_cast<int>(cudaGetLastError());
}

}  // namespace psg
