// ps_tc.cu -- self-test of the tcgen05 primitives that the mixed form uses:
// one CTA stages A (128 x K) in Tensor Memory and B (32 x K) in shared memory
// in the canonical layout, runs TF32 MMAs of shape 128 x 32 x 8 (or FP16
// MMAs of shape 128 x 32 x 16) into a Tensor Memory accumulator and reads
// D = A B^T back.  Exposed through the C ABI so that tests can check the
// operand and accumulator layouts against exact integer products.
#include <cuda_runtime.h>

#include <cstdint>

#include "ps_gb300.h"
#include "ps_tc.cuh"

namespace psg {
namespace {

constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kDCol = 480;             // accumulator columns [480, 512)
constexpr uint32_t kWaitTries = 1u << 22;   // mbarrier polls before giving up

// KIND 0: TF32 operands (K/8 MMAs); 1: FP16 operands (K/16 MMAs, two
// elements per Tensor Memory column).
template <int KIND>
__global__ void __launch_bounds__(128, 1)
tc_selftest_kernel(const float *A, const float *B, int K, float *D, int *status)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm);
    uint32_t *slot = reinterpret_cast<uint32_t *>(sm + 8);
    unsigned char *bs = sm + 1024;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tc::tmem_alloc(slot, kTmemCols);
    if (tid == 0) tc::mbar_init(mbar, 1);
    for (int e = tid; e < 32 * K; e += 128) {
        const int r = e / K, k = e - r * K;
        if constexpr (KIND == 0) {
            *reinterpret_cast<uint32_t *>(bs + tc::canon_offset(r, k, K)) = tc::to_tf32(B[e]);
        } else if ((k & 1) == 0) {
            *reinterpret_cast<uint32_t *>(bs + tc::canon_offset16(r, k, K)) = tc::pack_f16x2(B[e], B[e + 1]);
        }
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *slot;
    const uint32_t lane_base = static_cast<uint32_t>(warp * 32) << 16;
    const int m = warp * 32 + lane;
    constexpr int kPerCol = KIND == 0 ? 1 : 2;   // K elements per Tensor Memory column
    for (int k0 = 0; k0 < K; k0 += 8 * kPerCol) {
        uint32_t v[8];
        const float *a = A + static_cast<size_t>(m) * K + k0;
#pragma unroll
        for (int j = 0; j < 8; j++) v[j] = KIND == 0 ? tc::to_tf32(a[j]) : tc::pack_f16x2(a[2 * j], a[2 * j + 1]);
        tc::tmem_st8(tbase + lane_base + static_cast<uint32_t>(k0 / kPerCol), v);
    }
    tc::tmem_wait_st();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
        // one MMA per 32 bytes of K: 8 Tensor Memory columns of A, two core
        // matrices of B
        const uint32_t idesc = KIND == 0 ? tc::idesc_tf32(128, 32) : tc::idesc_f16(128, 32);
        const uint32_t b0 = tc::smem_u32(bs);
        const int kstep = 8 * kPerCol;
        const uint32_t sbo = static_cast<uint32_t>(K / (4 * kPerCol)) * 128;
        for (int ks = 0; ks < K / kstep; ks++) {
            const uint64_t bd = tc::smem_desc(b0 + static_cast<uint32_t>(ks) * 256, 128, sbo);
            if constexpr (KIND == 0)
                tc::mma_tf32_ts(tbase + kDCol, tbase + static_cast<uint32_t>(ks) * 8, bd, idesc, ks > 0);
            else
                tc::mma_f16_ts(tbase + kDCol, tbase + static_cast<uint32_t>(ks) * 8, bd, idesc, ks > 0);
        }
        tc::mma_commit(mbar);
    }
    const bool ok = __syncthreads_and(tc::mbar_wait(mbar, 0, kWaitTries));
    tc::fence_after_sync();
    if (ok) {
#pragma unroll
        for (int c0 = 0; c0 < 32; c0 += 8) {
            uint32_t v[8];
            tc::tmem_ld8(tbase + lane_base + kDCol + c0, v);
            tc::tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 8; j++) D[m * 32 + c0 + j] = __uint_as_float(v[j]);
        }
    } else if (tid == 0) {
        atomicOr(status, 1);
        // the MMAs may still be in flight: give them another bounded wait
        // before the columns are released
        tc::mbar_wait(mbar, 0, kWaitTries);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, kTmemCols);
}

// The bounded-wait path of the kernels, exercised on purpose: the CTA holds
// Tensor Memory, waits on an mbarrier phase that nothing will complete (no
// MMA is issued, nothing arrives), gives up after max_polls polls, records
// the timeout and frees its Tensor Memory -- what a fit slot does when a
// tensor-core wait expires.  Nothing is in flight when it gives up.
__global__ void __launch_bounds__(128, 1) tc_wait_selftest_kernel(uint32_t max_polls, int *status)
{
    __shared__ __align__(16) uint64_t mbar;
    __shared__ uint32_t slot;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) tc::tmem_alloc(&slot, 32);
    if (tid == 0) tc::mbar_init(&mbar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = slot;
    const bool ok = __syncthreads_and(tc::mbar_wait(&mbar, 0, max_polls));
    if (tid == 0) *status = ok ? 2 : 1;   // 1: the wait gave up (expected); 2: the phase completed
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 32);
}

}  // namespace
}  // namespace psg

namespace {

template <int KIND>
ps_status run_selftest(int32_t device, const float *A, const float *B, int32_t K, float *D)
{
    if (cudaSetDevice(device) != cudaSuccess) return PS_ERR_NO_DEVICE;
    float *dA = nullptr, *dB = nullptr, *dD = nullptr;
    int *dS = nullptr;
    ps_status st = PS_OK;
    const size_t smem = 1024 + static_cast<size_t>(32) * K * (KIND == 0 ? 4 : 2);
    int hs = 0;
    if (cudaMalloc(&dA, sizeof(float) * 128 * K) != cudaSuccess || cudaMalloc(&dB, sizeof(float) * 32 * K) != cudaSuccess ||
        cudaMalloc(&dD, sizeof(float) * 128 * 32) != cudaSuccess || cudaMalloc(&dS, sizeof(int)) != cudaSuccess) {
        st = PS_ERR_CUDA;
        goto done;
    }
    cudaMemcpy(dA, A, sizeof(float) * 128 * K, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, B, sizeof(float) * 32 * K, cudaMemcpyHostToDevice);
    cudaMemset(dD, 0, sizeof(float) * 128 * 32);
    cudaMemset(dS, 0, sizeof(int));
    if (cudaFuncSetAttribute(psg::tc_selftest_kernel<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem)) != cudaSuccess) {
        st = PS_ERR_CUDA;
        goto done;
    }
    psg::tc_selftest_kernel<KIND><<<1, 128, smem>>>(dA, dB, K, dD, dS);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        st = PS_ERR_CUDA;
        goto done;
    }
    cudaMemcpy(D, dD, sizeof(float) * 128 * 32, cudaMemcpyDeviceToHost);
    cudaMemcpy(&hs, dS, sizeof(int), cudaMemcpyDeviceToHost);
    if (hs) st = PS_ERR_TIMEOUT;
done:
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(dS);
    return st;
}

}  // namespace

extern "C" ps_status ps_tc_selftest(int32_t device, const float *A, const float *B, int32_t K, float *D)
{
    if (!A || !B || !D || K < 8 || K > 480 || K % 8) return PS_ERR_ARG;
    return run_selftest<0>(device, A, B, K, D);
}

extern "C" ps_status ps_tc_selftest_f16(int32_t device, const float *A, const float *B, int32_t K, float *D)
{
    if (!A || !B || !D || K < 16 || K > 960 || K % 16) return PS_ERR_ARG;
    return run_selftest<1>(device, A, B, K, D);
}

extern "C" ps_status ps_tc_wait_selftest(int32_t device, int32_t max_polls)
{
    if (max_polls < 1 || max_polls > (1 << 22)) return PS_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return PS_ERR_NO_DEVICE;
    int *dS = nullptr;
    if (cudaMalloc(&dS, sizeof(int)) != cudaSuccess) return PS_ERR_CUDA;
    int hs = 0;
    ps_status st = PS_OK;
    if (cudaMemset(dS, 0, sizeof(int)) != cudaSuccess) st = PS_ERR_CUDA;
    if (st == PS_OK) {
        psg::tc_wait_selftest_kernel<<<1, 128>>>(static_cast<uint32_t>(max_polls), dS);
        if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(&hs, dS, sizeof(int), cudaMemcpyDeviceToHost) !=
                                                          cudaSuccess)
            st = PS_ERR_CUDA;
        else if (hs == 1)
            st = PS_ERR_TIMEOUT;
        else if (hs != 2)
            st = PS_ERR_CUDA;
    }
    cudaFree(dS);
    return st;
}
