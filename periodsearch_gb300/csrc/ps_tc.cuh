// ps_tc.cuh -- Blackwell tensor-core primitives (tcgen05, Tensor Memory,
// mbarrier) as inline PTX for sm_103a, used by the mixed form's shape
// contraction and normal-matrix accumulation.
//
// The contraction is J^T[k][p] = sum_i Dsph^T[k][i] W^T[i][p] with A =
// Dsph^T (coefficients x facets) resident in Tensor Memory and B = W (points
// x facets, K-major) staged in shared memory in the no-swizzle canonical
// layout: 8-row x 16-byte core matrices, K-adjacent core matrices 128 bytes
// apart (leading byte offset), 8-row groups K/e core matrices apart (stride
// byte offset; e = 4 TF32 or 8 FP16 elements per 16 bytes).  In Tensor
// Memory a 32-bit column holds one TF32 element or two FP16 elements (the
// lower K index in the low half).  The accumulator D (M = 128 lanes x N
// columns, FP32) lives in Tensor Memory and is read back with tcgen05.ld
// (row m = lane m).
#pragma once

#include <cstdint>

namespace psg {
namespace tc {

// Instruction descriptor of tcgen05.mma.kind::tf32: D FP32, A and B TF32,
// both K-major, dense, shape M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N)
{
    return (1u << 4)                                  // D format F32
           | (2u << 7)                                // A format TF32
           | (2u << 10)                               // B format TF32
           | (static_cast<uint32_t>(N >> 3) << 17)    // N / 8
           | (static_cast<uint32_t>(M >> 4) << 24);   // M / 16
}

// Instruction descriptor of tcgen05.mma.kind::f16 with FP16 A and B: D
// FP32, both K-major, dense, shape M x N (K = 16 per MMA).
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N)
{
    return (1u << 4)                                  // D format F32
           | (0u << 7)                                // A format F16
           | (0u << 10)                               // B format F16
           | (static_cast<uint32_t>(N >> 3) << 17)    // N / 8
           | (static_cast<uint32_t>(M >> 4) << 24);   // M / 16
}

// Shared-memory matrix descriptor, no swizzle: start address, leading byte
// offset (K direction) and stride byte offset (M/N direction), all >> 4;
// bits 46-48 hold the fixed value 0b001.
__device__ inline uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4) | (static_cast<uint64_t>(lbo >> 4) << 16) |
           (static_cast<uint64_t>(sbo >> 4) << 32) | (1ull << 46);
}

// Byte offset of element (row r, k) of a K-major operand with K columns in
// the canonical no-swizzle layout (K-adjacent core matrices contiguous).
__host__ __device__ inline uint32_t canon_offset(int r, int k, int K)
{
    return static_cast<uint32_t>(((r >> 3) * (K >> 2) + (k >> 2)) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

// The same for 16-bit elements (8 per core-matrix row).
__host__ __device__ inline uint32_t canon_offset16(int r, int k, int K)
{
    return static_cast<uint32_t>(((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ inline uint32_t smem_u32(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// ---- Tensor Memory allocation (one warp, collective) ----
__device__ inline void tmem_alloc(uint32_t *slot_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot_smem)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ inline void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ inline void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ inline void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor core (async proxy)
__device__ inline void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- register <-> Tensor Memory (warp-collective, 32 lanes x 8 columns) ----
// Thread t of the warp accesses lane (taddr.lane + t), columns taddr.col .. +7.
__device__ inline void tmem_st8(uint32_t taddr, const uint32_t (&v)[8])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
                 "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
                 : "memory");
}

__device__ inline void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ inline void tmem_ld8(uint32_t taddr, uint32_t (&v)[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                 : "r"(taddr)
                 : "memory");
}

__device__ inline void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---- MMA: D[tmem] (+)= A[tmem] * B[smem]^T, issued by one thread ----
__device__ inline void mma_tf32_ts(uint32_t d_taddr, uint32_t a_taddr, uint64_t b_desc, uint32_t idesc,
                                   uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_taddr),
        "r"(a_taddr), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ inline void mma_f16_ts(uint32_t d_taddr, uint32_t a_taddr, uint64_t b_desc, uint32_t idesc,
                                  uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_taddr),
        "r"(a_taddr), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// ---- MMA: D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread ----
__device__ inline void mma_tf32_ss(uint32_t d_taddr, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                   uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_taddr),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrives once on the mbarrier when every MMA issued before by this thread
// has completed.
__device__ inline void mma_commit(uint64_t *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

// ---- mbarrier ----
__device__ inline void mbar_init(uint64_t *mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Waits for the phase with the given parity to complete; gives up after
// max_tries polls and returns false.
__device__ inline bool mbar_wait(uint64_t *mbar, uint32_t parity, uint32_t max_tries)
{
    const uint32_t a = smem_u32(mbar);
    for (uint32_t i = 0; i < max_tries; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// FP16 rounding (round to nearest even) of two FP32 values, packed with the
// first (the lower K index) in the low half: cvt.f16x2 puts its first
// source in the high half.
__device__ inline uint32_t pack_f16x2(float k0, float k1)
{
    uint32_t r;
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(k1), "f"(k0));
    return r;
}

// x rounded to FP16 (nearest even), as an FP32 value.
__device__ inline float round_f16(float x)
{
    float r;
    asm("{\n\t.reg .b16 h;\n\tcvt.rn.f16.f32 h, %1;\n\tcvt.f32.f16 %0, h;\n\t}" : "=f"(r) : "f"(x));
    return r;
}

// The FP32 value of the low or high FP16 half of a packed pair.
__device__ inline float f16_lo(uint32_t v)
{
    float f;
    asm("{\n\t.reg .b16 l, h;\n\tmov.b32 {l, h}, %1;\n\tcvt.f32.f16 %0, l;\n\t}" : "=f"(f) : "r"(v));
    return f;
}
__device__ inline float f16_hi(uint32_t v)
{
    float f;
    asm("{\n\t.reg .b16 l, h;\n\tmov.b32 {l, h}, %1;\n\tcvt.f32.f16 %0, h;\n\t}" : "=f"(f) : "r"(v));
    return f;
}

// TF32 rounding (round to nearest, ties away) of an FP32 value, as a bit pattern.
__device__ inline uint32_t to_tf32(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

}  // namespace tc
}  // namespace psg
