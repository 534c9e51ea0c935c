// umma.cuh -- 5th-generation tensor core (tcgen05) building blocks, inline PTX
// for sm_103a: tensor-memory allocation, shared-memory operand descriptors,
// the BF16 MMA with FP32 accumulation, completion through an mbarrier, and
// tensor-memory loads for the epilogues.
//
// Operand tiles live in shared memory K-major without swizzle: the tile is a
// grid of 8 x 8 "core matrices" (8 rows x 16 bytes, 128 contiguous bytes).
// Core matrices adjacent along K are 128 B apart (leading byte offset) and
// 8-row groups are K*16 B apart (stride byte offset), so element (r, k) of an
// R x K bf16 tile sits at
//     (r / 8) * (K * 16) + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2.
// One MMA consumes K = 16 (two core matrices along K); the next K-slice
// starts 256 B further.
//
// D[M x N] (+)= A[M x K] * B[N x K]^T, M = 128 (one TMEM lane per row of D,
// N FP32 columns), issued by one thread; completion is signalled on an
// mbarrier by tcgen05.commit.  Thread t of warp w (w < 4) of the epilogue
// reads TMEM lane 32 w + t.
#pragma once

#include <stdint.h>

#include "tma.cuh"

namespace sd {
namespace umma {

__host__ __device__ constexpr uint32_t tile_off(int r, int k, int K) {
    return (uint32_t)(((r >> 3) * (K << 4)) + ((k >> 3) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// Shared-memory matrix descriptor (tcgen05 format): start address >> 4 in bits
// 0-13, leading byte offset >> 4 in bits 16-29, stride byte offset >> 4 in bits
// 32-45, the fixed version field 0b001 at bit 46, base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, int K) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(128u >> 4) << 16;
    d |= (uint64_t)(((uint32_t)K * 16u) >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A BF16 (bits 7-9
// = 1), B BF16 (bits 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---- tensor memory ---------------------------------------------------------
// Warp-collective; the base address is written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---- MMA ---------------------------------------------------------------------
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// All MMAs issued so far by this thread arrive on bar once complete.
__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

// D (+)= A * B^T over K (multiple of 16); A is M x K, B is N x K, both tiles in
// the layout above.  Single thread.
__device__ __forceinline__ void mma_tile(uint32_t tmem_d, const void* a, const void* b, int K, uint32_t idesc,
                                         bool accumulate) {
    const uint32_t sa = smem_u32(a), sb = smem_u32(b);
    for (int k = 0; k < K / 16; ++k)
        mma_bf16(tmem_d, smem_desc(sa + 256u * k, K), smem_desc(sb + 256u * k, K), idesc,
                 (accumulate || k > 0) ? 1u : 0u);
}

// ---- tensor memory -> registers ---------------------------------------------
// 32 consecutive FP32 columns of this thread's lane (32x32b shape, .x32).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 16 consecutive FP32 columns (.x16).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// TMEM address of (lane, column).
__device__ __forceinline__ uint32_t taddr(uint32_t base, int lane, int col) {
    return base + ((uint32_t)lane << 16) + (uint32_t)col;
}

}  // namespace umma
}  // namespace sd
