/*
 * Fifth-generation tensor core (tcgen05) building blocks for sm_100-family
 * GPUs, as inline PTX: shared-memory matrix descriptors, the instruction
 * descriptor of kind::f16 MMAs, tensor-memory (TMEM) allocation, MMA issue,
 * completion through an mbarrier, and TMEM loads.
 *
 * Operand layouts used here (bf16, 128-byte swizzle, every swizzle atom of
 * 8 rows x 128 bytes aligned to 1024 bytes):
 *   K-major:  element (m, k) of an operand with 64-element K blocks is at
 *             block(k / 64) + (m / 8) * 1024 + (m % 8) * 128
 *             + ((k % 64 / 8) ^ (m % 8)) * 16 + (k % 8) * 2.
 *             Descriptor: start at the K block, plus 32 bytes per 16-element
 *             K step inside the atom; SBO = 1024 (next 8 rows); LBO unused.
 *   MN-major: the same bytes read with M and K swapped: element (m, k) at
 *             mblock(m / 64) + (k / 8) * 1024 + (k % 8) * 128
 *             + ((m % 64 / 8) ^ (k % 8)) * 16 + (m % 8) * 2.
 *             Descriptor: LBO = distance between 64-element M blocks,
 *             SBO = 1024 (next 8 rows of K); a 16-row K step adds 2048.
 * So a row-major tile A[r][c] stored K-major for "rows x cols" is at the
 * same time the MN-major operand of its transpose: one copy in shared memory
 * feeds both A x (M = rows) and A^T y (M = cols).
 */
#ifndef H2G_UMMA_CUH
#define H2G_UMMA_CUH

#include <cstdint>
#include <cuda_runtime.h>

namespace h2g {
namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

/* Shared-memory matrix descriptor (tcgen05 format): start address, leading
 * and stride byte offsets (16-byte units), version 1, base offset 0, and
 * the swizzle mode (2 = 128-byte swizzle). */
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

/* Instruction descriptor of tcgen05.mma kind::f16: bf16 A and B, FP32
 * accumulator, dense; a_mn / b_mn select the MN-major operand layouts. */
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, int a_mn, int b_mn)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

/* One warp allocates ncols TMEM columns (power of two >= 32); the base
 * address is written to shared memory. */
__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

/* D[tmem] (+)= A[smem] B[smem]; one thread issues. */
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         bool accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
                 "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)accumulate)
                 : "memory");
}

/* The mbarrier at `bar` receives one arrival when every MMA this thread
 * issued before has completed. */
__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
/* generic-proxy shared-memory writes become visible to the tensor core */
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

/* 16 consecutive 32-bit TMEM columns of the warp's 32 lanes (lane i of the
 * warp gets lane (taddr >> 16) + i); wait before use. */
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                 "%13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

/* Byte offset of element (m, k) of a K-major bf16 operand with 64-element K
 * blocks of `kblock_bytes` each (128-byte swizzle). */
__host__ __device__ constexpr uint32_t kmajor_off(int m, int k, uint32_t kblock_bytes)
{
    return (uint32_t)(k / 64) * kblock_bytes + (uint32_t)(m / 8) * 1024u + (uint32_t)(m % 8) * 128u +
           (uint32_t)(((k % 64) / 8) ^ (m % 8)) * 16u + (uint32_t)(k % 8) * 2u;
}

}  // namespace umma
}  // namespace h2g

#endif
