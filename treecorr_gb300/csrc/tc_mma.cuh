// tc_mma.cuh -- 5th-generation tensor core helpers for sm_100-family GPUs (tcgen05): TMEM
// allocation, shared-memory matrix descriptors, the instruction descriptor of kind::tf32,
// MMA issue, commit to an mbarrier with a bounded wait, and accumulator loads.
//
// Operand layout used here: K-major, no swizzle.  A "core matrix" is 8 rows x 16 bytes
// (4 TF32 values per row) stored as 128 contiguous bytes; an operand tile of R rows x 8 K
// values is two core matrices along K (leading byte offset 128) and R/8 along the rows
// (stride byte offset 256), i.e. element (r, k) of a K-step tile sits at
//   (r / 8) * 256 + (k / 4) * 128 + (r % 8) * 16 + (k % 4) * 4   bytes.
#pragma once

#include <cstdint>

namespace tc {

// Byte offset of element (r, k) inside one K-step (8 K values) tile.
__device__ __forceinline__ uint32_t umma_tile_off(int r, int k)
{
    return (uint32_t)((r >> 3) * 256 + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, leading (K) and stride (row) byte offsets,
// descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;            // version
    return d;                          // base offset 0, relative LBO mode, swizzle none
}

// Instruction descriptor, kind::tf32: FP32 accumulator, TF32 A and B, both K-major.
__host__ __device__ constexpr uint32_t umma_idesc_tf32(int M, int N)
{
    return (1u << 4)                      // D format: F32
         | (2u << 7)                      // A format: TF32
         | (2u << 10)                     // B format: TF32
         | ((uint32_t)(N >> 3) << 17)     // N / 8
         | ((uint32_t)(M >> 4) << 24);    // M / 16
}

// TMEM allocation by one whole warp; the address is written to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                 :: "r"(smem_u32(dst)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n"
                 :: "r"(taddr), "r"(ncols) : "memory");
}

// D (TMEM) = A * B^T (+ D when accumulate): issued by one thread.
__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n"
        "}\n"
        :: "r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

// Arrive on the mbarrier when the MMAs issued so far by this thread have completed.
__device__ __forceinline__ void umma_commit(uint64_t* mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
                 :: "r"(smem_u32(mbar)) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" :: "r"(smem_u32(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// Waits for the given phase parity; gives up after max_iter polls (returns false).
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, int max_iter)
{
    const uint32_t a = smem_u32(mbar);
    for (int it = 0; it < max_iter; ++it) {
        uint32_t done = 0;
        asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n"
            "}\n"
            : "=r"(done) : "r"(a), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

// Makes generic-proxy writes to shared memory visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// 8 consecutive FP32 accumulator columns of this thread's TMEM lane (warp w reads lanes
// 32 (w % 4) .. + 31; taddr carries the lane base in bits 16+ and the column below).
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8])
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                   "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr) : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = __uint_as_float(r[q]);
}

}  // namespace tc
