// tcgen05.cuh -- the 5th-generation tensor-core instructions of sm_100a / sm_103a (inline PTX):
// tensor-memory allocation, one-thread MMA issue with shared-memory operand descriptors, MMA
// completion through an mbarrier, and tensor-memory loads for the epilogue.
//
// Operand layout used here: K-major without swizzle.  A "core matrix" is 8 rows x 16 bytes
// (8 rows x 4 TF32 values), stored as 128 contiguous bytes; core matrices follow each other
// along K first (leading byte offset 128) and then along the rows (stride byte offset
// = 128 * K / 4).  The 64-bit shared-memory descriptor packs (PTX ISA, tcgen05 matrix
// descriptor): start address >> 4 in bits 0-13, leading byte offset >> 4 in bits 16-29, stride
// byte offset >> 4 in bits 32-45, the descriptor version 1 in bits 46-47, swizzle mode 0 (none)
// in bits 61-63.  The 32-bit instruction descriptor of kind::tf32 packs the accumulator format
// (F32 = 1) in bits 4-5, the A and B formats (TF32 = 2) in bits 7-9 and 10-12, K-major A and B
// (bits 15, 16 clear), N >> 3 in bits 17-22 and M >> 4 in bits 24-28.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace klsa {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t smem_desc_kmajor(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
    d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
    d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
    d |= static_cast<uint64_t>(1) << 46;   // descriptor version
    return d;                              // base offset 0, swizzle none
}

__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
           (static_cast<uint32_t>(M >> 4) << 24);
}

// one warp: allocate ncols columns of tensor memory, address written to *holder (shared)
__device__ __forceinline__ void tmem_alloc(uint32_t* holder, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(holder)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes become visible to the tensor core's (async proxy) reads
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D(tmem) (+)= A(smem) * B(smem)^T, kind::tf32, issued by one thread
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1u : 0u)
        : "memory");
}
// arrive on the mbarrier once every MMA issued so far by this thread has completed
__device__ __forceinline__ void commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// bounded wait for the phase with the given parity; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t limit) {
    const uint32_t a = smem_u32(mbar);
    for (uint32_t it = 0; it < limit; ++it) {
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

// 16 consecutive 32-bit columns of the warp's 32 tensor-memory lanes (lane i -> thread i)
__device__ __forceinline__ void ld_32x32b_x16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// FP32 -> TF32 (round to nearest, ties away), as the 32-bit pattern the tensor core reads
__device__ __forceinline__ float to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// byte offset of element (row, k) in a K-major, unswizzled tile of KC = K / 4 core-matrix
// columns (4-byte elements)
__device__ __forceinline__ uint32_t kmajor_offset(int row, int kidx, int KC) {
    return static_cast<uint32_t>((((row >> 3) * KC + (kidx >> 2)) << 7) + ((row & 7) << 4) + ((kidx & 3) << 2));
}

}  // namespace tc
}  // namespace klsa
