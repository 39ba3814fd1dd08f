// tc_mma.cuh — thin wrappers over the sm_100-family tensor-core (tcgen05)
// instructions used by the radiance-cache MLP, written as inline PTX.
//
//   TMEM      tcgen05.alloc / relinquish_alloc_permit / dealloc (one warp),
//             tcgen05.ld 32x32b (each warp reads its 32-lane quarter).
//   MMA       tcgen05.mma.cta_group::1.kind::f16: D(TMEM, FP32) (+)= A(SMEM) ·
//             B(SMEM), issued by one thread; tcgen05.commit arrives on an
//             mbarrier when the issued MMAs have completed.
//   Operands  no swizzle, tiled into "core matrices" of 8 x 8 elements
//             (16-bit), each 128 contiguous bytes in 8 rows of 16 bytes.
//             K-major: a core row holds 8 consecutive K of one M/N row.
//             MN-major: a core row holds 8 consecutive M/N of one K.
//             Either way the core matrix covering (M/N block mi, K block ki)
//             sits at mi * SBO + ki * LBO from the operand base; here every
//             operand uses LBO = 128 (cores adjacent along K are contiguous)
//             and SBO = (K / 8) * 128.
//   Waits     every mbarrier wait is bounded by %globaltimer; on timeout the
//             caller records an error and skips the rest of its work.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace orn {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_timer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---- mbarrier -----------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* m, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(m)), "r"(count));
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* m, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(m)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase with the given parity to complete; gives up after
// `timeout_ns` and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* m, uint32_t parity, uint64_t timeout_ns) {
    const uint64_t t0 = global_timer();
    while (!mbar_try_wait(m, parity)) {
        if (global_timer() - t0 > timeout_ns) return false;
    }
    return true;
}

// ---- fences ---------------------------------------------------------------------
// Generic-proxy shared-memory writes become visible to the async proxy
// (which the MMA reads operands through).
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---- TMEM -------------------------------------------------------------------------
// Executed by one whole warp; writes the TMEM base address to *dst (shared).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane.  `taddr` must
// carry the warp's lane quarter in bits 16+ (lane base = 32 * (warp % 4)).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---- descriptors -------------------------------------------------------------------
// Shared-memory matrix descriptor: start address, leading (K) and stride
// (M/N) byte offsets, all >> 4; descriptor version 1 at bits 46-47; no
// swizzle (layout type 0 at bits 61-63), base offset 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor for kind::f16: FP32 accumulator (bits 4-5 = 1),
// A and B both F16 (0) or both BF16 (1) (bits 7-9, 10-12), A and B K-major
// (bits 15, 16 = 0) or MN-major (1), N >> 3 at bits 17-22, M >> 4 at bits
// 24-28.
__host__ __device__ constexpr uint32_t idesc_f16(uint32_t m, uint32_t n, bool bf16, bool mn_major = false) {
    return (1u << 4) | ((bf16 ? 1u : 0u) << 7) | ((bf16 ? 1u : 0u) << 10) | ((mn_major ? 1u : 0u) << 15) |
           ((mn_major ? 1u : 0u) << 16) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

// D[tmem] (+)= A · B, one thread issues.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                        bool accumulate) {
    uint32_t acc = accumulate ? 1u : 0u;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(acc)
        : "memory");
}

// Arrive on `mbar` once all MMAs this thread issued have completed.
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_addr(mbar))
                 : "memory");
}

// Byte offset of element (r, k) of a K-major no-swizzle operand with K
// columns (LBO = 128, SBO = K/8 * 128).
__host__ __device__ __forceinline__ uint32_t kmajor_offset(uint32_t r, uint32_t k, uint32_t K) {
    return (r >> 3) * (K >> 3) * 128u + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Byte offset of element (r, k) of an MN-major no-swizzle operand with K
// columns (same LBO and SBO): 8 consecutive r of one k are 16 contiguous
// bytes, so a row of the source matrix stored k by k lands as whole
// 16-byte chunks.
__host__ __device__ __forceinline__ uint32_t mnmajor_offset(uint32_t r, uint32_t k, uint32_t K) {
    return (r >> 3) * (K >> 3) * 128u + (k >> 3) * 128u + (k & 7u) * 16u + (r & 7u) * 2u;
}

}  // namespace tc
}  // namespace orn
