// tc_selftest.cu — a one-tile tcgen05 GEMM used to check the operand and
// instruction descriptor encodings (tc_mma.cuh) against a host GEMM.
//
// D[128 x N] = A[128 x K] · B[N x K]^T with A and B given row-major (K
// contiguous) in global memory, staged into the K-major no-swizzle layout
// (or the MN-major one, mode bit 1), multiplied with K/16 tcgen05.mma
// instructions into TMEM and read back with tcgen05.ld.  Mode bit 0
// exchanges the two byte offsets in the operand descriptors (for the
// self-test to tell the encodings apart); every form addresses only the
// 64 KiB operand regions below.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstring>

#include "ornament_cuda.h"
#include "tc_mma.cuh"

namespace orn {

constexpr uint32_t kSelfTestRegion = 64 * 1024;

__global__ void __launch_bounds__(128)
tc_selftest_kernel(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B, float* __restrict__ D,
                   uint32_t K, uint32_t N, uint32_t bf16, uint32_t mode, uint32_t* status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    unsigned char* sa = smem;
    unsigned char* sb = smem + kSelfTestRegion;
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const bool swap_offsets = (mode & 1u) != 0, mn_major = (mode & 2u) != 0;
    // stage A (128 rows) and B (N rows): 16-byte chunks (K-major) or single
    // elements (MN-major)
    if (mn_major) {
        for (uint32_t k = 0; k < K; ++k) {
            *(uint16_t*)(sa + tc::mnmajor_offset(tid, k, K)) = A[(size_t)tid * K + k];
            if (tid < N) *(uint16_t*)(sb + tc::mnmajor_offset(tid, k, K)) = B[(size_t)tid * K + k];
        }
    } else {
        for (uint32_t k = 0; k < K; k += 8) {
            *(uint4*)(sa + tc::kmajor_offset(tid, k, K)) = *(const uint4*)(A + (size_t)tid * K + k);
            if (tid < N) *(uint4*)(sb + tc::kmajor_offset(tid, k, K)) = *(const uint4*)(B + (size_t)tid * K + k);
        }
    }
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base, 128);
        tc::tmem_relinquish();
    }
    if (tid == 0) tc::mbar_init(&mbar, 1);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const uint32_t lbo = 128u, sbo = (K / 8u) * 128u;
    if (tid == 0) {
        const uint32_t idesc = tc::idesc_f16(128, N, bf16 != 0, mn_major);
        for (uint32_t ks = 0; ks < K / 16u; ++ks) {
            uint32_t off = ks * 2u * 128u;
            uint64_t ad = swap_offsets ? tc::smem_desc(tc::smem_addr(sa) + off, sbo, lbo)
                                       : tc::smem_desc(tc::smem_addr(sa) + off, lbo, sbo);
            uint64_t bd = swap_offsets ? tc::smem_desc(tc::smem_addr(sb) + off, sbo, lbo)
                                       : tc::smem_desc(tc::smem_addr(sb) + off, lbo, sbo);
            tc::mma_f16(tmem, ad, bd, idesc, ks > 0);
        }
        tc::mma_commit(&mbar);
    }
    bool ok = tc::mbar_wait(&mbar, 0, 1000000000ull);
    // in-flight MMAs: wait once more; the columns are freed in any case (a
    // CTA leaving them allocated could block later allocations on the SM)
    if (!ok) ok = tc::mbar_wait(&mbar, 0, 1000000000ull);
    tc::fence_after_sync();
    if (ok) {
        for (uint32_t c = 0; c < N; c += 16) {
            float v[16];
            tc::tmem_ld16(tmem + ((32u * warp) << 16) + c, v);
            tc::tmem_ld_wait();
            for (int j = 0; j < 16; ++j) D[(size_t)tid * N + c + j] = v[j];
        }
    } else if (tid == 0) {
        atomicOr(status, 1u);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

}  // namespace orn

extern "C" int orn_tc_selftest(uint32_t K, uint32_t N, int bf16, int mode, const uint16_t* A,
                               const uint16_t* B, float* D) {
    if (!A || !B || !D || K == 0 || K > 256 || K % 16 || N < 16 || N > 128 || N % 16 || mode < 0 || mode > 3)
        return ORN_ERR_INVALID_ARGUMENT;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return ORN_ERR_NO_DEVICE;
    uint16_t *dA = nullptr, *dB = nullptr;
    float* dD = nullptr;
    uint32_t* dS = nullptr;
    int st = ORN_OK;
    const size_t smem = 2 * orn::kSelfTestRegion;
    if (cudaMalloc(&dA, 128 * K * 2) != cudaSuccess || cudaMalloc(&dB, N * K * 2) != cudaSuccess ||
        cudaMalloc(&dD, 128 * N * 4) != cudaSuccess || cudaMalloc(&dS, 4) != cudaSuccess) {
        st = ORN_ERR_OUT_OF_MEMORY;
    } else if (cudaMemcpy(dA, A, 128 * K * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
               cudaMemcpy(dB, B, N * K * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
               cudaMemset(dS, 0, 4) != cudaSuccess || cudaMemset(dD, 0, 128 * N * 4) != cudaSuccess ||
               cudaFuncSetAttribute(orn::tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem) != cudaSuccess) {
        st = ORN_ERR_CUDA;
    } else {
        orn::tc_selftest_kernel<<<1, 128, smem>>>(dA, dB, dD, K, N, bf16 ? 1u : 0u, (uint32_t)mode, dS);
        uint32_t s = 0;
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
            cudaMemcpy(&s, dS, 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(D, dD, 128 * N * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = ORN_ERR_CUDA;
        else if (s)
            st = ORN_ERR_TIMEOUT;
    }
    if (dA) cudaFree(dA);
    if (dB) cudaFree(dB);
    if (dD) cudaFree(dD);
    if (dS) cudaFree(dS);
    return st;
}
