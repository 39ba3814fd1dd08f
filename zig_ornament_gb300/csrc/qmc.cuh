// qmc.cuh — Owen-scrambled Sobol points for the cached renderer's optional
// sampler (orn_state.sampler = ORN_SAMPLER_SOBOL; the reference's sampler is
// the per-pixel PCG stream, which every parity path keeps).
//
// Sample i of a pixel takes, for each use ("pair": pixel jitter, lens,
// first-bounce direction, first light sample), the 2-D Sobol point of
// dimensions 0 and 1 — the van der Corput sequence and its (0,2) partner,
// whose generator columns follow c_k = c_{k-1} ^ (c_{k-1} >> 1) from
// c_0 = 2^31 — at a shuffled index, with both the index and the coordinates
// nested-uniform (Owen) scrambled by the hash-based construction of
// B. Burley, "Practical Hash-based Owen Scrambling", JCGT 9(4), 2020.  The
// seeds are per pixel and per pair, so pairs are decorrelated, every
// power-of-two prefix of a pixel's samples stays a stratified (0,m,2)-net in
// each pair, and every point is uniformly distributed (the estimator stays
// unbiased).
#pragma once

#include <stdint.h>

namespace orn {

enum QmcPair { QMC_PIXEL = 0, QMC_LENS = 1, QMC_BOUNCE = 2, QMC_LIGHT = 3 };

// Host and device (the host copy serves the orn_qmc_points check).
__host__ __device__ __forceinline__ uint32_t qmc_brev(uint32_t x) {
#ifdef __CUDA_ARCH__
    return __brev(x);
#else
    x = ((x >> 1) & 0x55555555u) | ((x & 0x55555555u) << 1);
    x = ((x >> 2) & 0x33333333u) | ((x & 0x33333333u) << 2);
    x = ((x >> 4) & 0x0f0f0f0fu) | ((x & 0x0f0f0f0fu) << 4);
    x = ((x >> 8) & 0x00ff00ffu) | ((x & 0x00ff00ffu) << 8);
    return (x >> 16) | (x << 16);
#endif
}

__host__ __device__ __forceinline__ uint32_t qmc_hash(uint32_t x) {
    // integer finaliser (xorshift-multiply), a seed mixer only
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// Laine-Karras style permutation of the reversed bits (Burley 2020, eq. 2).
__host__ __device__ __forceinline__ uint32_t qmc_lk_permute(uint32_t x, uint32_t seed) {
    x += seed;
    x ^= x * 0x6c50b47cu;
    x ^= x * 0xb82f1e52u;
    x ^= x * 0xc7afe638u;
    x ^= x * 0x8d22f6e6u;
    return x;
}

__host__ __device__ __forceinline__ uint32_t qmc_owen(uint32_t x, uint32_t seed) {
    return qmc_brev(qmc_lk_permute(qmc_brev(x), seed));
}

__host__ __device__ __forceinline__ uint32_t qmc_sobol1(uint32_t i) {
    uint32_t v = 0u, c = 0x80000000u;
    for (; i != 0u; i >>= 1) {
        if (i & 1u) v ^= c;
        c ^= c >> 1;
    }
    return v;
}

// Point `pair` of sample `index` of the pixel whose seed is `pixel_seed`.
__host__ __device__ __forceinline__ void qmc_point(uint32_t pixel_seed, uint32_t pair, uint32_t index, float* u0,
                                                   float* u1) {
    const uint32_t s = qmc_hash(pixel_seed ^ (0x9e3779b9u * (pair + 1u)));
    const uint32_t i = qmc_owen(index, s);
    const uint32_t x = qmc_owen(qmc_brev(i), qmc_hash(s ^ 0x68bc21ebu));
    const uint32_t y = qmc_owen(qmc_sobol1(i), qmc_hash(s ^ 0x02e5be93u));
    *u0 = (float)(x >> 8) * (1.0f / 16777216.0f);
    *u1 = (float)(y >> 8) * (1.0f / 16777216.0f);
}

}  // namespace orn
