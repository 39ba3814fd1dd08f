// radiance_cache.cu — the learned radiance cache: a small MLP trained
// online on the path tracer's own radiance samples, on the tensor cores.
//
// Network: 10 inputs (position normalised to the scene bounds, incoming
// direction, normal, roughness) → 12-band frequency encoding (sin and cos of
// 2^b·π·x, b = 0..11, for every input: 240 features) + the 10 raw inputs + a
// constant 1 + 5 zeros = 256 features → 5 hidden layers of 64 (ReLU) → 3
// outputs (RGB radiance; padded to 16 for the MMA).  No biases (the constant
// feature gives layer 1 one).  33,792 weights.
//
// Precision: forward (inference and training) in FP16 with FP32 accumulation
// in TMEM; backward in BF16 (gradients need BF16's range) with FP32
// accumulation; FP32 master weights, FP32 Adam.
//
// Every GEMM is a tcgen05.mma with M = 128 rows (a tile of 128 samples, one
// thread per sample, a group of 4 warps per tile in flight) and operands in
// shared memory (tc_mma.cuh):
//   rc_forward      X·W1ᵀ → ReLU → ·W2ᵀ … → ·W6ᵀ, activations kept in shared
//                   memory between layers, two tiles in flight per CTA;
//                   training also stores H1..H5 and the relative-L2 loss
//                   gradient dZ6.
//   rc_backward     dZ6·W6 ⊙ [H5>0] = dZ5, … down to dZ1 (BF16); a layer's
//                   H rows are fetched while its MMA runs.
//   rc_wgrad        dWlᵀ = Σ_tiles H(l-1)ᵀ·dZl: both operands MN-major
//                   (each sample's features are stored as they come, 16
//                   bytes at a time), double-buffered so the next tile is
//                   staged while the MMAs of the current one run,
//                   accumulated across sample tiles in TMEM, then added to
//                   the FP32 gradient.
//   rc_adam         Adam on the FP32 master weights; rewrites the FP16
//                   forward and BF16 backward operand copies in the K-major
//                   layout so kernels copy them to shared memory verbatim.
// All mbarrier waits are bounded (tc::mbar_wait); a timeout sets a status
// bit, the CTA waits once more for its MMAs, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "rc_kernels.h"
#include "tc_mma.cuh"

namespace orn {
namespace rc {

__device__ __forceinline__ uint16_t f2h(float x) { return __half_as_ushort(__float2half_rn(x)); }
__device__ __forceinline__ uint16_t f2b(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float h2f(uint16_t x) { return __half2float(__ushort_as_half(x)); }
__device__ __forceinline__ float b2f(uint16_t x) { return __bfloat162float(__ushort_as_bfloat16(x)); }

// The encoding of one sample's 10 inputs, produced 8 features at a time:
// emit8(f0, v) receives features f0..f0+7.  Input j gives features
// 24j + 2b (sin 2^b·π·x) and 24j + 2b + 1 (cos), b = 0..11, by angle
// doubling from one sincospi: sin 2a = 2 sin a cos a, cos 2a = (cos a - sin a)
// (cos a + sin a); the absolute error after 11 doublings stays below 2e-4,
// under the FP16 rounding of the features.  Features 240..249 are the raw
// inputs, 250 is 1 (the bias of layer 1), 251..255 are 0.
template <class F>
__device__ __forceinline__ void encode(const float* in, F&& emit8) {
    float g[8];
#pragma unroll 1
    for (int j = 0; j < kInputs; ++j) {
        float s, c;
        sincospif(in[j], &s, &c);
#pragma unroll
        for (int b = 0; b < kBands; ++b) {
            g[(2 * b) & 7] = s;
            g[(2 * b + 1) & 7] = c;
            if ((b & 3) == 3) emit8(24 * j + 2 * b - 6, g);
            const float s2 = 2.0f * s * c, c2 = (c - s) * (c + s);
            s = s2;
            c = c2;
        }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) g[j] = in[j];
    emit8(kEncoded, g);
    g[0] = in[8];
    g[1] = in[9];
    g[2] = 1.0f;
#pragma unroll
    for (int j = 3; j < 8; ++j) g[j] = 0.0f;
    emit8(kEncoded + 8, g);
}

__device__ __forceinline__ uint4 pack8(const uint16_t* h) {
    return make_uint4(h[0] | ((uint32_t)h[1] << 16), h[2] | ((uint32_t)h[3] << 16), h[4] | ((uint32_t)h[5] << 16),
                      h[6] | ((uint32_t)h[7] << 16));
}

// Offset (in elements) of layer l's backward operand inside the BF16 copy:
// layers 6, 5, 4, 3, 2 in that order (the order the backward kernel uses).
__host__ __device__ constexpr uint32_t bwd_offset(int l) {
    uint32_t o = 0;
    for (int i = kLayers - 1; i > l; --i) o += rc_layer_in(i) * rc_layer_out(i);
    return o;
}

// The 128 threads of a tile group meet at named barrier `id` (1 + the
// group; barrier 0 is __syncthreads'); the second form also returns whether
// `v` holds for all of them.
__device__ __forceinline__ void group_bar(uint32_t id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
__device__ __forceinline__ bool group_bar_and(uint32_t id, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 q, %1, 0;\n\t"
        "bar.red.and.pred p, %2, 128, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"(v ? 1u : 0u), "r"(id)
        : "memory");
    return r != 0;
}

// A tile group's synchronisation state for its MMA rounds: its mbarrier,
// the phase it waits for next, whether every wait so far completed, and its
// named barrier.
struct Sync {
    uint64_t* mbar;
    uint32_t phase;
    bool ok;
    uint32_t bar;
};

// Issues D(TMEM) = A · Bᵀ (+ D when `accumulate`), A: 128 x K at `a`, B:
// N x K at `b`, both K-major (or both MN-major when `mn_major`): makes the
// group's shared-memory writes visible to the tensor core, then the group's
// first thread issues the K/16 MMAs and commits them to the group's
// mbarrier.  Every thread of the group calls.
__device__ __forceinline__ void gemm_issue(Sync& s, uint32_t tmem, const unsigned char* a, const unsigned char* b,
                                           uint32_t K, uint32_t N, bool bf16, bool accumulate,
                                           bool mn_major = false) {
    tc::fence_async_smem();
    tc::fence_before_sync();
    group_bar(s.bar);
    tc::fence_after_sync();
    if ((threadIdx.x & 127u) == 0 && s.ok) {
        const uint32_t idesc = tc::idesc_f16(128, N, bf16, mn_major);
        const uint32_t sbo = (K / 8u) * 128u;
        for (uint32_t ks = 0; ks < K / 16u; ++ks) {
            const uint64_t ad = tc::smem_desc(tc::smem_addr(a) + ks * 256u, 128u, sbo);
            const uint64_t bd = tc::smem_desc(tc::smem_addr(b) + ks * 256u, 128u, sbo);
            tc::mma_f16(tmem, ad, bd, idesc, accumulate || ks > 0);
        }
        tc::mma_commit(s.mbar);
    }
}

// Waits (bounded) for the group's issued MMAs; all its threads agree on
// s.ok afterwards.
__device__ __forceinline__ void gemm_wait(Sync& s) {
    const bool ok = s.ok && tc::mbar_wait(s.mbar, s.phase, 2000000000ull);
    s.ok = group_bar_and(s.bar, ok);
    // on failure s.phase stays the phase of the round still in flight
    if (s.ok) s.phase ^= 1u;
    tc::fence_after_sync();
}

__device__ __forceinline__ void gemm_round(Sync& s, uint32_t tmem, const unsigned char* a, const unsigned char* b,
                                           uint32_t K, uint32_t N, bool bf16, bool accumulate) {
    gemm_issue(s, tmem, a, b, K, N, bf16, accumulate);
    gemm_wait(s);
}

// This thread's TMEM lane (its row of the tile), `ncols` FP32 columns.
__device__ __forceinline__ void read_row(uint32_t tmem, uint32_t ncols, float* v) {
    const uint32_t lane_base = (32u * ((threadIdx.x >> 5) & 3u)) << 16;
    for (uint32_t c = 0; c < ncols; c += 16) tc::tmem_ld16(tmem + lane_base + c, v + c);
    tc::tmem_ld_wait();
}

// Allocates `ncols` TMEM columns (warp 0) and initialises `nbar` mbarriers.
__device__ __forceinline__ uint32_t cta_setup(uint32_t* tmem_slot, uint64_t* mbar, uint32_t nbar, uint32_t ncols) {
    if (threadIdx.x < 32) {
        tc::tmem_alloc(tmem_slot, ncols);
        tc::tmem_relinquish();
    }
    if (threadIdx.x == 0)
        for (uint32_t i = 0; i < nbar; ++i) tc::mbar_init(mbar + i, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    return *tmem_slot;
}

// After a timed-out wait: give the group's MMAs in flight one more bounded
// wait, record the failure, then free the CTA's TMEM columns (on every
// path; `tmem_base` is the allocation's first column).  Freeing while an
// MMA might still write them is only reached when both waits (3 s) ran
// out; a CTA that exited holding its columns would instead leave them
// allocated for every later CTA on that SM, whose tcgen05.alloc could then
// wait forever, so the columns are always returned.
__device__ __forceinline__ void cta_teardown(Sync& s, uint32_t tmem_base, uint32_t ncols, uint32_t* status) {
    if (!s.ok) {
        tc::mbar_wait(s.mbar, s.phase, 1000000000ull);
        if ((threadIdx.x & 127u) == 0) atomicOr(status, 4u);   // ERR_MMA
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_dealloc(tmem_base, ncols);
}

// ---- forward ----------------------------------------------------------------------
// Two groups of 4 warps per CTA, each with a tile of 128 samples in flight
// (its own X buffer, mbarrier, named barrier and 64 TMEM columns), so one
// group's encoding and epilogues overlap the other's MMAs; group g takes
// tiles blockIdx.x + g * gridDim.x, then every 2 * gridDim.x-th.  Shared
// memory: the six FP16 weight operands (67,584 B) and per group X (128 x 256
// FP16); a layer's activations overwrite the start of X (the MMA that read
// the previous layer's has completed when they are written).
constexpr uint32_t kWfBytes = kWeightCount * 2;
constexpr uint32_t kXBytes = 128 * kFeatures * 2;
constexpr uint32_t kHBytes = 128 * kHidden * 2;
constexpr uint32_t kFwdGroups = 2;
constexpr uint32_t kFwdCols = kFwdGroups * kHidden;
constexpr uint32_t kForwardSmem = kWfBytes + kFwdGroups * kXBytes;
static_assert(kForwardSmem <= 227u * 1024u, "forward shared memory");

template <bool TRAIN>
__global__ void __launch_bounds__(128 * kFwdGroups, 1)
rc_forward(RcForward p) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar[kFwdGroups];
    __shared__ uint32_t tmem_slot;
    const uint32_t grp = threadIdx.x >> 7, t = threadIdx.x & 127u;
    unsigned char* W = smem;
    unsigned char* X = smem + kWfBytes + grp * kXBytes;
    const uint32_t n = p.n_dev ? min(*p.n_dev, p.n) : p.n;
    const uint32_t tiles = (n + 127) / 128;
    if (blockIdx.x >= tiles) return;
    for (uint32_t i = threadIdx.x; i < kWfBytes / 16; i += blockDim.x)
        ((uint4*)W)[i] = __ldg((const uint4*)p.weights_f16 + i);
    const uint32_t tmem_base = cta_setup(&tmem_slot, mbar, kFwdGroups, kFwdCols);
    const uint32_t tmem = tmem_base + grp * kHidden;
    Sync s{&mbar[grp], 0u, true, 1u + grp};
    float loss = 0.0f;
    for (uint32_t tile = blockIdx.x + grp * gridDim.x; tile < tiles && s.ok; tile += kFwdGroups * gridDim.x) {
        const uint32_t row = tile * 128 + t;
        const bool valid = row < n;
        float in[kInputs];
        for (int j = 0; j < kInputs; ++j) in[j] = valid ? p.inputs[(size_t)row * kInputs + j] : 0.0f;
        encode(in, [&](int f0, const float* g) {
            uint16_t h[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) h[j] = f2h(g[j]);
            *(uint4*)(X + tc::kmajor_offset(t, f0, kFeatures)) = pack8(h);
        });
        const unsigned char* A = X;
        uint32_t K = kFeatures;
        float v[kHidden];
        for (int l = 0; l < kLayers; ++l) {
            const uint32_t N = rc_layer_out(l);
            gemm_round(s, tmem, A, W + rc_layer_offset(l) * 2, K, N, false, false);
            if (!s.ok) break;
            read_row(tmem, N, v);
            if (l < kLayers - 1) {
                unsigned char* Hn = X;
                for (uint32_t c0 = 0; c0 < kHidden; c0 += 8) {
                    uint16_t h[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) h[j] = f2h(fmaxf(v[c0 + j], 0.0f));
                    const uint4 q = pack8(h);
                    *(uint4*)(Hn + tc::kmajor_offset(t, c0, kHidden)) = q;
                    if (TRAIN && valid) *(uint4*)(p.h_out + ((size_t)l * n + row) * kHidden + c0) = q;
                }
                A = Hn;
                K = kHidden;
            } else if (valid) {
                if (!TRAIN) {
                    if (p.pixel) {
                        // atomic: several sample streams of a pixel may query in
                        // one frame (one add each, so one query gives the same bits
                        // as a plain read-modify-write)
                        const uint32_t px = p.pixel[row];
                        const float4 th = p.throughput[row];
                        float* a = reinterpret_cast<float*>(p.acc + px);
                        atomicAdd(a + 0, th.x * fminf(fmaxf(v[0], 0.0f), 1.0e4f));
                        atomicAdd(a + 1, th.y * fminf(fmaxf(v[1], 0.0f), 1.0e4f));
                        atomicAdd(a + 2, th.z * fminf(fmaxf(v[2], 0.0f), 1.0e4f));
                    }
                    if (p.outputs)
                        for (int c = 0; c < kOutputs; ++c) p.outputs[(size_t)row * kOutputs + c] = v[c];
                } else {
                    // relative L2: per channel (y - r)^2 / (sg(y)^2 + 0.01), whose
                    // gradient is 2 (y - r) / (y^2 + 0.01)
                    uint16_t g[16];
#pragma unroll
                    for (int c = 0; c < 16; ++c) g[c] = 0;
                    const bool has = p.targets[(size_t)row * kOutputs] >= 0.0f;
                    for (int c = 0; c < kOutputs && has; ++c) {
                        const float y = v[c], r = p.targets[(size_t)row * kOutputs + c];
                        const float den = y * y + 0.01f;
                        loss += (y - r) * (y - r) / den;
                        g[c] = f2b(fminf(fmaxf(2.0f * (y - r) / den, -kGradClamp), kGradClamp));
                    }
                    if (p.outputs)
                        for (int c = 0; c < kOutputs; ++c) p.outputs[(size_t)row * kOutputs + c] = v[c];
                    uint4* dst = (uint4*)(p.dz_out + (size_t)row * kOutPad);
                    dst[0] = pack8(g);
                    dst[1] = pack8(g + 8);
                }
            }
        }
    }
    if (TRAIN && p.loss) {
        for (int o = 16; o > 0; o >>= 1) loss += __shfl_down_sync(0xffffffffu, loss, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(p.loss, loss);
    }
    cta_teardown(s, tmem_base, kFwdCols, p.status);
}

// ---- backward (data) ----------------------------------------------------------------
// Shared memory: the BF16 backward operands of layers 6..2 (34,816 B) and two
// 128 x 64 gradient buffers.
constexpr uint32_t kWbBytes = kBackwardWeightCount * 2;
constexpr uint32_t kBackwardSmem = kWbBytes + 2 * kHBytes;

__global__ void __launch_bounds__(128, 1)
rc_backward(RcBackward p) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    unsigned char* W = smem;
    unsigned char* Db[2] = {smem + kWbBytes, smem + kWbBytes + kHBytes};
    const uint32_t tiles = (p.n + 127) / 128;
    if (blockIdx.x >= tiles) return;
    for (uint32_t i = threadIdx.x; i < kWbBytes / 16; i += blockDim.x)
        ((uint4*)W)[i] = __ldg((const uint4*)p.weights_bf16 + i);
    const uint32_t tmem = cta_setup(&tmem_slot, &mbar, 1, kTmemCols);
    Sync s{&mbar, 0u, true, 1u};
    const uint32_t t = threadIdx.x;
    for (uint32_t tile = blockIdx.x; tile < tiles && s.ok; tile += gridDim.x) {
        const uint32_t row = tile * 128 + t;
        const bool valid = row < p.n;
        // dZ6 (128 x 16) is the first A operand
        uint4 g0 = make_uint4(0, 0, 0, 0), g1 = g0;
        if (valid) {
            g0 = *(const uint4*)(p.dz6 + (size_t)row * kOutPad);
            g1 = *(const uint4*)(p.dz6 + (size_t)row * kOutPad + 8);
        }
        *(uint4*)(Db[0] + tc::kmajor_offset(t, 0, kOutPad)) = g0;
        *(uint4*)(Db[0] + tc::kmajor_offset(t, 8, kOutPad)) = g1;
        const unsigned char* A = Db[0];
        uint32_t K = kOutPad;
        float v[kHidden];
        for (int l = kLayers - 1; l >= 1; --l) {
            // dH(l-1) = dZ(l) · W(l); the B operand is W(l)ᵀ (rows = layer inputs)
            gemm_issue(s, tmem, A, W + bwd_offset(l) * 2, K, kHidden, true, false);
            // the sample's H(l-1) row is fetched while the MMAs run
            const uint16_t* h = p.h + ((size_t)(l - 1) * p.n + (valid ? row : 0)) * kHidden;
            uint4 hrow[kHidden / 8];
#pragma unroll
            for (int c = 0; c < kHidden / 8; ++c)
                hrow[c] = valid ? *(const uint4*)(h + 8 * c) : make_uint4(0, 0, 0, 0);
            gemm_wait(s);
            if (!s.ok) break;
            read_row(tmem, kHidden, v);
            unsigned char* Dn = Db[(kLayers - l) & 1];
#pragma unroll
            for (uint32_t c0 = 0; c0 < kHidden; c0 += 8) {
                const uint16_t* hh = (const uint16_t*)&hrow[c0 / 8];
                uint16_t d[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) d[j] = f2b(h2f(hh[j]) > 0.0f ? v[c0 + j] : 0.0f);
                const uint4 q = pack8(d);
                *(uint4*)(Dn + tc::kmajor_offset(t, c0, kHidden)) = q;
                if (valid) *(uint4*)(p.dz + ((size_t)(l - 1) * p.n + row) * kHidden + c0) = q;
            }
            A = Dn;
            K = kHidden;
        }
    }
    cta_teardown(s, tmem, kTmemCols, p.status);
}

// ---- weight gradients -------------------------------------------------------------
// One job = (layer l, a block of up to 128 of its inputs).  For every tile of
// 128 samples the CTA stages A = H(l-1)ᵀ (inputs x samples) and B = dZ(l)ᵀ
// (outputs x samples), both MN-major with K = samples — thread t stores
// sample t's inputs and output gradients 8 at a time as 16-byte chunks,
// which keeps the stores free of bank conflicts (a K-major copy would be
// a transpose, 2 bytes per store) — and accumulates D[in x out] in TMEM
// across its tiles; D is then added to the FP32 gradient (gradient of
// W(l)[out][in] = D[in][out]).  The operands are double-buffered: tile i+1
// is staged while the MMAs of tile i run.
constexpr uint32_t kWgA = 128 * 128 * 2;
constexpr uint32_t kWgB = 64 * 128 * 2;
constexpr uint32_t kWgradSmem = 2 * (kWgA + kWgB);

__global__ void __launch_bounds__(128, 1)
rc_wgrad(RcWgrad p) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    const uint32_t job = blockIdx.x % kWgradJobs, split = blockIdx.x / kWgradJobs;
    const int l = job < 2 ? 0 : (int)job - 1;
    const uint32_t in_base = job < 2 ? job * 128u : 0u;
    const uint32_t in_n = rc_layer_in(l) - in_base < 128u ? rc_layer_in(l) - in_base : 128u;
    const uint32_t out_n = rc_layer_out(l);
    const uint32_t tiles = (p.n + 127) / 128;
    if (split >= tiles) return;
    const uint32_t t = threadIdx.x;
    // rows in_n..127 of A (inputs a layer does not have) stay zero
    for (uint32_t buf = 0; buf < 2; ++buf)
        for (uint32_t c0 = in_n; c0 < 128; c0 += 8)
            *(uint4*)(smem + buf * kWgA + tc::mnmajor_offset(c0, t, 128)) = make_uint4(0, 0, 0, 0);
    // Stages tile `tile` into operand buffer `buf`.
    auto stage = [&](uint32_t tile, uint32_t buf) {
        unsigned char* A = smem + buf * kWgA;
        unsigned char* B = smem + 2 * kWgA + buf * kWgB;
        const uint32_t row = tile * 128 + t;
        const bool valid = row < p.n;
        if (l == 0) {
            float in[kInputs];
            for (int j = 0; j < kInputs; ++j) in[j] = valid ? p.inputs[(size_t)row * kInputs + j] : 0.0f;
            // (features come in chunks of 8 at multiples of 8, and a block
            // starts at a multiple of 128, so a chunk is in or out whole)
            encode(in, [&](int f0, const float* g) {
                if ((uint32_t)f0 >= in_base && (uint32_t)f0 < in_base + 128u) {
                    uint16_t b[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) b[j] = valid ? f2b(g[j]) : (uint16_t)0;
                    *(uint4*)(A + tc::mnmajor_offset((uint32_t)f0 - in_base, t, 128)) = pack8(b);
                }
            });
        } else {
            const uint16_t* h = p.h + ((size_t)(l - 1) * p.n + (valid ? row : 0)) * kHidden;
#pragma unroll
            for (uint32_t c0 = 0; c0 < (uint32_t)kHidden; c0 += 8) {
                const uint4 hv = valid ? *(const uint4*)(h + c0) : make_uint4(0, 0, 0, 0);
                const uint16_t* hh = (const uint16_t*)&hv;
                uint16_t b[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) b[j] = f2b(h2f(hh[j]));
                *(uint4*)(A + tc::mnmajor_offset(c0, t, 128)) = pack8(b);
            }
        }
        const uint16_t* dz = l == kLayers - 1 ? p.dz6 + (size_t)(valid ? row : 0) * kOutPad
                                              : p.dz + ((size_t)l * p.n + (valid ? row : 0)) * kHidden;
        for (uint32_t c0 = 0; c0 < out_n; c0 += 8) {
            const uint4 dv = valid ? *(const uint4*)(dz + c0) : make_uint4(0, 0, 0, 0);
            *(uint4*)(B + tc::mnmajor_offset(c0, t, 128)) = dv;
        }
    };
    const uint32_t tmem = cta_setup(&tmem_slot, &mbar, 1, kTmemCols);
    Sync s{&mbar, 0u, true, 1u};
    stage(split, 0);
    uint32_t buf = 0;
    bool first = true;
    for (uint32_t tile = split; tile < tiles && s.ok; tile += p.splits) {
        gemm_issue(s, tmem, smem + buf * kWgA, smem + 2 * kWgA + buf * kWgB, 128, out_n, true, !first, true);
        // the other buffer's MMAs completed in the previous round
        if (tile + p.splits < tiles) stage(tile + p.splits, buf ^ 1u);
        gemm_wait(s);
        first = false;
        buf ^= 1u;
    }
    if (s.ok && !first) {
        float v[kHidden];
        read_row(tmem, out_n, v);
        if (t < in_n) {
            float* g = p.grads + rc_layer_offset(l);
            for (uint32_t o = 0; o < out_n; ++o) atomicAdd(&g[(size_t)o * rc_layer_in(l) + in_base + t], v[o]);
        }
    }
    cta_teardown(s, tmem, kTmemCols, p.status);
}

// ---- Adam and the operand copies ------------------------------------------------------
// One thread per weight w = (layer l, output o, input i): Adam on the FP32
// master copy (padded output rows 3..15 stay zero), then the FP16 forward
// operand (row o, column i of W(l)) and, for layers 2..6, the BF16 backward
// operand (row i, column o).  Clears the gradient for the next step.
__global__ void rc_adam(RcAdam p) {
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= kWeightCount) return;
    int l = 0;
    while (l < kLayers - 1 && w >= rc_layer_offset(l + 1)) ++l;
    const uint32_t local = w - rc_layer_offset(l);
    const uint32_t in_n = rc_layer_in(l), out_n = rc_layer_out(l);
    const uint32_t o = local / in_n, i = local % in_n;
    const bool real = o < (l == kLayers - 1 ? (uint32_t)kOutputs : out_n);
    float val = real ? p.params[w] : 0.0f;
    if (p.step > 0 && real) {
        const float g = p.grads[w] * p.grad_scale;
        const float m = p.beta1 * p.m[w] + (1.0f - p.beta1) * g;
        const float v = p.beta2 * p.v[w] + (1.0f - p.beta2) * g * g;
        p.m[w] = m;
        p.v[w] = v;
        const float mh = m / (1.0f - p.beta1_pow), vh = v / (1.0f - p.beta2_pow);
        val -= p.lr * mh / (sqrtf(vh) + p.eps);
        p.params[w] = val;
    }
    p.grads[w] = 0.0f;
    *(uint16_t*)((unsigned char*)p.weights_f16 + rc_layer_offset(l) * 2 + tc::kmajor_offset(o, i, in_n)) = f2h(val);
    if (l >= 1)
        *(uint16_t*)((unsigned char*)p.weights_bf16 + bwd_offset(l) * 2 + tc::kmajor_offset(i, o, out_n)) = f2b(val);
}

}  // namespace rc

// ---- launchers ---------------------------------------------------------------------------
namespace {
template <class K>
cudaError_t allow_smem(K kernel, uint32_t bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}
}  // namespace

cudaError_t rc_launch_forward(const RcForward& p, bool train, int grid, cudaStream_t s) {
    cudaError_t e = train ? allow_smem(rc::rc_forward<true>, rc::kForwardSmem)
                          : allow_smem(rc::rc_forward<false>, rc::kForwardSmem);
    if (e != cudaSuccess) return e;
    if (train) rc::rc_forward<true><<<grid, 128 * rc::kFwdGroups, rc::kForwardSmem, s>>>(p);
    else rc::rc_forward<false><<<grid, 128 * rc::kFwdGroups, rc::kForwardSmem, s>>>(p);
    return cudaGetLastError();
}

cudaError_t rc_launch_backward(const RcBackward& p, int grid, cudaStream_t s) {
    cudaError_t e = allow_smem(rc::rc_backward, rc::kBackwardSmem);
    if (e != cudaSuccess) return e;
    rc::rc_backward<<<grid, 128, rc::kBackwardSmem, s>>>(p);
    return cudaGetLastError();
}

cudaError_t rc_launch_wgrad(const RcWgrad& p, cudaStream_t s) {
    cudaError_t e = allow_smem(rc::rc_wgrad, rc::kWgradSmem);
    if (e != cudaSuccess) return e;
    rc::rc_wgrad<<<kWgradJobs * p.splits, 128, rc::kWgradSmem, s>>>(p);
    return cudaGetLastError();
}

cudaError_t rc_launch_adam(const RcAdam& p, cudaStream_t s) {
    rc::rc_adam<<<(kWeightCount + 255) / 256, 256, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace orn
