// pt_kernels.h — launch interface between the host C ABI (capi.cu) and the
// kernel translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ornament_cuda.h"

#include "pt_scene.h"

namespace orn {

constexpr int kMegaBlock = 128;
constexpr int kSmemStack = 32;
// Resident blocks per SM the megakernel is compiled for (register cap).
#ifndef ORN_MEGA_MIN_BLOCKS
#define ORN_MEGA_MIN_BLOCKS 6
#endif
constexpr int kMegaMinBlocks = ORN_MEGA_MIN_BLOCKS;   // traversal-stack entries per thread kept in shared memory

// Arguments of one megakernel launch (passed by value).
struct RenderLaunch {
    SceneDev scene;
    orn_constant_params cp;   // current_iteration = first pass of this launch
    uint32_t spp;             // passes in this launch
    uint32_t do_post;         // write the framebuffer after the last pass
    uint32_t pixel_count;
    float4* acc;
    float4* fb;
    uint32_t* rng;
    uint32_t* error;
    unsigned long long* counters;
    uint32_t* work_counter;    // next pixel to hand out (zeroed before each launch)
    double* acc64;             // FP64 accumulation (orn_render_f64 only)
    int shade_threshold;       // ready lanes needed before a warp shades
};

#ifndef ORN_SHADE_THRESHOLD
#define ORN_SHADE_THRESHOLD 8
#endif
constexpr int kShadeThreshold = ORN_SHADE_THRESHOLD;
// BVH node visits a traversing lane makes per pass of the megakernel's loop
// (amortises the loop's ballots).
#ifndef ORN_STEPS_PER_ITERATION
#define ORN_STEPS_PER_ITERATION 8
#endif
constexpr int kStepsPerIteration = ORN_STEPS_PER_ITERATION;

// Arguments of one wavefront iteration (wavefront.cu).  Path slots are
// structure-of-arrays; qstat holds per-iteration [queue count, slots waiting
// for a pixel, queue head, unused] for four iterations in rotation.
struct WaveLaunch {
    SceneDev scene;
    orn_constant_params cp;
    uint32_t spp;
    uint32_t do_post;
    uint32_t pixel_count;
    uint32_t slots;
    float4* acc;
    float4* fb;
    uint32_t* rng;
    uint32_t* error;
    unsigned long long* counters;
    uint32_t* pixel_counter;
    uint32_t* qstat;
    uint32_t* queue;
    uint32_t* mode;
    uint32_t* pixel;
    uint2* kb;
    uint32_t* rng_state;
    float4* accum;
    float4* color;
    float4* ro;
    float4* rd;
    float4* hit;
    int fetch_threshold;
};

#ifndef ORN_FETCH_THRESHOLD
#define ORN_FETCH_THRESHOLD 16
#endif
constexpr int kFetchThreshold = ORN_FETCH_THRESHOLD;

cudaError_t launch_mega(const RenderLaunch& p, int semantics, int math, bool count, bool fast, cudaStream_t s);
cudaError_t launch_mega_f64(const RenderLaunch& p, int semantics, bool fast, cudaStream_t s);
// relMSE = mean over pixels and RGB of (x - r)^2 / (r^2 + 1e-2), with x the
// per-pixel mean of `acc` (FP32 RGBA sums, or FP64 when acc64) and r of
// `ref64`; summed in FP64 into *out (zeroed by the caller).
cudaError_t launch_relmse(const float4* acc, const double* acc64, const double* ref64, uint32_t n,
                          double* out, cudaStream_t s);
cudaError_t launch_wf_logic(const WaveLaunch& p, uint32_t iter, int semantics, int math, bool count,
                            cudaStream_t s);
cudaError_t launch_wf_extend(const WaveLaunch& p, uint32_t iter, bool count, bool fast, cudaStream_t s);
cudaError_t launch_trace_rays(const SceneDev& sc, float t_min, const float* rays, size_t count,
                              orn_hit* hits, uint32_t* visits, uint32_t* error, cudaStream_t s);
cudaError_t launch_seed_rng(uint32_t* rng, uint32_t n, cudaStream_t s);
cudaError_t launch_post(const float4* acc, float4* fb, uint32_t W, uint32_t H, uint32_t flip_y,
                        float ci, float inv_gamma, int semantics, int math, cudaStream_t s);

}  // namespace orn
