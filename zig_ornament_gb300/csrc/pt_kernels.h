// pt_kernels.h — launch interface between the host C ABI (capi.cu) and the
// kernel translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ornament_cuda.h"

#include "pt_scene.h"

namespace orn {

constexpr int kMegaBlock = 128;

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
};

cudaError_t launch_mega(const RenderLaunch& p, int semantics, int math, bool count, cudaStream_t s);
cudaError_t launch_trace_rays(const SceneDev& sc, float t_min, const float* rays, size_t count,
                              orn_hit* hits, uint32_t* visits, uint32_t* error, cudaStream_t s);
cudaError_t launch_seed_rng(uint32_t* rng, uint32_t n, cudaStream_t s);
cudaError_t launch_post(const float4* acc, float4* fb, uint32_t W, uint32_t H, uint32_t flip_y,
                        float ci, float inv_gamma, int semantics, int math, cudaStream_t s);

}  // namespace orn
