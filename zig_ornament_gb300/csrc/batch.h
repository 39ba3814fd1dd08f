// batch.h — the batched persistent renderer (batch.cu): many contexts, one
// launch.  Shared between batch.cu and capi.cu (which owns orn_context).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ornament_cuda.h"
#include "pt_scene.h"

namespace orn {

constexpr uint32_t kMaxBatch = 64;   // scenes per launch (their views live in shared memory)

// One context's part of a batched frame: what orn_render would launch for
// it (all of this render()'s passes in one go).
struct BatchView {
    SceneDev scene;
    orn_constant_params cp;    // current_iteration = first pass of the frame
    uint32_t spp;              // passes this frame
    uint32_t pixel_begin;      // first pixel of this context in the frame's pixel space
    float4* acc;
    float4* fb;
    uint32_t* rng;
};

// Does the host side of orn_render for `ctx` (checks, targets, camera-dirty
// restart, current_iteration bookkeeping) and fills `view`; the batch stream
// is ordered after the context's queued work.  Returns an ORN_* status.
// With commit = false the context is left as it was (the autotuner's
// scratch frames).
int batch_prepare(orn_context* ctx, BatchView* view, bool* fast_slabs, uint32_t* semantics, int* device,
                  cudaStream_t batch_stream, bool commit);
// Orders the context's later work after `done` (recorded on the batch stream).
int batch_finish(orn_context* ctx, cudaEvent_t done);

struct BatchConfig {
    int block;           // 64, 128 or 192 threads
    int blocks_per_sm;   // resident blocks per SM the grid is sized for
    int shade_threshold; // ready lanes needed before a warp shades
};

// Launches one batched frame (views already in device memory).
cudaError_t launch_batch(const BatchView* views, uint32_t nviews, uint32_t total_pixels, uint32_t* work_counter,
                         uint32_t* error, int semantics, bool fast, const BatchConfig& cfg, cudaStream_t s);
// The largest resident block count per SM for a block size (0 if unknown).
int batch_max_blocks_per_sm(int block, int semantics, bool fast);

}  // namespace orn
