// pt_kernels.h — launch interface between the host C ABI (capi.cu) and the
// kernel translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ornament_cuda.h"

#include "pt_scene.h"

namespace orn {

// Threads per megakernel block (measured on the 1080p workload: 96 threads
// x 7 blocks, 21 warps per SM, 341 against 364 Msamples/s for 128 x 5).
#ifndef ORN_MEGA_BLOCK
#define ORN_MEGA_BLOCK 128
#endif
constexpr int kMegaBlock = ORN_MEGA_BLOCK;
// Traversal-stack entries per thread kept in shared memory (the rest of the
// 64-entry stack spills to local memory).
#ifndef ORN_SMEM_STACK
#define ORN_SMEM_STACK 32
#endif
constexpr int kSmemStack = ORN_SMEM_STACK;
// Resident blocks per SM the megakernel is compiled for (register cap).
// Measured on the 1080p workload (same box): 5 blocks 353, 6 blocks 335,
// 7 blocks 309 Msamples/s — fewer register spills outweigh fewer warps.
#ifndef ORN_MEGA_MIN_BLOCKS
#define ORN_MEGA_MIN_BLOCKS 5
#endif
constexpr int kMegaMinBlocks = ORN_MEGA_MIN_BLOCKS;

// Radiance-cache side of a cached megakernel launch.  Every pixel traces one
// sample, with next-event estimation: at a lambertian vertex whose scattered
// ray will be traced, a point on an emissive mesh triangle is sampled by area
// and connected by a shadow ray; the light sample and a scattered ray from
// that vertex that hits one of those emitters are combined with the balance
// heuristic against the density of the reference's own scatter direction
// (not a cosine lobe: its in_unit_sphere draws the polar angle uniformly,
// material.hip.h / random.hip.h).  The estimate keeps the reference's
// expectation, including its depth-limit term.
//
// The path's cache vertex is its first rough surface hit (lambertian, or
// metal with fuzz >= kCacheMinFuzz) from the second vertex on.  The network
// predicts the radiance leaving that vertex through its scattered ray (the
// light sample there stays explicit), divided by the surface colour a
// (clamped to >= 1e-3) so texture detail is not left to the network.  A
// regular pixel takes its light sample at the cache vertex, appends a query
// (pixel, network inputs, throughput x a) to the query queue and ends; the
// inference pass adds throughput x a x cache(inputs) afterwards.  Pixels of
// the training groups (one warp-sized group of 32 pixels in 2^train_shift,
// rotating with `frame`) trace the full path instead, record the network
// inputs at the cache vertex and, at the end of the path, the radiance
// gathered after the cache vertex's scatter divided by a (the training
// target) in their training slot.
constexpr int kCacheInputs = 10;   // position 3, direction 3, normal 3, roughness 1
constexpr float kCacheMinFuzz = 0.25f;   // metals below this fuzz are not cache vertices

struct CacheLaunch {
    uint32_t frame;            // the cache's frame counter (training decisions)
    float lo[3];               // scene bounds: position inputs are (p - lo) * inv_extent
    float inv_extent[3];
    uint32_t* query_count;     // zeroed before the launch
    uint32_t* query_pixel;
    float* query_in;           // [pixels][10]
    float4* query_thr;
    float* train_in;           // [slots][10]
    float* train_target;       // [slots][3]; x = -1 when the path had no cache vertex
    uint32_t train_slots;      // capacity (all streams)
    // training paths are chosen at the cache vertex: a path that reaches one
    // trains with probability min(1, train_slots / *vertices_prev) (the
    // previous frame's count of cache vertices) and takes the next free slot
    // of its lane's shard (train_count[lane] counts slots taken from
    // [shard * train_slots / 32, (shard + 1) * train_slots / 32)); *vertices
    // counts this frame's vertices
    uint32_t* train_count;     // [32], zeroed before the launch
    uint32_t* vertices;        // zeroed before the launch
    const uint32_t* vertices_prev;
    // next-event estimation: emissive mesh triangles, 4 float4 each (v0, e1,
    // e2 with the emission in .w; the emitter's inverse-transform id in the
    // x bits of the fourth), their cumulative areas, and a flag per material
    // whose mesh emitters are in the list
    uint32_t light_count;
    float light_area;
    const float4* lights;
    const float* light_cdf;
    const uint32_t* light_material;
    // sample streams per pixel in this launch: stream 0 continues the pixel's
    // own RNG state, stream s > 0 its own state in rng_extra[(s-1) * pixels +
    // pixel]; with more than one the samples are added to the accumulation
    // atomically (the host zeroes it first).
    uint32_t streams;
    uint32_t* rng_extra;
    uint32_t sobol;            // ORN_SAMPLER_SOBOL: pixel, lens, first bounce and light from qmc.cuh
};

// Training samples a cached frame collects per sample stream: one per
// 2^shift pixels, in whole groups of 32.
__host__ __device__ __forceinline__ uint32_t cache_train_slots(uint32_t pixels, uint32_t shift) {
    return ((pixels + (32u << shift) - 1u) >> (5 + shift)) * 32u;
}

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
    CacheLaunch cache;         // cached launches only
    const uint32_t* order;     // hand-out order of the pixels (null: raster order)
    uint32_t* cost;            // per-pixel traversal steps of this launch (or null)
    int wave_fetch;            // wavefront kernels: idle lanes a traversing warp gathers before taking rays
};

// Launch parameters of the persistent wavefront (wave.cu): one of the
// compiled block shapes (warps per block, of which shading, path slots per
// block, resident blocks per SM — see wave_shape_info), the idle lanes a
// traversing warp gathers before it takes new rays, and the node visits per
// traversal round (compiled for 32 and 64).  Every configuration renders
// the same images; only the speed differs.
struct WaveConfig {
    int shape;
    int fetch;
    int steps;
};
constexpr int kWaveShapes = 4;
constexpr WaveConfig kWaveDefault = {0, 4, 32};
// The cached wavefront (wave_cached.cu) has one shape and round length and
// takes this fetch threshold.
constexpr int kWaveFetchDefault = 4, kWaveStepsDefault = 32;
__host__ __device__ constexpr bool wave_config_valid(int shape, int fetch, int steps) {
    return shape >= 0 && shape < kWaveShapes && fetch >= 1 && fetch <= 32 && (steps == 32 || steps == 64);
}
// Warps, shading warps, path slots per block and resident blocks per SM of
// compiled shape `shape` (false when there is none).
bool wave_shape_info(int shape, int* warps, int* shading, int* slots, int* blocks_per_sm);

// What orn_render_noalloc (noalloc.cu) takes from a context (capi.cu keeps
// the context type private): its scene, device and semantics, whether the
// FMNMX slab test may be used with the call's camera, the device error word,
// a pinned host copy of it that each call queues after its work, the event
// recorded after that copy, and whether such a copy is outstanding.
struct NoAllocLink {
    const SceneDev* scene;
    int device;
    uint32_t semantics;
    bool fast_slabs;
    uint32_t* error_word;
    uint32_t* host_error;
    cudaEvent_t* done;
    bool* pending;
};

// Longest-first pixel order (order.cu): from the per-pixel costs of one
// launch, the hand-out order of the next (tiles of 32 pixels by decreasing
// summed cost).  Buffers: keys/vals/keys2/vals2 one entry per tile, `temp`
// of order_temp_bytes.
struct PixelOrder {
    const uint32_t* cost;
    uint32_t pixels;
    uint32_t* keys;
    uint32_t* vals;
    uint32_t* keys2;
    uint32_t* vals2;
    void* temp;
    size_t temp_bytes;
    uint32_t* order;
};
uint32_t order_tiles(uint32_t pixels);
cudaError_t order_temp_bytes(uint32_t pixels, size_t* bytes);
cudaError_t launch_pixel_order(const PixelOrder& o, cudaStream_t s);

#ifndef ORN_SHADE_THRESHOLD
#define ORN_SHADE_THRESHOLD 8
#endif
constexpr int kShadeThreshold = ORN_SHADE_THRESHOLD;
// the cached kernel's (its shading step is several times longer); measured
// on cached + batched 1920x1080 frames at 7 blocks per SM (ms per frame):
// 8 lanes 62.7, 16 54.9, 24 52.6, 28 53.6, 32 58.9
#ifndef ORN_CACHE_SHADE_THRESHOLD
#define ORN_CACHE_SHADE_THRESHOLD 24
#endif
constexpr int kCacheShadeThreshold = ORN_CACHE_SHADE_THRESHOLD;
// BVH node visits a traversing lane makes per pass of the megakernel's loop
// (amortises the loop's ballots).
#ifndef ORN_STEPS_PER_ITERATION
#define ORN_STEPS_PER_ITERATION 32
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
// Cached frame launch (one sample per pixel and stream, see CacheLaunch), on
// the megakernel or the persistent wavefront (wave_cached.cu).
cudaError_t launch_mega_cached(const RenderLaunch& p, int semantics, bool fast, cudaStream_t s);
cudaError_t launch_wave_cached(const RenderLaunch& p, int semantics, bool fast, cudaStream_t s);
cudaError_t launch_mega_f64(const RenderLaunch& p, int semantics, bool fast, cudaStream_t s);
// relMSE = mean over pixels and RGB of (x - r)^2 / (r^2 + 1e-2), with x the
// per-pixel mean of `acc` (FP32 RGBA sums, or FP64 when acc64) and r of
// `ref64`; the sum goes to out[0] and the number of skipped (non-finite)
// pixels to out[1], both FP64 and zeroed by the caller.
cudaError_t launch_relmse(const float4* acc, const double* acc64, const double* ref64, uint32_t n,
                          double* out, cudaStream_t s);
// The persistent wavefront (wave.cu): one launch renders p.spp passes of
// every pixel, like launch_mega.
cudaError_t launch_wave(const RenderLaunch& p, const WaveConfig& c, int semantics, bool count, bool fast,
                        cudaStream_t s);
cudaError_t launch_wf_logic(const WaveLaunch& p, uint32_t iter, int semantics, int math, bool count,
                            cudaStream_t s);
cudaError_t launch_wf_extend(const WaveLaunch& p, uint32_t iter, bool count, bool fast, cudaStream_t s);
cudaError_t launch_trace_rays(const SceneDev& sc, float t_min, const float* rays, size_t count,
                              orn_hit* hits, uint32_t* visits, uint32_t* error, cudaStream_t s);
cudaError_t launch_seed_rng(uint32_t* rng, uint32_t n, cudaStream_t s, uint32_t first = 0);   // rng[i] = first + i
cudaError_t launch_post(const float4* acc, float4* fb, uint32_t W, uint32_t H, uint32_t flip_y,
                        float ci, float inv_gamma, int semantics, int math, cudaStream_t s);

}  // namespace orn
