// order.cu — longest-first pixel hand-out for the persistent render kernels.
//
// A pixel's passes form a chain (its RNG state carries from one pass to the
// next, src/hip_backend/kernels/pathtracer.hip.cpp:15-56), so a launch has
// exactly pixel_count independent work items.  At low resolutions that is
// only a few per resident lane, and a raster hand-out leaves most lanes idle
// while the last expensive pixels finish.  Each launch therefore records
// every pixel's cost (traversal steps), and the next launch hands pixels out
// by tile of 32 consecutive pixels (one warp's worth, spatially coherent) in
// decreasing order of that cost: the classic longest-processing-time-first
// rule.  Which lane runs a pixel does not change its result.
#include <cub/device/device_radix_sort.cuh>

#include "pt_kernels.h"

namespace orn {
namespace {

constexpr uint32_t kTile = 32;

// One warp per tile: key = ~(summed cost) so that an ascending sort puts the
// costliest tile first; the partial last tile gets the largest key (last).
__global__ void tile_cost_kernel(const uint32_t* __restrict__ cost, uint32_t pixels, uint32_t tiles,
                                 uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    if (t >= tiles) return;   // whole warps leave together (blockDim is a multiple of 32)
    const uint32_t gid = t * kTile + lane;
    uint32_t c = gid < pixels ? cost[gid] : 0u;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) {
        const bool partial = (t + 1) * kTile > pixels;
        keys[t] = partial ? 0xffffffffu : ~min(c, 0xfffffffeu);
        vals[t] = t;
    }
}

__global__ void order_write_kernel(const uint32_t* __restrict__ sorted_tiles, uint32_t pixels,
                                   uint32_t* __restrict__ order) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pixels) return;
    order[i] = sorted_tiles[i / kTile] * kTile + (i % kTile);
}

}  // namespace

uint32_t order_tiles(uint32_t pixels) { return (pixels + kTile - 1) / kTile; }

cudaError_t order_temp_bytes(uint32_t pixels, size_t* bytes) {
    const int tiles = (int)order_tiles(pixels);
    return cub::DeviceRadixSort::SortPairs(nullptr, *bytes, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                           (const uint32_t*)nullptr, (uint32_t*)nullptr, tiles, 0, 32);
}

cudaError_t launch_pixel_order(const PixelOrder& o, cudaStream_t s) {
    const uint32_t tiles = order_tiles(o.pixels);
    tile_cost_kernel<<<(tiles * 32 + 255) / 256, 256, 0, s>>>(o.cost, o.pixels, tiles, o.keys, o.vals);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    size_t bytes = o.temp_bytes;
    e = cub::DeviceRadixSort::SortPairs(o.temp, bytes, o.keys, o.keys2, o.vals, o.vals2, (int)tiles, 0, 32, s);
    if (e != cudaSuccess) return e;
    order_write_kernel<<<(o.pixels + 255) / 256, 256, 0, s>>>(o.vals2, o.pixels, o.order);
    return cudaGetLastError();
}

}  // namespace orn
