// megakernel.cu — the plain sm_103a megakernel and its helpers.
//
// One thread owns one pixel and runs that pixel's sample passes in order
// inside the thread, keeping the FP32 accumulation in registers.  The
// reference launches one grid per pass (path_tracing_kernal,
// src/hip_backend/kernels/pathtracer.hip.cpp:30-42, driven by
// src/hip_backend/path_tracer.zig:121-133); because passes of different
// pixels never interact and a pixel's RNG state and accumulation are carried
// from pass to pass, running a pixel's passes back to back in one thread
// produces the same bits with one launch instead of `iterations` launches and
// without the per-pass accumulation/RNG round trips through HBM.  The last
// launch of a render applies post_processing (pathtracer.hip.cpp:58-70).
#include <cuda_fp16.h>

#include "pt_kernels.h"
#include "pt_device.cuh"
#include "pt_machine.cuh"

namespace orn {

enum LaneMode { LANE_IDLE = 0, LANE_TRAVERSE = 1, LANE_SHADE = 2, LANE_DONE = 3 };

// The render kernel: persistent threads, one path per lane, run as a
// warp-synchronous state machine (pt_machine.cuh).  Pixels are handed out
// 32 at a time from p.work_counter; each pixel runs its p.spp passes with the
// accumulation and RNG state in registers, then writes them back (and the
// post-processed framebuffer value when p.do_post).
template <int SEM, int MATH, bool COUNT, bool FAST>
__global__ void __launch_bounds__(kMegaBlock, kMegaMinBlocks)
mega_kernel(RenderLaunch p) {
    __shared__ uint32_t sstack[kSmemStack * kMegaBlock];
    TravStack<kSmemStack> stack;
    stack.sstack = sstack + threadIdx.x;
    stack.sstride = kMegaBlock;
    const unsigned kFull = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lanes_below = (1u << lane) - 1u;
    const uint32_t W = p.cp.width, H = p.cp.height;
    const float ci0 = p.cp.current_iteration;

    int mode = LANE_IDLE;
    bool exhausted = false;          // warp-uniform: the pixel counter ran out
    uint32_t gid = 0, k = 0, bounce = 0;
    Rng rng{0};
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    f3 ro = mk(0.0f, 0.0f, 0.0f), rd = ro, color = ro;
    HitRec h;
    h.t = 0.0f; h.material = 0; h.type = 0; h.inv = 0; h.tri = 0; h.u = 0.0f; h.v = 0.0f;
    Walker w;
    VisitCount vc = {0, 0, 0, 0, 0};
    SampleCount scn = {0, 0, 0, 0};
    uint32_t err = 0;

    // Starts sample k of the current pixel; returns the lane's next mode.
    // Samples with depth 0 finish immediately (the bounce loop never runs).
    auto start_samples = [&]() -> int {
        while (k < p.spp) {
            camera_ray<MATH>(p.cp, gid % W, gid / W, rng, &ro, &rd);
            color = mk(1.0f, 1.0f, 1.0f);
            bounce = 0;
            if (p.cp.depth > 0) {
                if (COUNT) scn.rays++;
                walker_begin(w, p.scene, ro, rd);
                return LANE_TRAVERSE;
            }
            float ci = ci0 + (float)k;
            if (ci > 1.0f) acc = make_float4(acc.x + color.x, acc.y + color.y, acc.z + color.z, acc.w + 1.0f);
            else acc = make_float4(color.x, color.y, color.z, 1.0f);
            ++k;
        }
        p.acc[gid] = acc;
        p.rng[gid] = rng.state;
        if (p.do_post) {
            uint32_t x = gid % W, y = gid / W;
            uint32_t fbi = p.cp.flip_y != 0 ? W * (H - y - 1) + x : gid;
            p.fb[fbi] = post_process<SEM, MATH>(acc, ci0 + (float)(p.spp - 1), p.cp.inverted_gamma);
        }
        return LANE_IDLE;
    };

    for (;;) {
        // Hand out pixels to idle lanes: one atomic per warp.
        unsigned idle = __ballot_sync(kFull, mode == LANE_IDLE);
        if (idle != 0u && !exhausted) {
            const unsigned leader = __ffs(idle) - 1u;
            const unsigned n = __popc(idle);
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(p.work_counter, n);
            base = __shfl_sync(kFull, base, leader);
            if (base + n >= p.pixel_count) exhausted = true;
            if (mode == LANE_IDLE) {
                uint32_t mine = base + __popc(idle & lanes_below);
                if (mine < p.pixel_count) {
                    gid = mine;
                    rng.state = p.rng[gid];
                    acc = ci0 > 1.0f ? p.acc[gid] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    k = 0;
                    mode = start_samples();
                }
            }
        }
        if (exhausted && mode == LANE_IDLE) mode = LANE_DONE;
        if (__ballot_sync(kFull, mode == LANE_TRAVERSE || mode == LANE_SHADE) == 0u &&
            __ballot_sync(kFull, mode == LANE_IDLE) == 0u)
            break;

        if (mode == LANE_TRAVERSE) {
#pragma unroll 1
            for (int s = 0; s < kStepsPerIteration; ++s) {
                if (!walker_step<COUNT, kSmemStack, FAST>(w, p.scene, ro, rd, p.cp.ray_cast_epsilon, &h, stack, &vc, &err)) {
                    mode = LANE_SHADE;
                    break;
                }
            }
        }

        const unsigned ready = __ballot_sync(kFull, mode == LANE_SHADE);
        const unsigned busy = __ballot_sync(kFull, mode == LANE_TRAVERSE);
        if (ready != 0u && ((int)__popc(ready) >= p.shade_threshold || busy == 0u)) {
            if (mode == LANE_SHADE) {
                bool cont;
                if (!w.any) {
                    if (err) color = mk(0.0f, 0.0f, 0.0f);
                    else color = sky_color(color, rd);
                    cont = false;
                } else {
                    cont = shade_hit<SEM, MATH, COUNT>(p.scene, p.cp, rng, h, &ro, &rd, &color, &scn);
                }
                if (cont && ++bounce < p.cp.depth) {
                    if (COUNT) scn.rays++;
                    walker_begin(w, p.scene, ro, rd);
                    mode = LANE_TRAVERSE;
                } else {
                    float ci = ci0 + (float)k;
                    if (ci > 1.0f) acc = make_float4(acc.x + color.x, acc.y + color.y, acc.z + color.z, acc.w + 1.0f);
                    else acc = make_float4(color.x, color.y, color.z, 1.0f);
                    ++k;
                    mode = start_samples();
                }
            }
        }
        __syncwarp();
    }
    if (err) atomicOr(p.error, err);
    if (COUNT) {
        atomicAdd(p.counters + 1, (unsigned long long)scn.rays);
        atomicAdd(p.counters + 2, (unsigned long long)vc.visits);
        atomicAdd(p.counters + 3, (unsigned long long)vc.internal);
        atomicAdd(p.counters + 4, (unsigned long long)vc.sphere);
        atomicAdd(p.counters + 5, (unsigned long long)vc.mesh);
        atomicAdd(p.counters + 6, (unsigned long long)vc.tri);
        atomicAdd(p.counters + 7, (unsigned long long)scn.sphere_hits);
        atomicAdd(p.counters + 8, (unsigned long long)scn.mesh_hits);
        atomicAdd(p.counters + 9, (unsigned long long)scn.textured);
        if (blockIdx.x == 0 && threadIdx.x == 0)
            atomicAdd(p.counters + 0, (unsigned long long)p.spp * p.pixel_count);
    }
}

// Bvh::hit on a ray list (parity / debugging entry point).
__global__ void __launch_bounds__(128)
trace_rays_kernel(SceneDev sc, float t_min, const float* __restrict__ rays, size_t count,
                  orn_hit* __restrict__ hits, uint32_t* __restrict__ visits, uint32_t* error) {
    __shared__ uint32_t sstack[kSmemStack * 128];
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float* r = rays + 6 * i;
    f3 ro = mk(r[0], r[1], r[2]), rd = mk(r[3], r[4], r[5]);
    HitRec h;
    h.t = 0.0f; h.material = 0; h.type = 0; h.inv = 0; h.tri = 0; h.u = 0.0f; h.v = 0.0f;
    VisitCount vc = {0, 0, 0, 0, 0};
    uint32_t err = 0;
    bool any = trace_ray<true, kSmemStack>(sc, ro, rd, t_min, &h, &vc, &err, sstack + threadIdx.x, 128);
    orn_hit o;
    o.hit = any ? 1u : 0u;
    o.t = any ? h.t : 0.0f;
    o.material_index = any ? h.material : 0u;
    o.node_type = any ? h.type : 0u;
    o.inverted_transform_id = any ? h.inv : 0u;
    bool mesh = any && h.type == ORN_NODE_MESH;
    o.tri_id = mesh ? h.tri : 0u;
    o.uv[0] = mesh ? h.u : 0.0f;
    o.uv[1] = mesh ? h.v : 0.0f;
    hits[i] = o;
    if (visits) visits[i] = vc.visits;
    if (err) atomicOr(error, err);
}

// Reseeds every pixel's RNG state with its pixel index
// (src/hip_backend/buffers.zig:27-31).
__global__ void seed_rng_kernel(uint32_t* rng, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rng[i] = i;
}

// Post-processing alone (post_processing_kernal, pathtracer.hip.cpp:44-56).
template <int SEM, int MATH>
__global__ void post_kernel(const float4* __restrict__ acc, float4* __restrict__ fb,
                            uint32_t W, uint32_t H, uint32_t flip_y, float ci, float inv_gamma) {
    uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= W * H) return;
    uint32_t x = gid % W, y = gid / W;
    uint32_t fbi = flip_y ? W * (H - y - 1) + x : gid;
    fb[fbi] = post_process<SEM, MATH>(acc[gid], ci, inv_gamma);
}

// ---- host-side launchers -----------------------------------------------------
// Persistent grid: as many blocks as fit on the device at once (never more
// than the pixels need).
template <int SEM, int MATH, bool COUNT, bool FAST>
static cudaError_t launch_mega_tt(const RenderLaunch& p, cudaStream_t s) {
    static int blocks_per_sm = 0, sms = 0;
    if (blocks_per_sm == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, mega_kernel<SEM, MATH, COUNT, FAST>, kMegaBlock, 0);
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    uint32_t need = (p.pixel_count + kMegaBlock - 1) / kMegaBlock;
    uint32_t grid = (uint32_t)(blocks_per_sm * sms);
    if (need < grid) grid = need;
    cudaError_t e = cudaMemsetAsync(p.work_counter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    mega_kernel<SEM, MATH, COUNT, FAST><<<grid, kMegaBlock, 0, s>>>(p);
    return cudaGetLastError();
}

template <int SEM>
static cudaError_t launch_mega_t(const RenderLaunch& p, bool count, bool fast, cudaStream_t s) {
    if (fast) return count ? launch_mega_tt<SEM, MATH_PORTABLE, true, true>(p, s)
                           : launch_mega_tt<SEM, MATH_PORTABLE, false, true>(p, s);
    return count ? launch_mega_tt<SEM, MATH_PORTABLE, true, false>(p, s)
                 : launch_mega_tt<SEM, MATH_PORTABLE, false, false>(p, s);
}

// The render kernels always use the portable transcendentals (bit-exact
// with the CPU restatement); `math` is accepted for the launch interface.
cudaError_t launch_mega(const RenderLaunch& p, int semantics, int math, bool count, bool fast, cudaStream_t s) {
    (void)math;
    return semantics == SEM_WGSL ? launch_mega_t<SEM_WGSL>(p, count, fast, s)
                                 : launch_mega_t<SEM_HIP>(p, count, fast, s);
}

cudaError_t launch_trace_rays(const SceneDev& sc, float t_min, const float* rays, size_t count,
                              orn_hit* hits, uint32_t* visits, uint32_t* error, cudaStream_t s) {
    if (count == 0) return cudaSuccess;
    size_t blocks = (count + 127) / 128;
    trace_rays_kernel<<<(unsigned)blocks, 128, 0, s>>>(sc, t_min, rays, count, hits, visits, error);
    return cudaGetLastError();
}

cudaError_t launch_seed_rng(uint32_t* rng, uint32_t n, cudaStream_t s) {
    seed_rng_kernel<<<(n + 255) / 256, 256, 0, s>>>(rng, n);
    return cudaGetLastError();
}

cudaError_t launch_post(const float4* acc, float4* fb, uint32_t W, uint32_t H, uint32_t flip_y,
                        float ci, float inv_gamma, int semantics, int math, cudaStream_t s) {
    uint32_t n = W * H;
    dim3 grid((n + 255) / 256);
    if (semantics == SEM_WGSL) {
        if (math == MATH_DEVICE) post_kernel<SEM_WGSL, MATH_DEVICE><<<grid, 256, 0, s>>>(acc, fb, W, H, flip_y, ci, inv_gamma);
        else post_kernel<SEM_WGSL, MATH_PORTABLE><<<grid, 256, 0, s>>>(acc, fb, W, H, flip_y, ci, inv_gamma);
    } else {
        if (math == MATH_DEVICE) post_kernel<SEM_HIP, MATH_DEVICE><<<grid, 256, 0, s>>>(acc, fb, W, H, flip_y, ci, inv_gamma);
        else post_kernel<SEM_HIP, MATH_PORTABLE><<<grid, 256, 0, s>>>(acc, fb, W, H, flip_y, ci, inv_gamma);
    }
    return cudaGetLastError();
}

}  // namespace orn
