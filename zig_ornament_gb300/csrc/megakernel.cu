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

namespace orn {

template <int SEM, int MATH, bool COUNT>
__global__ void __launch_bounds__(kMegaBlock)
mega_kernel(RenderLaunch p) {
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= p.pixel_count) return;
    const uint32_t W = p.cp.width, H = p.cp.height;
    const uint32_t x = gid % W, y = gid / W;
    Rng rng{p.rng[gid]};
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (p.cp.current_iteration > 1.0f) acc = p.acc[gid];
    VisitCount vc = {0, 0, 0, 0, 0};
    SampleCount scn = {0, 0, 0, 0};
    uint32_t err = 0;
    float ci = p.cp.current_iteration;
    for (uint32_t k = 0; k < p.spp; ++k) {
        ci = p.cp.current_iteration + (float)k;
        f3 c = trace_sample<SEM, MATH, COUNT>(p.scene, p.cp, x, y, rng, &vc, &scn, &err);
        if (ci > 1.0f) acc = make_float4(acc.x + c.x, acc.y + c.y, acc.z + c.z, acc.w + 1.0f);
        else acc = make_float4(c.x, c.y, c.z, 1.0f);
    }
    p.acc[gid] = acc;
    p.rng[gid] = rng.state;
    if (p.do_post) {
        uint32_t fbi = gid;
        if (p.cp.flip_y != 0) fbi = W * (H - y - 1) + x;
        p.fb[fbi] = post_process<SEM, MATH>(acc, ci, p.cp.inverted_gamma);
    }
    if (err) atomicOr(p.error, err);
    if (COUNT) {
        atomicAdd(p.counters + 0, (unsigned long long)p.spp);
        atomicAdd(p.counters + 1, (unsigned long long)scn.rays);
        atomicAdd(p.counters + 2, (unsigned long long)vc.visits);
        atomicAdd(p.counters + 3, (unsigned long long)vc.internal);
        atomicAdd(p.counters + 4, (unsigned long long)vc.sphere);
        atomicAdd(p.counters + 5, (unsigned long long)vc.mesh);
        atomicAdd(p.counters + 6, (unsigned long long)vc.tri);
        atomicAdd(p.counters + 7, (unsigned long long)scn.sphere_hits);
        atomicAdd(p.counters + 8, (unsigned long long)scn.mesh_hits);
        atomicAdd(p.counters + 9, (unsigned long long)scn.textured);
    }
}

// Bvh::hit on a ray list (parity / debugging entry point).
__global__ void __launch_bounds__(128)
trace_rays_kernel(SceneDev sc, float t_min, const float* __restrict__ rays, size_t count,
                  orn_hit* __restrict__ hits, uint32_t* __restrict__ visits, uint32_t* error) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float* r = rays + 6 * i;
    f3 ro = mk(r[0], r[1], r[2]), rd = mk(r[3], r[4], r[5]);
    HitRec h;
    h.t = 0.0f; h.material = 0; h.type = 0; h.inv = 0; h.tri = 0; h.u = 0.0f; h.v = 0.0f;
    VisitCount vc = {0, 0, 0, 0, 0};
    uint32_t err = 0;
    bool any = trace_ray<true>(sc, ro, rd, t_min, &h, &vc, &err);
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
template <int SEM, int MATH>
static cudaError_t launch_mega_t(const RenderLaunch& p, bool count, cudaStream_t s) {
    dim3 grid((p.pixel_count + kMegaBlock - 1) / kMegaBlock);
    if (count) mega_kernel<SEM, MATH, true><<<grid, kMegaBlock, 0, s>>>(p);
    else mega_kernel<SEM, MATH, false><<<grid, kMegaBlock, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_mega(const RenderLaunch& p, int semantics, int math, bool count, cudaStream_t s) {
    if (semantics == SEM_WGSL) {
        return math == MATH_DEVICE ? launch_mega_t<SEM_WGSL, MATH_DEVICE>(p, count, s)
                                   : launch_mega_t<SEM_WGSL, MATH_PORTABLE>(p, count, s);
    }
    return math == MATH_DEVICE ? launch_mega_t<SEM_HIP, MATH_DEVICE>(p, count, s)
                               : launch_mega_t<SEM_HIP, MATH_PORTABLE>(p, count, s);
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
