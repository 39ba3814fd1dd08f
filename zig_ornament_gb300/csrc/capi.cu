// capi.cu — host side of libornament_cuda: the C ABI declared in
// include/ornament_cuda.h.
//
// A context mirrors the HIP backend's PathTracer
// (src/hip_backend/path_tracer.zig:12-236): it owns the device copy of the
// scene arrays, the lazily created target buffers (framebuffer,
// accumulation, per-pixel RNG state), the State fields and the camera with
// its dirty flag.  render() follows PathTracer.render/update (:121-168):
// a dirty camera resets current_iteration, each of the `iterations` passes
// advances it by one, and post-processing uses the last value.  The passes
// are issued as one or more megakernel launches on the context's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "ornament_cuda.h"
#include "qmc.cuh"
#include "pt_kernels.h"
#include "batch.h"
#include "rc_host.h"
#include "tune_cache.h"

using orn::RenderLaunch;
using orn::SceneDev;
using orn::TexDesc;

struct orn_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    std::vector<void*> scene_allocs;
    SceneDev scene{};
    uint32_t scene_textures_count = 0;
    uint32_t tlas_len = 0, blas_len = 0;
    double world_extent = 0.0;        // largest |coordinate| of the TLAS bounds
    double max_inverse_entry = 0.0;   // largest |entry| of the inverse transforms
    float scene_lo[3] = {0.0f, 0.0f, 0.0f}, scene_hi[3] = {0.0f, 0.0f, 0.0f};   // TLAS bounds

    orn_state state{};
    orn_camera camera{};
    bool camera_set = false;
    bool camera_dirty = true;
    float current_iteration = 0.0f;

    uint32_t width = 500, height = 500;   // State.init resolution
    bool target_valid = false;
    float4* acc = nullptr;
    float4* fb = nullptr;
    uint32_t* rng = nullptr;
    // longest-first pixel order (order.cu): per-pixel costs of the last
    // launch, the order derived from them, and the sort's buffers
    uint32_t* px_cost = nullptr;
    uint32_t* px_order = nullptr;
    uint32_t* tile_buf = nullptr;     // 4 arrays of one entry per tile
    void* sort_temp = nullptr;
    size_t sort_temp_bytes = 0;
    bool order_valid = false;

    uint32_t* d_error = nullptr;
    uint32_t* d_work = nullptr;
    // orn_render_noalloc's report of device-side errors without waiting: a
    // pinned copy of d_error queued after its work, the event recorded after
    // that copy, and whether a copy is outstanding (mutable: that entry point
    // takes a const context)
    mutable uint32_t* na_host_error = nullptr;
    mutable cudaEvent_t na_done = nullptr;
    mutable bool na_pending = false;
    unsigned long long* d_counters = nullptr;
    bool counters_enabled = false;
    bool rendered = false;
    uint64_t launches = 0;
    std::string last_error;
    // radiance cache (ORN_KERNEL_CACHED): the attached cache, the query queue
    // (one entry per pixel at most) and the training slots
    orn_cache* cache = nullptr;
    uint32_t cq_pixels = 0, cq_slots = 0, cq_shift = 0, cq_streams = 0;
    uint32_t* rng_extra = nullptr;    // RNG states of sample streams 1.. of cached frames
    uint32_t* cq_count = nullptr;
    uint32_t* cv_counters = nullptr;  // [32 training-slot shards, cache vertices (two frames, alternating)]
    uint32_t cv_flip = 0;
    uint32_t* cq_pixel = nullptr;
    float* cq_in = nullptr;
    float4* cq_thr = nullptr;
    float* ct_in = nullptr;
    float* ct_target = nullptr;
    // emitters the cached renderer samples directly (build_lights)
    uint32_t light_count = 0;
    float light_area = 0.0f;
    const float4* d_lights = nullptr;
    const float* d_light_cdf = nullptr;
    const uint32_t* d_light_material = nullptr;
    // launch parameters of the persistent wavefront (ORN_KERNEL_WAVEFRONT),
    // set by orn_wave_set_config or orn_wave_tune
    orn::WaveConfig wave_cfg = orn::kWaveDefault;
    bool wave_tuned = false;
};

namespace {

int fail(orn_context* ctx, int status, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return status;
}

int cuda_fail(orn_context* ctx, cudaError_t e, const char* what) {
    std::string msg = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) return fail(ctx, ORN_ERR_OUT_OF_MEMORY, msg);
    if (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice || e == cudaErrorInsufficientDriver)
        return fail(ctx, ORN_ERR_NO_DEVICE, msg);
    return fail(ctx, ORN_ERR_CUDA, msg);
}

#define ORN_CUDA(ctx, call)                                         \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call);  \
    } while (0)

orn_state default_state() {
    orn_state s;
    std::memset(&s, 0, sizeof(s));
    s.depth = 10;
    s.flip_y = 0;
    s.inverted_gamma = 1.0f;
    s.iterations = 1;
    s.ray_cast_epsilon = 0.001f;
    s.semantics = ORN_SEMANTICS_HIP;
    s.kernel = ORN_KERNEL_MEGA;
    s.spp_per_launch = 0;
    return s;
}

// Blob validation: every index the kernels follow must be in range, and
// internal nodes must point at lower ids (children are appended before
// their parent in src/bvh.zig), which rules out cycles.
int validate_blob(orn_context* ctx, const orn_scene_blob* b) {
    if (!b) return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "blob is NULL");
    if (b->tlas_nodes_len == 0 || !b->tlas_nodes)
        return fail(ctx, ORN_ERR_EMPTY_SCENE, "scene cannot be empty (no TLAS nodes)");
    if ((b->blas_nodes_len && !b->blas_nodes) || (b->normals_len && !b->normals) ||
        (b->normal_indices_len && !b->normal_indices) || (b->uvs_len && !b->uvs) ||
        (b->uv_indices_len && !b->uv_indices) || (b->transforms_len && !b->transforms) ||
        (b->materials_len && !b->materials) || (b->textures_len && !b->textures))
        return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "blob array pointer is NULL with nonzero length");
    if ((uint64_t)b->tlas_nodes_len + b->blas_nodes_len > 0x3FFFFFFFull)
        return fail(ctx, ORN_ERR_BAD_SCENE, "too many nodes (at most 2^30)");
    for (uint32_t i = 0; i < b->tlas_nodes_len; ++i) {
        const orn_bvh_node& n = b->tlas_nodes[i];
        switch (n.node_type) {
            case ORN_NODE_INTERNAL:
                if (n.left_or_custom_id >= i || n.right_or_material_index >= i)
                    return fail(ctx, ORN_ERR_BAD_SCENE, "TLAS internal node child out of range");
                break;
            case ORN_NODE_SPHERE:
            case ORN_NODE_MESH:
                if ((uint64_t)n.transform_id * 2 + 1 >= b->transforms_len)
                    return fail(ctx, ORN_ERR_BAD_SCENE, "TLAS leaf transform_id out of range");
                if (n.right_or_material_index >= b->materials_len)
                    return fail(ctx, ORN_ERR_BAD_SCENE, "TLAS leaf material out of range");
                if (n.node_type == ORN_NODE_MESH && n.left_or_custom_id >= b->blas_nodes_len)
                    return fail(ctx, ORN_ERR_BAD_SCENE, "mesh leaf BLAS root out of range");
                break;
            default:
                return fail(ctx, ORN_ERR_BAD_SCENE, "invalid TLAS node type");
        }
    }
    for (uint32_t i = 0; i < b->blas_nodes_len; ++i) {
        const orn_bvh_node& n = b->blas_nodes[i];
        if (n.node_type == ORN_NODE_INTERNAL) {
            if (n.left_or_custom_id >= i || n.right_or_material_index >= i)
                return fail(ctx, ORN_ERR_BAD_SCENE, "BLAS internal node child out of range");
        } else if (n.node_type == ORN_NODE_TRIANGLE) {
            uint64_t last = (uint64_t)n.left_or_custom_id * 3 + 2;
            if (last >= b->normal_indices_len || last >= b->uv_indices_len)
                return fail(ctx, ORN_ERR_BAD_SCENE, "triangle id out of range of the index arrays");
        } else {
            return fail(ctx, ORN_ERR_BAD_SCENE, "invalid BLAS node type");
        }
    }
    for (uint32_t i = 0; i < b->normal_indices_len; ++i)
        if (b->normal_indices[i] >= b->normals_len)
            return fail(ctx, ORN_ERR_BAD_SCENE, "normal index out of range");
    for (uint32_t i = 0; i < b->uv_indices_len; ++i)
        if (b->uv_indices[i] >= b->uvs_len) return fail(ctx, ORN_ERR_BAD_SCENE, "uv index out of range");
    for (uint32_t i = 0; i < b->textures_len; ++i) {
        const orn_texture& t = b->textures[i];
        uint32_t texel = t.format == ORN_TEXEL_RGBA8 ? 4u : 8u;
        if (!t.data || t.width == 0 || t.height == 0 || t.format > ORN_TEXEL_RGBA16F ||
            t.bytes_per_row < t.width * texel)
            return fail(ctx, ORN_ERR_BAD_SCENE, "invalid texture");
    }
    return ORN_OK;
}

template <typename T>
int upload(orn_context* ctx, const T* host, size_t count, T** dev) {
    *dev = nullptr;
    size_t bytes = std::max<size_t>(count * sizeof(T), 16);
    void* p = nullptr;
    ORN_CUDA(ctx, cudaMalloc(&p, bytes));
    ctx->scene_allocs.push_back(p);
    if (count) ORN_CUDA(ctx, cudaMemcpy(p, host, count * sizeof(T), cudaMemcpyHostToDevice));
    *dev = (T*)p;
    return ORN_OK;
}

// Light list of the cached renderer's next-event estimation: every triangle
// of every mesh leaf of the TLAS whose material is an untextured diffuse
// light, in world space (object vertices times the leaf's forward transform,
// the second matrix of its pair), as (v0, e1 = v1 - v0, e2 = v2 - v0) with
// the emission in the .w components and the leaf's inverse-transform id
// (what a hit on it records), plus the cumulative areas and a flag per
// material (1 = its mesh emitters are in the list).
int build_lights(orn_context* ctx, const orn_scene_blob* b) {
    std::vector<uint32_t> flag(std::max<uint32_t>(b->materials_len, 1u), 0u);
    auto nee_material = [&](uint32_t m) {
        if (m >= b->materials_len) return false;
        const orn_material& mat = b->materials[m];
        return mat.type == ORN_DIFFUSE_LIGHT && mat.albedo_texture_index >= b->textures_len;
    };
    std::vector<float4> tris;
    std::vector<float> cdf;
    double total = 0.0;
    for (uint32_t i = 0; i < b->tlas_nodes_len; ++i) {
        const orn_bvh_node& leaf = b->tlas_nodes[i];
        if (leaf.node_type != ORN_NODE_MESH || !nee_material(leaf.right_or_material_index)) continue;
        const uint32_t mid = leaf.right_or_material_index;
        flag[mid] = 1u;
        const size_t fid = (size_t)leaf.transform_id * 2 + 1;
        if (fid >= b->transforms_len) continue;
        const float* F = b->transforms + fid * 16;
        auto world = [&](const float* v) {
            double r[3];
            for (int k = 0; k < 3; ++k)
                r[k] = (double)F[4 * k] * v[0] + (double)F[4 * k + 1] * v[1] + (double)F[4 * k + 2] * v[2] +
                       (double)F[4 * k + 3];
            return std::array<double, 3>{r[0], r[1], r[2]};
        };
        const orn_material& mat = b->materials[mid];
        std::vector<uint32_t> stack{leaf.left_or_custom_id};
        while (!stack.empty()) {
            const uint32_t n = stack.back();
            stack.pop_back();
            if (n >= b->blas_nodes_len) continue;
            const orn_bvh_node& bn = b->blas_nodes[n];
            if (bn.node_type == ORN_NODE_INTERNAL) {
                stack.push_back(bn.left_or_custom_id);
                stack.push_back(bn.right_or_material_index);
                continue;
            }
            if (bn.node_type != ORN_NODE_TRIANGLE) continue;
            auto v0 = world(bn.left_aabb_min_or_v0), v1 = world(bn.left_aabb_max_or_v1),
                 v2 = world(bn.right_aabb_min_or_v2);
            double e1[3], e2[3];
            for (int k = 0; k < 3; ++k) {
                e1[k] = v1[k] - v0[k];
                e2[k] = v2[k] - v0[k];
            }
            const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                         cz = e1[0] * e2[1] - e1[1] * e2[0];
            const double area = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
            if (!(area > 0.0) || !std::isfinite(area)) continue;
            tris.push_back(make_float4((float)v0[0], (float)v0[1], (float)v0[2], mat.albedo[0]));
            tris.push_back(make_float4((float)e1[0], (float)e1[1], (float)e1[2], mat.albedo[1]));
            tris.push_back(make_float4((float)e2[0], (float)e2[1], (float)e2[2], mat.albedo[2]));
            uint32_t inv_id = leaf.transform_id * 2u;
            float inv_f;
            std::memcpy(&inv_f, &inv_id, 4);
            tris.push_back(make_float4(inv_f, 0.0f, 0.0f, 0.0f));
            total += area;
            cdf.push_back((float)total);
        }
    }
    ctx->light_count = (uint32_t)cdf.size();
    ctx->light_area = (float)total;
    float4* dl = nullptr;
    float* dc = nullptr;
    uint32_t* dm = nullptr;
    int s;
    if ((s = upload(ctx, tris.data(), tris.size(), &dl))) return s;
    if ((s = upload(ctx, cdf.data(), cdf.size(), &dc))) return s;
    if ((s = upload(ctx, flag.data(), flag.size(), &dm))) return s;
    ctx->d_lights = dl;
    ctx->d_light_cdf = dc;
    ctx->d_light_material = dm;
    return ORN_OK;
}

// Re-lays the reference's BvhNode arrays into the kernel's node array.
void relayout_nodes(const orn_scene_blob* b, std::vector<float4>* out) {
    const uint32_t T = b->tlas_nodes_len, B = b->blas_nodes_len;
    out->assign((size_t)(T + B) * 4, make_float4(0, 0, 0, 0));
    auto u2f = [](uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; };
    // reference to node `i` of the TLAS (blas=false) or BLAS, with its type
    auto ref = [&](uint32_t i, bool blas) -> uint32_t {
        const orn_bvh_node& c = blas ? b->blas_nodes[i] : b->tlas_nodes[i];
        return ((blas ? T : 0u) + i) | (c.node_type << 30);
    };
    auto put = [&](size_t idx, const orn_bvh_node& n, uint32_t child_offset) {
        float4* o = out->data() + idx * 4;
        const float* a = n.left_aabb_min_or_v0;
        const float* bb = n.left_aabb_max_or_v1;
        const float* c = n.right_aabb_min_or_v2;
        const float* e = n.right_aabb_max_or_v3;
        switch (n.node_type) {
            case ORN_NODE_INTERNAL:
                o[0] = make_float4(a[0], a[1], a[2], u2f(ref(n.left_or_custom_id, child_offset != 0)));
                o[1] = make_float4(bb[0], bb[1], bb[2], u2f(ref(n.right_or_material_index, child_offset != 0)));
                o[2] = make_float4(c[0], c[1], c[2], u2f(ORN_NODE_INTERNAL));
                o[3] = make_float4(e[0], e[1], e[2], 0.0f);
                break;
            case ORN_NODE_TRIANGLE: {
                // the vertices as given, so triangles sharing an edge see the
                // same floats (the watertight test relies on it), and the two
                // edges the reference's test subtracts on the fly
                // (bvh.hip.h:81-82) — the same single-precision subtractions
                const float e1[3] = {bb[0] - a[0], bb[1] - a[1], bb[2] - a[2]};
                const float e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
                o[0] = make_float4(a[0], a[1], a[2], u2f(n.left_or_custom_id));
                o[1] = make_float4(bb[0], bb[1], bb[2], e2[0]);
                o[2] = make_float4(c[0], c[1], c[2], e2[1]);
                o[3] = make_float4(e1[0], e1[1], e1[2], e2[2]);
                break;
            }
            default: {  // sphere / mesh leaf: inverse rows 0..2 inline
                const float* m = b->transforms + (size_t)n.transform_id * 2 * 16;
                o[0] = make_float4(m[0], m[1], m[2], m[3]);
                o[1] = make_float4(m[4], m[5], m[6], m[7]);
                o[2] = make_float4(m[8], m[9], m[10], u2f(n.node_type));
                uint32_t root = n.node_type == ORN_NODE_MESH ? ref(n.left_or_custom_id, true) : 0u;
                o[3] = make_float4(m[11], u2f(n.right_or_material_index), u2f(n.transform_id), u2f(root));
                break;
            }
        }
    };
    for (uint32_t i = 0; i < T; ++i) put(i, b->tlas_nodes[i], 0);
    for (uint32_t i = 0; i < B; ++i) put((size_t)T + i, b->blas_nodes[i], T);
}

int ensure_target(orn_context* ctx) {
    if (ctx->target_valid) return ORN_OK;
    size_t n = (size_t)ctx->width * ctx->height;
    if (n == 0) return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "resolution is zero");
    if (n >= 0xFFFFFFFFull) return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "resolution too large");
    ORN_CUDA(ctx, cudaMalloc(&ctx->acc, n * sizeof(float4)));
    ORN_CUDA(ctx, cudaMalloc(&ctx->fb, n * sizeof(float4)));
    ORN_CUDA(ctx, cudaMalloc(&ctx->rng, n * sizeof(uint32_t)));
    ORN_CUDA(ctx, cudaMemsetAsync(ctx->acc, 0, n * sizeof(float4), ctx->stream));
    ORN_CUDA(ctx, cudaMemsetAsync(ctx->fb, 0, n * sizeof(float4), ctx->stream));
    ORN_CUDA(ctx, orn::launch_seed_rng(ctx->rng, (uint32_t)n, ctx->stream));
    const size_t tiles = orn::order_tiles((uint32_t)n);
    ORN_CUDA(ctx, cudaMalloc(&ctx->px_cost, n * sizeof(uint32_t)));
    ORN_CUDA(ctx, cudaMalloc(&ctx->px_order, n * sizeof(uint32_t)));
    ORN_CUDA(ctx, cudaMalloc(&ctx->tile_buf, 4 * tiles * sizeof(uint32_t)));
    ORN_CUDA(ctx, orn::order_temp_bytes((uint32_t)n, &ctx->sort_temp_bytes));
    ORN_CUDA(ctx, cudaMalloc(&ctx->sort_temp, std::max<size_t>(ctx->sort_temp_bytes, 16)));
    ctx->order_valid = false;
    ctx->target_valid = true;
    return ORN_OK;
}

// Points a launch at the pixel order (when one exists and the state asks for
// it) and at the cost buffer the launch fills.
void use_pixel_order(orn_context* ctx, RenderLaunch* p) {
    const bool on = ctx->state.pixel_order == ORN_PIXEL_ORDER_COST;
    p->order = on && ctx->order_valid ? ctx->px_order : nullptr;
    p->cost = on ? ctx->px_cost : nullptr;
}

// After a launch that recorded costs: the order for the next launch.
int update_pixel_order(orn_context* ctx, const RenderLaunch& p) {
    if (!p.cost) return ORN_OK;
    const size_t tiles = orn::order_tiles(p.pixel_count);
    orn::PixelOrder o;
    o.cost = ctx->px_cost;
    o.pixels = p.pixel_count;
    o.keys = ctx->tile_buf;
    o.vals = ctx->tile_buf + tiles;
    o.keys2 = ctx->tile_buf + 2 * tiles;
    o.vals2 = ctx->tile_buf + 3 * tiles;
    o.temp = ctx->sort_temp;
    o.temp_bytes = ctx->sort_temp_bytes;
    o.order = ctx->px_order;
    ORN_CUDA(ctx, orn::launch_pixel_order(o, ctx->stream));
    ctx->launches += 2;   // tile costs and the order (the radix sort between them is CUB's)
    ctx->order_valid = true;
    return ORN_OK;
}

void free_cache_buffers(orn_context* ctx) {
    void* ptrs[] = {ctx->cq_count, ctx->cq_pixel, ctx->cq_in, ctx->cq_thr, ctx->ct_in, ctx->ct_target,
                    ctx->rng_extra, ctx->cv_counters};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    ctx->rng_extra = nullptr;
    ctx->cv_counters = nullptr;
    ctx->cq_streams = 0;
    ctx->cq_count = nullptr;
    ctx->cq_pixel = nullptr;
    ctx->cq_in = nullptr;
    ctx->cq_thr = nullptr;
    ctx->ct_in = nullptr;
    ctx->ct_target = nullptr;
    ctx->cq_pixels = ctx->cq_slots = 0;
}

void free_target(orn_context* ctx) {
    void* ptrs[] = {ctx->acc, ctx->fb, ctx->rng, ctx->px_cost, ctx->px_order, ctx->tile_buf, ctx->sort_temp};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    ctx->acc = nullptr;
    ctx->fb = nullptr;
    ctx->rng = nullptr;
    ctx->px_cost = nullptr;
    ctx->px_order = nullptr;
    ctx->tile_buf = nullptr;
    ctx->sort_temp = nullptr;
    ctx->order_valid = false;
    ctx->target_valid = false;
}

// Synchronises and turns the device error word into a status.
int sync_and_check(orn_context* ctx) {
    ORN_CUDA(ctx, cudaSetDevice(ctx->device));
    ORN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    uint32_t err = 0;
    ORN_CUDA(ctx, cudaMemcpy(&err, ctx->d_error, 4, cudaMemcpyDeviceToHost));
    if (err) {
        ORN_CUDA(ctx, cudaMemset(ctx->d_error, 0, 4));
        if (err & orn::ERR_STACK)
            return fail(ctx, ORN_ERR_STACK_OVERFLOW, "a ray needed more than 64 traversal stack entries");
        if (err & orn::ERR_MMA) return fail(ctx, ORN_ERR_TIMEOUT, "a radiance-cache tensor-core wait timed out");
        if (err & orn::ERR_WAIT) return fail(ctx, ORN_ERR_TIMEOUT, "a wavefront queue wait timed out");
        return fail(ctx, ORN_ERR_TIMEOUT, "a ray exceeded the per-ray node-visit limit");
    }
    return ORN_OK;
}

orn_constant_params make_params(const orn_context* ctx, float current_iteration) {
    orn_constant_params cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.camera = ctx->camera;
    cp.depth = ctx->state.depth;
    cp.width = ctx->width;
    cp.height = ctx->height;
    cp.flip_y = ctx->state.flip_y ? 1u : 0u;
    cp.inverted_gamma = ctx->state.inverted_gamma;
    cp.ray_cast_epsilon = ctx->state.ray_cast_epsilon;
    cp.textures_count = ctx->scene_textures_count;
    cp.current_iteration = current_iteration;
    return cp;
}

// Whether every ray of a render satisfies the condition of the FMNMX slab
// test (aabb_hit_fast: ray origin and node bounds finite and below 1e30 in
// magnitude).  Render rays start at the camera (origin plus a lens offset)
// or at a hit point, which lies inside the scene's world bounds; in a BLAS
// the origin is that point mapped by an inverse transform.  With S the
// largest world-space magnitude (scene bounds, camera origin plus lens) and
// C the largest inverse-transform entry, object-space origins are bounded by
// 4*C*(S+1).
bool render_fast_slabs(const orn_context* ctx) {
    if (ctx->scene.exact_slabs) return false;
    const orn_camera& cam = ctx->camera;
    double s = ctx->world_extent;
    for (int i = 0; i < 3; ++i) {
        double o = std::fabs((double)cam.origin[i]);
        double l = 2.0 * (std::fabs((double)cam.u[i]) + std::fabs((double)cam.v[i])) * std::fabs((double)cam.lens_radius);
        if (!std::isfinite(o) || !std::isfinite(l)) return false;
        s = std::max(s, o + l);
    }
    if (!(s < 1e29)) return false;
    return 4.0 * ctx->max_inverse_entry * (s + 1.0) < 1e29;
}

// The cached renderer (on the wavefront or the megakernel).
bool is_cached(const orn_context* ctx) {
    return ctx->state.kernel == ORN_KERNEL_CACHED || ctx->state.kernel == ORN_KERNEL_CACHED_WAVEFRONT;
}

// Query queue and training slots of the cached renderer, sized for the
// current resolution and the cache's training fraction.
// Sample streams per pixel of a cached frame: orn_state.spp_per_launch
// (0 = 1), at most 64.
uint32_t cache_streams(const orn_context* ctx) {
    return std::min<uint32_t>(std::max<uint32_t>(ctx->state.spp_per_launch, 1u), 64u);
}

int ensure_cache_buffers(orn_context* ctx) {
    const uint32_t n = ctx->width * ctx->height;
    const uint32_t shift = ctx->cache->config.train_shift;
    const uint32_t streams = cache_streams(ctx);
    if (ctx->cq_count && ctx->cq_pixels == n && ctx->cq_shift == shift && ctx->cq_streams == streams) return ORN_OK;
    if ((uint64_t)n * streams >= 0xFFFFFFFFull)
        return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "pixels x sample streams exceeds 2^32");
    free_cache_buffers(ctx);
    const uint32_t slots = orn::cache_train_slots(n, shift) * streams;   // every stream trains
    const size_t queries = (size_t)n * streams;   // one query per stream and pixel at most
    ORN_CUDA(ctx, cudaMalloc(&ctx->cq_count, 4));
    ORN_CUDA(ctx, cudaMalloc(&ctx->cv_counters, 34 * sizeof(uint32_t)));
    ORN_CUDA(ctx, cudaMemsetAsync(ctx->cv_counters, 0, 34 * sizeof(uint32_t), ctx->stream));
    ORN_CUDA(ctx, cudaMalloc(&ctx->cq_pixel, queries * 4));
    ORN_CUDA(ctx, cudaMalloc(&ctx->cq_in, queries * orn::kCacheInputs * 4));
    ORN_CUDA(ctx, cudaMalloc(&ctx->cq_thr, queries * sizeof(float4)));
    if (streams > 1) {
        // stream s of pixel i starts from state s * pixels + i (stream 0 is
        // the pixel's own state, seeded with i)
        ORN_CUDA(ctx, cudaMalloc(&ctx->rng_extra, (size_t)(streams - 1) * n * 4));
        ORN_CUDA(ctx, orn::launch_seed_rng(ctx->rng_extra, (streams - 1) * n, ctx->stream, n));
    }
    ctx->cq_streams = streams;
    ORN_CUDA(ctx, cudaMalloc(&ctx->ct_in, (size_t)slots * orn::kCacheInputs * 4));
    ORN_CUDA(ctx, cudaMalloc(&ctx->ct_target, (size_t)slots * 3 * 4));
    // training inputs must stay finite even in slots no path writes
    ORN_CUDA(ctx, cudaMemsetAsync(ctx->ct_in, 0, (size_t)slots * orn::kCacheInputs * 4, ctx->stream));
    ctx->cq_pixels = n;
    ctx->cq_slots = slots;
    ctx->cq_shift = shift;
    return ORN_OK;
}

// `passes` cached frames, each: one sample per pixel with the cached
// megakernel, the query pass (inference) adding the cached radiance, then
// up to steps_per_frame training steps on this frame's training slots; the
// framebuffer is post-processed after the last frame.
int render_cached(orn_context* ctx, RenderLaunch p, uint32_t passes, float ci_start) {
    orn_cache* c = ctx->cache;
    const bool fast = render_fast_slabs(ctx);
    const uint32_t n = ctx->width * ctx->height;
    const uint32_t batch = c->config.batch;
    const uint32_t nb = (ctx->cq_slots + batch - 1) / batch;
    const uint32_t steps = std::min(c->config.steps_per_frame, nb);
    p.do_post = 0;
    p.spp = 1;
    p.shade_threshold = orn::kCacheShadeThreshold;
    p.wave_fetch = orn::kWaveFetchDefault;
    const uint32_t streams = ctx->cq_streams;
    p.cache.streams = streams;
    p.cache.rng_extra = ctx->rng_extra;
    p.cache.sobol = ctx->state.sampler == ORN_SAMPLER_SOBOL ? 1u : 0u;
    if (streams > 1 && ci_start <= 1.0f)   // restarted accumulation: the streams add to zero
        ORN_CUDA(ctx, cudaMemsetAsync(ctx->acc, 0, (size_t)n * sizeof(float4), ctx->stream));
    for (int k = 0; k < 3; ++k) {
        p.cache.lo[k] = ctx->scene_lo[k];
        const float ext = ctx->scene_hi[k] - ctx->scene_lo[k];
        p.cache.inv_extent[k] = ext > 0.0f ? 1.0f / ext : 0.0f;
    }
    p.cache.query_count = ctx->cq_count;
    p.cache.query_pixel = ctx->cq_pixel;
    p.cache.query_in = ctx->cq_in;
    p.cache.query_thr = ctx->cq_thr;
    p.cache.train_in = ctx->ct_in;
    p.cache.train_target = ctx->ct_target;
    p.cache.train_slots = ctx->cq_slots;
    p.cache.train_count = ctx->cv_counters;
    p.cache.light_count = ctx->light_count;
    p.cache.light_area = ctx->light_area;
    p.cache.lights = ctx->d_lights;
    p.cache.light_cdf = ctx->d_light_cdf;
    p.cache.light_material = ctx->d_light_material;
    for (uint32_t f = 0; f < passes; ++f) {
        p.cp = make_params(ctx, ci_start + (float)(f * streams));
        p.cache.frame = (uint32_t)c->frames;
        // this frame counts cache vertices into one counter and reads the
        // other (the previous frame's)
        p.cache.vertices = ctx->cv_counters + 32 + ctx->cv_flip;
        p.cache.vertices_prev = ctx->cv_counters + 33 - ctx->cv_flip;
        ctx->cv_flip ^= 1u;
        ORN_CUDA(ctx, cudaMemsetAsync(ctx->cv_counters, 0, 32 * sizeof(uint32_t), ctx->stream));
        ORN_CUDA(ctx, cudaMemsetAsync(p.cache.vertices, 0, 4, ctx->stream));
        ORN_CUDA(ctx, cudaMemsetAsync(ctx->cq_count, 0, 4, ctx->stream));
        // slots no training path writes this frame read as "no target" (NaN)
        ORN_CUDA(ctx, cudaMemsetAsync(ctx->ct_target, 0xFF, (size_t)ctx->cq_slots * 12, ctx->stream));
        if (ctx->state.kernel == ORN_KERNEL_CACHED_WAVEFRONT)
            ORN_CUDA(ctx, orn::launch_wave_cached(p, (int)ctx->state.semantics, fast, ctx->stream));
        else
            ORN_CUDA(ctx, orn::launch_mega_cached(p, (int)ctx->state.semantics, fast, ctx->stream));
        ctx->launches++;
        int st = orn::cache_apply_queries(c, ctx->cq_count, n * streams, ctx->cq_in, ctx->cq_pixel, ctx->cq_thr, ctx->acc,
                                          ctx->d_error, ctx->stream);
        if (st) return fail(ctx, st, c->last_error);
        for (uint32_t k = 0; k < steps; ++k) {
            const uint32_t b = (uint32_t)((c->frames * steps + k) % nb);
            const uint32_t off = b * batch;
            const uint32_t m = std::min(batch, ctx->cq_slots - off);
            st = orn::cache_train_step(c, ctx->ct_in + (size_t)off * orn::kCacheInputs, ctx->ct_target + (size_t)off * 3,
                                       m, true, ctx->d_error, ctx->stream);
            if (st) return fail(ctx, st, c->last_error);
        }
        c->frames++;
    }
    if (p.pixel_count) {
        ORN_CUDA(ctx, orn::launch_post(ctx->acc, ctx->fb, ctx->width, ctx->height, ctx->state.flip_y ? 1u : 0u,
                                       ci_start + (float)(passes * streams - 1), ctx->state.inverted_gamma,
                                       (int)ctx->state.semantics, orn::MATH_PORTABLE, ctx->stream));
    }
    return ORN_OK;
}

}  // namespace

namespace orn {

// For orn_render_noalloc (noalloc.cu): the device-resident scene of a
// context, what a render with `camera` needs to launch the wavefront (the
// FMNMX slab condition is render_fast_slabs' check for that camera), and the
// context's error word with its pinned copy.
bool noalloc_link(const orn_context* ctx, const orn_camera* camera, NoAllocLink* out) {
    if (!ctx || !camera || !out || !ctx->na_host_error || !ctx->na_done) return false;
    out->scene = &ctx->scene;
    out->device = ctx->device;
    out->semantics = ctx->state.semantics;
    out->error_word = ctx->d_error;
    out->host_error = ctx->na_host_error;
    out->done = &ctx->na_done;
    out->pending = &ctx->na_pending;
    bool fast = !ctx->scene.exact_slabs;
    double s = ctx->world_extent;
    for (int i = 0; i < 3 && fast; ++i) {
        double o = std::fabs((double)camera->origin[i]);
        double l = 2.0 * (std::fabs((double)camera->u[i]) + std::fabs((double)camera->v[i])) *
                   std::fabs((double)camera->lens_radius);
        if (!std::isfinite(o) || !std::isfinite(l)) fast = false;
        else s = std::max(s, o + l);
    }
    if (fast && !(s < 1e29)) fast = false;
    if (fast && !(4.0 * ctx->max_inverse_entry * (s + 1.0) < 1e29)) fast = false;
    out->fast_slabs = fast;
    return true;
}

int batch_prepare(orn_context* ctx, BatchView* view, bool* fast_slabs, uint32_t* semantics, int* device,
                  cudaStream_t batch_stream, bool commit) {
    if (!ctx || !view) return ORN_ERR_INVALID_ARGUMENT;
    if (!ctx->camera_set) return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "no camera set (orn_set_camera)");
    ORN_CUDA(ctx, cudaSetDevice(ctx->device));
    int st = ensure_target(ctx);
    if (st) return st;
    const float ci = ctx->camera_dirty ? 0.0f : ctx->current_iteration;
    const uint32_t passes = std::max<uint32_t>(ctx->state.iterations, 1u);
    const float ci_start = ci + 1.0f;
    if (commit) {
        ctx->camera_dirty = false;
        ctx->current_iteration = ci + (float)passes;
    }
    view->scene = ctx->scene;
    view->cp = make_params(ctx, ci_start);
    view->spp = passes;
    view->pixel_begin = 0;
    view->acc = ctx->acc;
    view->fb = ctx->fb;
    view->rng = ctx->rng;
    *fast_slabs = render_fast_slabs(ctx);
    *semantics = ctx->state.semantics;
    *device = ctx->device;
    // the batch stream starts after the context's own queued work
    cudaEvent_t ev = nullptr;
    ORN_CUDA(ctx, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ev, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(batch_stream, ev, 0);
    cudaEventDestroy(ev);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "ordering the batch after the context");
    if (commit) {
        ctx->rendered = true;
        ctx->launches++;
    }
    return ORN_OK;
}

int batch_finish(orn_context* ctx, cudaEvent_t done) {
    ORN_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, done, 0));
    return ORN_OK;
}

}  // namespace orn

extern "C" {

uint32_t orn_abi_version(void) { return ORN_ABI_VERSION; }

int orn_get_device(const orn_context* ctx, int* device) {
    if (!ctx || !device) return ORN_ERR_INVALID_ARGUMENT;
    *device = ctx->device;
    return ORN_OK;
}

int orn_qmc_points(uint32_t pixel, uint32_t pair, uint32_t first, uint32_t count, float* out) {
    if (!out || pair > orn::QMC_LIGHT) return ORN_ERR_INVALID_ARGUMENT;
    const uint32_t seed = orn::qmc_hash(pixel + 1u);   // the cached kernel's pixel seed
    for (uint32_t k = 0; k < count; ++k) orn::qmc_point(seed, pair, first + k, out + 2 * (size_t)k, out + 2 * (size_t)k + 1);
    return ORN_OK;
}

const char* orn_status_string(int status) {
    switch (status) {
        case ORN_OK: return "ok";
        case ORN_ERR_INVALID_ARGUMENT: return "invalid argument";
        case ORN_ERR_EMPTY_SCENE: return "empty scene";
        case ORN_ERR_OUT_OF_MEMORY: return "out of memory";
        case ORN_ERR_CUDA: return "CUDA error";
        case ORN_ERR_NO_DEVICE: return "no CUDA device";
        case ORN_ERR_BAD_SCENE: return "invalid scene data";
        case ORN_ERR_STACK_OVERFLOW: return "traversal stack overflow";
        case ORN_ERR_BUFFER_TOO_SMALL: return "buffer too small";
        case ORN_ERR_TIMEOUT: return "device-side limit reached";
        case ORN_ERR_UNSUPPORTED: return "unsupported input";
        case ORN_ERR_BAD_IMAGE: return "corrupt image data";
        default: return "unknown status";
    }
}

const char* orn_last_error(const orn_context* ctx) {
    return ctx ? ctx->last_error.c_str() : "context is NULL";
}

int orn_create(const orn_scene_blob* blob, int device, orn_context** out) {
    if (!out) return ORN_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int st = validate_blob(nullptr, blob);
    if (st != ORN_OK) return st;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return ORN_ERR_NO_DEVICE;
    if (device < 0) device = count - 1;
    if (device >= count) return ORN_ERR_NO_DEVICE;
    orn_context* ctx = new (std::nothrow) orn_context();
    if (!ctx) return ORN_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    ctx->state = default_state();
    st = [&]() -> int {
        ORN_CUDA(ctx, cudaSetDevice(device));
        ORN_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ORN_CUDA(ctx, cudaEventCreate(&ctx->ev_start));
        ORN_CUDA(ctx, cudaEventCreate(&ctx->ev_stop));
        ORN_CUDA(ctx, cudaMalloc(&ctx->d_error, 4));
        ORN_CUDA(ctx, cudaMemset(ctx->d_error, 0, 4));
        ORN_CUDA(ctx, cudaMalloc(&ctx->d_work, 4));
        ORN_CUDA(ctx, cudaMallocHost(&ctx->na_host_error, 4));
        *ctx->na_host_error = 0;
        ORN_CUDA(ctx, cudaEventCreateWithFlags(&ctx->na_done, cudaEventDisableTiming));
        ORN_CUDA(ctx, cudaMalloc(&ctx->d_counters, ORN_COUNTER_COUNT * sizeof(unsigned long long)));
        ORN_CUDA(ctx, cudaMemset(ctx->d_counters, 0, ORN_COUNTER_COUNT * sizeof(unsigned long long)));
        std::vector<float4> nodes;
        relayout_nodes(blob, &nodes);
        float4* d_nodes = nullptr;
        int s = upload(ctx, nodes.data(), nodes.size(), &d_nodes);
        if (s) return s;
        float4* d_x = nullptr;
        if ((s = upload(ctx, (const float4*)blob->transforms, (size_t)blob->transforms_len * 4, &d_x))) return s;
        float4* d_n = nullptr;
        if ((s = upload(ctx, (const float4*)blob->normals, (size_t)blob->normals_len, &d_n))) return s;
        uint32_t* d_ni = nullptr;
        if ((s = upload(ctx, blob->normal_indices, blob->normal_indices_len, &d_ni))) return s;
        float2* d_uv = nullptr;
        if ((s = upload(ctx, (const float2*)blob->uvs, (size_t)blob->uvs_len, &d_uv))) return s;
        uint32_t* d_ui = nullptr;
        if ((s = upload(ctx, blob->uv_indices, blob->uv_indices_len, &d_ui))) return s;
        float4* d_m = nullptr;
        if ((s = upload(ctx, (const float4*)blob->materials, (size_t)blob->materials_len * 2, &d_m))) return s;
        // Textures: one device copy per distinct host image (the builder
        // appends a texture once per material that uses it).
        std::map<std::pair<const void*, uint64_t>, const unsigned char*> seen;
        std::vector<TexDesc> descs(blob->textures_len);
        for (uint32_t i = 0; i < blob->textures_len; ++i) {
            const orn_texture& t = blob->textures[i];
            uint32_t texel = t.format == ORN_TEXEL_RGBA8 ? 4u : 8u;
            uint32_t pitch = t.width * texel;
            auto key = std::make_pair(t.data, ((uint64_t)t.width << 32) | t.height);
            const unsigned char* dptr = nullptr;
            auto it = seen.find(key);
            if (it != seen.end()) {
                dptr = it->second;
            } else {
                void* p = nullptr;
                ORN_CUDA(ctx, cudaMalloc(&p, (size_t)pitch * t.height));
                ctx->scene_allocs.push_back(p);
                ORN_CUDA(ctx, cudaMemcpy2D(p, pitch, t.data, t.bytes_per_row, pitch, t.height,
                                           cudaMemcpyHostToDevice));
                dptr = (const unsigned char*)p;
                seen[key] = dptr;
            }
            descs[i] = TexDesc{dptr, t.width, t.height, pitch, t.format};
        }
        TexDesc* d_t = nullptr;
        if ((s = upload(ctx, descs.data(), descs.size(), &d_t))) return s;
        ctx->scene.nodes = d_nodes;
        ctx->scene.tlas_len = blob->tlas_nodes_len;
        ctx->scene.node_count = blob->tlas_nodes_len + blob->blas_nodes_len;
        ctx->scene.root_ref = (blob->tlas_nodes_len - 1) |
                              (blob->tlas_nodes[blob->tlas_nodes_len - 1].node_type << 30);
        // The FMNMX slab test needs every internal-node bound finite and
        // below 1e30 in magnitude (pt_device.cuh, aabb_hit_fast).
        bool huge = false;
        auto check_bounds = [&](const orn_bvh_node* nodes, uint32_t n) {
            for (uint32_t i = 0; i < n && !huge; ++i) {
                if (nodes[i].node_type != ORN_NODE_INTERNAL) continue;
                const float* f[4] = {nodes[i].left_aabb_min_or_v0, nodes[i].left_aabb_max_or_v1,
                                     nodes[i].right_aabb_min_or_v2, nodes[i].right_aabb_max_or_v3};
                for (int k = 0; k < 4; ++k)
                    for (int j = 0; j < 3; ++j)
                        if (!(std::fabs(f[k][j]) < 1e30f)) huge = true;
            }
        };
        check_bounds(blob->tlas_nodes, blob->tlas_nodes_len);
        check_bounds(blob->blas_nodes, blob->blas_nodes_len);
        for (uint32_t i = 0; i < blob->tlas_nodes_len; ++i) {
            const orn_bvh_node& n = blob->tlas_nodes[i];
            const float* f[4] = {n.left_aabb_min_or_v0, n.left_aabb_max_or_v1, n.right_aabb_min_or_v2,
                                 n.right_aabb_max_or_v3};
            int boxes = n.node_type == ORN_NODE_INTERNAL ? 4 : 2;
            for (int k = 0; k < boxes; ++k)
                for (int j = 0; j < 3; ++j) {
                    double v = std::fabs((double)f[k][j]);
                    if (!std::isfinite(v)) huge = true;
                    else ctx->world_extent = std::max(ctx->world_extent, v);
                }
        }
        // scene bounds (radiance-cache position inputs): the union of the
        // TLAS internal nodes' child boxes, else +-world_extent
        {
            double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
            for (uint32_t i = 0; i < blob->tlas_nodes_len; ++i) {
                const orn_bvh_node& n = blob->tlas_nodes[i];
                if (n.node_type != ORN_NODE_INTERNAL) continue;
                const float* mins[2] = {n.left_aabb_min_or_v0, n.right_aabb_min_or_v2};
                const float* maxs[2] = {n.left_aabb_max_or_v1, n.right_aabb_max_or_v3};
                for (int k = 0; k < 2; ++k)
                    for (int j = 0; j < 3; ++j) {
                        if (std::isfinite(mins[k][j])) lo[j] = std::min(lo[j], (double)mins[k][j]);
                        if (std::isfinite(maxs[k][j])) hi[j] = std::max(hi[j], (double)maxs[k][j]);
                    }
            }
            for (int j = 0; j < 3; ++j) {
                if (!(lo[j] <= hi[j])) {
                    lo[j] = -ctx->world_extent;
                    hi[j] = ctx->world_extent;
                }
                ctx->scene_lo[j] = (float)lo[j];
                ctx->scene_hi[j] = (float)hi[j];
            }
        }
        for (uint32_t t = 0; t < blob->transforms_len; t += 2)
            for (int j = 0; j < 16; ++j) {
                double v = std::fabs((double)blob->transforms[(size_t)t * 16 + j]);
                if (!std::isfinite(v)) huge = true;
                else ctx->max_inverse_entry = std::max(ctx->max_inverse_entry, v);
            }
        ctx->scene.exact_slabs = huge ? 1u : 0u;
#ifdef ORN_FORCE_EXACT_SLABS
        ctx->scene.exact_slabs = 1u;
#endif
        ctx->scene.xforms = d_x;
        ctx->scene.normals = d_n;
        ctx->scene.normal_indices = d_ni;
        ctx->scene.uvs = d_uv;
        ctx->scene.uv_indices = d_ui;
        ctx->scene.materials = d_m;
        ctx->scene.textures = d_t;
        ctx->scene.textures_len = blob->textures_len;
        ctx->scene_textures_count = blob->scene_textures_count;
        ctx->tlas_len = blob->tlas_nodes_len;
        ctx->blas_len = blob->blas_nodes_len;
        return build_lights(ctx, blob);
    }();
    if (st != ORN_OK) {
        orn_destroy(ctx);
        return st;
    }
    *out = ctx;
    return ORN_OK;
}

int orn_destroy(orn_context* ctx) {
    if (!ctx) return ORN_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_target(ctx);
    for (void* p : ctx->scene_allocs) cudaFree(p);
    if (ctx->d_error) cudaFree(ctx->d_error);
    if (ctx->d_work) cudaFree(ctx->d_work);
    if (ctx->na_host_error) cudaFreeHost(ctx->na_host_error);
    if (ctx->na_done) cudaEventDestroy(ctx->na_done);
    if (ctx->d_counters) cudaFree(ctx->d_counters);
    free_cache_buffers(ctx);
    if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
    if (ctx->ev_stop) cudaEventDestroy(ctx->ev_stop);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return ORN_OK;
}

int orn_set_state(orn_context* ctx, const orn_state* s) {
    if (!ctx || !s) return ORN_ERR_INVALID_ARGUMENT;
    if (s->semantics > ORN_SEMANTICS_WGSL || s->kernel > ORN_KERNEL_CACHED_WAVEFRONT ||
        s->triangle_test > ORN_TRIANGLE_WATERTIGHT || s->pixel_order > ORN_PIXEL_ORDER_RASTER ||
        s->sampler > ORN_SAMPLER_SOBOL)
        return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "unknown semantics, kernel or triangle test");
    ctx->state = *s;
    ctx->scene.watertight = s->triangle_test == ORN_TRIANGLE_WATERTIGHT ? 1u : 0u;
    return ORN_OK;
}

int orn_get_state(const orn_context* ctx, orn_state* out) {
    if (!ctx || !out) return ORN_ERR_INVALID_ARGUMENT;
    *out = ctx->state;
    return ORN_OK;
}

int orn_set_camera(orn_context* ctx, const orn_camera* camera) {
    if (!ctx || !camera) return ORN_ERR_INVALID_ARGUMENT;
    ctx->camera = *camera;
    ctx->camera_set = true;
    ctx->camera_dirty = true;
    return ORN_OK;
}

int orn_set_resolution(orn_context* ctx, uint32_t width, uint32_t height) {
    if (!ctx || width == 0 || height == 0) return ORN_ERR_INVALID_ARGUMENT;
    if ((uint64_t)width * height >= 0xFFFFFFFFull)
        return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "resolution too large");
    cudaSetDevice(ctx->device);
    if (ctx->target_valid) {
        cudaStreamSynchronize(ctx->stream);
        free_target(ctx);
    }
    ctx->width = width;
    ctx->height = height;
    return ORN_OK;
}

int orn_get_resolution(const orn_context* ctx, uint32_t* w, uint32_t* h) {
    if (!ctx || !w || !h) return ORN_ERR_INVALID_ARGUMENT;
    *w = ctx->width;
    *h = ctx->height;
    return ORN_OK;
}

int orn_peek_constant_params(const orn_context* ctx, orn_constant_params* out) {
    if (!ctx || !out) return ORN_ERR_INVALID_ARGUMENT;
    float ci = ctx->camera_dirty ? 0.0f : ctx->current_iteration;
    *out = make_params(ctx, ci + 1.0f);
    return ORN_OK;
}

int orn_attach_cache(orn_context* ctx, orn_cache* cache) {
    if (!ctx) return ORN_ERR_INVALID_ARGUMENT;
    if (cache && cache->device != ctx->device)
        return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "the cache lives on another device");
    if (ctx->cache != cache) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        free_cache_buffers(ctx);
    }
    ctx->cache = cache;
    return ORN_OK;
}

int orn_render(orn_context* ctx) {
    if (!ctx) return ORN_ERR_INVALID_ARGUMENT;
    if (!ctx->camera_set) return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "no camera set (orn_set_camera)");
    ORN_CUDA(ctx, cudaSetDevice(ctx->device));
    int st = ensure_target(ctx);
    if (st) return st;
    if (ctx->camera_dirty) {
        ctx->current_iteration = 0.0f;
        ctx->camera_dirty = false;
    }
    // iterations <= 1 takes the fused path of the reference: one pass.
    const uint32_t passes = std::max<uint32_t>(ctx->state.iterations, 1u);
    const float ci_start = ctx->current_iteration + 1.0f;
    // a cached frame takes cache_streams() samples per pixel
    ctx->current_iteration += (float)passes * (is_cached(ctx) ? cache_streams(ctx) : 1u);
    uint32_t chunk = ctx->state.spp_per_launch;
    if (chunk == 0) chunk = passes <= 64 ? passes : 32;
    RenderLaunch p;
    std::memset(&p, 0, sizeof(p));
    p.scene = ctx->scene;
    p.pixel_count = ctx->width * ctx->height;
    p.acc = ctx->acc;
    p.fb = ctx->fb;
    p.rng = ctx->rng;
    p.error = ctx->d_error;
    p.counters = ctx->d_counters;
    p.work_counter = ctx->d_work;
    p.shade_threshold = orn::kShadeThreshold;
    p.wave_fetch = ctx->wave_cfg.fetch;
    if (ctx->counters_enabled)
        ORN_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, ORN_COUNTER_COUNT * sizeof(unsigned long long), ctx->stream));
    if (is_cached(ctx)) {
        if (!ctx->cache)
            return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "ORN_KERNEL_CACHED needs a cache (orn_attach_cache)");
        st = ensure_cache_buffers(ctx);
        if (st) return st;
        ORN_CUDA(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
        st = render_cached(ctx, p, passes, ci_start);
        if (st) return st;
        ORN_CUDA(ctx, cudaEventRecord(ctx->ev_stop, ctx->stream));
        ctx->rendered = true;
        return ORN_OK;
    }
    ORN_CUDA(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
    for (uint32_t done = 0; done < passes;) {
        uint32_t n = std::min(chunk, passes - done);
        p.cp = make_params(ctx, ci_start + (float)done);
        p.spp = n;
        p.do_post = (done + n == passes) ? 1u : 0u;
        use_pixel_order(ctx, &p);
        if (ctx->state.kernel == ORN_KERNEL_WAVEFRONT) {
            ORN_CUDA(ctx, orn::launch_wave(p, ctx->wave_cfg, (int)ctx->state.semantics, ctx->counters_enabled,
                                           render_fast_slabs(ctx), ctx->stream));
        } else {
            ORN_CUDA(ctx, orn::launch_mega(p, (int)ctx->state.semantics, orn::MATH_PORTABLE,
                                           ctx->counters_enabled, render_fast_slabs(ctx), ctx->stream));
        }
        ctx->launches++;
        st = update_pixel_order(ctx, p);
        if (st) return st;
        done += n;
    }
    ORN_CUDA(ctx, cudaEventRecord(ctx->ev_stop, ctx->stream));
    ctx->rendered = true;
    return ORN_OK;
}

int orn_synchronize(orn_context* ctx) {
    if (!ctx) return ORN_ERR_INVALID_ARGUMENT;
    return sync_and_check(ctx);
}

int orn_last_render_ms(orn_context* ctx, float* ms) {
    if (!ctx || !ms) return ORN_ERR_INVALID_ARGUMENT;
    if (!ctx->rendered) return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "nothing rendered yet");
    int st = sync_and_check(ctx);
    if (st) return st;
    ORN_CUDA(ctx, cudaEventElapsedTime(ms, ctx->ev_start, ctx->ev_stop));
    return ORN_OK;
}

int orn_get_framebuffer(orn_context* ctx, float* dst, size_t pixel_count) {
    if (!ctx || !dst) return ORN_ERR_INVALID_ARGUMENT;
    ORN_CUDA(ctx, cudaSetDevice(ctx->device));
    int st = ensure_target(ctx);
    if (st) return st;
    size_t n = (size_t)ctx->width * ctx->height;
    if (pixel_count < n) return fail(ctx, ORN_ERR_BUFFER_TOO_SMALL, "framebuffer destination too small");
    ORN_CUDA(ctx, cudaMemcpyAsync(dst, ctx->fb, n * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    return sync_and_check(ctx);
}

int orn_get_accumulation(orn_context* ctx, float* dst, size_t pixel_count) {
    if (!ctx || !dst) return ORN_ERR_INVALID_ARGUMENT;
    ORN_CUDA(ctx, cudaSetDevice(ctx->device));
    int st = ensure_target(ctx);
    if (st) return st;
    size_t n = (size_t)ctx->width * ctx->height;
    if (pixel_count < n) return fail(ctx, ORN_ERR_BUFFER_TOO_SMALL, "accumulation destination too small");
    ORN_CUDA(ctx, cudaMemcpyAsync(dst, ctx->acc, n * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    return sync_and_check(ctx);
}

int orn_get_progress(orn_context* ctx, float* accumulation, uint32_t* rng_state, size_t pixel_count,
                     float* current_iteration) {
    if (!ctx || !accumulation || !rng_state || !current_iteration) return ORN_ERR_INVALID_ARGUMENT;
    ORN_CUDA(ctx, cudaSetDevice(ctx->device));
    int st = ensure_target(ctx);
    if (st) return st;
    size_t n = (size_t)ctx->width * ctx->height;
    if (pixel_count < n) return fail(ctx, ORN_ERR_BUFFER_TOO_SMALL, "progress destination too small");
    ORN_CUDA(ctx, cudaMemcpyAsync(accumulation, ctx->acc, n * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    ORN_CUDA(ctx, cudaMemcpyAsync(rng_state, ctx->rng, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    st = sync_and_check(ctx);
    if (st) return st;
    *current_iteration = ctx->camera_dirty ? 0.0f : ctx->current_iteration;
    return ORN_OK;
}

int orn_set_progress(orn_context* ctx, const float* accumulation, const uint32_t* rng_state,
                     size_t pixel_count, float current_iteration) {
    if (!ctx || !accumulation || !rng_state || current_iteration < 0.0f) return ORN_ERR_INVALID_ARGUMENT;
    ORN_CUDA(ctx, cudaSetDevice(ctx->device));
    int st = ensure_target(ctx);
    if (st) return st;
    size_t n = (size_t)ctx->width * ctx->height;
    if (pixel_count != n) return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "progress size does not match the resolution");
    ORN_CUDA(ctx, cudaMemcpyAsync(ctx->acc, accumulation, n * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
    ORN_CUDA(ctx, cudaMemcpyAsync(ctx->rng, rng_state, n * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream));
    st = sync_and_check(ctx);
    if (st) return st;
    ctx->current_iteration = current_iteration;
    ctx->camera_dirty = false;
    return ORN_OK;
}

int orn_trace_rays(orn_context* ctx, const orn_ray* rays, size_t count, orn_hit* hits, uint32_t* visits) {
    if (!ctx || (count && (!rays || !hits))) return ORN_ERR_INVALID_ARGUMENT;
    if (count == 0) return ORN_OK;
    ORN_CUDA(ctx, cudaSetDevice(ctx->device));
    float* d_rays = nullptr;
    orn_hit* d_hits = nullptr;
    uint32_t* d_visits = nullptr;
    int st = [&]() -> int {
        ORN_CUDA(ctx, cudaMalloc(&d_rays, count * sizeof(orn_ray)));
        ORN_CUDA(ctx, cudaMalloc(&d_hits, count * sizeof(orn_hit)));
        if (visits) ORN_CUDA(ctx, cudaMalloc(&d_visits, count * sizeof(uint32_t)));
        ORN_CUDA(ctx, cudaMemcpyAsync(d_rays, rays, count * sizeof(orn_ray), cudaMemcpyHostToDevice, ctx->stream));
        ORN_CUDA(ctx, orn::launch_trace_rays(ctx->scene, ctx->state.ray_cast_epsilon, d_rays, count, d_hits,
                                             d_visits, ctx->d_error, ctx->stream));
        ORN_CUDA(ctx, cudaMemcpyAsync(hits, d_hits, count * sizeof(orn_hit), cudaMemcpyDeviceToHost, ctx->stream));
        if (visits)
            ORN_CUDA(ctx, cudaMemcpyAsync(visits, d_visits, count * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
        return sync_and_check(ctx);
    }();
    cudaStreamSynchronize(ctx->stream);
    if (d_rays) cudaFree(d_rays);
    if (d_hits) cudaFree(d_hits);
    if (d_visits) cudaFree(d_visits);
    return st;
}

int orn_render_f64(orn_context* ctx, uint32_t spp, double* mean_rgba, size_t pixel_count) {
    if (!ctx || !mean_rgba || spp == 0) return ORN_ERR_INVALID_ARGUMENT;
    if (!ctx->camera_set) return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "no camera set (orn_set_camera)");
    const size_t n = (size_t)ctx->width * ctx->height;
    if (pixel_count < n) return fail(ctx, ORN_ERR_BUFFER_TOO_SMALL, "mean destination too small");
    ORN_CUDA(ctx, cudaSetDevice(ctx->device));
    double* acc64 = nullptr;
    uint32_t* rng = nullptr;
    int st = [&]() -> int {
        ORN_CUDA(ctx, cudaMalloc(&acc64, n * 4 * sizeof(double)));
        ORN_CUDA(ctx, cudaMalloc(&rng, n * sizeof(uint32_t)));
        ORN_CUDA(ctx, orn::launch_seed_rng(rng, (uint32_t)n, ctx->stream));
        RenderLaunch p;
        std::memset(&p, 0, sizeof(p));
        p.scene = ctx->scene;
        p.pixel_count = (uint32_t)n;
        p.rng = rng;
        p.acc64 = acc64;
        p.error = ctx->d_error;
        p.counters = ctx->d_counters;
        p.work_counter = ctx->d_work;
        p.shade_threshold = orn::kShadeThreshold;
        const bool fast = render_fast_slabs(ctx);
        const uint32_t chunk = 64;
        for (uint32_t done = 0; done < spp;) {
            uint32_t k = std::min(chunk, spp - done);
            p.cp = make_params(ctx, 1.0f + (float)done);
            p.spp = k;
            if (ctx->target_valid) use_pixel_order(ctx, &p);
            ORN_CUDA(ctx, orn::launch_mega_f64(p, (int)ctx->state.semantics, fast, ctx->stream));
            ctx->launches++;
            if (ctx->target_valid) {
                int ost = update_pixel_order(ctx, p);
                if (ost) return ost;
            }
            done += k;
        }
        std::vector<double> host(n * 4);
        ORN_CUDA(ctx, cudaMemcpyAsync(host.data(), acc64, n * 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        int s2 = sync_and_check(ctx);
        if (s2) return s2;
        for (size_t i = 0; i < n; ++i) {
            double w = host[4 * i + 3];
            for (int c = 0; c < 3; ++c) mean_rgba[4 * i + c] = host[4 * i + c] / w;
            mean_rgba[4 * i + 3] = 1.0;
        }
        return ORN_OK;
    }();
    cudaStreamSynchronize(ctx->stream);
    if (acc64) cudaFree(acc64);
    if (rng) cudaFree(rng);
    return st;
}

int orn_relmse(orn_context* ctx, const double* reference_mean_rgba, size_t pixel_count, double* relmse,
               uint64_t* skipped_pixels) {
    if (!ctx || !reference_mean_rgba || !relmse) return ORN_ERR_INVALID_ARGUMENT;
    const size_t n = (size_t)ctx->width * ctx->height;
    if (pixel_count != n) return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "reference size does not match the resolution");
    if (!ctx->target_valid || !ctx->rendered) return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "nothing rendered yet");
    ORN_CUDA(ctx, cudaSetDevice(ctx->device));
    double* ref = nullptr;
    double* out = nullptr;
    int st = [&]() -> int {
        ORN_CUDA(ctx, cudaMalloc(&ref, n * 4 * sizeof(double)));
        ORN_CUDA(ctx, cudaMalloc(&out, 2 * sizeof(double)));
        ORN_CUDA(ctx, cudaMemsetAsync(out, 0, 2 * sizeof(double), ctx->stream));
        ORN_CUDA(ctx, cudaMemcpyAsync(ref, reference_mean_rgba, n * 4 * sizeof(double), cudaMemcpyHostToDevice,
                                      ctx->stream));
        ORN_CUDA(ctx, orn::launch_relmse(ctx->acc, nullptr, ref, (uint32_t)n, out, ctx->stream));
        double sums[2] = {0.0, 0.0};
        ORN_CUDA(ctx, cudaMemcpyAsync(sums, out, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        int s2 = sync_and_check(ctx);
        if (s2) return s2;
        const double used = (double)n - sums[1];
        *relmse = used > 0.0 ? sums[0] / (3.0 * used) : 0.0;
        if (skipped_pixels) *skipped_pixels = (uint64_t)sums[1];
        return ORN_OK;
    }();
    cudaStreamSynchronize(ctx->stream);
    if (ref) cudaFree(ref);
    if (out) cudaFree(out);
    return st;
}

int orn_get_stream(const orn_context* ctx, void** stream) {
    if (!ctx || !stream) return ORN_ERR_INVALID_ARGUMENT;
    *stream = (void*)ctx->stream;
    return ORN_OK;
}

int orn_launch_count(const orn_context* ctx, uint64_t* launches) {
    if (!ctx || !launches) return ORN_ERR_INVALID_ARGUMENT;
    *launches = ctx->launches;
    return ORN_OK;
}

int orn_enable_counters(orn_context* ctx, int enable) {
    if (!ctx) return ORN_ERR_INVALID_ARGUMENT;
    ctx->counters_enabled = enable != 0;
    return ORN_OK;
}

int orn_get_counters(orn_context* ctx, uint64_t* out, size_t count) {
    if (!ctx || !out) return ORN_ERR_INVALID_ARGUMENT;
    int st = sync_and_check(ctx);
    if (st) return st;
    unsigned long long tmp[ORN_COUNTER_COUNT];
    ORN_CUDA(ctx, cudaMemcpy(tmp, ctx->d_counters, sizeof(tmp), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < count && i < ORN_COUNTER_COUNT; ++i) out[i] = tmp[i];
    return ORN_OK;
}

}  // extern "C"

// ---- persistent-wavefront launch parameters and their autotuner ------------------
extern "C" {

int orn_wave_get_config(const orn_context* ctx, orn_wave_config* out) {
    if (!ctx || !out) return ORN_ERR_INVALID_ARGUMENT;
    out->shape = (uint32_t)ctx->wave_cfg.shape;
    out->fetch = (uint32_t)ctx->wave_cfg.fetch;
    out->steps = (uint32_t)ctx->wave_cfg.steps;
    out->tuned = ctx->wave_tuned ? 1u : 0u;
    return ORN_OK;
}

int orn_wave_set_config(orn_context* ctx, const orn_wave_config* c) {
    if (!ctx || !c) return ORN_ERR_INVALID_ARGUMENT;
    if (c->shape >= (uint32_t)orn::kWaveShapes || c->fetch > 32u || c->steps > 64u ||
        !orn::wave_config_valid((int)c->shape, (int)c->fetch, (int)c->steps))
        return fail(ctx, ORN_ERR_INVALID_ARGUMENT,
                    "invalid wavefront configuration (shape 0..3, fetch 1..32, steps 32 or 64)");
    ctx->wave_cfg = orn::WaveConfig{(int)c->shape, (int)c->fetch, (int)c->steps};
    ctx->wave_tuned = false;
    return ORN_OK;
}

int orn_wave_tune(orn_context* ctx, const char* cache_path, orn_wave_config* chosen) {
    if (!ctx) return ORN_ERR_INVALID_ARGUMENT;
    if (!ctx->camera_set) return fail(ctx, ORN_ERR_INVALID_ARGUMENT, "no camera set (orn_set_camera)");
    ORN_CUDA(ctx, cudaSetDevice(ctx->device));
    int st = ensure_target(ctx);
    if (st) return st;
    st = sync_and_check(ctx);
    if (st) return st;
    const uint32_t n = ctx->width * ctx->height;
    // the passes of one launch as orn_render would issue them, at most 8
    // and at most ~16 M samples per candidate launch
    const uint32_t passes = std::max<uint32_t>(ctx->state.iterations, 1u);
    uint32_t chunk = ctx->state.spp_per_launch;
    if (chunk == 0) chunk = passes <= 64 ? passes : 32;
    const uint32_t tune_spp =
        std::max<uint32_t>(1u, std::min<uint32_t>({chunk, 8u, (uint32_t)((16u << 20) / std::max<uint32_t>(n, 1u))}));
    const bool fast = render_fast_slabs(ctx);
    cudaDeviceProp prop;
    char dev_name[256] = {0};
    int sms = 0;
    if (cudaGetDeviceProperties(&prop, ctx->device) == cudaSuccess) {
        std::snprintf(dev_name, sizeof(dev_name), "%s", prop.name);
        sms = prop.multiProcessorCount;
    }
    char key[512];
    std::snprintf(key, sizeof(key), "%s|sm%d|wavefront|pixels=%u|spp=%u|depth=%u|sem=%u|fast=%d|tlas=%u|blas=%u",
                  dev_name, sms, n, tune_spp, ctx->state.depth, ctx->state.semantics, fast ? 1 : 0, ctx->tlas_len,
                  ctx->blas_len);
    auto entries = orn::read_tune_cache(cache_path);
    auto hit = entries.find(key);
    if (hit != entries.end()) {
        const auto& f = hit->second.fields;
        auto a = f.find("shape"), b = f.find("fetch"), c = f.find("steps");
        // an entry outside the valid range (a hand-edited or foreign file) is
        // tuned again
        if (a != f.end() && b != f.end() && c != f.end() &&
            orn::wave_config_valid((int)a->second, (int)b->second, (int)c->second)) {
            ctx->wave_cfg = orn::WaveConfig{(int)a->second, (int)b->second, (int)c->second};
            ctx->wave_tuned = true;
            if (chosen) orn_wave_get_config(ctx, chosen);
            return ORN_OK;
        }
    }
    // Scratch targets and a copy of the RNG states: the context's image,
    // progress and pixel order are untouched.
    float4 *acc = nullptr, *fb = nullptr;
    uint32_t* rng = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto release = [&]() {
        if (acc) cudaFree(acc);
        if (fb) cudaFree(fb);
        if (rng) cudaFree(rng);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    if (cudaMalloc(&acc, (size_t)n * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&fb, (size_t)n * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&rng, (size_t)n * sizeof(uint32_t)) != cudaSuccess) {
        release();
        return fail(ctx, ORN_ERR_OUT_OF_MEMORY, "wavefront tuning scratch targets");
    }
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        release();
        return fail(ctx, ORN_ERR_CUDA, "wavefront tuning events");
    }
    RenderLaunch p;
    std::memset(&p, 0, sizeof(p));
    p.scene = ctx->scene;
    p.pixel_count = n;
    p.acc = acc;
    p.fb = fb;
    p.rng = rng;
    p.error = ctx->d_error;
    p.counters = ctx->d_counters;
    p.work_counter = ctx->d_work;
    p.shade_threshold = orn::kShadeThreshold;
    p.cp = make_params(ctx, 1.0f);
    p.spp = tune_spp;
    p.do_post = 1;
    p.order = ctx->state.pixel_order == ORN_PIXEL_ORDER_COST && ctx->order_valid ? ctx->px_order : nullptr;
    p.cost = nullptr;
    const int fetches[3] = {2, 4, 8};
    const int steps[2] = {32, 64};
    orn::WaveConfig best = ctx->wave_cfg;
    float best_ms = 3.0e38f;
    cudaError_t e = cudaSuccess;
    for (int shape = 0; shape < orn::kWaveShapes && e == cudaSuccess; ++shape) {
        for (int fi = 0; fi < 3 && e == cudaSuccess; ++fi) {
            for (int si = 0; si < 2 && e == cudaSuccess; ++si) {
                const orn::WaveConfig c{shape, fetches[fi], steps[si]};
                p.wave_fetch = c.fetch;
                float ms = 0.0f;
                for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {   // the first run warms the caches
                    e = cudaMemcpyAsync(rng, ctx->rng, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                                        ctx->stream);
                    if (e == cudaSuccess) e = cudaEventRecord(e0, ctx->stream);
                    if (e == cudaSuccess)
                        e = orn::launch_wave(p, c, (int)ctx->state.semantics, false, fast, ctx->stream);
                    if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
                    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                }
                if (e == cudaSuccess && ms < best_ms) {
                    best_ms = ms;
                    best = c;
                }
                ctx->launches += 2;
            }
        }
    }
    cudaStreamSynchronize(ctx->stream);
    release();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "wavefront tuning launch");
    st = sync_and_check(ctx);
    if (st) return st;
    ctx->wave_cfg = best;
    ctx->wave_tuned = true;
    if (cache_path) {
        orn::TuneEntry te;
        te.fields["shape"] = best.shape;
        te.fields["fetch"] = best.fetch;
        te.fields["steps"] = best.steps;
        te.ms = best_ms;
        entries[key] = te;
        orn::write_tune_cache(cache_path, entries, {"shape", "fetch", "steps"});
    }
    if (chosen) orn_wave_get_config(ctx, chosen);
    return ORN_OK;
}

}  // extern "C"
