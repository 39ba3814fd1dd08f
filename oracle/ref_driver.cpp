// Test infrastructure (oracle): drives the reference's own HIP kernels,
// compiled unmodified for the host through oracle/shim.
//
// This translation unit #includes src/hip_backend/kernels/pathtracer.hip.cpp
// from the zig_ornament sources (the include path is given by
// oracle/build_oracle.py; nothing of the reference is copied here).  It
// exposes a C API that mirrors the HIP backend's host loop:
//   ref_render      PathTracer.render (src/hip_backend/path_tracer.zig:121-133)
//                   + update() (:150-168): `spp` calls of path_tracing_kernal,
//                   then post_processing_kernal — or the fused kernel when
//                   spp == 1 — over every pixel, with blockDim/blockIdx/
//                   threadIdx set per pixel as a 256-wide 1-D launch would.
//   ref_trace_rays  Bvh::hit (src/hip_backend/kernels/bvh.hip.h:145-276) on
//                   caller-supplied rays.
// Only tests/ and bench.py load the library this file builds.
#include "pathtracer.hip.cpp"

#include <cstring>
#include <vector>
#include <omp.h>

#include "ornament_cuda.h"

thread_local orn_shim_dim3 blockDim = {256, 1, 1};
thread_local orn_shim_dim3 blockIdx = {0, 1, 1};
thread_local orn_shim_dim3 threadIdx = {0, 1, 1};

float orn_shim_half_to_float(uint16_t h) {
    uint32_t s = (uint32_t)(h >> 15) << 31;
    uint32_t e = (h >> 10) & 0x1f;
    uint32_t m = h & 0x3ff;
    uint32_t bits;
    if (e == 0) {
        if (m == 0) {
            bits = s;
        } else {  // subnormal half: normalise
            int shift = 0;
            while ((m & 0x400) == 0) { m <<= 1; shift++; }
            m &= 0x3ff;
            bits = s | ((uint32_t)(127 - 15 - shift + 1) << 23) | (m << 13);
        }
    } else if (e == 31) {
        bits = s | 0x7f800000u | (m << 13);
    } else {
        bits = s | ((e - 15 + 127) << 23) | (m << 13);
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

namespace {

struct RefScene {
    KernalGlobals kg;
    std::vector<orn_shim_texture> textures;
    std::vector<hipTextureObject_t> texture_objects;
};

void fill_globals(RefScene* s, const orn_scene_blob* b) {
    std::memset(&s->kg, 0, sizeof(s->kg));
    s->kg.bvh.tlas_nodes = {(BvhNode*)b->tlas_nodes, b->tlas_nodes_len};
    s->kg.bvh.blas_nodes = {(BvhNode*)b->blas_nodes, b->blas_nodes_len};
    s->kg.bvh.normals = {(float4*)b->normals, b->normals_len};
    s->kg.bvh.normal_indices = {(uint32_t*)b->normal_indices, b->normal_indices_len};
    s->kg.bvh.uvs = {(float2*)b->uvs, b->uvs_len};
    s->kg.bvh.uv_indices = {(uint32_t*)b->uv_indices, b->uv_indices_len};
    s->kg.bvh.transforms = {(float4x4*)b->transforms, b->transforms_len};
    s->kg.materials = {(Material*)b->materials, b->materials_len};
    s->textures.resize(b->textures_len);
    s->texture_objects.resize(b->textures_len);
    for (uint32_t i = 0; i < b->textures_len; ++i) {
        const orn_texture& t = b->textures[i];
        s->textures[i] = {(const unsigned char*)t.data, t.width, t.height,
                          t.bytes_per_row, t.format};
        s->texture_objects[i] = &s->textures[i];
    }
    s->kg.textures = {s->texture_objects.data(), b->textures_len};
}

void set_constant_params(const orn_constant_params* cp, float current_iteration) {
    static_assert(sizeof(ConstantParams) == sizeof(orn_constant_params),
                  "ConstantParams layout");
    std::memcpy(&constant_params, cp, sizeof(ConstantParams));
    constant_params.current_iteration = current_iteration;
}

void set_thread_ids(uint32_t gid) {
    blockDim = {256, 1, 1};
    blockIdx = {gid / 256, 0, 0};
    threadIdx = {gid % 256, 0, 0};
}

}  // namespace

extern "C" {

int ref_struct_sizes(uint32_t* out, int n) {
    uint32_t s[5] = {(uint32_t)sizeof(BvhNode), (uint32_t)sizeof(Material),
                     (uint32_t)sizeof(ConstantParams), (uint32_t)sizeof(Camera),
                     (uint32_t)sizeof(float4x4)};
    for (int i = 0; i < n && i < 5; ++i) out[i] = s[i];
    return 0;
}

// `acc` and `fb` hold pixel_count float4; `rng` pixel_count u32.  The pass
// loop follows PathTracer.render: the constant-params upload of update()
// happens before each pass with current_iteration = ci_start + pass.
int ref_render(const orn_scene_blob* blob, const orn_constant_params* cp,
               uint32_t spp, float ci_start, float* acc, uint32_t* rng,
               float* fb, int threads) {
    if (!blob || !cp || !acc || !rng || !fb || spp == 0) return 1;
    RefScene s;
    fill_globals(&s, blob);
    uint32_t pixel_count = cp->width * cp->height;
    s.kg.framebuffer = (float4*)fb;
    s.kg.accumulation_buffer = (float4*)acc;
    s.kg.rng_seed_buffer = rng;
    s.kg.pixel_count = pixel_count;
    uint32_t launch_threads = (pixel_count + 255) / 256 * 256;
    if (threads <= 0) threads = omp_get_max_threads();
    if (spp > 1) {
        for (uint32_t pass = 0; pass < spp; ++pass) {
            set_constant_params(cp, ci_start + (float)pass);
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
            for (uint32_t gid = 0; gid < launch_threads; ++gid) {
                set_thread_ids(gid);
                path_tracing_kernal(s.kg);
            }
        }
#pragma omp parallel for schedule(static) num_threads(threads)
        for (uint32_t gid = 0; gid < launch_threads; ++gid) {
            set_thread_ids(gid);
            post_processing_kernal(s.kg);
        }
    } else {
        set_constant_params(cp, ci_start);
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
        for (uint32_t gid = 0; gid < launch_threads; ++gid) {
            set_thread_ids(gid);
            path_tracing_and_post_processing_kernal(s.kg);
        }
    }
    return 0;
}

// rays: 6 floats each (origin, direction).  Writes orn_hit per ray.
int ref_trace_rays(const orn_scene_blob* blob, float ray_cast_epsilon,
                   const float* rays, size_t count, orn_hit* hits, int threads) {
    if (!blob || !rays || !hits) return 1;
    RefScene s;
    fill_globals(&s, blob);
    orn_constant_params cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.ray_cast_epsilon = ray_cast_epsilon;
    set_constant_params(&cp, 1.0f);
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads)
    for (size_t i = 0; i < count; ++i) {
        const float* r = rays + 6 * i;
        Ray ray(make_float3(r[0], r[1], r[2]), make_float3(r[3], r[4], r[5]));
        float t = 0.0f;
        uint32_t material_index = 0;
        BvhNodeType node_type = InternalNode;
        uint32_t inv_id = 0, tri_id = 0;
        float2 uv = make_float2(0.0f, 0.0f);
        bool h = s.kg.bvh.hit(ray, &t, &material_index, &node_type, &inv_id, &tri_id, &uv);
        orn_hit out;
        std::memset(&out, 0, sizeof(out));
        if (h) {
            out.hit = 1;
            out.t = t;
            out.material_index = material_index;
            out.node_type = (uint32_t)node_type;
            out.inverted_transform_id = inv_id;
            out.tri_id = (node_type == Mesh) ? tri_id : 0u;
            out.uv[0] = (node_type == Mesh) ? uv.x : 0.0f;
            out.uv[1] = (node_type == Mesh) ? uv.y : 0.0f;
        }
        hits[i] = out;
    }
    return 0;
}

}  // extern "C"

// ---- unit-level hooks for golden vectors --------------------------------
extern "C" {

// RndGen (random.hip.h:8-30): n draws of gen_uint32 and gen_float from seed.
int ref_pcg(uint32_t seed, size_t n, uint32_t* u32_out, float* f_out) {
    RndGen a(seed), b(seed);
    for (size_t i = 0; i < n; ++i) {
        u32_out[i] = a.gen_uint32();
        f_out[i] = b.gen_float();
    }
    return 0;
}

// Bvh::safe_invdir (bvh.hip.h:43-52) on n directions (3 floats each).
int ref_safe_invdir(const float* d, size_t n, float* out) {
    Bvh bvh;
    std::memset(&bvh, 0, sizeof(bvh));
    for (size_t i = 0; i < n; ++i) {
        float3 r = bvh.safe_invdir(make_float3(d[3 * i], d[3 * i + 1], d[3 * i + 2]));
        out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
    }
    return 0;
}

// Bvh::triangle_hit (bvh.hip.h:72-117): per case 6 ray floats, 9 vertex
// floats, t_min, t_max -> t, u, v (u, v = -1 when not written).
int ref_triangle_hit(const float* c, size_t n, float* out) {
    Bvh bvh;
    std::memset(&bvh, 0, sizeof(bvh));
    for (size_t i = 0; i < n; ++i) {
        const float* p = c + 17 * i;
        Ray r(make_float3(p[0], p[1], p[2]), make_float3(p[3], p[4], p[5]));
        float2 uv = make_float2(-1.0f, -1.0f);
        float t = bvh.triangle_hit(r, make_float3(p[6], p[7], p[8]), make_float3(p[9], p[10], p[11]),
                                   make_float3(p[12], p[13], p[14]), p[15], p[16], &uv);
        out[3 * i] = t; out[3 * i + 1] = uv.x; out[3 * i + 2] = uv.y;
    }
    return 0;
}

// Bvh::sphere_hit (bvh.hip.h:119-143): per case 6 ray floats, t_min, t_max.
int ref_sphere_hit(const float* c, size_t n, float* out) {
    Bvh bvh;
    std::memset(&bvh, 0, sizeof(bvh));
    for (size_t i = 0; i < n; ++i) {
        const float* p = c + 8 * i;
        Ray r(make_float3(p[0], p[1], p[2]), make_float3(p[3], p[4], p[5]));
        out[i] = bvh.sphere_hit(r, p[6], p[7]);
    }
    return 0;
}

// Bvh::aabb_hit (bvh.hip.h:54-70): per case min(3), max(3), invdir(3),
// oxinvdir(3), t_min, t_max -> (min_t, max_t).
int ref_aabb_hit(const float* c, size_t n, float* out) {
    Bvh bvh;
    std::memset(&bvh, 0, sizeof(bvh));
    for (size_t i = 0; i < n; ++i) {
        const float* p = c + 14 * i;
        float2 r = bvh.aabb_hit(make_float3(p[0], p[1], p[2]), make_float3(p[3], p[4], p[5]),
                                make_float3(p[6], p[7], p[8]), make_float3(p[9], p[10], p[11]), p[12], p[13]);
        out[2 * i] = r.x; out[2 * i + 1] = r.y;
    }
    return 0;
}

}  // extern "C"
