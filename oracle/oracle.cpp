// oracle.cpp — CPU restatement of zig_ornament's path-tracing hot path.
//
// TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py
// (its CPU-baseline leg and the reference arm) load the library built from
// this file; the product never does.  It is pinned bit-for-bit against the
// reference's own HIP kernels compiled for the host (oracle/ref_driver.cpp)
// (tests/test_oracle_golden.py::test_oracle_matches_compiled_reference)
// and against committed golden vectors in tests/golden/.
//
// Every function follows the reference's arithmetic in the same operation
// order (no FMA contraction: build with -ffp-contract=off), citing the
// HIP source file:line it restates (paths inside zig_ornament,
// src/hip_backend/kernels/…; the WGSL twins under src/wgpu_backend/shaders/
// compute the same formulas).
//
// Switches:
//   semantics  0 = HIP (metal always scatters, wrap addressing,
//                  post-processing clamp = max(min(x,1),0))
//              1 = WGSL (metal absorbs when dot(scattered, n) <= 0,
//                  material.wgsl:22-27; clamp-to-edge addressing; clamp =
//                  min(max(x,0),1))
//   math       0 = host libm (powf/acosf/atan2f/sincosf), the functions the
//                  reference build calls
//              1 = the project's portable transcendentals (pmath.h), the ones
//                  the GPU kernel calls
// Extra outputs the reference does not have: per-ray node-visit counts, work
// counters, and an FP64 accumulation buffer (FP64 only in the accumulation).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <omp.h>

#include "ornament_cuda.h"
#include "pmath.h"

namespace {

struct V3 { float x, y, z; };
struct V4 { float x, y, z, w; };

inline V3 v3(float x, float y, float z) { return {x, y, z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 mul(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 scale(float c, V3 a) { return {c * a.x, c * a.y, c * a.z}; }   // vec_math: c * a.x
inline V3 divs(V3 a, float c) { return {a.x / c, a.y / c, a.z / c}; }
inline V3 neg(V3 a) { return {-a.x, -a.y, -a.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 normalize(V3 a) { return divs(a, sqrtf(dot(a, a))); }
// vec_math.hip.h: reflect(e1, e2) = e1 - 2 * dot(e2, e1) * e2
inline V3 reflect(V3 e1, V3 e2) { return sub(e1, scale(2.0f * dot(e2, e1), e2)); }
// vec_math.hip.h: refract(i, n, eta)
inline V3 refract(V3 i, V3 n, float eta) {
    float k = 1.0f - eta * eta * (1.0f - dot(n, i) * dot(n, i));
    if (k < 0.0f) return v3(0.0f, 0.0f, 0.0f);
    return sub(scale(eta, i), scale(eta * dot(n, i) + sqrtf(k), n));
}
// RT_MIN / RT_MAX (vec_math.hip.h:42-43)
inline float rt_min(float a, float b) { return b < a ? b : a; }
inline float rt_max(float a, float b) { return b > a ? b : a; }
inline float dot4(const float* r, float x, float y, float z, float w) {
    return r[0] * x + r[1] * y + r[2] * z + r[3] * w;
}

struct Tex {
    const unsigned char* data;
    uint32_t w, h, pitch, format;
};

struct Scene {
    const orn_bvh_node* tlas; uint32_t tlas_len;
    const orn_bvh_node* blas; uint32_t blas_len;
    const float* normals;
    const uint32_t* normal_indices;
    const float* uvs;
    const uint32_t* uv_indices;
    const float* transforms;
    const orn_material* materials;
    std::vector<Tex> textures;
    uint32_t textures_count;  // ConstantParams.textures_count
};

struct Counters {
    uint64_t c[ORN_COUNTER_COUNT];
};

struct Math {
    int portable;
    float pow(float a, float b) const { return portable ? pm_powf(a, b) : powf(a, b); }
    float acos(float a) const { return portable ? pm_acosf(a) : acosf(a); }
    float atan2(float a, float b) const { return portable ? pm_atan2f(a, b) : atan2f(a, b); }
    void sincos(float a, float* s, float* c) const {
        if (portable) pm_sincosf(a, s, c); else sincosf(a, s, c);
    }
};

// ---- RNG: random.hip.h:14-30 ------------------------------------------
struct Rng {
    uint32_t state;
    uint32_t next() {
        uint32_t old_state = state + 747796405u + 2891336453u;
        uint32_t word = ((old_state >> ((old_state >> 28) + 4)) ^ old_state) * 277803737u;
        state = (word >> 22) ^ word;
        return state;
    }
    float f() { return (float)next() * (1.0f / 4294967296.0f); }
    // random.hip.h:47-63
    V3 in_unit_sphere(const Math& m) {
        float r = m.pow(f(), 0.33333f);
        float theta = 3.14159265358979f * f();
        float phi = 2.0f * 3.14159265358979f * f();
        float st, ct, sp, cp;
        m.sincos(theta, &st, &ct);
        m.sincos(phi, &sp, &cp);
        return v3(r * st * cp, r * st * sp, r * ct);
    }
    // random.hip.h:83-95
    V3 in_unit_disk(const Math& m) {
        float r = sqrtf(f());
        float alpha = 2.0f * 3.14159265358979f * f();
        float sa, ca;
        m.sincos(alpha, &sa, &ca);
        return v3(r * ca, r * sa, 0.0f);
    }
};

// ---- Bvh::hit restated: bvh.hip.h:145-276 ---------------------------------
struct Hit {
    float t;
    uint32_t material;
    uint32_t type;   // 1 sphere, 2 mesh
    uint32_t inv;
    uint32_t tri;
    float u, v;
};

inline V3 safe_invdir(V3 d) {  // bvh.hip.h:43-52
    const float eps = 1e-5f;
    float x = fabsf(d.x) > eps ? d.x : (d.x < 0.0f ? -eps : eps);
    float y = fabsf(d.y) > eps ? d.y : (d.y < 0.0f ? -eps : eps);
    float z = fabsf(d.z) > eps ? d.z : (d.z < 0.0f ? -eps : eps);
    return v3(1.0f / x, 1.0f / y, 1.0f / z);
}

inline bool aabb_hit(const float* mn, const float* mx, V3 inv, V3 oxinv, float t_min, float t_max) {
    // bvh.hip.h:54-70
    float fx = mx[0] * inv.x + oxinv.x, fy = mx[1] * inv.y + oxinv.y, fz = mx[2] * inv.z + oxinv.z;
    float nx = mn[0] * inv.x + oxinv.x, ny = mn[1] * inv.y + oxinv.y, nz = mn[2] * inv.z + oxinv.z;
    float tmax_x = rt_max(fx, nx), tmax_y = rt_max(fy, ny), tmax_z = rt_max(fz, nz);
    float tmin_x = rt_min(fx, nx), tmin_y = rt_min(fy, ny), tmin_z = rt_min(fz, nz);
    float max_t = fminf(rt_min(rt_min(tmax_x, tmax_y), tmax_z), t_max);
    float min_t = fmaxf(rt_max(rt_max(tmin_x, tmin_y), tmin_z), t_min);
    return min_t <= max_t;
}

inline float triangle_hit(V3 o, V3 d, V3 v1, V3 v2, V3 v3_, float t_min, float t_max,
                          float* hu, float* hv) {  // bvh.hip.h:72-117
    V3 e1 = sub(v2, v1);
    V3 e2 = sub(v3_, v1);
    V3 s1 = cross(d, e2);
    float det = dot(s1, e1);
    float invd = 1.0f / det;
    V3 dd = sub(o, v1);
    float u = dot(dd, s1) * invd;
    if (u < 0.0f || u > 1.0f) return t_max;
    V3 s2 = cross(dd, e1);
    float v = dot(d, s2) * invd;
    if (v < 0.0f || u + v > 1.0f) return t_max;
    float t = dot(e2, s2) * invd;
    if (t < t_min || t > t_max) return t_max;
    *hu = u;
    *hv = v;
    return t;
}

inline float sphere_hit(V3 o, V3 d, float t_min, float t_max) {  // bvh.hip.h:119-143
    V3 oc = o;  // centre (0,0,0): o - 0
    oc = sub(o, v3(0.0f, 0.0f, 0.0f));
    float a = d.x * d.x + d.y * d.y + d.z * d.z;
    float half_b = dot(oc, d);
    float c = (oc.x * oc.x + oc.y * oc.y + oc.z * oc.z) - 1.0f * 1.0f;
    float disc = half_b * half_b - a * c;
    if (disc < 0.0f) return t_max;
    float sq = sqrtf(disc);
    float t = (-half_b - sq) / a;
    if (t < t_min || t_max < t) {
        t = (-half_b + sq) / a;
        if (t < t_min || t_max < t) return t_max;
    }
    return t;
}

// transform.hip.h:19-32 (M stored row-major, m * v = row dot products)
inline void transform_ray(const float* m, V3 o, V3 d, V3* oo, V3* od) {
    *oo = v3(dot4(m + 0, o.x, o.y, o.z, 1.0f), dot4(m + 4, o.x, o.y, o.z, 1.0f),
             dot4(m + 8, o.x, o.y, o.z, 1.0f));
    *od = v3(dot4(m + 0, d.x, d.y, d.z, 0.0f), dot4(m + 4, d.x, d.y, d.z, 0.0f),
             dot4(m + 8, d.x, d.y, d.z, 0.0f));
}

constexpr uint32_t kSentinel = 0xffffffffu;

bool bvh_hit(const Scene& s, V3 ro, V3 rd, float t_min, Hit* out, uint32_t* visits,
             Counters* cnt, int* overflow) {
    float t_max = 3.40282e+38f;
    int top = 0;
    uint32_t addr = s.tlas_len - 1;
    uint32_t stack[64];
    stack[0] = addr;
    bool tlas = true;
    bool any = false;
    V3 o = ro, d = rd;
    V3 inv = safe_invdir(d);
    V3 oxinv = mul(neg(o), inv);
    const V3 world_inv = inv, world_oxinv = oxinv;
    uint32_t material = 0, inv_id = 0;
    uint32_t n_visits = 0;
    while (top >= 0) {
        const orn_bvh_node& node = tlas ? s.tlas[addr] : s.blas[addr];
        ++n_visits;
        switch (node.node_type) {
            case ORN_NODE_INTERNAL: {
                if (cnt) cnt->c[3]++;
                bool l = aabb_hit(node.left_aabb_min_or_v0, node.left_aabb_max_or_v1, inv, oxinv, t_min, t_max);
                bool r = aabb_hit(node.right_aabb_min_or_v2, node.right_aabb_max_or_v3, inv, oxinv, t_min, t_max);
                if (l) { if (top >= 63) { *overflow = 1; return false; } stack[++top] = node.left_or_custom_id; }
                if (r) { if (top >= 63) { *overflow = 1; return false; } stack[++top] = node.right_or_material_index; }
                break;
            }
            case ORN_NODE_SPHERE: {
                if (cnt) cnt->c[4]++;
                uint32_t id = node.transform_id * 2;
                V3 to, td;
                transform_ray(s.transforms + (size_t)id * 16, o, d, &to, &td);
                float t = sphere_hit(to, td, t_min, t_max);
                if (t < t_max) {
                    any = true;
                    t_max = t;
                    out->t = t;
                    out->material = node.right_or_material_index;
                    out->type = ORN_NODE_SPHERE;
                    out->inv = id;
                }
                break;
            }
            case ORN_NODE_MESH: {
                if (cnt) cnt->c[5]++;
                tlas = false;
                if (top >= 62) { *overflow = 1; return false; }
                stack[++top] = kSentinel;
                stack[++top] = node.left_or_custom_id;
                inv_id = node.transform_id * 2;
                material = node.right_or_material_index;
                V3 to, td;
                transform_ray(s.transforms + (size_t)inv_id * 16, o, d, &to, &td);
                o = to;
                d = td;
                inv = safe_invdir(d);
                oxinv = mul(neg(o), inv);
                break;
            }
            case ORN_NODE_TRIANGLE: {
                if (cnt) cnt->c[6]++;
                float u = 0.0f, v = 0.0f;
                V3 a = v3(node.left_aabb_min_or_v0[0], node.left_aabb_min_or_v0[1], node.left_aabb_min_or_v0[2]);
                V3 b = v3(node.left_aabb_max_or_v1[0], node.left_aabb_max_or_v1[1], node.left_aabb_max_or_v1[2]);
                V3 c = v3(node.right_aabb_min_or_v2[0], node.right_aabb_min_or_v2[1], node.right_aabb_min_or_v2[2]);
                float t = triangle_hit(o, d, a, b, c, t_min, t_max, &u, &v);
                if (t < t_max) {
                    any = true;
                    t_max = t;
                    out->t = t;
                    out->material = material;
                    out->type = ORN_NODE_MESH;
                    out->inv = inv_id;
                    out->tri = node.left_or_custom_id * 3;
                    out->u = u;
                    out->v = v;
                }
                break;
            }
            default: break;
        }
        addr = stack[top];
        top--;
        if (addr == kSentinel) {
            tlas = true;
            o = ro;
            d = rd;
            inv = world_inv;
            oxinv = world_oxinv;
            addr = stack[top];
            top--;
        }
    }
    if (visits) *visits = n_visits;
    if (cnt) { cnt->c[2] += n_visits; cnt->c[1]++; }
    return any;
}

// ---- texture sampling ------------------------------------------------------
float half_to_float(uint16_t h) {
    uint32_t s = (uint32_t)(h >> 15) << 31, e = (h >> 10) & 0x1f, m = h & 0x3ff, bits;
    if (e == 0) {
        if (m == 0) bits = s;
        else {
            int shift = 0;
            while ((m & 0x400) == 0) { m <<= 1; shift++; }
            m &= 0x3ff;
            bits = s | ((uint32_t)(127 - 15 - shift + 1) << 23) | (m << 13);
        }
    } else if (e == 31) bits = s | 0x7f800000u | (m << 13);
    else bits = s | ((e - 15 + 127) << 23) | (m << 13);
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

int tex_index(float c, uint32_t n, int clamp_mode) {
    if (!(c == c)) c = 0.0f;
    float x;
    if (clamp_mode) {
        x = floorf(c * (float)n);
    } else {
        float f = c - floorf(c);
        x = floorf(f * (float)n);
    }
    if (x > (float)(n - 1)) x = (float)(n - 1);
    if (x < 0.0f) x = 0.0f;
    return (int)x;
}

V3 sample(const Tex& t, float u, float v, int clamp_mode) {
    int x = tex_index(u, t.w, clamp_mode), y = tex_index(v, t.h, clamp_mode);
    const unsigned char* row = t.data + (size_t)y * t.pitch;
    if (t.format == ORN_TEXEL_RGBA8) {
        const unsigned char* p = row + (size_t)x * 4;
        return v3(p[0] / 255.0f, p[1] / 255.0f, p[2] / 255.0f);
    }
    const uint16_t* p = (const uint16_t*)(row + (size_t)x * 8);
    return v3(half_to_float(p[0]), half_to_float(p[1]), half_to_float(p[2]));
}

// ---- one sample: pathtracer.hip.cpp:72-154 ----------------------------------
struct Params {
    orn_constant_params cp;
    int semantics;
    Math math;
};

V3 get_color(const Scene& s, const Params& p, const orn_material& m, float u, float v, int* textured) {
    // material.hip.h:30-33 (HIP: index < textures.len; WGSL: < textures_count)
    uint32_t id = m.albedo_texture_index;
    bool use = p.semantics == ORN_SEMANTICS_WGSL
                   ? (id < p.cp.textures_count && id < (uint32_t)s.textures.size())
                   : id < (uint32_t)s.textures.size();
    if (use) {
        *textured = 1;
        return sample(s.textures[id], u, v, p.semantics == ORN_SEMANTICS_WGSL);
    }
    return v3(m.albedo[0], m.albedo[1], m.albedo[2]);
}

V4 trace_sample(const Scene& s, const Params& p, uint32_t px, uint32_t py, Rng& rng,
                Counters* cnt, int* overflow) {
    const orn_constant_params& cp = p.cp;
    const Math& mth = p.math;
    float u = ((float)px + rng.f()) / (float)(cp.width - 1);
    float v = ((float)py + rng.f()) / (float)(cp.height - 1);
    // camera.hip.h:25-33
    const orn_camera& cam = cp.camera;
    V3 disk = rng.in_unit_disk(mth);
    V3 rdv = scale(cam.lens_radius, disk);
    V3 cu = v3(cam.u[0], cam.u[1], cam.u[2]), cv = v3(cam.v[0], cam.v[1], cam.v[2]);
    V3 origin = v3(cam.origin[0], cam.origin[1], cam.origin[2]);
    V3 offset = add(scale(rdv.x, cu), scale(rdv.y, cv));
    V3 llc = v3(cam.lower_left_corner[0], cam.lower_left_corner[1], cam.lower_left_corner[2]);
    V3 hor = v3(cam.horizontal[0], cam.horizontal[1], cam.horizontal[2]);
    V3 ver = v3(cam.vertical[0], cam.vertical[1], cam.vertical[2]);
    V3 ro = add(origin, offset);
    V3 rd = sub(sub(add(add(llc, scale(u, hor)), scale(v, ver)), origin), offset);
    V3 color = v3(1.0f, 1.0f, 1.0f);
    for (uint32_t i = 0; i < cp.depth; ++i) {
        Hit h{};
        if (!bvh_hit(s, ro, rd, cp.ray_cast_epsilon, &h, nullptr, cnt, overflow)) {
            if (*overflow) return {0, 0, 0, 0};
            V3 ud = normalize(rd);
            float tt = 0.5f * (ud.y + 1.0f);
            V3 sky = add(scale(1.0f - tt, v3(1.0f, 1.0f, 1.0f)), scale(tt, v3(0.5f, 0.7f, 1.0f)));
            color = mul(color, sky);
            break;
        }
        uint32_t transform_id = h.inv + 1;
        V3 hp = add(ro, scale(h.t, rd));
        V3 normal;
        bool front;
        float hu = 0.0f, hv = 0.0f;
        if (h.type == ORN_NODE_SPHERE) {
            if (cnt) cnt->c[7]++;
            const float* m = s.transforms + (size_t)transform_id * 16;
            V3 center = v3(dot4(m + 0, 0.0f, 0.0f, 0.0f, 1.0f), dot4(m + 4, 0.0f, 0.0f, 0.0f, 1.0f),
                           dot4(m + 8, 0.0f, 0.0f, 0.0f, 1.0f));
            V3 on = normalize(sub(hp, center));
            float theta = mth.acos(-on.y);
            float phi = mth.atan2(-on.z, on.x) + 3.14159265358979f;
            hu = phi / (2.0f * 3.14159265358979f);
            hv = theta / 3.14159265358979f;
            if (dot(rd, on) > 0.0f) { normal = neg(on); front = false; }
            else { normal = on; front = true; }
        } else {
            if (cnt) cnt->c[8]++;
            const float* n0 = s.normals + (size_t)s.normal_indices[h.tri] * 4;
            const float* n1 = s.normals + (size_t)s.normal_indices[h.tri + 1] * 4;
            const float* n2 = s.normals + (size_t)s.normal_indices[h.tri + 2] * 4;
            const float* t0 = s.uvs + (size_t)s.uv_indices[h.tri] * 2;
            const float* t1 = s.uvs + (size_t)s.uv_indices[h.tri + 1] * 2;
            const float* t2 = s.uvs + (size_t)s.uv_indices[h.tri + 2] * 2;
            float w = 1.0f - h.u - h.v;
            float nn[3];
            for (int k = 0; k < 3; ++k) nn[k] = w * n0[k] + h.u * n1[k] + h.v * n2[k];
            hu = w * t0[0] + h.u * t1[0] + h.v * t2[0];
            hv = w * t0[1] + h.u * t1[1] + h.v * t2[1];
            // transform_normal (transform.hip.h:28-32): transpose(M^-1) * (n, 0)
            const float* m = s.transforms + (size_t)h.inv * 16;
            V3 tn = v3(m[0] * nn[0] + m[4] * nn[1] + m[8] * nn[2] + m[12] * 0.0f,
                       m[1] * nn[0] + m[5] * nn[1] + m[9] * nn[2] + m[13] * 0.0f,
                       m[2] * nn[0] + m[6] * nn[1] + m[10] * nn[2] + m[14] * 0.0f);
            V3 on = normalize(tn);
            if (dot(rd, on) > 0.0f) { normal = neg(on); front = false; }
            else { normal = on; front = true; }
        }
        const orn_material& mat = s.materials[h.material];
        int textured = 0;
        // material.hip.h:87-105
        if (mat.type == ORN_LAMBERTIAN) {
            V3 dir = add(normal, normalize(rng.in_unit_sphere(mth)));
            if (fabsf(dir.x) < 1e-8f && fabsf(dir.y) < 1e-8f && fabsf(dir.z) < 1e-8f) dir = normal;
            V3 att = get_color(s, p, mat, hu, hv, &textured);
            ro = hp;
            rd = dir;
            color = mul(color, att);
        } else if (mat.type == ORN_METAL) {
            V3 dir = add(reflect(normalize(rd), normal), scale(mat.fuzz, rng.in_unit_sphere(mth)));
            V3 att = get_color(s, p, mat, hu, hv, &textured);
            if (p.semantics == ORN_SEMANTICS_WGSL && !(dot(dir, normal) > 0.0f)) {
                // material.wgsl:26 — scatter returns false: emit() of a metal is 0
                color = mul(color, v3(0.0f, 0.0f, 0.0f));
                if (cnt && textured) cnt->c[9]++;
                break;
            }
            ro = hp;
            rd = dir;
            color = mul(color, att);
        } else if (mat.type == ORN_DIELECTRIC) {
            float ratio = front ? 1.0f / mat.ior : mat.ior;
            V3 ud = normalize(rd);
            float cos_t = fminf(dot(neg(ud), normal), 1.0f);
            float sin_t = sqrtf(1.0f - cos_t * cos_t);
            bool cannot = ratio * sin_t > 1.0f;
            bool refl = cannot;
            if (!cannot) {
                float r0 = (1.0f - ratio) / (1.0f + ratio);
                r0 = r0 * r0;
                float refl_p = r0 + (1.0f - r0) * mth.pow(1.0f - cos_t, 5.0f);
                refl = refl_p > rng.f();
            }
            V3 dir = refl ? reflect(ud, normal) : refract(ud, normal, ratio);
            ro = hp;
            rd = dir;
            color = mul(color, v3(1.0f, 1.0f, 1.0f));
        } else {
            V3 e = mat.type == ORN_DIFFUSE_LIGHT ? get_color(s, p, mat, hu, hv, &textured)
                                                 : v3(0.0f, 0.0f, 0.0f);
            color = mul(color, e);
            if (cnt && textured) cnt->c[9]++;
            break;
        }
        if (cnt && textured) cnt->c[9]++;
    }
    return {color.x, color.y, color.z, 1.0f};
}

void load_scene(Scene* s, const orn_scene_blob* b, uint32_t textures_count) {
    s->tlas = b->tlas_nodes; s->tlas_len = b->tlas_nodes_len;
    s->blas = b->blas_nodes; s->blas_len = b->blas_nodes_len;
    s->normals = b->normals;
    s->normal_indices = b->normal_indices;
    s->uvs = b->uvs;
    s->uv_indices = b->uv_indices;
    s->transforms = b->transforms;
    s->materials = b->materials;
    s->textures.resize(b->textures_len);
    for (uint32_t i = 0; i < b->textures_len; ++i)
        s->textures[i] = {(const unsigned char*)b->textures[i].data, b->textures[i].width,
                          b->textures[i].height, b->textures[i].bytes_per_row, b->textures[i].format};
    s->textures_count = textures_count;
}

}  // namespace

extern "C" {

// Bvh::hit over a ray list; visits may be NULL.
int oracle_trace_rays(const orn_scene_blob* blob, float ray_cast_epsilon, const float* rays,
                      size_t count, orn_hit* hits, uint32_t* visits, int threads) {
    if (!blob || !rays || !hits || blob->tlas_nodes_len == 0) return ORN_ERR_INVALID_ARGUMENT;
    Scene s;
    load_scene(&s, blob, blob->scene_textures_count);
    if (threads <= 0) threads = omp_get_max_threads();
    int overflow_any = 0;
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) reduction(| : overflow_any)
    for (size_t i = 0; i < count; ++i) {
        const float* r = rays + 6 * i;
        Hit h{};
        uint32_t nv = 0;
        int overflow = 0;
        bool any = bvh_hit(s, v3(r[0], r[1], r[2]), v3(r[3], r[4], r[5]), ray_cast_epsilon, &h, &nv,
                           nullptr, &overflow);
        overflow_any |= overflow;
        orn_hit o;
        std::memset(&o, 0, sizeof(o));
        if (any) {
            o.hit = 1;
            o.t = h.t;
            o.material_index = h.material;
            o.node_type = h.type;
            o.inverted_transform_id = h.inv;
            o.tri_id = h.type == ORN_NODE_MESH ? h.tri : 0u;
            o.uv[0] = h.type == ORN_NODE_MESH ? h.u : 0.0f;
            o.uv[1] = h.type == ORN_NODE_MESH ? h.v : 0.0f;
        }
        hits[i] = o;
        if (visits) visits[i] = nv;
    }
    return overflow_any ? ORN_ERR_STACK_OVERFLOW : ORN_OK;
}

// PathTracer.render restated (src/hip_backend/path_tracer.zig:121-168):
// `spp` sample passes with current_iteration = ci_start, ci_start+1, …, then
// post-processing with the last value.  Each pixel's passes run in order in
// one thread, which gives the same per-pixel RNG stream and accumulation
// order as one launch per pass.  acc/fb: pixel_count float4; rng: u32 each.
// acc64 (optional): FP64 accumulation of the same samples (sum only).
// Pixels pixel_begin, pixel_begin + pixel_stride, ... below pixel_end are
// rendered (a bounded sample of the frame); post-processing covers the same
// pixels.
int oracle_render(const orn_scene_blob* blob, const orn_constant_params* cp, uint32_t spp,
                  float ci_start, int semantics, int portable_math, float* acc, uint32_t* rng,
                  float* fb, double* acc64, uint32_t pixel_begin, uint32_t pixel_end,
                  uint32_t pixel_stride, int threads, uint64_t* counters) {
    if (!blob || !cp || !acc || !rng || !fb || spp == 0) return ORN_ERR_INVALID_ARGUMENT;
    if (blob->tlas_nodes_len == 0) return ORN_ERR_EMPTY_SCENE;
    Scene s;
    load_scene(&s, blob, cp->textures_count);
    const uint32_t W = cp->width, H = cp->height;
    const uint32_t pixel_count = W * H;
    if (pixel_end > pixel_count) pixel_end = pixel_count;
    if (pixel_stride == 0) pixel_stride = 1;
    const uint32_t n_px = pixel_end > pixel_begin ? (pixel_end - pixel_begin + pixel_stride - 1) / pixel_stride : 0;
    if (threads <= 0) threads = omp_get_max_threads();
    Params p;
    p.cp = *cp;
    p.semantics = semantics;
    p.math.portable = portable_math;
    const float ci_last = ci_start + (float)(spp - 1);
    Counters total{};
    int overflow_any = 0;
#pragma omp parallel num_threads(threads) reduction(| : overflow_any)
    {
        Counters local{};
#pragma omp for schedule(dynamic, 64)
        for (uint32_t ip = 0; ip < n_px; ++ip) {
            const uint32_t gid = pixel_begin + ip * pixel_stride;
            uint32_t x = gid % W, y = gid / W;
            Rng r{rng[gid]};
            V4 a = {acc[4 * gid], acc[4 * gid + 1], acc[4 * gid + 2], acc[4 * gid + 3]};
            int overflow = 0;
            for (uint32_t k = 0; k < spp; ++k) {
                float ci = ci_start + (float)k;
                V4 c = trace_sample(s, p, x, y, r, counters ? &local : nullptr, &overflow);
                local.c[0]++;
                if (ci > 1.0f) a = {a.x + c.x, a.y + c.y, a.z + c.z, a.w + c.w};
                else a = c;
                if (acc64) {
                    double* d = acc64 + 4 * (size_t)gid;
                    if (ci > 1.0f) { d[0] += c.x; d[1] += c.y; d[2] += c.z; d[3] += c.w; }
                    else { d[0] = c.x; d[1] = c.y; d[2] = c.z; d[3] = c.w; }
                }
            }
            overflow_any |= overflow;
            acc[4 * gid] = a.x; acc[4 * gid + 1] = a.y; acc[4 * gid + 2] = a.z; acc[4 * gid + 3] = a.w;
            rng[gid] = r.state;
            // post_processing: pathtracer.hip.cpp:58-70 / pathtracer.wgsl:81-93
            float q[4] = {a.x / ci_last, a.y / ci_last, a.z / ci_last, a.w / ci_last};
            for (int k = 0; k < 4; ++k)
                q[k] = semantics == ORN_SEMANTICS_WGSL ? fminf(fmaxf(q[k], 0.0f), 1.0f)
                                                       : fmaxf(fminf(q[k], 1.0f), 0.0f);
            for (int k = 0; k < 3; ++k) q[k] = p.math.pow(q[k], cp->inverted_gamma);
            uint32_t fbi = gid;
            if (cp->flip_y != 0) fbi = W * (H - y - 1) + x;
            for (int k = 0; k < 4; ++k) fb[4 * (size_t)fbi + k] = q[k];
        }
#pragma omp critical
        for (int k = 0; k < ORN_COUNTER_COUNT; ++k) total.c[k] += local.c[k];
    }
    if (counters)
        for (int k = 0; k < ORN_COUNTER_COUNT; ++k) counters[k] = total.c[k];
    return overflow_any ? ORN_ERR_STACK_OVERFLOW : ORN_OK;
}

// The portable transcendentals, exported for the accuracy tests.
float oracle_pm_powf(float a, float b) { return pm_powf(a, b); }
float oracle_pm_acosf(float a) { return pm_acosf(a); }
float oracle_pm_atan2f(float a, float b) { return pm_atan2f(a, b); }
void oracle_pm_sincosf(float a, float* s, float* c) { pm_sincosf(a, s, c); }
// Vectorised forms for numpy.
void oracle_pm_eval(int fn, const float* a, const float* b, float* out, float* out2, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        switch (fn) {
            case 0: out[i] = pm_powf(a[i], b[i]); break;
            case 1: out[i] = pm_acosf(a[i]); break;
            case 2: out[i] = pm_atan2f(a[i], b[i]); break;
            default: pm_sincosf(a[i], &out[i], &out2[i]); break;
        }
    }
}
void oracle_libm_eval(int fn, const float* a, const float* b, float* out, float* out2, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        switch (fn) {
            case 0: out[i] = powf(a[i], b[i]); break;
            case 1: out[i] = acosf(a[i]); break;
            case 2: out[i] = atan2f(a[i], b[i]); break;
            default: sincosf(a[i], &out[i], &out2[i]); break;
        }
    }
}

}  // extern "C"

// ---- unit-level hooks (same case layouts as the reference driver's) -------
extern "C" {

int oracle_pcg(uint32_t seed, size_t n, uint32_t* u32_out, float* f_out) {
    Rng a{seed}, b{seed};
    for (size_t i = 0; i < n; ++i) {
        u32_out[i] = a.next();
        f_out[i] = b.f();
    }
    return 0;
}

int oracle_safe_invdir(const float* d, size_t n, float* out) {
    for (size_t i = 0; i < n; ++i) {
        V3 r = safe_invdir(v3(d[3 * i], d[3 * i + 1], d[3 * i + 2]));
        out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
    }
    return 0;
}

int oracle_triangle_hit(const float* c, size_t n, float* out) {
    for (size_t i = 0; i < n; ++i) {
        const float* p = c + 17 * i;
        float u = -1.0f, v = -1.0f;
        float t = triangle_hit(v3(p[0], p[1], p[2]), v3(p[3], p[4], p[5]), v3(p[6], p[7], p[8]),
                               v3(p[9], p[10], p[11]), v3(p[12], p[13], p[14]), p[15], p[16], &u, &v);
        out[3 * i] = t; out[3 * i + 1] = u; out[3 * i + 2] = v;
    }
    return 0;
}

int oracle_sphere_hit(const float* c, size_t n, float* out) {
    for (size_t i = 0; i < n; ++i) {
        const float* p = c + 8 * i;
        out[i] = sphere_hit(v3(p[0], p[1], p[2]), v3(p[3], p[4], p[5]), p[6], p[7]);
    }
    return 0;
}

int oracle_aabb_hit(const float* c, size_t n, float* out) {
    for (size_t i = 0; i < n; ++i) {
        const float* p = c + 14 * i;
        V3 inv = v3(p[6], p[7], p[8]), ox = v3(p[9], p[10], p[11]);
        // same values as aabb_hit, returned as the (min_t, max_t) pair
        float fx = p[3] * inv.x + ox.x, fy = p[4] * inv.y + ox.y, fz = p[5] * inv.z + ox.z;
        float nx = p[0] * inv.x + ox.x, ny = p[1] * inv.y + ox.y, nz = p[2] * inv.z + ox.z;
        out[2 * i + 1] = fminf(rt_min(rt_min(rt_max(fx, nx), rt_max(fy, ny)), rt_max(fz, nz)), p[13]);
        out[2 * i] = fmaxf(rt_max(rt_max(rt_min(fx, nx), rt_min(fy, ny)), rt_min(fz, nz)), p[12]);
    }
    return 0;
}

}  // extern "C"
