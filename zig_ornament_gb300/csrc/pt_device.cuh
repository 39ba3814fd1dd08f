// pt_device.cuh — device-side core of the sm_103a path tracer.
//
// What it computes is zig_ornament's per-pixel path-tracing hot path
// (src/hip_backend/kernels/pathtracer.hip.cpp:72-154 and the headers it
// includes; the WGSL twins under src/wgpu_backend/shaders/ compute the same
// formulas).  How it computes it is GB300-specific:
//
//  * One node array for TLAS and BLAS (BLAS ids offset by the TLAS length),
//    64-byte nodes fetched as two 32-byte read-only vector loads
//    (ld.global.nc.v8) before the branch on the node's kind.  Sphere and
//    mesh-entry leaves carry rows 0-2 of their inverse transform inline, so
//    a leaf visit is one node fetch instead of node + transform; triangle
//    leaves carry the three vertices as given.
//  * The reference's explicit stack loop (bvh.hip.h:145-276: push left,
//    push right, pop; a 0xffffffff sentinel marks the BLAS exit) is run as
//    "keep the next node in a register, push only the deferred child" with
//    the BLAS exit detected by stack depth.  Nodes are visited in exactly
//    the reference's order, so hits and per-ray visit counts are identical.
//  * All arithmetic keeps the reference's operation order; the translation
//    unit is compiled with -fmad=false so no multiply-add is contracted.
//    With MATH_PORTABLE the transcendentals come from pmath.h and every
//    sample is bit-identical to the CPU restatement.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ornament_cuda.h"
#include "pmath.h"
#include "pt_scene.h"

namespace orn {

constexpr uint32_t kMaxVisitsPerRay = 1u << 24;
constexpr int kStackSize = 64;

struct f3 { float x, y, z; };
__device__ __forceinline__ f3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 add(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 sub(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 mul(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ f3 scale(float c, f3 a) { return {c * a.x, c * a.y, c * a.z}; }
__device__ __forceinline__ f3 neg(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ f3 normalize(f3 a) {
    float l = sqrtf(dot(a, a));
    return {a.x / l, a.y / l, a.z / l};
}
__device__ __forceinline__ f3 reflect(f3 e1, f3 e2) { return sub(e1, scale(2.0f * dot(e2, e1), e2)); }
__device__ __forceinline__ f3 refract(f3 i, f3 n, float eta) {
    float k = 1.0f - eta * eta * (1.0f - dot(n, i) * dot(n, i));
    if (k < 0.0f) return mk(0.0f, 0.0f, 0.0f);
    return sub(scale(eta, i), scale(eta * dot(n, i) + sqrtf(k), n));
}
__device__ __forceinline__ float rt_min(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float rt_max(float a, float b) { return b > a ? b : a; }
__device__ __forceinline__ float dot4(float4 r, float x, float y, float z, float w) {
    return r.x * x + r.y * y + r.z * z + r.w * w;
}
__device__ __forceinline__ uint32_t bits(float f) { return __float_as_uint(f); }
__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

// Two float4 with one 256-bit read-only load (sm_100+).  A lane's request
// then fills a whole 32-byte L1 sector instead of half of one; nodes are
// 64-byte aligned.
__device__ __forceinline__ void ldg8(const float4* p, float4* lo, float4* hi) {
#ifdef ORN_NODE_LOAD_V4
    *lo = __ldg(p);
    *hi = __ldg(p + 1);
    return;
#endif
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(lo->x), "=f"(lo->y), "=f"(lo->z), "=f"(lo->w), "=f"(hi->x), "=f"(hi->y), "=f"(hi->z),
                   "=f"(hi->w)
                 : "l"(p));
}

template <int MATH> struct DevMath;
template <> struct DevMath<MATH_PORTABLE> {
    __device__ static float pow(float a, float b) { return pm_powf(a, b); }
    __device__ static float acos(float a) { return pm_acosf(a); }
    __device__ static float atan2(float a, float b) { return pm_atan2f(a, b); }
    __device__ static void sincos(float a, float* s, float* c) { pm_sincosf(a, s, c); }
};
template <> struct DevMath<MATH_DEVICE> {
    __device__ static float pow(float a, float b) { return powf(a, b); }
    __device__ static float acos(float a) { return acosf(a); }
    __device__ static float atan2(float a, float b) { return atan2f(a, b); }
    __device__ static void sincos(float a, float* s, float* c) { sincosf(a, s, c); }
};

// ---- RNG (random.hip.h:14-30, 47-63, 83-95) -------------------------------
struct Rng {
    uint32_t state;
    __device__ __forceinline__ uint32_t next() {
        uint32_t old_state = state + 747796405u + 2891336453u;
        uint32_t word = ((old_state >> ((old_state >> 28) + 4)) ^ old_state) * 277803737u;
        state = (word >> 22) ^ word;
        return state;
    }
    __device__ __forceinline__ float f() { return __uint2float_rn(next()) * (1.0f / 4294967296.0f); }
    template <int MATH> __device__ __forceinline__ f3 in_unit_sphere() {
        float r = DevMath<MATH>::pow(f(), 0.33333f);
        float theta = 3.14159265358979f * f();
        float phi = 2.0f * 3.14159265358979f * f();
        float st, ct, sp, cp;
        DevMath<MATH>::sincos(theta, &st, &ct);
        DevMath<MATH>::sincos(phi, &sp, &cp);
        return mk(r * st * cp, r * st * sp, r * ct);
    }
    template <int MATH> __device__ __forceinline__ f3 in_unit_disk() {
        float r = sqrtf(f());
        float alpha = 2.0f * 3.14159265358979f * f();
        float sa, ca;
        DevMath<MATH>::sincos(alpha, &sa, &ca);
        return mk(r * ca, r * sa, 0.0f);
    }
};

// ---- traversal (bvh.hip.h:43-143, 145-276) ------------------------------------
__device__ __forceinline__ f3 safe_invdir(f3 d) {
    const float eps = 1e-5f;
    float x = fabsf(d.x) > eps ? d.x : (d.x < 0.0f ? -eps : eps);
    float y = fabsf(d.y) > eps ? d.y : (d.y < 0.0f ? -eps : eps);
    float z = fabsf(d.z) > eps ? d.z : (d.z < 0.0f ? -eps : eps);
    // __frcp_rn: the correctly rounded reciprocal, the same value as 1.0f / x
    return mk(__frcp_rn(x), __frcp_rn(y), __frcp_rn(z));
}

__device__ __forceinline__ bool aabb_hit(float4 mn, float4 mx, f3 inv, f3 oxinv, float t_min, float t_max) {
    float fx = mx.x * inv.x + oxinv.x, fy = mx.y * inv.y + oxinv.y, fz = mx.z * inv.z + oxinv.z;
    float nx = mn.x * inv.x + oxinv.x, ny = mn.y * inv.y + oxinv.y, nz = mn.z * inv.z + oxinv.z;
    float max_t = fminf(rt_min(rt_min(rt_max(fx, nx), rt_max(fy, ny)), rt_max(fz, nz)), t_max);
    float min_t = fmaxf(rt_max(rt_max(rt_min(fx, nx), rt_min(fy, ny)), rt_min(fz, nz)), t_min);
    return min_t <= max_t;
}

// The same slab test with fminf/fmaxf (one FMNMX each) in place of the
// reference's RT_MIN/RT_MAX (a compare and a select each).  For inputs
// without NaN the two forms return numerically equal values (they can only
// disagree on the sign of a zero result), and `min_t <= max_t` does not see
// zero signs, so the decision is identical.  The slab values are NaN-free
// whenever the ray origin and the box bounds are finite with magnitude below
// 1e30: |invdir| <= 1e5 by construction (safe_invdir), so every product and
// sum stays finite.  Callers use this form only under that condition
// (Walker::fast_slabs, SceneDev::exact_slabs).
__device__ __forceinline__ bool aabb_hit_fast(float4 mn, float4 mx, f3 inv, f3 oxinv, float t_min, float t_max) {
    float fx = mx.x * inv.x + oxinv.x, fy = mx.y * inv.y + oxinv.y, fz = mx.z * inv.z + oxinv.z;
    float nx = mn.x * inv.x + oxinv.x, ny = mn.y * inv.y + oxinv.y, nz = mn.z * inv.z + oxinv.z;
    float max_t = fminf(fminf(fminf(fmaxf(fx, nx), fmaxf(fy, ny)), fmaxf(fz, nz)), t_max);
    float min_t = fmaxf(fmaxf(fmaxf(fminf(fx, nx), fminf(fy, ny)), fminf(fz, nz)), t_min);
    return min_t <= max_t;
}

// A node's 64 bytes (two 256-bit read-only loads), loaded once per visit
// before the branch on the node's kind: a warp whose lanes visit nodes of
// different kinds then waits for one load latency per step, not one per kind.
struct Node {
    float4 a, b, c, e;
    __device__ __forceinline__ void load(const float4* p) {
        ldg8(p, &a, &b);
        ldg8(p + 2, &c, &e);
    }
};

// Both child tests of an internal node (bvh.hip.h:177-196): whether the ray
// (segment [t_min, t_max]) hits the left / right child's box, and the two
// child references.  FAST: the FMNMX form (aabb_hit_fast's condition).
template <bool FAST>
__device__ __forceinline__ void internal_test(const Node& nd, f3 inv, f3 oxinv, float t_min, float t_max,
                                              bool* hl, bool* hr, uint32_t* lref, uint32_t* rref) {
    *lref = bits(nd.a.w);
    *rref = bits(nd.b.w);
    if (FAST) {
        *hl = aabb_hit_fast(nd.a, nd.b, inv, oxinv, t_min, t_max);
        *hr = aabb_hit_fast(nd.c, nd.e, inv, oxinv, t_min, t_max);
    } else {
        *hl = aabb_hit(nd.a, nd.b, inv, oxinv, t_min, t_max);
        *hr = aabb_hit(nd.c, nd.e, inv, oxinv, t_min, t_max);
    }
}

// True when every component of o is finite with magnitude below 1e30.
__device__ __forceinline__ bool slab_safe(f3 o) {
    return fabsf(o.x) < 1e30f && fabsf(o.y) < 1e30f && fabsf(o.z) < 1e30f;
}

// Möller–Trumbore exactly as bvh.hip.h:72-117 (e1 = v1 - v0, e2 = v2 - v0):
// true when the hit distance t satisfies t_min <= t < t_max; (u, v) are the
// weights of v1 and v2.
// With the edges e1, e2 given (the triangle node stores them, computed with
// the same single-precision subtractions).
__device__ __forceinline__ bool tri_mt_edges(f3 o, f3 d, f3 v0, f3 e1, f3 e2, float t_min, float t_max,
                                             float* t_out, float* u_out, float* v_out) {
    const f3 s1 = cross(d, e2);
    const float det = dot(s1, e1);
    const float invd = __frcp_rn(det);   // correctly rounded, as 1.0f / det
    const f3 dd = sub(o, v0);
    const float u = dot(dd, s1) * invd;
    if (u < 0.0f || u > 1.0f) return false;
    const f3 s2 = cross(dd, e1);
    const float v = dot(d, s2) * invd;
    if (v < 0.0f || u + v > 1.0f) return false;
    const float t = dot(e2, s2) * invd;
    if (t < t_min || t > t_max || !(t < t_max)) return false;
    *t_out = t;
    *u_out = u;
    *v_out = v;
    return true;
}

__device__ __forceinline__ bool tri_mt(f3 o, f3 d, f3 v0, f3 v1, f3 v2, float t_min, float t_max, float* t_out,
                                       float* u_out, float* v_out) {
    const f3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    const f3 s1 = cross(d, e2);
    const float det = dot(s1, e1);
    const float invd = 1.0f / det;
    const f3 dd = sub(o, v0);
    const float u = dot(dd, s1) * invd;
    if (u < 0.0f || u > 1.0f) return false;
    const f3 s2 = cross(dd, e1);
    const float v = dot(d, s2) * invd;
    if (v < 0.0f || u + v > 1.0f) return false;
    const float t = dot(e2, s2) * invd;
    if (t < t_min || t > t_max || !(t < t_max)) return false;
    *t_out = t;
    *u_out = u;
    *v_out = v;
    return true;
}

__device__ __forceinline__ float comp(f3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

// Watertight ray/triangle test (Woop, Benthin, Wald, "Watertight Ray/Triangle
// Intersection", JCGT 2013): the ray is sheared so that it runs along +z
// from the origin, the triangle's 2-D edge functions U, V, W decide the hit
// (recomputed in double when one is exactly zero), so a ray through an edge
// or vertex shared by two triangles hits at least one of them.  Same
// acceptance rule and (u, v) meaning as tri_mt.  A non-parity option: it
// can decide edge cases differently from the reference's test.  Kept out of
// line so the reference test's path through the traversal loop keeps its
// registers.
static __device__ __noinline__ bool tri_watertight(f3 o, f3 d, f3 v0, f3 v1, f3 v2, float t_min, float t_max,
                                               float* t_out, float* u_out, float* v_out) {
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz == 2 ? 0 : kz + 1, ky = kx == 2 ? 0 : kx + 1;
    const float dz = comp(d, kz);
    if (dz < 0.0f) {
        const int tmp = kx;
        kx = ky;
        ky = tmp;
    }
    const float sx = comp(d, kx) / dz, sy = comp(d, ky) / dz, sz = 1.0f / dz;
    const f3 A = sub(v0, o), B = sub(v1, o), C = sub(v2, o);
    const float Ax = comp(A, kx) - sx * comp(A, kz), Ay = comp(A, ky) - sy * comp(A, kz);
    const float Bx = comp(B, kx) - sx * comp(B, kz), By = comp(B, ky) - sy * comp(B, kz);
    const float Cx = comp(C, kx) - sx * comp(C, kz), Cy = comp(C, ky) - sy * comp(C, kz);
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    float T = U * (sz * comp(A, kz)) + V * (sz * comp(B, kz)) + W * (sz * comp(C, kz));
    if (det < 0.0f) {
        det = -det;
        T = -T;
        V = -V;
        W = -W;
    }
    const float rcp = 1.0f / det;
    const float t = T * rcp;
    if (t < t_min || t > t_max || !(t < t_max)) return false;
    *t_out = t;
    *u_out = V * rcp;
    *v_out = W * rcp;
    return true;
}

struct HitRec {
    float t;
    uint32_t material;
    uint32_t type;   // ORN_NODE_SPHERE / ORN_NODE_MESH
    uint32_t inv;    // inverse transform index
    uint32_t tri;    // 3 * triangle id
    float u, v;
};

struct VisitCount {
    uint32_t visits, internal, sphere, mesh, tri;
};

// Closest hit of one ray; returns whether anything was hit.  `err` gets
// ERR_* bits when the ray is abandoned (the result is then a miss).
// Traversal stack: the first SS entries live in shared memory (entry i of
// this thread at sstack[i * sstride], so a warp's accesses hit 32 distinct
// banks), deeper entries spill to a per-thread local array; the total depth
// is the reference's 64.
template <int SS>
struct TravStack {
    uint32_t* sstack;
    int sstride;
    uint32_t lstack[kStackSize - SS > 0 ? kStackSize - SS : 1];
    __device__ __forceinline__ void put(int i, uint32_t v) {
        if (SS >= kStackSize || i < SS) sstack[i * sstride] = v;
        else lstack[i - SS] = v;
    }
    __device__ __forceinline__ uint32_t get(int i) const {
        if (SS >= kStackSize || i < SS) return sstack[i * sstride];
        return lstack[i - SS];
    }
};

template <bool COUNT, int SS>
__device__ __forceinline__ bool trace_ray(const SceneDev& sc, f3 ro, f3 rd, float t_min,
                                          HitRec* out, VisitCount* vc, uint32_t* err,
                                          uint32_t* sstack, int sstride) {
    float t_max = (float)3.40282e+38;
    TravStack<SS> stack;
    stack.sstack = sstack;
    stack.sstride = sstride;
    int sp = 0;
    uint32_t node = sc.root_ref;
    bool in_blas = false;
    int blas_sp = 0;
    f3 o = ro, d = rd;
    f3 inv = safe_invdir(d);
    f3 oxinv = mul(neg(o), inv);
    const f3 winv = inv, woxinv = oxinv;
    const bool wfast = !sc.exact_slabs && slab_safe(ro);
    bool fast = wfast;
    uint32_t material = 0, inv_id = 0;
    bool any = false;
    uint32_t visits = 0;
    for (;;) {
        if (++visits > kMaxVisitsPerRay) { *err |= ERR_VISITS; return false; }
        Node nd;
        nd.load(sc.nodes + 4 * (size_t)(node & kRefIndexMask));
        const float4 a = nd.a, b = nd.b, c = nd.c, e = nd.e;
        const uint32_t type = node >> 30;
        bool have_next = false;
        uint32_t next = 0;
        if (type == ORN_NODE_INTERNAL) {
            if (COUNT) vc->internal++;
            bool hl, hr;
            uint32_t lref, rref;
            if (fast) internal_test<true>(nd, inv, oxinv, t_min, t_max, &hl, &hr, &lref, &rref);
            else internal_test<false>(nd, inv, oxinv, t_min, t_max, &hl, &hr, &lref, &rref);
            if (hr) {
                next = rref;
                have_next = true;
                if (hl) {
                    if (sp >= kStackSize) { *err |= ERR_STACK; return false; }
                    stack.put(sp++, lref);
                }
            } else if (hl) {
                next = lref;
                have_next = true;
            }
        } else if (type == ORN_NODE_TRIANGLE) {
            if (COUNT) vc->tri++;
            const f3 v0 = mk(a.x, a.y, a.z);
            float t, u, v;
            const bool hit = sc.watertight
                                 ? tri_watertight(o, d, v0, mk(b.x, b.y, b.z), mk(c.x, c.y, c.z), t_min, t_max, &t, &u, &v)
                                 : tri_mt_edges(o, d, v0, mk(e.x, e.y, e.z), mk(b.w, c.w, e.w), t_min, t_max, &t, &u, &v);
            if (hit) {
                any = true;
                t_max = t;
                out->t = t;
                out->material = material;
                out->type = ORN_NODE_MESH;
                out->inv = inv_id;
                out->tri = bits(a.w) * 3u;
                out->u = u;
                out->v = v;
            }
        } else {
            // sphere or mesh entry; inverse rows 0..2: a, b, (c.xyz, e.x)
            float4 r2 = make_float4(c.x, c.y, c.z, e.x);
            f3 to = mk(dot4(a, o.x, o.y, o.z, 1.0f), dot4(b, o.x, o.y, o.z, 1.0f),
                       dot4(r2, o.x, o.y, o.z, 1.0f));
            f3 td = mk(dot4(a, d.x, d.y, d.z, 0.0f), dot4(b, d.x, d.y, d.z, 0.0f),
                       dot4(r2, d.x, d.y, d.z, 0.0f));
            uint32_t mat = bits(e.y);
            uint32_t inv_index = bits(e.z) * 2u;
            if (type == ORN_NODE_SPHERE) {
                if (COUNT) vc->sphere++;
                // sphere_hit, unit sphere at the origin
                float aa = td.x * td.x + td.y * td.y + td.z * td.z;
                float half_b = dot(to, td);
                float cc = (to.x * to.x + to.y * to.y + to.z * to.z) - 1.0f * 1.0f;
                float disc = half_b * half_b - aa * cc;
                float t = t_max;
                if (!(disc < 0.0f)) {
                    float sq = sqrtf(disc);
                    t = (-half_b - sq) / aa;
                    if (t < t_min || t_max < t) {
                        t = (-half_b + sq) / aa;
                        if (t < t_min || t_max < t) t = t_max;
                    }
                }
                if (t < t_max) {
                    any = true;
                    t_max = t;
                    out->t = t;
                    out->material = mat;
                    out->type = ORN_NODE_SPHERE;
                    out->inv = inv_index;
                }
            } else {
                if (COUNT) vc->mesh++;
                in_blas = true;
                blas_sp = sp;
                inv_id = inv_index;
                material = mat;
                o = to;
                d = td;
                inv = safe_invdir(d);
                oxinv = mul(neg(o), inv);
                fast = !sc.exact_slabs && slab_safe(to);
                next = bits(e.w);
                have_next = true;
            }
        }
        if (!have_next) {
            if (in_blas && sp == blas_sp) {
                in_blas = false;
                o = ro;
                d = rd;
                inv = winv;
                oxinv = woxinv;
                fast = wfast;
            }
            if (sp == 0) break;
            next = stack.get(--sp);
        }
        node = next;
    }
    if (COUNT) vc->visits += visits;
    return any;
}

// ---- texture fetch (material.hip.h:30-33) ---------------------------------------
__device__ __forceinline__ int tex_index(float c, uint32_t n, bool clamp_mode) {
    if (!(c == c)) c = 0.0f;
    float x = clamp_mode ? floorf(c * (float)n) : floorf((c - floorf(c)) * (float)n);
    if (x > (float)(n - 1)) x = (float)(n - 1);
    if (x < 0.0f) x = 0.0f;
    return (int)x;
}

__device__ __forceinline__ float half_bits_to_float(uint32_t h) {
    return __half2float(__ushort_as_half((unsigned short)h));
}

__device__ __forceinline__ f3 tex_sample(const TexDesc& t, float u, float v, bool clamp_mode) {
    int x = tex_index(u, t.width, clamp_mode), y = tex_index(v, t.height, clamp_mode);
    const unsigned char* row = t.data + (size_t)y * t.pitch;
    if (t.format == ORN_TEXEL_RGBA8) {
        uint32_t p = __ldg((const unsigned int*)(row + (size_t)x * 4));
        return mk((float)(p & 0xffu) / 255.0f, (float)((p >> 8) & 0xffu) / 255.0f,
                  (float)((p >> 16) & 0xffu) / 255.0f);
    }
    uint2 p = __ldg((const uint2*)(row + (size_t)x * 8));
    return mk(half_bits_to_float(p.x & 0xffffu), half_bits_to_float(p.x >> 16),
              half_bits_to_float(p.y & 0xffffu));
}

struct SampleCount {
    uint32_t rays, sphere_hits, mesh_hits, textured;
};

// ---- one sample (pathtracer.hip.cpp:72-146), in pieces ----------------------
// Camera ray for pixel (px, py): 2 jitter draws, then the lens-disk draws
// (camera.hip.h:25-33), consumed even when the aperture is 0.
template <int MATH>
__device__ __forceinline__ void camera_ray(const orn_constant_params& cp, uint32_t px, uint32_t py, Rng& rng,
                                           f3* ro, f3* rd) {
    float u = ((float)px + rng.f()) / (float)(cp.width - 1);
    float v = ((float)py + rng.f()) / (float)(cp.height - 1);
    const orn_camera& cam = cp.camera;
    f3 disk = rng.in_unit_disk<MATH>();
    f3 rdv = scale(cam.lens_radius, disk);
    f3 cu = mk(cam.u[0], cam.u[1], cam.u[2]), cv = mk(cam.v[0], cam.v[1], cam.v[2]);
    f3 origin = mk(cam.origin[0], cam.origin[1], cam.origin[2]);
    f3 offset = add(scale(rdv.x, cu), scale(rdv.y, cv));
    f3 llc = mk(cam.lower_left_corner[0], cam.lower_left_corner[1], cam.lower_left_corner[2]);
    f3 hor = mk(cam.horizontal[0], cam.horizontal[1], cam.horizontal[2]);
    f3 ver = mk(cam.vertical[0], cam.vertical[1], cam.vertical[2]);
    *ro = add(origin, offset);
    *rd = sub(sub(add(add(llc, scale(u, hor)), scale(v, ver)), origin), offset);
}

// The same camera ray from given uniforms (jitter ju, jv; lens l0, l1) —
// the cached renderer's Sobol sampler.
template <int MATH>
__device__ __forceinline__ void camera_ray_from(const orn_constant_params& cp, uint32_t px, uint32_t py, float ju,
                                                float jv, float l0, float l1, f3* ro, f3* rd) {
    float u = ((float)px + ju) / (float)(cp.width - 1);
    float v = ((float)py + jv) / (float)(cp.height - 1);
    const orn_camera& cam = cp.camera;
    const float r = sqrtf(l0);
    float sa, ca;
    DevMath<MATH>::sincos(2.0f * 3.14159265358979f * l1, &sa, &ca);
    f3 rdv = scale(cam.lens_radius, mk(r * ca, r * sa, 0.0f));
    f3 cu = mk(cam.u[0], cam.u[1], cam.u[2]), cv = mk(cam.v[0], cam.v[1], cam.v[2]);
    f3 origin = mk(cam.origin[0], cam.origin[1], cam.origin[2]);
    f3 offset = add(scale(rdv.x, cu), scale(rdv.y, cv));
    f3 llc = mk(cam.lower_left_corner[0], cam.lower_left_corner[1], cam.lower_left_corner[2]);
    f3 hor = mk(cam.horizontal[0], cam.horizontal[1], cam.horizontal[2]);
    f3 ver = mk(cam.vertical[0], cam.vertical[1], cam.vertical[2]);
    *ro = add(origin, offset);
    *rd = sub(sub(add(add(llc, scale(u, hor)), scale(v, ver)), origin), offset);
}

// Miss: sky gradient (pathtracer.hip.cpp:87-93).
__device__ __forceinline__ f3 sky_color(f3 color, f3 rd) {
    f3 ud = normalize(rd);
    float tt = 0.5f * (ud.y + 1.0f);
    f3 sky = add(scale(1.0f - tt, mk(1.0f, 1.0f, 1.0f)), scale(tt, mk(0.5f, 0.7f, 1.0f)));
    return mul(color, sky);
}

// Surface point of a hit (pathtracer.hip.cpp:95-131): position, the normal
// facing the incoming ray, the side, and the texture coordinates.
struct HitGeom {
    f3 hp, normal;
    bool front;
    float hu, hv;
};

template <int MATH, bool COUNT>
__device__ __forceinline__ HitGeom hit_geometry(const SceneDev& sc, const HitRec& h, f3 ro, f3 rd, SampleCount* scn) {
    typedef DevMath<MATH> M;
    HitGeom g;
    uint32_t transform_id = h.inv + 1u;
    g.hp = add(ro, scale(h.t, rd));
    if (h.type == ORN_NODE_SPHERE) {
        if (COUNT) scn->sphere_hits++;
        const float4* m = sc.xforms + 4 * (size_t)transform_id;
        f3 center = mk(dot4(ldg4(m), 0.0f, 0.0f, 0.0f, 1.0f), dot4(ldg4(m + 1), 0.0f, 0.0f, 0.0f, 1.0f),
                       dot4(ldg4(m + 2), 0.0f, 0.0f, 0.0f, 1.0f));
        f3 on = normalize(sub(g.hp, center));
        float theta = M::acos(-on.y);
        float phi = M::atan2(-on.z, on.x) + 3.14159265358979f;
        g.hu = phi / (2.0f * 3.14159265358979f);
        g.hv = theta / 3.14159265358979f;
        if (dot(rd, on) > 0.0f) { g.normal = neg(on); g.front = false; }
        else { g.normal = on; g.front = true; }
    } else {
        if (COUNT) scn->mesh_hits++;
        float4 n0 = ldg4(sc.normals + __ldg(sc.normal_indices + h.tri));
        float4 n1 = ldg4(sc.normals + __ldg(sc.normal_indices + h.tri + 1));
        float4 n2 = ldg4(sc.normals + __ldg(sc.normal_indices + h.tri + 2));
        float2 t0 = __ldg(sc.uvs + __ldg(sc.uv_indices + h.tri));
        float2 t1 = __ldg(sc.uvs + __ldg(sc.uv_indices + h.tri + 1));
        float2 t2 = __ldg(sc.uvs + __ldg(sc.uv_indices + h.tri + 2));
        float w = 1.0f - h.u - h.v;
        float nx = w * n0.x + h.u * n1.x + h.v * n2.x;
        float ny = w * n0.y + h.u * n1.y + h.v * n2.y;
        float nz = w * n0.z + h.u * n1.z + h.v * n2.z;
        g.hu = w * t0.x + h.u * t1.x + h.v * t2.x;
        g.hv = w * t0.y + h.u * t1.y + h.v * t2.y;
        const float4* m = sc.xforms + 4 * (size_t)h.inv;
        float4 m0 = ldg4(m), m1 = ldg4(m + 1), m2 = ldg4(m + 2), m3 = ldg4(m + 3);
        f3 tn = mk(m0.x * nx + m1.x * ny + m2.x * nz + m3.x * 0.0f,
                   m0.y * nx + m1.y * ny + m2.y * nz + m3.y * 0.0f,
                   m0.z * nx + m1.z * ny + m2.z * nz + m3.z * 0.0f);
        f3 on = normalize(tn);
        if (dot(rd, on) > 0.0f) { g.normal = neg(on); g.front = false; }
        else { g.normal = on; g.front = true; }
    }
    return g;
}

// Hit shading and material (pathtracer.hip.cpp:95-145, material.hip.h):
// returns true when the path continues with the scattered ray in (ro, rd),
// false when it ends (emission or absorption) with `color` final.
// `preset` (the cached renderer's Sobol sampler): a lambertian scatter takes
// the polar and azimuthal uniforms of its in_unit_sphere direction from
// (pu_theta, pu_phi) instead of the stream (the radius is normalised away).
template <int SEM, int MATH, bool COUNT>
__device__ __forceinline__ bool shade_geom(const SceneDev& sc, const orn_constant_params& cp, Rng& rng,
                                           const HitRec& h, const HitGeom& g, f3* ro_io, f3* rd_io,
                                           f3* color_io, SampleCount* scn, bool preset = false,
                                           float pu_theta = 0.0f, float pu_phi = 0.0f) {
    typedef DevMath<MATH> M;
    const f3 rd = *rd_io;
    f3 color = *color_io;
    const f3 hp = g.hp, normal = g.normal;
    const bool front = g.front;
    const float hu = g.hu, hv = g.hv;
    float4 ma = ldg4(sc.materials + 2 * (size_t)h.material);
    float4 mb = ldg4(sc.materials + 2 * (size_t)h.material + 1);
    uint32_t mtype = bits(mb.z);
    uint32_t tex_id = bits(ma.w);
    bool use_tex = SEM == SEM_WGSL ? (tex_id < cp.textures_count && tex_id < sc.textures_len)
                                   : tex_id < sc.textures_len;
    if (mtype == ORN_LAMBERTIAN) {
        f3 s;
        if (preset) {
            float st, ct, sp, cph;
            DevMath<MATH>::sincos(3.14159265358979f * pu_theta, &st, &ct);
            DevMath<MATH>::sincos(2.0f * 3.14159265358979f * pu_phi, &sp, &cph);
            s = mk(st * cph, st * sp, ct);
        } else {
            s = rng.in_unit_sphere<MATH>();
        }
        f3 dir = add(normal, normalize(s));
        if (fabsf(dir.x) < 1e-8f && fabsf(dir.y) < 1e-8f && fabsf(dir.z) < 1e-8f) dir = normal;
        f3 att = use_tex ? tex_sample(sc.textures[tex_id], hu, hv, SEM == SEM_WGSL) : mk(ma.x, ma.y, ma.z);
        if (COUNT && use_tex) scn->textured++;
        *ro_io = hp;
        *rd_io = dir;
        *color_io = mul(color, att);
        return true;
    }
    if (mtype == ORN_METAL) {
        f3 dir = add(reflect(normalize(rd), normal), scale(mb.x, rng.in_unit_sphere<MATH>()));
        f3 att = use_tex ? tex_sample(sc.textures[tex_id], hu, hv, SEM == SEM_WGSL) : mk(ma.x, ma.y, ma.z);
        if (COUNT && use_tex) scn->textured++;
        if (SEM == SEM_WGSL && !(dot(dir, normal) > 0.0f)) {
            *color_io = mul(color, mk(0.0f, 0.0f, 0.0f));
            return false;
        }
        *ro_io = hp;
        *rd_io = dir;
        *color_io = mul(color, att);
        return true;
    }
    if (mtype == ORN_DIELECTRIC) {
        float ior = mb.y;
        float ratio = front ? 1.0f / ior : ior;
        f3 ud = normalize(rd);
        float cos_t = fminf(dot(neg(ud), normal), 1.0f);
        float sin_t = sqrtf(1.0f - cos_t * cos_t);
        bool refl = ratio * sin_t > 1.0f;
        if (!refl) {
            float r0 = (1.0f - ratio) / (1.0f + ratio);
            r0 = r0 * r0;
            float pr = r0 + (1.0f - r0) * M::pow(1.0f - cos_t, 5.0f);
            refl = pr > rng.f();
        }
        f3 dir = refl ? reflect(ud, normal) : refract(ud, normal, ratio);
        *ro_io = hp;
        *rd_io = dir;
        *color_io = mul(color, mk(1.0f, 1.0f, 1.0f));
        return true;
    }
    f3 em = mk(0.0f, 0.0f, 0.0f);
    if (mtype == ORN_DIFFUSE_LIGHT) {
        em = use_tex ? tex_sample(sc.textures[tex_id], hu, hv, SEM == SEM_WGSL) : mk(ma.x, ma.y, ma.z);
        if (COUNT && use_tex) scn->textured++;
    }
    *color_io = mul(color, em);
    return false;
}

template <int SEM, int MATH, bool COUNT>
__device__ __forceinline__ bool shade_hit(const SceneDev& sc, const orn_constant_params& cp, Rng& rng,
                                          const HitRec& h, f3* ro_io, f3* rd_io, f3* color_io,
                                          SampleCount* scn) {
    const HitGeom g = hit_geometry<MATH, COUNT>(sc, h, *ro_io, *rd_io, scn);
    return shade_geom<SEM, MATH, COUNT>(sc, cp, rng, h, g, ro_io, rd_io, color_io, scn);
}

// One whole sample with the straightforward loop structure (used by the
// debug kernels; the render kernel runs the same pieces as a state machine).
template <int SEM, int MATH, bool COUNT, int SS>
__device__ __forceinline__ f3 trace_sample(const SceneDev& sc, const orn_constant_params& cp,
                                           uint32_t px, uint32_t py, Rng& rng, VisitCount* vc,
                                           SampleCount* scn, uint32_t* err, uint32_t* sstack,
                                           int sstride) {
    f3 ro, rd;
    camera_ray<MATH>(cp, px, py, rng, &ro, &rd);
    f3 color = mk(1.0f, 1.0f, 1.0f);
    for (uint32_t i = 0; i < cp.depth; ++i) {
        HitRec h;
        h.tri = 0;
        h.u = 0.0f;
        h.v = 0.0f;
        if (COUNT) scn->rays++;
        if (!trace_ray<COUNT, SS>(sc, ro, rd, cp.ray_cast_epsilon, &h, vc, err, sstack, sstride)) {
            if (*err) return mk(0.0f, 0.0f, 0.0f);
            color = sky_color(color, rd);
            break;
        }
        if (!shade_hit<SEM, MATH, COUNT>(sc, cp, rng, h, &ro, &rd, &color, scn)) break;
    }
    return color;
}

// Solid-angle density of the reference's lambertian scatter direction
// w = normalize(n + s), s = normalize(in_unit_sphere()) (material.hip.h,
// random.hip.h), whose polar angle about the world z axis is uniform in
// [0, pi]: p_s(s) = 1 / (2 pi^2 sin(theta_s)).  The map s -> w takes the unit
// sphere around n (through the origin) to directions with cos(a) = n.w and
// |n + s| = 2 cos(a), so p(w) = 4 cos(a) p_s(s) with s = 2 cos(a) w - n.
// (The direction is not cosine-distributed.)
__device__ __forceinline__ float scatter_pdf(f3 n, f3 w) {
    const float ca = dot(n, w);
    if (!(ca > 0.0f)) return 0.0f;
    const f3 sv = sub(scale(2.0f * ca, w), n);
    const float sin_s = fmaxf(sqrtf(sv.x * sv.x + sv.y * sv.y), 1e-7f);
    return 2.0f * ca / (9.8696044f * sin_s);
}

// post_processing (pathtracer.hip.cpp:58-70; pathtracer.wgsl:81-93)
template <int SEM, int MATH>
__device__ __forceinline__ float4 post_process(float4 acc, float ci, float inv_gamma) {
    float q[4] = {acc.x / ci, acc.y / ci, acc.z / ci, acc.w / ci};
#pragma unroll
    for (int k = 0; k < 4; ++k)
        q[k] = SEM == SEM_WGSL ? fminf(fmaxf(q[k], 0.0f), 1.0f) : fmaxf(fminf(q[k], 1.0f), 0.0f);
#pragma unroll
    for (int k = 0; k < 3; ++k) q[k] = DevMath<MATH>::pow(q[k], inv_gamma);
    return make_float4(q[0], q[1], q[2], q[3]);
}

}  // namespace orn
