// pt_machine.cuh — the megakernel as a warp-synchronous state machine.
//
// A path tracer's work per sample varies by two orders of magnitude (a sky
// pixel costs ~20 node visits, a pixel on a glass object several hundred),
// and the nested loops of the straightforward form (samples → bounces →
// traversal) let the lanes of a warp drift apart: measured with ncu on
// sm_103a, the nested-loop megakernel ran with 1.08 active threads per warp.
//
// Here every lane holds one path and the warp runs ONE loop whose condition
// comes from warp ballots, so the lanes stay converged:
//   * each iteration, every lane in the TRAVERSE state visits one BVH node;
//   * lanes whose ray finished traversal wait in SHADE until enough of the
//     warp is ready (or nobody is traversing), then all ready lanes shade
//     together (material scatter, next bounce, next sample, pixel done);
//   * lanes without a pixel take the next ones from a global counter, one
//     atomic per warp (persistent threads, dynamic load balance).
// Each pixel's own sequence of operations is unchanged — the same RNG draws,
// the same float operations in the same order — so the result is
// bit-identical to the reference's per-pass loop.
#pragma once

#include "pt_device.cuh"

namespace orn {

// Traversal state of one ray, advanced one node per step
// (bvh.hip.h:145-276 visit order; see trace_ray).  `node` is a typed node
// reference (pt_scene.h).
struct Walker {
    uint32_t node;
    int sp;
    int blas_sp;
    bool in_blas;
    bool any;
    f3 o, d, inv, oxinv;
    float t_max;
    uint32_t material, inv_id;
    uint32_t visits;
    // any-hit shadow rays (walker_step<..., ANY = true>): a hit before occl_t
    // on an instance other than occl_inv ends the traversal (occluded);
    // occl_inv = ~0 for ordinary rays
    uint32_t occl_inv;
    float occl_t;
};

__device__ __forceinline__ void walker_begin(Walker& w, const SceneDev& sc, f3 ro, f3 rd) {
    w.node = sc.root_ref;
    w.sp = 0;
    w.blas_sp = 0;
    w.in_blas = false;
    w.any = false;
    w.occl_inv = 0xffffffffu;
    w.occl_t = 0.0f;
    w.o = ro;
    w.d = rd;
    w.inv = safe_invdir(rd);
    w.oxinv = mul(neg(ro), w.inv);
    w.t_max = (float)3.40282e+38;
    w.material = 0;
    w.inv_id = 0;
    w.visits = 0;
}

// Visits the lane's current node; returns false when the traversal has
// finished.  The three node kinds are separate branches; a warp runs each
// branch that any of its lanes needs (grouping lanes by node kind measured
// slower on sm_103a: the lanes kept waiting cost more than the divergence).
// FAST selects the FMNMX slab test (aabb_hit_fast); the host decides per
// render whether every ray of the render satisfies its condition
// (render_fast_slabs in capi.cu).
// CHECK: count the visit and apply the per-ray visit limit here; a caller
// that passes false counts the visits of a whole round of steps itself
// (walker_account_round) and the COUNT statistics are then unavailable.
template <bool COUNT, int SS, bool FAST, bool ANY = false, bool CHECK = true>
__device__ __forceinline__ bool walker_step(Walker& w, const SceneDev& sc, f3 ro, f3 rd, float t_min,
                                            HitRec* out, TravStack<SS>& stack, VisitCount* vc,
                                            uint32_t* err) {
    static_assert(CHECK || !COUNT, "visit statistics need the per-step count");
    if (CHECK && ++w.visits > kMaxVisitsPerRay) { *err |= ERR_VISITS; w.any = false; return false; }
    const uint32_t type = w.node >> 30;
    bool have_next = false;
    uint32_t next = 0;
    // the node's 64 bytes, loaded before the branch on its kind (measured
    // on the 1080p workload: 345 against 278 Msamples/s with a load inside
    // each branch, whose latencies a warp then waits for one after another)
    Node nd;
    nd.load(sc.nodes + 4 * (size_t)(w.node & kRefIndexMask));
    if (type == ORN_NODE_INTERNAL) {
        if (COUNT) vc->internal++;
        bool hl, hr;
        uint32_t lref, rref;
        internal_test<FAST>(nd, w.inv, w.oxinv, t_min, w.t_max, &hl, &hr, &lref, &rref);
        if (hr) {
            next = rref;
            have_next = true;
            if (hl) {
                if (w.sp >= kStackSize) { *err |= ERR_STACK; w.any = false; return false; }
                stack.put(w.sp++, lref);
            }
        } else if (hl) {
            next = lref;
            have_next = true;
        }
    } else if (type == ORN_NODE_TRIANGLE) {
        if (COUNT) vc->tri++;
        const float4 a = nd.a, b = nd.b, c = nd.c, e = nd.e;
        const f3 v0 = mk(a.x, a.y, a.z);
        float t, u, v;
        const bool hit = sc.watertight
                             ? tri_watertight(w.o, w.d, v0, mk(b.x, b.y, b.z), mk(c.x, c.y, c.z), t_min, w.t_max, &t, &u, &v)
                             : tri_mt_edges(w.o, w.d, v0, mk(e.x, e.y, e.z), mk(b.w, c.w, e.w), t_min, w.t_max, &t, &u, &v);
        if (hit) {
            w.any = true;
            w.t_max = t;
            out->t = t;
            out->material = w.material;
            out->type = ORN_NODE_MESH;
            out->inv = w.inv_id;
            out->tri = bits(a.w) * 3u;
            out->u = u;
            out->v = v;
            if (ANY && w.occl_inv != 0xffffffffu && w.inv_id != w.occl_inv && t < w.occl_t) {
                if (COUNT) vc->visits += w.visits;
                return false;   // an occluder: the closest hit cannot be the sampled light
            }
        }
    } else {
        const float4 a = nd.a, b = nd.b, c = nd.c, e = nd.e;
        float4 r2 = make_float4(c.x, c.y, c.z, e.x);
        f3 to = mk(dot4(a, w.o.x, w.o.y, w.o.z, 1.0f), dot4(b, w.o.x, w.o.y, w.o.z, 1.0f),
                   dot4(r2, w.o.x, w.o.y, w.o.z, 1.0f));
        f3 td = mk(dot4(a, w.d.x, w.d.y, w.d.z, 0.0f), dot4(b, w.d.x, w.d.y, w.d.z, 0.0f),
                   dot4(r2, w.d.x, w.d.y, w.d.z, 0.0f));
        uint32_t mat = bits(e.y);
        uint32_t inv_index = bits(e.z) * 2u;
        if (type == ORN_NODE_SPHERE) {
            if (COUNT) vc->sphere++;
            float aa = td.x * td.x + td.y * td.y + td.z * td.z;
            float half_b = dot(to, td);
            float cc = (to.x * to.x + to.y * to.y + to.z * to.z) - 1.0f * 1.0f;
            float disc = half_b * half_b - aa * cc;
            float t = w.t_max;
            if (!(disc < 0.0f)) {
                float sq = sqrtf(disc);
                t = (-half_b - sq) / aa;
                if (t < t_min || w.t_max < t) {
                    t = (-half_b + sq) / aa;
                    if (t < t_min || w.t_max < t) t = w.t_max;
                }
            }
            if (t < w.t_max) {
                w.any = true;
                w.t_max = t;
                out->t = t;
                out->material = mat;
                out->type = ORN_NODE_SPHERE;
                out->inv = inv_index;
                if (ANY && w.occl_inv != 0xffffffffu && t < w.occl_t) {
                    if (COUNT) vc->visits += w.visits;
                    return false;   // spheres never carry sampled lights
                }
            }
        } else {
            if (COUNT) vc->mesh++;
            w.in_blas = true;
            w.blas_sp = w.sp;
            w.inv_id = inv_index;
            w.material = mat;
            w.o = to;
            w.d = td;
            w.inv = safe_invdir(td);
            w.oxinv = mul(neg(to), w.inv);
            next = bits(e.w);
            have_next = true;
        }
    }
    if (!have_next) {
        if (w.in_blas && w.sp == w.blas_sp) {
            w.in_blas = false;
            w.o = ro;
            w.d = rd;
            // recomputed rather than kept: six registers fewer for every
            // step (measured +0.8 % on the 1080p step)
            w.inv = safe_invdir(rd);
            w.oxinv = mul(neg(ro), w.inv);
        }
        if (w.sp == 0) {
            if (COUNT) vc->visits += w.visits;
            return false;
        }
        next = stack.get(--w.sp);
    }
    w.node = next;
    return true;
}

// After a round of `steps` walker_step<..., CHECK = false> calls on a ray
// that is still traversing: counts them and applies the per-ray visit limit
// (the limit then acts up to one round late); false when the ray is given up.
__device__ __forceinline__ bool walker_account_round(Walker& w, uint32_t steps, uint32_t* err) {
    w.visits += steps;
    if (w.visits > kMaxVisitsPerRay) {
        *err |= ERR_VISITS;
        w.any = false;
        return false;
    }
    return true;
}

}  // namespace orn
