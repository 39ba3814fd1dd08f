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
#include "qmc.cuh"

namespace orn {

enum LaneMode { LANE_IDLE = 0, LANE_TRAVERSE = 1, LANE_SHADE = 2, LANE_DONE = 3 };


// Per-pixel accumulation: FP32 RGBA as the reference keeps it
// (pathtracer.hip.cpp:148-153), or FP64 for the high-sample-count oracle
// render (orn_render_f64), where only the accumulation is double.
template <bool F64> struct Accum;
template <> struct Accum<false> {
    float4 v;
    __device__ void load(const RenderLaunch& p, uint32_t gid, float ci0) {
        v = ci0 > 1.0f ? p.acc[gid] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    __device__ void add(float ci, f3 c) {
        if (ci > 1.0f) v = make_float4(v.x + c.x, v.y + c.y, v.z + c.z, v.w + 1.0f);
        else v = make_float4(c.x, c.y, c.z, 1.0f);
    }
    __device__ void store(const RenderLaunch& p, uint32_t gid) { p.acc[gid] = v; }
};
template <> struct Accum<true> {
    double x, y, z, w;
    __device__ void load(const RenderLaunch& p, uint32_t gid, float ci0) {
        if (ci0 > 1.0f) {
            const double* a = p.acc64 + 4 * (size_t)gid;
            x = a[0]; y = a[1]; z = a[2]; w = a[3];
        } else {
            x = y = z = w = 0.0;
        }
    }
    __device__ void add(float ci, f3 c) {
        if (ci > 1.0f) { x += (double)c.x; y += (double)c.y; z += (double)c.z; w += 1.0; }
        else { x = c.x; y = c.y; z = c.z; w = 1.0; }
    }
    __device__ void store(const RenderLaunch& p, uint32_t gid) {
        double* a = p.acc64 + 4 * (size_t)gid;
        a[0] = x; a[1] = y; a[2] = z; a[3] = w;
    }
};

// The render kernel: persistent threads, one path per lane, run as a
// warp-synchronous state machine (pt_machine.cuh).  Pixels are handed out
// 32 at a time from p.work_counter; each pixel runs its p.spp passes with the
// accumulation and RNG state in registers, then writes them back (and the
// post-processed framebuffer value when p.do_post).
//
// CACHE: the radiance-cache variant (one sample per pixel; CacheLaunch in
// pt_kernels.h).  A regular pixel's path stops at its cache vertex (the
// first rough surface from the second vertex on) and leaves a query there; a
// training pixel's path runs to the end and records the network inputs at
// the cache vertex and the radiance that left it.
// Resident blocks per SM the CACHE variant is compiled for (register cap).
// Measured on cached + batched 1920x1080 frames (ms per frame): 3 blocks
// (152 registers, no spills) 63.5, 4 (128) 59.9, 5 (96) 58.1, 6 (80) 55.6,
// 7 (72) 55.0, 8 (64) 59.4 — more warps in flight outweigh the register
// spills up to 7.
#ifndef ORN_CACHE_MIN_BLOCKS
#define ORN_CACHE_MIN_BLOCKS 7
#endif
template <int SEM, int MATH, bool COUNT, bool FAST, bool F64 = false, bool CACHE = false, bool SOBOL = false>
__global__ void __launch_bounds__(kMegaBlock, CACHE ? ORN_CACHE_MIN_BLOCKS : kMegaMinBlocks)
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
    uint32_t steps = 0;              // traversal steps of the current pixel (its cost)
    uint32_t stream = 0;             // cached launches: the sample stream of the current item
    const uint32_t items = CACHE ? p.pixel_count * p.cache.streams : p.pixel_count;
    const bool atomic_acc = CACHE && p.cache.streams > 1u;
    bool vertex = false;             // cached launches: this shading step reached a cache vertex
    Rng rng{0};
    Accum<F64> acc;
    acc.load(p, 0, 0.0f);
    f3 ro = mk(0.0f, 0.0f, 0.0f), rd = ro, color = ro;
    HitRec h;
    h.t = 0.0f; h.material = 0; h.type = 0; h.inv = 0; h.tri = 0; h.u = 0.0f; h.v = 0.0f;
    Walker w;
    VisitCount vc = {0, 0, 0, 0, 0};
    SampleCount scn = {0, 0, 0, 0};
    uint32_t err = 0;
    // radiance cache: the pixel's training slot (or ~0), whether the current
    // sample recorded its cache vertex, and its throughput up to there
    uint32_t tslot = 0xffffffffu;
    bool v2 = false;
    f3 pre = mk(1.0f, 1.0f, 1.0f);
    // cached variant: radiance gathered so far (L; Lpre before the cache
    // vertex), and a pending light sample (its contribution, and the
    // scattered ray to trace after its shadow ray)
    f3 L = mk(0.0f, 0.0f, 0.0f), Lpre = L, nee_c = L, sro = L, srd = L, nprev = L;
    bool shadow = false, nee_prev = false, shadow_end = false, shadow_pre = false;
    uint32_t shadow_inv = 0;
    f3 qthr = mk(0.0f, 0.0f, 0.0f);   // a query's throughput x surface colour

    // Adds a finished sample to the pixel: in registers, or atomically when
    // several streams of a cached launch share the pixel.
    auto add_sample = [&](f3 c) {
        if (atomic_acc) {
            float* a = reinterpret_cast<float*>(p.acc + gid);
            atomicAdd(a + 0, c.x);
            atomicAdd(a + 1, c.y);
            atomicAdd(a + 2, c.z);
            atomicAdd(a + 3, 1.0f);
        } else {
            acc.add(ci0 + (float)k, c);
        }
    };

    // Starts sample k of the current pixel; returns the lane's next mode.
    // Samples with depth 0 finish immediately (the bounce loop never runs).
    auto start_samples = [&]() -> int {
        while (k < p.spp) {
            if (CACHE && SOBOL) {
                // the pixel's seed and the sample's index since the last camera
                // change (one pass per launch: index = first pass - 1 + stream)
                const uint32_t qseed = qmc_hash(gid + 1u), qidx = (uint32_t)ci0 - 1u + stream;
                float ju, jv, l0, l1;
                qmc_point(qseed, QMC_PIXEL, qidx, &ju, &jv);
                qmc_point(qseed, QMC_LENS, qidx, &l0, &l1);
                camera_ray_from<MATH>(p.cp, gid % W, gid / W, ju, jv, l0, l1, &ro, &rd);
            } else {
                camera_ray<MATH>(p.cp, gid % W, gid / W, rng, &ro, &rd);
            }
            color = mk(1.0f, 1.0f, 1.0f);
            bounce = 0;
            if (CACHE) {
                v2 = false;
                shadow = false;
                shadow_end = false;
                shadow_pre = false;
                nee_prev = false;
                L = mk(0.0f, 0.0f, 0.0f);
            }
            if (p.cp.depth > 0) {
                if (COUNT) scn.rays++;
                walker_begin(w, p.scene, ro, rd);
                return LANE_TRAVERSE;
            }
            add_sample(color);
            ++k;
        }
        if (CACHE && stream > 0u) {
            p.cache.rng_extra[(size_t)(stream - 1u) * p.pixel_count + gid] = rng.state;
        } else {
            if (!atomic_acc) acc.store(p, gid);
            p.rng[gid] = rng.state;
        }
        if (p.cost) p.cost[gid] = steps;
        if constexpr (!F64 && !CACHE) {
            if (p.do_post) {
                uint32_t x = gid % W, y = gid / W;
                uint32_t fbi = p.cp.flip_y != 0 ? W * (H - y - 1) + x : gid;
                p.fb[fbi] = post_process<SEM, MATH>(acc.v, ci0 + (float)(p.spp - 1), p.cp.inverted_gamma);
            }
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
            if (base + n >= items) exhausted = true;
            if (mode == LANE_IDLE) {
                uint32_t mine = base + __popc(idle & lanes_below);
                if (mine < items) {
                    steps = 0;
                    k = 0;
                    if constexpr (CACHE) {
                        stream = mine / p.pixel_count;
                        gid = mine - stream * p.pixel_count;
                        rng.state = stream > 0u ? p.cache.rng_extra[(size_t)(stream - 1u) * p.pixel_count + gid]
                                                : p.rng[gid];
                        if (atomic_acc) acc.load(p, gid, 0.0f);   // zero: the samples are added atomically
                        else acc.load(p, gid, ci0);
                        tslot = 0xffffffffu;   // decided at the cache vertex
                    } else {
                        gid = p.order ? p.order[mine] : mine;
                        rng.state = p.rng[gid];
                        acc.load(p, gid, ci0);
                    }
                    mode = start_samples();
                }
            }
        }
        if (exhausted && mode == LANE_IDLE) mode = LANE_DONE;
        if (__ballot_sync(kFull, mode == LANE_TRAVERSE || mode == LANE_SHADE) == 0u &&
            __ballot_sync(kFull, mode == LANE_IDLE) == 0u)
            break;

        if (mode == LANE_TRAVERSE) {
            // a round of up to kStepsPerIteration node visits; the plain kernel
            // counts them (pixel cost, per-ray visit limit) once per round.
            // (Ending a round early once enough lanes wait to be shaded,
            // checked every 4 / 8 / 16 steps, measured 3.5 / 1.8 / 1.0 %
            // slower: the extra ballots cost more than the waiting lanes.)
            constexpr bool kPerStep = COUNT || CACHE || F64;
            uint32_t s = 0;
#pragma unroll 1
            while (s < (uint32_t)kStepsPerIteration) {
                ++s;
                if (!walker_step<COUNT, kSmemStack, FAST, CACHE, kPerStep>(w, p.scene, ro, rd, p.cp.ray_cast_epsilon,
                                                                           &h, stack, &vc, &err)) {
                    mode = LANE_SHADE;
                    break;
                }
            }
            steps += s;
            if (!kPerStep && mode == LANE_TRAVERSE && !walker_account_round(w, s, &err)) mode = LANE_SHADE;
        }

        const unsigned ready = __ballot_sync(kFull, mode == LANE_SHADE);
        const unsigned busy = __ballot_sync(kFull, mode == LANE_TRAVERSE);
        if (ready != 0u && ((int)__popc(ready) >= p.shade_threshold || busy == 0u)) {
            if (mode == LANE_SHADE) {
                if constexpr (CACHE) {
                    bool end = false, query = false;
                    vertex = false;
                    float qin[kCacheInputs];
                    if (shadow) {
                        // the shadow ray of a light sample finished: add the sample
                        // if unoccluded, then trace the scattered ray
                        shadow = false;
                        if (w.any && !err && h.type == ORN_NODE_MESH && h.inv == shadow_inv &&
                            __ldg(p.cache.light_material + h.material) != 0u) {
                            if (shadow_pre) Lpre = add(Lpre, nee_c);
                            else L = add(L, nee_c);
                        }
                        shadow_pre = false;
                        if (shadow_end) {
                            // a regular path's cache vertex: the sample is complete
                            shadow_end = false;
                            end = true;
                        } else {
                            ro = sro;
                            rd = srd;
                            walker_begin(w, p.scene, ro, rd);
                            mode = LANE_TRAVERSE;
                        }
                    } else if (!w.any) {
                        if (!err) L = add(L, sky_color(color, rd));
                        end = true;
                    } else {
                        const float4 ma = ldg4(p.scene.materials + 2 * (size_t)h.material);
                        const float4 mb = ldg4(p.scene.materials + 2 * (size_t)h.material + 1);
                        const uint32_t mtype = bits(mb.z);
                        const HitGeom g = hit_geometry<MATH, COUNT>(p.scene, h, ro, rd, &scn);
                        if (mtype > ORN_DIELECTRIC) {
                            // emitter (or unknown type): the path ends with color x emission,
                            // unless the previous vertex sampled this emitter directly
                            // (shade_geom's emission, computed here: a second inlined
                            // copy of shade_geom cost instruction-cache misses)
                            const uint32_t etex = bits(ma.w);
                            const bool etex_on = SEM == SEM_WGSL
                                                     ? (etex < p.cp.textures_count && etex < p.scene.textures_len)
                                                     : etex < p.scene.textures_len;
                            f3 em = mk(0.0f, 0.0f, 0.0f);
                            if (mtype == ORN_DIFFUSE_LIGHT)
                                em = etex_on ? tex_sample(p.scene.textures[etex], g.hu, g.hv, SEM == SEM_WGSL)
                                             : mk(ma.x, ma.y, ma.z);
                            f3 c2 = mul(color, em);
                            const bool sampled = nee_prev && h.type == ORN_NODE_MESH &&
                                                 __ldg(p.cache.light_material + h.material) != 0u;
                            if (sampled) {
                                // the previous vertex also sampled this emitter: balance-heuristic
                                // weight of the scattered ray, p_w / (p_w + p_light)
                                const float rl = sqrtf(dot(rd, rd));
                                const f3 wd = scale(1.0f / rl, rd);
                                const float dist = h.t * rl;
                                const float cl = fabsf(dot(g.normal, wd));
                                const float pw = scatter_pdf(nprev, wd);
                                const float pl = cl > 0.0f ? dist * dist / (cl * p.cache.light_area) : 3.0e38f;
                                c2 = scale(pw / (pw + pl), c2);
                            }
                            L = add(L, c2);
                            end = true;
                        } else {
                            const bool rough = mtype == ORN_LAMBERTIAN || (mtype == ORN_METAL && mb.x >= kCacheMinFuzz);
                            // the surface colour (lambertian and metal attenuation)
                            auto surface_att = [&]() -> f3 {
                                const uint32_t tex_id = bits(ma.w);
                                const bool use_tex = SEM == SEM_WGSL
                                                         ? (tex_id < p.cp.textures_count && tex_id < p.scene.textures_len)
                                                         : tex_id < p.scene.textures_len;
                                return use_tex ? tex_sample(p.scene.textures[tex_id], g.hu, g.hv, SEM == SEM_WGSL)
                                               : mk(ma.x, ma.y, ma.z);
                            };
                            bool at_cache = false;
                            f3 aclamp = mk(1.0f, 1.0f, 1.0f);
                            if (bounce >= 1u && !v2 && rough) {
                                // the cache vertex.  The network learns the radiance that
                                // leaves it through its scattered ray, divided by the surface
                                // colour (clamped away from 0), so textures stay exact.
                                at_cache = true;
                                const f3 ud = normalize(rd);
                                const float q[kCacheInputs] = {
                                    (g.hp.x - p.cache.lo[0]) * p.cache.inv_extent[0],
                                    (g.hp.y - p.cache.lo[1]) * p.cache.inv_extent[1],
                                    (g.hp.z - p.cache.lo[2]) * p.cache.inv_extent[2],
                                    0.5f * (ud.x + 1.0f), 0.5f * (ud.y + 1.0f), 0.5f * (ud.z + 1.0f),
                                    0.5f * (g.normal.x + 1.0f), 0.5f * (g.normal.y + 1.0f), 0.5f * (g.normal.z + 1.0f),
                                    mtype == ORN_LAMBERTIAN ? 1.0f : mb.x};
#pragma unroll
                                for (int j = 0; j < kCacheInputs; ++j) qin[j] = fminf(fmaxf(q[j], 0.0f), 1.0f);
                                const f3 a = surface_att();
                                aclamp = mk(fmaxf(a.x, 1e-3f), fmaxf(a.y, 1e-3f), fmaxf(a.z, 1e-3f));
                                vertex = true;
                                // trains with probability min(1, slots / vertices of
                                // the previous frame), decided per group of 32 pixels
                                // (a hash of group, frame and stream) so that a warp's
                                // lanes mostly all train or all stop here
                                const uint32_t prev = __ldg(p.cache.vertices_prev);
                                const uint32_t coin = qmc_hash((gid >> 5) * 0x9e3779b9u ^
                                                               p.cache.frame * 0x85ebca6bu ^ stream * 0xc2b2ae35u);
                                if (prev <= p.cache.train_slots ||
                                    (float)(coin >> 8) * (1.0f / 16777216.0f) * (float)prev < (float)p.cache.train_slots) {
                                    // 32 counters, one per lane index, each owning a 32nd
                                    // of the slots: a warp's lanes never wait on one
                                    // address (train_slots is a multiple of 32)
                                    const uint32_t shard = lane;
                                    const uint32_t per = p.cache.train_slots >> 5;
                                    const uint32_t slot = atomicAdd(p.cache.train_count + shard, 1u);
                                    if (slot < per) tslot = shard * per + slot;
                                }
                                if (tslot == 0xffffffffu) {
                                    query = true;
                                    qthr = mul(color, aclamp);
                                } else {
#pragma unroll
                                    for (int j = 0; j < kCacheInputs; ++j)
                                        p.cache.train_in[(size_t)tslot * kCacheInputs + j] = qin[j];
                                }
                            }
                            // next-event estimation where the scattered ray is traced
                            const bool nee = mtype == ORN_LAMBERTIAN && p.cache.light_count > 0u &&
                                             bounce + 1u < p.cp.depth;
                            bool shadow_ray = false;
                            f3 ldir = mk(0.0f, 0.0f, 0.0f);
                            float ldist = 0.0f;
                            if (nee) {
                                const float target = rng.f() * p.cache.light_area;
                                float u1, u2;
                                if (SOBOL && bounce == 0u) {
                                    qmc_point(qmc_hash(gid + 1u), QMC_LIGHT, (uint32_t)ci0 - 1u + stream, &u1, &u2);
                                } else {
                                    u1 = rng.f();
                                    u2 = rng.f();
                                }
                                uint32_t lo = 0, hi = p.cache.light_count - 1u;
                                while (lo < hi) {
                                    const uint32_t mid = (lo + hi) >> 1;
                                    if (__ldg(p.cache.light_cdf + mid) < target) lo = mid + 1u;
                                    else hi = mid;
                                }
                                const float4 t0 = ldg4(p.cache.lights + 4 * (size_t)lo);
                                const float4 t1 = ldg4(p.cache.lights + 4 * (size_t)lo + 1);
                                const float4 t2 = ldg4(p.cache.lights + 4 * (size_t)lo + 2);
                                shadow_inv = bits(ldg4(p.cache.lights + 4 * (size_t)lo + 3).x);
                                const f3 e1 = mk(t1.x, t1.y, t1.z), e2 = mk(t2.x, t2.y, t2.z);
                                const float su = sqrtf(u1);
                                const f3 y = add(mk(t0.x, t0.y, t0.z), add(scale(su * (1.0f - u2), e1), scale(su * u2, e2)));
                                const f3 nl = normalize(cross(e1, e2));
                                const f3 dv = sub(y, g.hp);
                                const float d2 = dot(dv, dv);
                                ldist = sqrtf(d2);
                                ldir = scale(1.0f / ldist, dv);
                                const float cx = dot(g.normal, ldir), cl = fabsf(dot(nl, ldir));
                                if (cx > 0.0f && cl > 0.0f && d2 > 0.0f) {
                                    // balance heuristic: att x Le x p_w / (p_light + p_w),
                                    // p_light = d^2 / (cos_l A) the light sample's solid-angle
                                    // density, p_w the scattered ray's
                                    const float pw = scatter_pdf(g.normal, ldir);
                                    const float pl = d2 / (cl * p.cache.light_area);
                                    const float wgt = pw / (pl + pw);
                                    nee_c = mul(color, mul(surface_att(), scale(wgt, mk(t0.w, t1.w, t2.w))));
                                    shadow_ray = true;
                                }
                            }
                            const f3 hp = g.hp;
                            bool trace_shadow = false;
                            if (query) {
                                // a regular path ends at its cache vertex: the direct light
                                // there explicitly, the rest from the cache
                                if (shadow_ray) {
                                    trace_shadow = true;
                                    shadow_end = true;
                                } else {
                                    end = true;
                                }
                            } else {
                                if (at_cache) {
                                    // a training path: from here on gather the radiance the
                                    // cache learns; this vertex's own light sample counts for
                                    // the pixel only
                                    pre = mul(color, aclamp);
                                    Lpre = L;
                                    color = mk(1.0f / aclamp.x, 1.0f / aclamp.y, 1.0f / aclamp.z);
                                    L = mk(0.0f, 0.0f, 0.0f);
                                    v2 = true;
                                    shadow_pre = shadow_ray;
                                }
                                const bool preset = SOBOL && bounce == 0u;
                                float pt = 0.0f, pp = 0.0f;
                                if (preset) qmc_point(qmc_hash(gid + 1u), QMC_BOUNCE, (uint32_t)ci0 - 1u + stream, &pt, &pp);
                                const bool cont = shade_geom<SEM, MATH, COUNT>(p.scene, p.cp, rng, h, g, &ro, &rd, &color,
                                                                               &scn, preset, pt, pp);
                                nee_prev = nee;
                                nprev = g.normal;
                                if (!cont) {
                                    end = true;   // absorbed
                                } else if (++bounce >= p.cp.depth) {
                                    L = add(L, color);   // depth limit: the reference ends with the throughput
                                    end = true;
                                } else if (shadow_ray) {
                                    trace_shadow = true;
                                } else {
                                    walker_begin(w, p.scene, ro, rd);
                                    mode = LANE_TRAVERSE;
                                }
                            }
                            if (trace_shadow) {
                                // trace the shadow ray first; (ro, rd) carry it, since the
                                // walker restores the world ray from them on leaving a BLAS.
                                // The shadow ray is the very vector the reference's scatter
                                // would produce toward the light, n + s = 2 cos(a) w, so its
                                // t_min (in units of that vector) excludes the same
                                // self-intersections as a scattered ray's.  It searches a
                                // little past the light point: the sample counts only if the
                                // closest hit is that emitter, as a scattered ray's emission
                                // would (coplanar overlapping emitters count once).
                                const float cx2 = 2.0f * dot(g.normal, ldir);
                                sro = ro;
                                srd = rd;
                                ro = hp;
                                rd = scale(cx2, ldir);
                                walker_begin(w, p.scene, ro, rd);
                                w.t_max = ldist / cx2 * (1.0f + 1e-3f);
                                // any-hit: stop at an occluder before the light point
                                w.occl_inv = shadow_inv;
                                w.occl_t = ldist / cx2;
                                shadow = true;
                                mode = LANE_TRAVERSE;
                            }
                        }
                    }
                    // count this warp's cache vertices (one atomic)
                    const unsigned vm = __ballot_sync(ready, vertex);
                    if (vm != 0u && lane == __ffs(vm) - 1u) atomicAdd(p.cache.vertices, (unsigned)__popc(vm));
                    // append this warp's queries to the queue (one atomic)
                    const unsigned qm = __ballot_sync(ready, query);
                    if (qm != 0u) {
                        const unsigned leader = __ffs(qm) - 1u;
                        uint32_t base = 0;
                        if (lane == leader) base = atomicAdd(p.cache.query_count, (unsigned)__popc(qm));
                        base = __shfl_sync(ready, base, leader);
                        if (query) {
                            const uint32_t qi = base + __popc(qm & lanes_below);
                            p.cache.query_pixel[qi] = gid;
#pragma unroll
                            for (int j = 0; j < kCacheInputs; ++j) p.cache.query_in[(size_t)qi * kCacheInputs + j] = qin[j];
                            p.cache.query_thr[qi] = make_float4(qthr.x, qthr.y, qthr.z, 0.0f);
                        }
                    }
                    if (end) {
                        // a query's cached radiance is added by the inference pass
                        f3 c = L;
                        if (tslot != 0xffffffffu) {
                            float* tg = p.cache.train_target + (size_t)tslot * 3;
                            tg[0] = v2 ? L.x : -1.0f;
                            tg[1] = v2 ? L.y : 0.0f;
                            tg[2] = v2 ? L.z : 0.0f;
                            if (v2) c = add(Lpre, mul(pre, L));
                        }
                        add_sample(c);
                        ++k;
                        mode = start_samples();
                    }
                } else {
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
                        acc.add(ci0 + (float)k, color);
                        ++k;
                        mode = start_samples();
                    }
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
__global__ void seed_rng_kernel(uint32_t* rng, uint32_t n, uint32_t first) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rng[i] = first + i;
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

// relMSE against an FP64 reference: per pixel and RGB channel
// (x - r)^2 / (r^2 + 1e-2) with x the pixel's mean sample value, summed in
// FP64 into out[0]; pixels whose estimate or reference is not finite are
// skipped and counted in out[1] (as a double).
__global__ void __launch_bounds__(256)
relmse_kernel(const float4* __restrict__ acc, const double* __restrict__ acc64, const double* __restrict__ ref64,
              uint32_t n, double* out) {
    __shared__ double part[256];
    __shared__ unsigned skipped;
    if (threadIdx.x == 0) skipped = 0;
    __syncthreads();
    double sum = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double x[3], w;
        if (acc64) {
            const double* a = acc64 + 4 * (size_t)i;
            w = a[3];
            x[0] = a[0] / w; x[1] = a[1] / w; x[2] = a[2] / w;
        } else {
            float4 a = acc[i];
            w = (double)a.w;
            x[0] = (double)a.x / w; x[1] = (double)a.y / w; x[2] = (double)a.z / w;
        }
        const double* r = ref64 + 4 * (size_t)i;
        bool finite = true;
#pragma unroll
        for (int c = 0; c < 3; ++c) finite = finite && isfinite(x[c]) && isfinite(r[c]);
        if (!finite) {
            atomicAdd(&skipped, 1u);
            continue;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            double d = x[c] - r[c];
            sum += d * d / (r[c] * r[c] + 1e-2);
        }
    }
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(out, part[0]);
        if (skipped) atomicAdd(out + 1, (double)skipped);
    }
}

cudaError_t launch_relmse(const float4* acc, const double* acc64, const double* ref64, uint32_t n, double* out,
                          cudaStream_t s) {
    uint32_t blocks = (n + 255) / 256;
    if (blocks > 1216) blocks = 1216;
    relmse_kernel<<<blocks, 256, 0, s>>>(acc, acc64, ref64, n, out);
    return cudaGetLastError();
}

// ---- host-side launchers -----------------------------------------------------
// Persistent grid: as many blocks as fit on the device at once (never more
// than the pixels need).
template <int SEM, int MATH, bool COUNT, bool FAST, bool F64 = false, bool CACHE = false, bool SOBOL = false>
static cudaError_t launch_mega_tt(const RenderLaunch& p, cudaStream_t s) {
    static int blocks_per_sm = 0, sms = 0;
    if (blocks_per_sm == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
#ifdef ORN_MEGA_CARVEOUT
        // shared-memory share of the unified L1/shared space, in percent
        cudaFuncSetAttribute(mega_kernel<SEM, MATH, COUNT, FAST, F64, CACHE, SOBOL>,
                             cudaFuncAttributePreferredSharedMemoryCarveout, ORN_MEGA_CARVEOUT);
#endif
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, mega_kernel<SEM, MATH, COUNT, FAST, F64, CACHE, SOBOL>,
                                                      kMegaBlock, 0);
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    const uint64_t items = CACHE ? (uint64_t)p.pixel_count * p.cache.streams : p.pixel_count;
    uint32_t need = (uint32_t)((items + kMegaBlock - 1) / kMegaBlock);
    uint32_t grid = (uint32_t)(blocks_per_sm * sms);
    if (need < grid) grid = need;
    cudaError_t e = cudaMemsetAsync(p.work_counter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    mega_kernel<SEM, MATH, COUNT, FAST, F64, CACHE, SOBOL><<<grid, kMegaBlock, 0, s>>>(p);
    return cudaGetLastError();
}

// The Sobol sampler is a separate instantiation, so the stream sampler's
// kernel carries none of its code.
template <bool SOBOL>
static cudaError_t launch_mega_cached_t(const RenderLaunch& p, int semantics, bool fast, cudaStream_t s) {
    if (semantics == SEM_WGSL)
        return fast ? launch_mega_tt<SEM_WGSL, MATH_PORTABLE, false, true, false, true, SOBOL>(p, s)
                    : launch_mega_tt<SEM_WGSL, MATH_PORTABLE, false, false, false, true, SOBOL>(p, s);
    return fast ? launch_mega_tt<SEM_HIP, MATH_PORTABLE, false, true, false, true, SOBOL>(p, s)
                : launch_mega_tt<SEM_HIP, MATH_PORTABLE, false, false, false, true, SOBOL>(p, s);
}

cudaError_t launch_mega_cached(const RenderLaunch& p, int semantics, bool fast, cudaStream_t s) {
    return p.cache.sobol ? launch_mega_cached_t<true>(p, semantics, fast, s)
                         : launch_mega_cached_t<false>(p, semantics, fast, s);
}

template <int SEM>
static cudaError_t launch_mega_t(const RenderLaunch& p, bool count, bool fast, cudaStream_t s) {
    if (fast) return count ? launch_mega_tt<SEM, MATH_PORTABLE, true, true>(p, s)
                           : launch_mega_tt<SEM, MATH_PORTABLE, false, true>(p, s);
    return count ? launch_mega_tt<SEM, MATH_PORTABLE, true, false>(p, s)
                 : launch_mega_tt<SEM, MATH_PORTABLE, false, false>(p, s);
}

cudaError_t launch_mega_f64(const RenderLaunch& p, int semantics, bool fast, cudaStream_t s) {
    if (semantics == SEM_WGSL)
        return fast ? launch_mega_tt<SEM_WGSL, MATH_PORTABLE, false, true, true>(p, s)
                    : launch_mega_tt<SEM_WGSL, MATH_PORTABLE, false, false, true>(p, s);
    return fast ? launch_mega_tt<SEM_HIP, MATH_PORTABLE, false, true, true>(p, s)
                : launch_mega_tt<SEM_HIP, MATH_PORTABLE, false, false, true>(p, s);
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

cudaError_t launch_seed_rng(uint32_t* rng, uint32_t n, cudaStream_t s, uint32_t first) {
    seed_rng_kernel<<<(n + 255) / 256, 256, 0, s>>>(rng, n, first);
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
