// wave_cached.cu — the radiance-cache renderer on the persistent wavefront.
//
// One cached frame (see CacheLaunch in pt_kernels.h): every pixel and
// sample stream traces one sample with next-event estimation; a regular
// path ends at its cache vertex (the first rough surface from the second
// vertex on) with a query for the network, a training path runs to its end
// and records the network inputs at the cache vertex and the radiance that
// left it.  The path logic is the cached megakernel's (megakernel.cu,
// CACHE = true), operation for operation; what changes is where it runs.
// Two warps of a block only shade; the others run wave_warp (wave_queue.cuh)
// and switch between
//
//   traversal   every ray of the block's paths — scattered rays and the
//               any-hit shadow rays of light samples (ANY);
//   shading     the per-vertex logic on full warps, by the warps that have
//               run out of rays: light sampling, the cache-vertex decision
//               (query / training slot), material scatter, and the sample's
//               end (accumulation, training target) and the next item.
//
// In the megakernel this logic runs on the few lanes of a warp that are
// ready together, in a kernel whose size (128 registers, instruction-cache
// misses) limits residency.  The reference's per-pass loop and the estimator
// are unchanged (src/hip_backend/path_tracer.zig:121-133;
// src/hip_backend/kernels/pathtracer.hip.cpp:72-154).
#include <cuda_fp16.h>

#include "qmc.cuh"
#include "wave_queue.cuh"

namespace orn {

using namespace wave;

namespace {

// Per-slot bits of the cached path state.
enum : uint32_t { B_V2 = 1u, B_SHADOW = 2u, B_NEE_PREV = 4u, B_SHADOW_END = 8u, B_SHADOW_PRE = 16u };

// The block's path pool for cached frames (one sample per item).
template <int P>
struct CPool {
    uint32_t gid[P], stream[P], rng[P], bounce[P], flag[P], steps[P];
    uint32_t tslot[P], bits[P], shadow_inv[P];
    float color[3][P], ro[3][P], rd[3][P];
    float L[3][P], Lpre[3][P], nee_c[3][P], sro[3][P], srd[3][P], nprev[3][P], pre[3][P];
    float ray_tmax[P], occl_t[P];
    uint32_t occl_inv[P];
    float t[P], u[P], v[P];
    uint32_t material[P], type[P], inv[P], tri[P];
    uint32_t rq[P], hq[P];
    uint32_t rq_head, rq_tail, hq_head, hq_tail;
    uint32_t active, exhausted, abort;
};

template <int P>
__device__ __forceinline__ f3 ld3(const float (&a)[3][P], uint32_t i) {
    return mk(a[0][i], a[1][i], a[2][i]);
}
template <int P>
__device__ __forceinline__ void st3(float (&a)[3][P], uint32_t i, f3 v) {
    a[0][i] = v.x;
    a[1][i] = v.y;
    a[2][i] = v.z;
}

}  // namespace

// Resident blocks per SM the kernel is compiled for (register cap).
// Measured on cached + batched 1920x1080 frames (ms per frame): 2 blocks of
// 8 warps (128 registers) 64.6; 3 blocks of 8 warps with 192 slots (80
// registers, 1.6 KB of spills per thread) 102.9; 4 blocks of 6 warps 117.7;
// 2 blocks of 10 warps 65.8.  Unlike the cached megakernel, spilling the
// shading code costs more than the extra warps bring.
#ifndef ORN_WAVE_CACHED_MINB
#define ORN_WAVE_CACHED_MINB 2
#endif
template <int SEM, bool FAST, bool SOBOL, int NW, int NS, int P>
__global__ void __launch_bounds__(32 * NW, ORN_WAVE_CACHED_MINB)
wave_cached_kernel(RenderLaunch p) {
    extern __shared__ __align__(16) unsigned char wave_smem[];
    CPool<P>& pool = *reinterpret_cast<CPool<P>*>(wave_smem);
    uint32_t* sstack = reinterpret_cast<uint32_t*>(wave_smem + ((sizeof(CPool<P>) + 15) / 16) * 16);
    const unsigned kFull = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lanes_below = (1u << lane) - 1u;
    constexpr int MATH = MATH_PORTABLE;
    pool_init<P>(pool);

    uint32_t err = 0;
    VisitCount vc = {0, 0, 0, 0, 0};
    SampleCount scn = {0, 0, 0, 0};
    const uint32_t W = p.cp.width;
    const float ci0 = p.cp.current_iteration;
    const uint32_t items = p.pixel_count * p.cache.streams;
    const bool atomic_acc = p.cache.streams > 1u;

    // The path logic of one shading round: the lane's slot (or kEmpty) was
    // taken from the hit queue; new rays go to the ray queue.
    auto shade = [&](uint32_t slot) -> bool {
        bool emit = false, need = false, end = false, query = false, vertex = false;
        uint32_t gid = 0, stream = 0, bounce = 0, tslot = kEmpty, pf = 0, shadow_inv = 0;
        Rng rng{0};
        f3 ro = mk(0.0f, 0.0f, 0.0f), rd = ro, color = ro, L = ro, Lpre = ro, nee_c = ro, sro = ro, srd = ro,
           nprev = ro, pre = mk(1.0f, 1.0f, 1.0f), qthr = ro;
        float ray_tmax = 3.40282e+38f, occl_t = 0.0f;
        uint32_t occl_inv = kEmpty;
        float qin[kCacheInputs];
#pragma unroll
        for (int j = 0; j < kCacheInputs; ++j) qin[j] = 0.0f;

        // A new sample of item (stream, gid): its camera ray.
        auto start_sample = [&]() {
            if (SOBOL) {
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
            pf = 0;
            L = mk(0.0f, 0.0f, 0.0f);
            ray_tmax = 3.40282e+38f;
            occl_inv = kEmpty;
            occl_t = 0.0f;
        };
        // The item's one sample is complete: accumulation (atomic with several
        // streams) and RNG state.
        auto finish_item = [&](f3 c) {
            if (atomic_acc) {
                float* a = reinterpret_cast<float*>(p.acc + gid);
                atomicAdd(a + 0, c.x);
                atomicAdd(a + 1, c.y);
                atomicAdd(a + 2, c.z);
                atomicAdd(a + 3, 1.0f);
            } else {
                float4 a = ci0 > 1.0f ? p.acc[gid] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (ci0 > 1.0f) a = make_float4(a.x + c.x, a.y + c.y, a.z + c.z, a.w + 1.0f);
                else a = make_float4(c.x, c.y, c.z, 1.0f);
                p.acc[gid] = a;
            }
            if (stream > 0u) p.cache.rng_extra[(size_t)(stream - 1u) * p.pixel_count + gid] = rng.state;
            else p.rng[gid] = rng.state;
        };

        if (slot != kEmpty) {
            if (pool.flag[slot] == NEED_PIXEL) {
                need = true;
            } else {
                gid = pool.gid[slot];
                stream = pool.stream[slot];
                rng.state = pool.rng[slot];
                bounce = pool.bounce[slot];
                tslot = pool.tslot[slot];
                pf = pool.bits[slot];
                shadow_inv = pool.shadow_inv[slot];
                color = ld3(pool.color, slot);
                ro = ld3(pool.ro, slot);
                rd = ld3(pool.rd, slot);
                L = ld3(pool.L, slot);
                Lpre = ld3(pool.Lpre, slot);
                nee_c = ld3(pool.nee_c, slot);
                sro = ld3(pool.sro, slot);
                srd = ld3(pool.srd, slot);
                nprev = ld3(pool.nprev, slot);
                pre = ld3(pool.pre, slot);
                const uint32_t flag = pool.flag[slot];
                const bool any = flag == HIT_ANY, failed = flag == HIT_FAILED;
                HitRec h;
                h.t = pool.t[slot];
                h.material = pool.material[slot];
                h.type = pool.type[slot];
                h.inv = pool.inv[slot];
                h.tri = pool.tri[slot];
                h.u = pool.u[slot];
                h.v = pool.v[slot];
                if (pf & B_SHADOW) {
                    // the shadow ray of a light sample finished: add the sample if
                    // unoccluded, then trace the scattered ray
                    pf &= ~B_SHADOW;
                    if (any && h.type == ORN_NODE_MESH && h.inv == shadow_inv &&
                        __ldg(p.cache.light_material + h.material) != 0u) {
                        if (pf & B_SHADOW_PRE) Lpre = add(Lpre, nee_c);
                        else L = add(L, nee_c);
                    }
                    pf &= ~B_SHADOW_PRE;
                    if (pf & B_SHADOW_END) {
                        // a regular path's cache vertex: the sample is complete
                        pf &= ~B_SHADOW_END;
                        end = true;
                    } else {
                        ro = sro;
                        rd = srd;
                        emit = true;
                    }
                } else if (!any) {
                    if (!failed) L = add(L, sky_color(color, rd));
                    end = true;
                } else {
                    const float4 ma = ldg4(p.scene.materials + 2 * (size_t)h.material);
                    const float4 mb = ldg4(p.scene.materials + 2 * (size_t)h.material + 1);
                    const uint32_t mtype = bits(mb.z);
                    const HitGeom g = hit_geometry<MATH, false>(p.scene, h, ro, rd, &scn);
                    if (mtype > ORN_DIELECTRIC) {
                        // emitter (or unknown type): the path ends with color x emission,
                        // unless the previous vertex sampled this emitter directly
                        const uint32_t etex = bits(ma.w);
                        const bool etex_on = SEM == SEM_WGSL
                                                 ? (etex < p.cp.textures_count && etex < p.scene.textures_len)
                                                 : etex < p.scene.textures_len;
                        f3 em = mk(0.0f, 0.0f, 0.0f);
                        if (mtype == ORN_DIFFUSE_LIGHT)
                            em = etex_on ? tex_sample(p.scene.textures[etex], g.hu, g.hv, SEM == SEM_WGSL)
                                         : mk(ma.x, ma.y, ma.z);
                        f3 c2 = mul(color, em);
                        const bool sampled = (pf & B_NEE_PREV) && h.type == ORN_NODE_MESH &&
                                             __ldg(p.cache.light_material + h.material) != 0u;
                        if (sampled) {
                            // balance-heuristic weight of the scattered ray, p_w / (p_w + p_light)
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
                        if (bounce >= 1u && !(pf & B_V2) && rough) {
                            // the cache vertex: the network learns the radiance leaving
                            // it through its scattered ray, over the surface colour
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
                            // trains with probability min(1, slots / vertices of the
                            // previous frame), decided per group of 32 pixels
                            const uint32_t prev = __ldg(p.cache.vertices_prev);
                            const uint32_t coin = qmc_hash((gid >> 5) * 0x9e3779b9u ^ p.cache.frame * 0x85ebca6bu ^
                                                           stream * 0xc2b2ae35u);
                            if (prev <= p.cache.train_slots ||
                                (float)(coin >> 8) * (1.0f / 16777216.0f) * (float)prev < (float)p.cache.train_slots) {
                                // 32 counters, each owning a 32nd of the slots; the shard
                                // comes from the item (a shading warp's lanes hold
                                // whichever slots the hit queue gave them, often fewer
                                // than 32, so a lane-indexed shard would fill unevenly)
                                const uint32_t shard = (gid + stream * 13u) & 31u;
                                const uint32_t per = p.cache.train_slots >> 5;
                                const uint32_t ts = atomicAdd(p.cache.train_count + shard, 1u);
                                if (ts < per) tslot = shard * per + ts;
                            }
                            if (tslot == kEmpty) {
                                query = true;
                                qthr = mul(color, aclamp);
                            } else {
#pragma unroll
                                for (int j = 0; j < kCacheInputs; ++j)
                                    p.cache.train_in[(size_t)tslot * kCacheInputs + j] = qin[j];
                            }
                        }
                        // next-event estimation where the scattered ray is traced
                        const bool nee = mtype == ORN_LAMBERTIAN && p.cache.light_count > 0u && bounce + 1u < p.cp.depth;
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
                                pf |= B_SHADOW_END;
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
                                pf |= B_V2;
                                if (shadow_ray) pf |= B_SHADOW_PRE;
                                else pf &= ~B_SHADOW_PRE;
                            }
                            const bool preset = SOBOL && bounce == 0u;
                            float pt = 0.0f, pp = 0.0f;
                            if (preset) qmc_point(qmc_hash(gid + 1u), QMC_BOUNCE, (uint32_t)ci0 - 1u + stream, &pt, &pp);
                            const bool cont = shade_geom<SEM, MATH, false>(p.scene, p.cp, rng, h, g, &ro, &rd, &color,
                                                                           &scn, preset, pt, pp);
                            if (nee) pf |= B_NEE_PREV;
                            else pf &= ~B_NEE_PREV;
                            nprev = g.normal;
                            if (!cont) {
                                end = true;   // absorbed
                            } else if (++bounce >= p.cp.depth) {
                                L = add(L, color);   // depth limit: the reference ends with the throughput
                                end = true;
                            } else if (shadow_ray) {
                                trace_shadow = true;
                            } else {
                                emit = true;
                            }
                        }
                        if (trace_shadow) {
                            // trace the shadow ray first (the vector the reference's
                            // scatter would produce toward the light, n + s = 2 cos(a) w),
                            // a little past the light point, any-hit against occluders
                            const float cx2 = 2.0f * dot(g.normal, ldir);
                            sro = ro;
                            srd = rd;
                            ro = hp;
                            rd = scale(cx2, ldir);
                            ray_tmax = ldist / cx2 * (1.0f + 1e-3f);
                            occl_inv = shadow_inv;
                            occl_t = ldist / cx2;
                            pf |= B_SHADOW;
                            emit = true;
                        }
                    }
                }
            }
        }
        // count this warp's cache vertices (one atomic)
        const unsigned vm = __ballot_sync(kFull, vertex);
        if (vm != 0u && lane == __ffs(vm) - 1u) atomicAdd(p.cache.vertices, (unsigned)__popc(vm));
        // append this warp's queries to the queue (one atomic)
        const unsigned qm = __ballot_sync(kFull, query);
        if (qm != 0u) {
            const unsigned leader = __ffs(qm) - 1u;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(p.cache.query_count, (unsigned)__popc(qm));
            base = __shfl_sync(kFull, base, leader);
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
            if (tslot != kEmpty) {
                float* tg = p.cache.train_target + (size_t)tslot * 3;
                const bool v2 = (pf & B_V2) != 0u;
                tg[0] = v2 ? L.x : -1.0f;
                tg[1] = v2 ? L.y : 0.0f;
                tg[2] = v2 ? L.z : 0.0f;
                if (v2) c = add(Lpre, mul(pre, L));
            }
            finish_item(c);
            need = true;
        }
        // Lanes whose slot needs an item take the next ones (one atomic per warp).
        for (;;) {
            const unsigned nm = __ballot_sync(kFull, need);
            if (nm == 0u) break;
            if (warp_flag(vload(pool.exhausted) != 0u)) {
                if (need) {
                    atomicSub(&pool.active, 1u);
                    need = false;
                    slot = kEmpty;
                }
                continue;
            }
            const unsigned leader = __ffs(nm) - 1u;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(p.work_counter, (unsigned)__popc(nm));
            base = __shfl_sync(kFull, base, leader);
            if (base + __popc(nm) >= items && lane == leader) atomicExch(&pool.exhausted, 1u);
            if (need) {
                const uint32_t mine = base + __popc(nm & lanes_below);
                if (mine < items) {
                    stream = mine / p.pixel_count;
                    gid = mine - stream * p.pixel_count;
                    rng.state = stream > 0u ? p.cache.rng_extra[(size_t)(stream - 1u) * p.pixel_count + gid]
                                            : p.rng[gid];
                    tslot = kEmpty;   // decided at the cache vertex
                    start_sample();
                    if (p.cp.depth > 0) {
                        emit = true;
                        need = false;
                    } else {
                        finish_item(color);   // depth 0: the sample is white; the slot asks again
                    }
                } else {
                    atomicSub(&pool.active, 1u);
                    need = false;
                    slot = kEmpty;
                }
            }
        }
        if (emit) {
            pool.gid[slot] = gid;
            pool.stream[slot] = stream;
            pool.rng[slot] = rng.state;
            pool.bounce[slot] = bounce;
            pool.tslot[slot] = tslot;
            pool.bits[slot] = pf;
            pool.shadow_inv[slot] = shadow_inv;
            st3(pool.color, slot, color);
            st3(pool.ro, slot, ro);
            st3(pool.rd, slot, rd);
            st3(pool.L, slot, L);
            st3(pool.Lpre, slot, Lpre);
            st3(pool.nee_c, slot, nee_c);
            st3(pool.sro, slot, sro);
            st3(pool.srd, slot, srd);
            st3(pool.nprev, slot, nprev);
            st3(pool.pre, slot, pre);
            pool.ray_tmax[slot] = ray_tmax;
            pool.occl_inv[slot] = occl_inv;
            pool.occl_t[slot] = occl_t;
            __threadfence_block();
        }
        return q_push<P>(pool.rq, &pool.rq_tail, emit, slot, lane);
    };
    if ((threadIdx.x >> 5) < (uint32_t)NS)
        wave_warp<false, FAST, true, P, ROLE_SHADE, kWaveStepsDefault>(pool, p, sstack + threadIdx.x,
                                                                       (int)blockDim.x, lane, vc, err, shade);
    else
        wave_warp<false, FAST, true, P, ROLE_BOTH, kWaveStepsDefault>(pool, p, sstack + threadIdx.x,
                                                                      (int)blockDim.x, lane, vc, err, shade);
    if (err) atomicOr(p.error, err);
}

// ---- host-side launcher ------------------------------------------------------------
namespace {

#ifndef ORN_WAVE_CACHED_WARPS
#define ORN_WAVE_CACHED_WARPS 8
#endif
#ifndef ORN_WAVE_CACHED_SLOTS
#define ORN_WAVE_CACHED_SLOTS 320
#endif
#ifndef ORN_WAVE_CACHED_SHADERS
#define ORN_WAVE_CACHED_SHADERS 2
#endif
constexpr int kCachedW = ORN_WAVE_CACHED_WARPS, kCachedP = ORN_WAVE_CACHED_SLOTS, kCachedS = ORN_WAVE_CACHED_SHADERS;

template <int SEM, bool FAST, bool SOBOL>
cudaError_t launch_t(const RenderLaunch& p, cudaStream_t s) {
    constexpr int kBlock = 32 * kCachedW;
    constexpr size_t kSmem = ((sizeof(CPool<kCachedP>) + 15) / 16) * 16 + sizeof(uint32_t) * kSmemStack * kBlock;
    static int blocks_per_sm = 0, sms = 0;
    auto kern = wave_cached_kernel<SEM, FAST, SOBOL, kCachedW, kCachedS, kCachedP>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
    if (e != cudaSuccess) return e;
    if (blocks_per_sm == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, kBlock, kSmem);
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    const uint64_t items = (uint64_t)p.pixel_count * p.cache.streams;
    uint32_t need = (uint32_t)((items + kCachedP - 1) / kCachedP);
    uint32_t grid = (uint32_t)(blocks_per_sm * sms);
    if (need < grid) grid = need;
    e = cudaMemsetAsync(p.work_counter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    kern<<<grid, kBlock, kSmem, s>>>(p);
    return cudaGetLastError();
}

template <bool SOBOL>
cudaError_t launch_s(const RenderLaunch& p, int semantics, bool fast, cudaStream_t s) {
    if (semantics == SEM_WGSL) return fast ? launch_t<SEM_WGSL, true, SOBOL>(p, s) : launch_t<SEM_WGSL, false, SOBOL>(p, s);
    return fast ? launch_t<SEM_HIP, true, SOBOL>(p, s) : launch_t<SEM_HIP, false, SOBOL>(p, s);
}

}  // namespace

cudaError_t launch_wave_cached(const RenderLaunch& p, int semantics, bool fast, cudaStream_t s) {
    return p.cache.sobol ? launch_s<true>(p, semantics, fast, s) : launch_s<false>(p, semantics, fast, s);
}

}  // namespace orn
