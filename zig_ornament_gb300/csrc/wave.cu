// wave.cu — the persistent wavefront: per-block path pools with ray and hit
// queues in shared memory.
//
// The reference's render loop (src/hip_backend/path_tracer.zig:121-133,
// one launch of path_tracing_kernal per pass, per-pixel work in
// src/hip_backend/kernels/pathtracer.hip.cpp:72-154) is run as one
// persistent launch.  Each block owns a pool of P path slots in shared
// memory and two queues of slot indices:
//
//   ray queue  slots whose next ray is ready to trace;
//   hit queue  slots whose ray was traced (or that need a pixel).
//
// The block's warps (wave_queue.cuh) split the work: all but one traverse
// (traversal_warp; nine of ten in the default block shape) — idle lanes
// take the next rays from the ray queue (ballot-compacted, one reservation
// per warp) once enough of them are idle (p.wave_fetch, default four),
// each lane visits BVH nodes (walker_step, the megakernel's traversal) and,
// when its ray is done, writes the hit record into the slot and appends the
// slot to the hit queue — and one shades: it takes up to 32 slots from the
// hit queue and runs the path logic with a full warp —
// material scatter and the next bounce, or the sample's accumulation and
// the next sample's camera ray, or the pixel's completion (accumulation,
// RNG state, framebuffer, traversal cost) and the next pixel from the
// launch's counter (in the longest-first order when one is given).  New
// rays go to the ray queue.
//
// Against the megakernel this separates the two kinds of work: a lane whose
// ray finished no longer waits for the rest of its warp to finish theirs
// before it is shaded, and shading code (material scatter, portable
// transcendentals) runs on full warps instead of the few lanes that happen
// to be ready.  A pixel's samples still run in order in its slot with the
// pixel's RNG state, so every pixel is bit-identical to the reference's
// passes.  Every wait (an entry not yet written, a position not yet
// cleared, no work while the block is not finished) is bounded by
// %globaltimer; a wait that runs out sets ERR_WAIT, and every warp of the
// block returns.
#include <cuda_fp16.h>

#include "wave_queue.cuh"

namespace orn {

using namespace wave;

namespace {

// The block's path pool (structure of arrays in dynamic shared memory).
template <int P>
struct Pool {
    uint32_t gid[P], k[P], bounce[P], rng[P], steps[P], flag[P];
    float acc[4][P];
    float color[3][P];
    float ro[3][P], rd[3][P];
    float t[P], u[P], v[P];
    uint32_t material[P], type[P], inv[P], tri[P];
    uint32_t rq[P], hq[P];
    uint32_t rq_head, rq_tail, hq_head, hq_tail;
    uint32_t active;      // slots not retired
    uint32_t exhausted;   // the launch's pixel counter ran out
    uint32_t abort;       // a bounded wait ran out
};

}  // namespace

// NW warps per block, NS of them shading, P path slots, launch bounds for
// MINB resident blocks per SM (the register cap), STEPS node visits per
// traversal round.
template <int SEM, bool COUNT, bool FAST, int NW, int NS, int P, int MINB, int STEPS>
__global__ void __launch_bounds__(32 * NW, MINB)
wave_kernel(RenderLaunch p) {
    extern __shared__ __align__(16) unsigned char wave_smem[];
    Pool<P>& pool = *reinterpret_cast<Pool<P>*>(wave_smem);
    uint32_t* sstack = reinterpret_cast<uint32_t*>(wave_smem + ((sizeof(Pool<P>) + 15) / 16) * 16);
    const unsigned kFull = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31u;
    pool_init<P>(pool);

    uint32_t err = 0;
    VisitCount vc = {0, 0, 0, 0, 0};
    SampleCount scn = {0, 0, 0, 0};
    const uint32_t W = p.cp.width, H = p.cp.height;
    const float ci0 = p.cp.current_iteration;

    // The path logic of one shading round: the lane's slot (or kEmpty) was
    // taken from the hit queue; new rays go to the ray queue.
    auto shade = [&](uint32_t slot) -> bool {
        bool emit = false, need = false;
        uint32_t gid = 0, k = 0, bounce = 0;
        Rng rng{0};
        float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        f3 ro = mk(0.0f, 0.0f, 0.0f), rd = ro, color = ro;
        // Starts samples k.. of the slot's pixel (depth-0 samples finish at
        // once); true when a camera ray was made, false when the pixel is
        // complete (its results are then written).
        auto start_samples = [&]() -> bool {
            while (k < p.spp) {
                camera_ray<MATH_PORTABLE>(p.cp, gid % W, gid / W, rng, &ro, &rd);
                color = mk(1.0f, 1.0f, 1.0f);
                bounce = 0;
                if (p.cp.depth > 0) return true;
                const float ci = ci0 + (float)k;
                if (ci > 1.0f) acc = make_float4(acc.x + color.x, acc.y + color.y, acc.z + color.z, acc.w + 1.0f);
                else acc = make_float4(color.x, color.y, color.z, 1.0f);
                ++k;
            }
            p.acc[gid] = acc;
            p.rng[gid] = rng.state;
            if (p.cost) p.cost[gid] = pool.steps[slot];
            if (p.do_post) {
                const uint32_t x = gid % W, y = gid / W;
                const uint32_t fbi = p.cp.flip_y != 0 ? W * (H - y - 1) + x : gid;
                p.fb[fbi] = post_process<SEM, MATH_PORTABLE>(acc, ci0 + (float)(p.spp - 1), p.cp.inverted_gamma);
            }
            return false;
        };
        if (slot != kEmpty) {
            if (pool.flag[slot] == NEED_PIXEL) {
                need = true;
            } else {
                gid = pool.gid[slot];
                k = pool.k[slot];
                bounce = pool.bounce[slot];
                rng.state = pool.rng[slot];
                acc = make_float4(pool.acc[0][slot], pool.acc[1][slot], pool.acc[2][slot], pool.acc[3][slot]);
                color = mk(pool.color[0][slot], pool.color[1][slot], pool.color[2][slot]);
                ro = mk(pool.ro[0][slot], pool.ro[1][slot], pool.ro[2][slot]);
                rd = mk(pool.rd[0][slot], pool.rd[1][slot], pool.rd[2][slot]);
                const uint32_t flag = pool.flag[slot];
                bool cont;
                if (flag != HIT_ANY) {
                    color = flag == HIT_FAILED ? mk(0.0f, 0.0f, 0.0f) : sky_color(color, rd);
                    cont = false;
                } else {
                    HitRec h;
                    h.t = pool.t[slot];
                    h.material = pool.material[slot];
                    h.type = pool.type[slot];
                    h.inv = pool.inv[slot];
                    h.tri = pool.tri[slot];
                    h.u = pool.u[slot];
                    h.v = pool.v[slot];
                    cont = shade_hit<SEM, MATH_PORTABLE, COUNT>(p.scene, p.cp, rng, h, &ro, &rd, &color, &scn);
                }
                if (cont && ++bounce < p.cp.depth) {
                    emit = true;
                } else {
                    const float ci = ci0 + (float)k;
                    if (ci > 1.0f) acc = make_float4(acc.x + color.x, acc.y + color.y, acc.z + color.z, acc.w + 1.0f);
                    else acc = make_float4(color.x, color.y, color.z, 1.0f);
                    ++k;
                    emit = start_samples();
                    need = !emit;
                }
            }
        }
        // Lanes whose slot needs a pixel take the next ones (one atomic per
        // warp); a depth-0 pixel completes at once and asks again.
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
            if (base + __popc(nm) >= p.pixel_count && lane == leader) atomicExch(&pool.exhausted, 1u);
            if (need) {
                const uint32_t mine = base + __popc(nm & ((1u << lane) - 1u));
                if (mine < p.pixel_count) {
                    gid = p.order ? p.order[mine] : mine;
                    rng.state = p.rng[gid];
                    acc = ci0 > 1.0f ? p.acc[gid] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    k = 0;
                    pool.steps[slot] = 0;
                    emit = start_samples();
                    need = !emit;
                } else {
                    atomicSub(&pool.active, 1u);
                    need = false;
                    slot = kEmpty;
                }
            }
        }
        if (emit) {
            if (COUNT) scn.rays++;
            pool.gid[slot] = gid;
            pool.k[slot] = k;
            pool.bounce[slot] = bounce;
            pool.rng[slot] = rng.state;
            pool.acc[0][slot] = acc.x;
            pool.acc[1][slot] = acc.y;
            pool.acc[2][slot] = acc.z;
            pool.acc[3][slot] = acc.w;
            pool.color[0][slot] = color.x;
            pool.color[1][slot] = color.y;
            pool.color[2][slot] = color.z;
            pool.ro[0][slot] = ro.x;
            pool.ro[1][slot] = ro.y;
            pool.ro[2][slot] = ro.z;
            pool.rd[0][slot] = rd.x;
            pool.rd[1][slot] = rd.y;
            pool.rd[2][slot] = rd.z;
            __threadfence_block();
        }
        return q_push<P>(pool.rq, &pool.rq_tail, emit, slot, lane);
    };
    const uint32_t warp = threadIdx.x >> 5;
    if (warp >= (uint32_t)NS) {
        // traversal warps: their lanes' stacks are the first 32 * (NW - NS)
        // columns of the shared stack array
        traversal_warp<COUNT, FAST, P, STEPS>(pool, p, sstack + (threadIdx.x - 32 * NS), 32 * (NW - NS), lane, vc,
                                              err);
    } else {
        // the shading warp: up to 32 queued hits per round
        bool ok = true;
        uint64_t idle_since = 0;
        for (;;) {
            if (warp_flag(vload(pool.abort) != 0u)) break;
            const uint32_t slot = q_pop<P>(pool.hq, &pool.hq_head, &pool.hq_tail, kFull, lane, &ok);
            if (!__all_sync(kFull, ok)) {
                pool.abort = 1;
                err |= ERR_WAIT;
                break;
            }
            if (__ballot_sync(kFull, slot != kEmpty) == 0u) {
                if (warp_flag(vload(pool.exhausted) != 0u && vload(pool.active) == 0u)) break;
                const uint64_t now = wave_timer();
                if (idle_since == 0) idle_since = now;
                else if (now - idle_since > kWaitLimitNs) {
                    pool.abort = 1;
                    err |= ERR_WAIT;
                    break;
                }
                __nanosleep(64);
                continue;
            }
            idle_since = 0;
            if (!shade(slot)) {
                pool.abort = 1;
                err |= ERR_WAIT;
                break;
            }
        }
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

// ---- host-side launcher ------------------------------------------------------------
namespace {

// The compiled block shapes (WaveConfig::shape, orn_wave_config.shape):
// warps per block, shading warps among them, path slots per block (more
// slots than traversal lanes, so lanes find rays while other paths wait to
// be shaded) and the resident blocks per SM the registers are capped for.
// Measured on the 1080p plain workload (Msamples/s; the megakernel 365):
// 10 warps (9 + 1) x 2 blocks 354, 11 + 1 x 2 blocks 329, 7 + 1 x 3 blocks
// 320 (80 registers); also tried: 8 + 2 x 2 blocks 325, 6 + 2 x 3 blocks
// 284, 5 + 1 x 4 blocks 308, 7 + 1 x 2 blocks 304, 14 + 2 x 1 block 305.
template <int SHAPE>
struct Shape;
template <>
struct Shape<0> {
    static constexpr int W = 10, S = 1, P = 320, B = 2;
};
template <>
struct Shape<1> {
    static constexpr int W = 8, S = 1, P = 256, B = 3;
};
template <>
struct Shape<2> {
    static constexpr int W = 12, S = 1, P = 384, B = 2;
};
template <>
struct Shape<3> {
    static constexpr int W = 11, S = 1, P = 352, B = 2;
};

template <int SHAPE>
constexpr size_t shape_smem() {
    using T = Shape<SHAPE>;
    return ((sizeof(Pool<T::P>) + 15) / 16) * 16 + sizeof(uint32_t) * kSmemStack * 32 * (T::W - T::S);
}

template <int SEM, bool COUNT, bool FAST, int SHAPE, int STEPS>
cudaError_t launch_wave_t(const RenderLaunch& p, cudaStream_t s) {
    using T = Shape<SHAPE>;
    constexpr int kBlock = 32 * T::W;
    constexpr size_t kSmem = shape_smem<SHAPE>();
    static int blocks_per_sm = 0, sms = 0;
    auto kern = wave_kernel<SEM, COUNT, FAST, T::W, T::S, T::P, T::B, STEPS>;
    // more than 48 KB of dynamic shared memory: an opt-in per device
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
    if (e != cudaSuccess) return e;
    if (blocks_per_sm == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, kBlock, kSmem);
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    // enough blocks for every pixel to have a slot, at most one wave of resident blocks
    uint32_t need = (p.pixel_count + T::P - 1) / T::P;
    uint32_t grid = (uint32_t)(blocks_per_sm * sms);
    if (need < grid) grid = need;
    e = cudaMemsetAsync(p.work_counter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    kern<<<grid, kBlock, kSmem, s>>>(p);
    return cudaGetLastError();
}

template <int SEM, bool FAST, int STEPS>
cudaError_t launch_wave_steps(const RenderLaunch& p, int shape, cudaStream_t s) {
    switch (shape) {
        case 1: return launch_wave_t<SEM, false, FAST, 1, STEPS>(p, s);
        case 2: return launch_wave_t<SEM, false, FAST, 2, STEPS>(p, s);
        case 3: return launch_wave_t<SEM, false, FAST, 3, STEPS>(p, s);
        default: return launch_wave_t<SEM, false, FAST, 0, STEPS>(p, s);
    }
}

// Counting launches (a diagnostics mode) are compiled for shape 0 with 32
// steps per round only.
template <int SEM, bool FAST>
cudaError_t launch_wave_shape(const RenderLaunch& p, const WaveConfig& c, bool count, cudaStream_t s) {
    if (count) return launch_wave_t<SEM, true, FAST, 0, 32>(p, s);
    return c.steps == 64 ? launch_wave_steps<SEM, FAST, 64>(p, c.shape, s)
                         : launch_wave_steps<SEM, FAST, 32>(p, c.shape, s);
}

}  // namespace

bool wave_shape_info(int shape, int* warps, int* shading, int* slots, int* blocks_per_sm) {
    int w = 0, sh = 0, sl = 0, b = 0;
    switch (shape) {
        case 0: w = Shape<0>::W; sh = Shape<0>::S; sl = Shape<0>::P; b = Shape<0>::B; break;
        case 1: w = Shape<1>::W; sh = Shape<1>::S; sl = Shape<1>::P; b = Shape<1>::B; break;
        case 2: w = Shape<2>::W; sh = Shape<2>::S; sl = Shape<2>::P; b = Shape<2>::B; break;
        case 3: w = Shape<3>::W; sh = Shape<3>::S; sl = Shape<3>::P; b = Shape<3>::B; break;
        default: return false;
    }
    if (warps) *warps = w;
    if (shading) *shading = sh;
    if (slots) *slots = sl;
    if (blocks_per_sm) *blocks_per_sm = b;
    return true;
}

cudaError_t launch_wave(const RenderLaunch& p, const WaveConfig& c, int semantics, bool count, bool fast,
                        cudaStream_t s) {
    if (!wave_config_valid(c.shape, c.fetch, c.steps) || p.wave_fetch != c.fetch) return cudaErrorInvalidValue;
    if (semantics == SEM_WGSL)
        return fast ? launch_wave_shape<SEM_WGSL, true>(p, c, count, s)
                    : launch_wave_shape<SEM_WGSL, false>(p, c, count, s);
    return fast ? launch_wave_shape<SEM_HIP, true>(p, c, count, s) : launch_wave_shape<SEM_HIP, false>(p, c, count, s);
}

}  // namespace orn
