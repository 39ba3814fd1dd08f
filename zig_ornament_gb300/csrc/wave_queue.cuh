// wave_queue.cuh — shared-memory work queues of the persistent wavefront
// kernels (wave.cu, wave_cached.cu) and the loop their warps run.
//
// Queues are rings of P entries holding path-slot indices (a slot is in at
// most one queue at a time, so a ring never holds more than P entries).  A
// producer reserves positions with one atomicAdd per warp and fills each
// with a compare-and-swap from the empty marker (the position's previous
// entry may still be on its way out); a consumer reserves only entries below
// the producers' reservations (compare-and-swap on the head) and takes each
// with an exchange back to empty (the producer may not have written it
// yet).  Every wait is bounded by %globaltimer.
#pragma once

#include "pt_kernels.h"
#include "pt_device.cuh"
#include "pt_machine.cuh"

namespace orn {
namespace wave {

constexpr uint32_t kEmpty = 0xffffffffu;
constexpr uint64_t kWaitLimitNs = 5000000000ull;   // 5 s: any real wait is microseconds
enum SlotFlag { HIT_MISS = 0, HIT_ANY = 1, HIT_FAILED = 2, NEED_PIXEL = 3 };
// What a warp of a wavefront block does (wave_warp): both kinds of work, only
// shading, or only traversal.
enum WarpRole { ROLE_BOTH = 0, ROLE_SHADE = 1, ROLE_TRAVERSE = 2 };

__device__ __forceinline__ uint64_t wave_timer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

template <typename T>
__device__ __forceinline__ T vload(const T& x) {
    return *(const volatile T*)&x;
}

// A block flag as lane 0 of the warp reads it, so that every lane of the
// warp takes the same branch.
__device__ __forceinline__ bool warp_flag(bool v) { return __shfl_sync(0xffffffffu, v ? 1 : 0, 0) != 0; }

// Entries in a queue, as lane 0 reads the counters (the same for the whole
// warp; a hint, the queue may change right after).
__device__ __forceinline__ uint32_t q_count(const uint32_t* head, const uint32_t* tail) {
    return __shfl_sync(0xffffffffu, vload(*tail) - vload(*head), 0);
}

// Appends `item` for every lane with `have` (all 32 lanes call); false when
// a wait ran out.
template <int P>
__device__ __forceinline__ bool q_push(uint32_t* q, uint32_t* tail, bool have, uint32_t item, uint32_t lane) {
    const unsigned m = __ballot_sync(0xffffffffu, have);
    if (m == 0u) return true;
    const unsigned leader = __ffs(m) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(tail, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    bool ok = true;
    if (have) {
        const uint32_t pos = (base + __popc(m & ((1u << lane) - 1u))) % P;
        // the position's previous entry may still be on its way out
        if (atomicCAS(q + pos, kEmpty, item) != kEmpty) {
            const uint64_t t0 = wave_timer();
            while (atomicCAS(q + pos, kEmpty, item) != kEmpty) {
                if (wave_timer() - t0 > kWaitLimitNs) { ok = false; break; }
                __nanosleep(32);
            }
        }
    }
    return __all_sync(0xffffffffu, ok);
}

// Takes up to popc(want) entries for the lanes in `want`, in lane order
// (all 32 lanes call); returns the lane's entry or kEmpty.  `*ok` turns
// false when a wait ran out.
template <int P>
__device__ __forceinline__ uint32_t q_pop(uint32_t* q, uint32_t* head, const uint32_t* tail, unsigned want,
                                          uint32_t lane, bool* ok) {
    const unsigned leader = __ffs(want) - 1u;
    uint32_t base = 0, take = 0;
    if (lane == leader) {
        const uint32_t n = __popc(want);
        for (int tries = 0; tries < 64; ++tries) {
            const uint32_t h = vload(*head), t = vload(*tail);
            take = min(n, t - h);
            if (take == 0u) break;
            if (atomicCAS(head, h, h + take) == h) {
                base = h;
                break;
            }
            take = 0;
        }
    }
    base = __shfl_sync(0xffffffffu, base, leader);
    take = __shfl_sync(0xffffffffu, take, leader);
    uint32_t item = kEmpty;
    if ((want >> lane) & 1u) {
        const uint32_t rank = __popc(want & ((1u << lane) - 1u));
        if (rank < take) {
            const uint32_t pos = (base + rank) % P;
            item = atomicExch(q + pos, kEmpty);
            if (item == kEmpty) {   // reserved by a producer, not yet written
                const uint64_t t0 = wave_timer();
                while ((item = atomicExch(q + pos, kEmpty)) == kEmpty) {
                    if (wave_timer() - t0 > kWaitLimitNs) { *ok = false; break; }
                    __nanosleep(32);
                }
            }
        }
    }
    __threadfence_block();
    return item;
}

// The loop every warp of a wavefront block runs.  A warp switches between
// the two kinds of work by the state of its own lanes and of the queues:
//   * while any lane has a ray in flight it traverses: every such lane
//     visits up to STEPS BVH nodes per round (walker_step), a finished ray's
//     hit record goes into its slot and the slot into the hit queue, and
//     idle lanes take the next rays from the ray queue once p.wave_fetch of
//     them are idle;
//   * once none has, it shades — 32 queued hits at a time, or whatever is
//     queued when no ray is waiting — through `shade(slot)` (called by all
//     32 lanes with the lane's slot or kEmpty; it runs the path logic, queues
//     the new rays and returns false when a wait ran out), and otherwise
//     takes new rays.
// So traversal keeps every lane it can busy, and shading runs on full warps
// by whichever warps have run out of rays, in whatever proportion the scene
// needs.  A ROLE_SHADE warp never traverses: it shades whatever hits are
// queued, so the ray queue is refilled while every other warp still has rays
// in flight; a ROLE_TRAVERSE warp never shades.  Measured on the 1080p plain
// workload (7 + 1 warps per block): traversal-only warps beside one shading
// warp 331 Msamples/s, warps that also shade when they run dry 275; on cached
// frames, where shading is heavier, two shading warps beside six that do both
// were fastest.  With ANY (shadow rays of the cached renderer) the slot also gives
// the ray's t_max and occluder test (pool.ray_tmax, occl_inv, occl_t).
// Returns when the block is finished (no pixel left, every slot retired)
// or a wait ran out (pool.abort, ERR_WAIT).
template <bool COUNT, bool FAST, bool ANY, int P, WarpRole ROLE, int STEPS, class Pool, class Shade>
__device__ __forceinline__ void wave_warp(Pool& pool, const RenderLaunch& p, uint32_t* sstack, int stride,
                                          uint32_t lane, VisitCount& vc, uint32_t& err, Shade&& shade) {
    // (a compile-time role: a traversal-only loop carries no shading code, so
    // the walker state does not compete with it for registers)
    constexpr bool shade_only = ROLE == ROLE_SHADE, traverse_only = ROLE == ROLE_TRAVERSE;
    const unsigned kFull = 0xffffffffu;
    TravStack<kSmemStack> stack;
    stack.sstack = sstack;
    stack.sstride = stride;
    const float t_min = p.cp.ray_cast_epsilon;
    const int fetch = p.wave_fetch;
    uint32_t slot = kEmpty, steps = 0;
    f3 ro = mk(0.0f, 0.0f, 0.0f), rd = ro;
    HitRec h;
    Walker w;
    bool ok = true;
    uint64_t idle_since = 0;
    auto fail = [&]() {
        pool.abort = 1;
        err |= ERR_WAIT;
    };
    for (;;) {
        if (warp_flag(vload(pool.abort) != 0u)) break;
        if (__ballot_sync(kFull, slot != kEmpty) == 0u) {
            // no ray in flight: shade, or take rays, or wait
            const uint32_t nh = q_count(&pool.hq_head, &pool.hq_tail);
            const uint32_t nr = shade_only ? 0u : q_count(&pool.rq_head, &pool.rq_tail);
            if (!traverse_only && (nh >= 32u || (nh > 0u && nr == 0u))) {
                const uint32_t s = q_pop<P>(pool.hq, &pool.hq_head, &pool.hq_tail, kFull, lane, &ok);
                if (!__all_sync(kFull, ok)) { fail(); break; }
                if (!shade(s)) { fail(); break; }
                idle_since = 0;
                continue;
            }
            if (nr == 0u) {
                if ((nh == 0u || traverse_only) && warp_flag(vload(pool.exhausted) != 0u && vload(pool.active) == 0u))
                    break;
                const uint64_t now = wave_timer();
                if (idle_since == 0) idle_since = now;
                else if (now - idle_since > kWaitLimitNs) { fail(); break; }
                __nanosleep(64);
                continue;
            }
        }
        const unsigned idle = __ballot_sync(kFull, slot == kEmpty);
        if (idle != 0u && ((int)__popc(idle) >= fetch || idle == kFull)) {
            const uint32_t got = q_pop<P>(pool.rq, &pool.rq_head, &pool.rq_tail, idle, lane, &ok);
            if (got != kEmpty) {
                slot = got;
                ro = mk(pool.ro[0][slot], pool.ro[1][slot], pool.ro[2][slot]);
                rd = mk(pool.rd[0][slot], pool.rd[1][slot], pool.rd[2][slot]);
                h.t = 0.0f; h.material = 0; h.type = 0; h.inv = 0; h.tri = 0; h.u = 0.0f; h.v = 0.0f;
                walker_begin(w, p.scene, ro, rd);
                if constexpr (ANY) {
                    w.t_max = pool.ray_tmax[slot];
                    w.occl_inv = pool.occl_inv[slot];
                    w.occl_t = pool.occl_t[slot];
                }
                steps = 0;
            }
            if (!__all_sync(kFull, ok)) { fail(); break; }
        }
        if (__ballot_sync(kFull, slot != kEmpty) == 0u) continue;   // the rays went to other warps
        idle_since = 0;
        bool fin = false;
        uint32_t flag = HIT_MISS;
        if (slot != kEmpty) {
#pragma unroll 1
            for (int s = 0; s < STEPS; ++s) {
                ++steps;
                const uint32_t e0 = err;
                if (!walker_step<COUNT, kSmemStack, FAST, ANY>(w, p.scene, ro, rd, t_min, &h, stack, &vc, &err)) {
                    fin = true;
                    flag = err != e0 ? HIT_FAILED : (w.any ? HIT_ANY : HIT_MISS);
                    break;
                }
            }
        }
        if (fin) {
            pool.t[slot] = h.t;
            pool.u[slot] = h.u;
            pool.v[slot] = h.v;
            pool.material[slot] = h.material;
            pool.type[slot] = h.type;
            pool.inv[slot] = h.inv;
            pool.tri[slot] = h.tri;
            pool.flag[slot] = flag;
            pool.steps[slot] += steps;
            __threadfence_block();
        }
        if (!q_push<P>(pool.hq, &pool.hq_tail, fin, slot, lane)) { fail(); break; }
        if (fin) slot = kEmpty;
    }
}

// A warp that only traverses (the plain wavefront's traversal warps): idle
// lanes take rays from the ray queue once p.wave_fetch of them are idle (or
// all are), every lane with a ray visits up to STEPS BVH nodes per round (a
// compile-time count: measured 1.8 % faster than the same count read from
// the launch), and a finished ray's hit record goes into its slot, the slot
// into the hit queue.  The same traversal as wave_warp's, in a loop that carries
// no shading code (measured: 331 against 274 Msamples/s for wave_warp with
// the traversal-only role on the 1080p workload).  Returns when the block is
// finished or a wait ran out.
template <bool COUNT, bool FAST, int P, int STEPS, class Pool>
__device__ __forceinline__ void traversal_warp(Pool& pool, const RenderLaunch& p, uint32_t* sstack, int stride,
                                               uint32_t lane, VisitCount& vc, uint32_t& err) {
    const unsigned kFull = 0xffffffffu;
    TravStack<kSmemStack> stack;
    stack.sstack = sstack;
    stack.sstride = stride;
    const float t_min = p.cp.ray_cast_epsilon;
    const int fetch = p.wave_fetch;
    uint32_t slot = kEmpty, steps = 0;
    f3 ro = mk(0.0f, 0.0f, 0.0f), rd = ro;
    HitRec h;
    Walker w;
    bool ok = true;
    uint64_t idle_since = 0;
    for (;;) {
        if (warp_flag(vload(pool.abort) != 0u)) break;
        const unsigned idle = __ballot_sync(kFull, slot == kEmpty);
        if (idle != 0u && ((int)__popc(idle) >= fetch || idle == kFull)) {
            const uint32_t got = q_pop<P>(pool.rq, &pool.rq_head, &pool.rq_tail, idle, lane, &ok);
            if (got != kEmpty) {
                slot = got;
                ro = mk(pool.ro[0][slot], pool.ro[1][slot], pool.ro[2][slot]);
                rd = mk(pool.rd[0][slot], pool.rd[1][slot], pool.rd[2][slot]);
                h.t = 0.0f; h.material = 0; h.type = 0; h.inv = 0; h.tri = 0; h.u = 0.0f; h.v = 0.0f;
                walker_begin(w, p.scene, ro, rd);
                steps = 0;
            }
            if (!__all_sync(kFull, ok)) {
                pool.abort = 1;
                err |= ERR_WAIT;
                break;
            }
        }
        if (__ballot_sync(kFull, slot != kEmpty) == 0u) {
            // nothing to trace: the block is finished, or its rays are being shaded
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
        bool fin = false;
        uint32_t flag = HIT_MISS;
        if (slot != kEmpty) {
            // visits counted once per round, as in the megakernel
            uint32_t s = 0;
            const uint32_t e0 = err;
#pragma unroll 1
            while (s < (uint32_t)STEPS) {
                ++s;
                if (!walker_step<COUNT, kSmemStack, FAST, false, COUNT>(w, p.scene, ro, rd, t_min, &h, stack, &vc,
                                                                        &err)) {
                    fin = true;
                    break;
                }
            }
            steps += s;
            if (!COUNT && !fin && !walker_account_round(w, s, &err)) fin = true;
            if (fin) flag = err != e0 ? HIT_FAILED : (w.any ? HIT_ANY : HIT_MISS);
        }
        if (fin) {
            pool.t[slot] = h.t;
            pool.u[slot] = h.u;
            pool.v[slot] = h.v;
            pool.material[slot] = h.material;
            pool.type[slot] = h.type;
            pool.inv[slot] = h.inv;
            pool.tri[slot] = h.tri;
            pool.flag[slot] = flag;
            pool.steps[slot] += steps;
            __threadfence_block();
        }
        if (!q_push<P>(pool.hq, &pool.hq_tail, fin, slot, lane)) {
            pool.abort = 1;
            err |= ERR_WAIT;
            break;
        }
        if (fin) slot = kEmpty;
    }
}

// Every slot starts in the hit queue asking for a pixel; the queues' and
// the block's counters start at zero.
template <int P, class Pool>
__device__ __forceinline__ void pool_init(Pool& pool) {
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
        pool.flag[i] = NEED_PIXEL;
        pool.hq[i] = i;
        pool.rq[i] = kEmpty;
    }
    if (threadIdx.x == 0) {
        pool.rq_head = pool.rq_tail = 0;
        pool.hq_head = 0;
        pool.hq_tail = P;
        pool.active = P;
        pool.exhausted = 0;
        pool.abort = 0;
    }
    __syncthreads();
}

}  // namespace wave
}  // namespace orn
