// wavefront.cu — persistent wavefront path tracer with compacted ray queues.
//
// Same result as the megakernel (and the reference's per-pass loop), bit
// for bit, computed in two alternating kernels over a pool of P path slots:
//
//   wf_logic   one thread per slot.  A slot whose ray has been traced is
//              shaded (material scatter → next bounce; miss/emission/depth →
//              the sample is accumulated and the next sample's camera ray is
//              made; after the last sample the pixel's accumulation, RNG
//              state and framebuffer value are written).  A slot without a
//              pixel takes the next one from a global counter (one atomic
//              per warp).  Every slot that has a new ray appends itself to
//              the ray queue; the warp's appends are compacted with
//              __ballot_sync/__popc into one atomicAdd.
//   wf_extend  persistent threads.  Each lane traverses one queued ray at a
//              time (one BVH node per loop iteration, pt_machine.cuh) and
//              writes the closest hit back to its slot; as soon as enough
//              lanes of a warp are free they take the next rays from the
//              queue, so lanes do not idle while others finish long rays.
//
// Each slot runs its pixel's samples in order with the pixel's RNG state, so
// per-pixel arithmetic is identical to the reference's.  The host drives the
// iterations and stops once a (lagged) readback of the queue length is zero;
// no kernel ever waits on another.
#include <cuda_fp16.h>

#include "pt_kernels.h"
#include "pt_device.cuh"
#include "pt_machine.cuh"

namespace orn {

enum SlotMode { SLOT_NEED_PIXEL = 0, SLOT_TRACED = 1, SLOT_RETIRED = 2 };

template <int SEM, int MATH, bool COUNT>
__global__ void __launch_bounds__(256)
wf_logic(WaveLaunch p, uint32_t iter) {
    const unsigned kFull = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lanes_below = (1u << lane) - 1u;
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = slot < p.slots;
    uint32_t* stat = p.qstat + 4 * (iter & 3);   // [queue count, pending slots, queue head]
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // the counters of iteration iter+2 were last used by iteration iter-2
        uint32_t* next = p.qstat + 4 * ((iter + 2) & 3);
        next[0] = 0;
        next[1] = 0;
        next[2] = 0;
        if (COUNT && iter == 0) atomicAdd(p.counters + 0, (unsigned long long)p.spp * p.pixel_count);
    }
    const uint32_t W = p.cp.width, H = p.cp.height;
    const float ci0 = p.cp.current_iteration;
    uint32_t mode = valid ? p.mode[slot] : SLOT_RETIRED;
    bool emit = false;
    uint32_t gid = 0, k = 0, bounce = 0;
    Rng rng{0};
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    f3 ro = mk(0.0f, 0.0f, 0.0f), rd = ro, color = ro;
    SampleCount scn = {0, 0, 0, 0};
    uint32_t err = 0;

    // Starts samples k.. of pixel gid (depth-0 samples finish at once);
    // returns true when a camera ray was made, false when the pixel is done.
    auto start_samples = [&]() -> bool {
        while (k < p.spp) {
            camera_ray<MATH>(p.cp, gid % W, gid / W, rng, &ro, &rd);
            color = mk(1.0f, 1.0f, 1.0f);
            bounce = 0;
            if (p.cp.depth > 0) return true;
            float ci = ci0 + (float)k;
            if (ci > 1.0f) acc = make_float4(acc.x + color.x, acc.y + color.y, acc.z + color.z, acc.w + 1.0f);
            else acc = make_float4(color.x, color.y, color.z, 1.0f);
            ++k;
        }
        p.acc[gid] = acc;
        p.rng[gid] = rng.state;
        if (p.do_post) {
            uint32_t x = gid % W, y = gid / W;
            uint32_t fbi = p.cp.flip_y != 0 ? W * (H - y - 1) + x : gid;
            p.fb[fbi] = post_process<SEM, MATH>(acc, ci0 + (float)(p.spp - 1), p.cp.inverted_gamma);
        }
        return false;
    };

    if (mode == SLOT_TRACED) {
        gid = p.pixel[slot];
        uint2 kb = p.kb[slot];
        k = kb.x;
        bounce = kb.y;
        rng.state = p.rng_state[slot];
        acc = p.accum[slot];
        float4 c4 = p.color[slot], o4 = p.ro[slot], d4 = p.rd[slot];
        color = mk(c4.x, c4.y, c4.z);
        ro = mk(o4.x, o4.y, o4.z);
        rd = mk(d4.x, d4.y, d4.z);
        float4 h0 = p.hit[2 * slot], h1 = p.hit[2 * slot + 1];
        HitRec h;
        h.t = h0.x;
        h.material = bits(h0.y);
        h.type = bits(h0.z);
        h.inv = bits(h0.w);
        h.tri = bits(h1.x);
        h.u = h1.y;
        h.v = h1.z;
        const bool any = bits(h1.w) != 0u;
        const bool failed = bits(h1.w) == 2u;
        bool cont;
        if (!any) {
            color = failed ? mk(0.0f, 0.0f, 0.0f) : sky_color(color, rd);
            cont = false;
        } else {
            cont = shade_hit<SEM, MATH, COUNT>(p.scene, p.cp, rng, h, &ro, &rd, &color, &scn);
        }
        if (cont && ++bounce < p.cp.depth) {
            emit = true;
        } else {
            float ci = ci0 + (float)k;
            if (ci > 1.0f) acc = make_float4(acc.x + color.x, acc.y + color.y, acc.z + color.z, acc.w + 1.0f);
            else acc = make_float4(color.x, color.y, color.z, 1.0f);
            ++k;
            emit = start_samples();
            if (!emit) mode = SLOT_NEED_PIXEL;
        }
    }
    // Slots without a pixel take the next ones (one atomic per warp).
    const unsigned need = __ballot_sync(kFull, mode == SLOT_NEED_PIXEL);
    if (need != 0u) {
        const unsigned leader = __ffs(need) - 1u;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(p.pixel_counter, (unsigned)__popc(need));
        base = __shfl_sync(kFull, base, leader);
        if (mode == SLOT_NEED_PIXEL) {
            uint32_t mine = base + __popc(need & lanes_below);
            if (mine < p.pixel_count) {
                gid = mine;
                rng.state = p.rng[gid];
                acc = ci0 > 1.0f ? p.acc[gid] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                k = 0;
                emit = start_samples();
                mode = emit ? SLOT_TRACED : SLOT_NEED_PIXEL;
                // a pixel whose samples all finished without rays (depth 0)
                // leaves the slot free for the next iteration
            } else {
                mode = SLOT_RETIRED;
            }
        }
    }
    if (emit) mode = SLOT_TRACED;
    // Append the slots with a new ray to the queue (compacted per warp).
    const unsigned em = __ballot_sync(kFull, emit);
    if (em != 0u) {
        const unsigned leader = __ffs(em) - 1u;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&stat[0], (unsigned)__popc(em));
        base = __shfl_sync(kFull, base, leader);
        if (emit) p.queue[base + __popc(em & lanes_below)] = slot;
    }
    // Slots that will ask for a pixel next iteration keep the loop going.
    const unsigned waiting = __ballot_sync(kFull, mode == SLOT_NEED_PIXEL);
    if (waiting != 0u && lane == __ffs(waiting) - 1u) atomicAdd(&stat[1], (unsigned)__popc(waiting));
    if (valid) {
        p.mode[slot] = mode;
        if (mode == SLOT_TRACED) {
            p.pixel[slot] = gid;
            p.kb[slot] = make_uint2(k, bounce);
            p.rng_state[slot] = rng.state;
            p.accum[slot] = acc;
            p.color[slot] = make_float4(color.x, color.y, color.z, 0.0f);
            p.ro[slot] = make_float4(ro.x, ro.y, ro.z, 0.0f);
            p.rd[slot] = make_float4(rd.x, rd.y, rd.z, 0.0f);
        }
    }
    if (err) atomicOr(p.error, err);
    if (COUNT) {
        atomicAdd(p.counters + 1, (unsigned long long)(emit ? 1u : 0u));
        atomicAdd(p.counters + 7, (unsigned long long)scn.sphere_hits);
        atomicAdd(p.counters + 8, (unsigned long long)scn.mesh_hits);
        atomicAdd(p.counters + 9, (unsigned long long)scn.textured);
    }
}

template <bool COUNT, bool FAST>
__global__ void __launch_bounds__(kMegaBlock)
wf_extend(WaveLaunch p, uint32_t iter) {
    __shared__ uint32_t sstack[kSmemStack * kMegaBlock];
    TravStack<kSmemStack> stack;
    stack.sstack = sstack + threadIdx.x;
    stack.sstride = kMegaBlock;
    const unsigned kFull = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lanes_below = (1u << lane) - 1u;
    const uint32_t count = *(volatile uint32_t*)&p.qstat[4 * (iter & 3)];
    uint32_t* head = &p.qstat[4 * (iter & 3) + 2];
    const float t_min = p.cp.ray_cast_epsilon;
    bool drained = count == 0;
    uint32_t slot = 0xffffffffu;
    f3 ro = mk(0.0f, 0.0f, 0.0f), rd = ro;
    HitRec h;
    Walker w;
    VisitCount vc = {0, 0, 0, 0, 0};
    uint32_t err = 0;
    for (;;) {
        const unsigned idle = __ballot_sync(kFull, slot == 0xffffffffu);
        if (!drained && idle != 0u && ((int)__popc(idle) >= p.fetch_threshold || idle == kFull)) {
            const unsigned leader = __ffs(idle) - 1u;
            const unsigned n = __popc(idle);
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(head, n);
            base = __shfl_sync(kFull, base, leader);
            if (base + n >= count) drained = true;
            if (slot == 0xffffffffu) {
                uint32_t mine = base + __popc(idle & lanes_below);
                if (mine < count) {
                    slot = p.queue[mine];
                    float4 o4 = p.ro[slot], d4 = p.rd[slot];
                    ro = mk(o4.x, o4.y, o4.z);
                    rd = mk(d4.x, d4.y, d4.z);
                    h.t = 0.0f; h.material = 0; h.type = 0; h.inv = 0; h.tri = 0; h.u = 0.0f; h.v = 0.0f;
                    walker_begin(w, p.scene, ro, rd);
                }
            }
        }
        if (drained && __ballot_sync(kFull, slot != 0xffffffffu) == 0u) break;
        if (slot != 0xffffffffu) {
            uint32_t e0 = err;
            if (!walker_step<COUNT, kSmemStack, FAST>(w, p.scene, ro, rd, t_min, &h, stack, &vc, &err)) {
                uint32_t flag = (err != e0) ? 2u : (w.any ? 1u : 0u);
                p.hit[2 * slot] = make_float4(h.t, __uint_as_float(h.material), __uint_as_float(h.type),
                                              __uint_as_float(h.inv));
                p.hit[2 * slot + 1] = make_float4(__uint_as_float(h.tri), h.u, h.v, __uint_as_float(flag));
                slot = 0xffffffffu;
            }
        }
    }
    if (err) atomicOr(p.error, err);
    if (COUNT) {
        atomicAdd(p.counters + 2, (unsigned long long)vc.visits);
        atomicAdd(p.counters + 3, (unsigned long long)vc.internal);
        atomicAdd(p.counters + 4, (unsigned long long)vc.sphere);
        atomicAdd(p.counters + 5, (unsigned long long)vc.mesh);
        atomicAdd(p.counters + 6, (unsigned long long)vc.tri);
    }
}

// ---- host-side launchers -----------------------------------------------------
template <int SEM, int MATH>
static cudaError_t logic_t(const WaveLaunch& p, uint32_t iter, bool count, cudaStream_t s) {
    dim3 grid((p.slots + 255) / 256);
    if (count) wf_logic<SEM, MATH, true><<<grid, 256, 0, s>>>(p, iter);
    else wf_logic<SEM, MATH, false><<<grid, 256, 0, s>>>(p, iter);
    return cudaGetLastError();
}

cudaError_t launch_wf_logic(const WaveLaunch& p, uint32_t iter, int semantics, int math, bool count,
                            cudaStream_t s) {
    if (semantics == SEM_WGSL)
        return math == MATH_DEVICE ? logic_t<SEM_WGSL, MATH_DEVICE>(p, iter, count, s)
                                   : logic_t<SEM_WGSL, MATH_PORTABLE>(p, iter, count, s);
    return math == MATH_DEVICE ? logic_t<SEM_HIP, MATH_DEVICE>(p, iter, count, s)
                               : logic_t<SEM_HIP, MATH_PORTABLE>(p, iter, count, s);
}

template <bool COUNT, bool FAST>
static cudaError_t extend_t(const WaveLaunch& p, uint32_t iter, cudaStream_t s) {
    static int blocks_per_sm = 0, sms = 0;
    if (blocks_per_sm == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, wf_extend<COUNT, FAST>, kMegaBlock, 0);
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    uint32_t grid = (uint32_t)(blocks_per_sm * sms);
    uint32_t need = (p.slots + kMegaBlock - 1) / kMegaBlock;
    if (need < grid) grid = need;
    wf_extend<COUNT, FAST><<<grid, kMegaBlock, 0, s>>>(p, iter);
    return cudaGetLastError();
}

cudaError_t launch_wf_extend(const WaveLaunch& p, uint32_t iter, bool count, bool fast, cudaStream_t s) {
    if (fast) return count ? extend_t<true, true>(p, iter, s) : extend_t<false, true>(p, iter, s);
    return count ? extend_t<true, false>(p, iter, s) : extend_t<false, false>(p, iter, s);
}

}  // namespace orn
