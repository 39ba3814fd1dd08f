// batch.cu — batched persistent renderer: one render() of many contexts
// (scenes of any size, resolution and sample count) in one launch, replayed
// as a CUDA graph, with a launch shape chosen by an autotuner whose choice is
// kept in a JSON file.
//
// Each context keeps its own scene arrays and targets.  A frame's pixel
// space is the concatenation of the contexts' pixels; persistent warps take
// 32-pixel runs from one counter, so a context with a small frame does not
// leave the GPU idle while a large one finishes, and one launch replaces one
// launch (or more) per context.  The per-context views (scene pointers,
// ConstantParams, targets) stay in global memory, read through the L1; a
// lane keeps its scene's node array and root in registers for traversal and
// reads the rest of its view when it starts a pixel or shades, so traversal
// and shading are the megakernel's (pt_machine.cuh, pt_device.cuh) with
// per-lane scenes, and each pixel's bits equal those of orn_render on its
// context.  Shared memory holds only the traversal stacks, which leaves the
// L1 to the node fetches.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "batch.h"
#include "pt_kernels.h"
#include "pt_device.cuh"
#include "pt_machine.cuh"
#include "tune_cache.h"

namespace orn {

namespace {

enum BatchLane { B_IDLE = 0, B_TRAVERSE = 1, B_SHADE = 2, B_DONE = 3 };

// Resident blocks per SM each block size is compiled for (80 registers a
// thread at 128 and 192).
template <int BLOCK> constexpr int batch_min_blocks() { return BLOCK == 64 ? 8 : (BLOCK == 128 ? 6 : 4); }

template <int SEM, bool FAST, int BLOCK>
__global__ void __launch_bounds__(BLOCK, batch_min_blocks<BLOCK>())
batch_kernel(const BatchView* __restrict__ views, uint32_t nviews, uint32_t total_pixels, uint32_t* work_counter,
             uint32_t* error, int shade_threshold) {
    __shared__ uint32_t sstack[kSmemStack * BLOCK];
    const BatchView* __restrict__ sv = views;
    TravStack<kSmemStack> stack;
    stack.sstack = sstack + threadIdx.x;
    stack.sstride = BLOCK;
    const unsigned kFull = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lanes_below = (1u << lane) - 1u;

    int mode = B_IDLE;
    bool exhausted = false;
    uint32_t sc = 0, gid = 0, k = 0, bounce = 0;
    // the lane's scene as traversal sees it: walker_begin / walker_step read
    // only the node array, the root and the triangle-test choice
    SceneDev tsc;
    tsc.nodes = nullptr;
    tsc.root_ref = 0;
    tsc.exact_slabs = 0;
    tsc.watertight = 0;
    Rng rng{0};
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    f3 ro = mk(0.0f, 0.0f, 0.0f), rd = ro, color = ro;
    HitRec h;
    h.t = 0.0f; h.material = 0; h.type = 0; h.inv = 0; h.tri = 0; h.u = 0.0f; h.v = 0.0f;
    Walker w;
    VisitCount vc = {0, 0, 0, 0, 0};
    SampleCount scn = {0, 0, 0, 0};
    uint32_t err = 0;

    auto add_sample = [&](float ci) {
        if (ci > 1.0f) acc = make_float4(acc.x + color.x, acc.y + color.y, acc.z + color.z, acc.w + 1.0f);
        else acc = make_float4(color.x, color.y, color.z, 1.0f);
    };
    // Starts sample k of pixel gid of context sc (as the megakernel does).
    auto start_samples = [&]() -> int {
        const BatchView& V = sv[sc];
        const uint32_t W = V.cp.width, H = V.cp.height;
        while (k < V.spp) {
            camera_ray<MATH_PORTABLE>(V.cp, gid % W, gid / W, rng, &ro, &rd);
            color = mk(1.0f, 1.0f, 1.0f);
            bounce = 0;
            if (V.cp.depth > 0) {
                walker_begin(w, tsc, ro, rd);
                return B_TRAVERSE;
            }
            add_sample(V.cp.current_iteration + (float)k);
            ++k;
        }
        V.acc[gid] = acc;
        V.rng[gid] = rng.state;
        const uint32_t x = gid % W, y = gid / W;
        const uint32_t fbi = V.cp.flip_y != 0 ? W * (H - y - 1) + x : gid;
        V.fb[fbi] = post_process<SEM, MATH_PORTABLE>(acc, V.cp.current_iteration + (float)(V.spp - 1),
                                                     V.cp.inverted_gamma);
        return B_IDLE;
    };

    for (;;) {
        const unsigned idle = __ballot_sync(kFull, mode == B_IDLE);
        if (idle != 0u && !exhausted) {
            const unsigned leader = __ffs(idle) - 1u;
            const unsigned n = __popc(idle);
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(work_counter, n);
            base = __shfl_sync(kFull, base, leader);
            if (base + n >= total_pixels) exhausted = true;
            if (mode == B_IDLE) {
                const uint32_t mine = base + __popc(idle & lanes_below);
                if (mine < total_pixels) {
                    // the context owning pixel `mine`: last view with pixel_begin <= mine
                    uint32_t lo = 0, hi = nviews - 1u;
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi + 1u) >> 1;
                        if (sv[mid].pixel_begin <= mine) lo = mid;
                        else hi = mid - 1u;
                    }
                    sc = lo;
                    tsc.nodes = sv[sc].scene.nodes;
                    tsc.root_ref = sv[sc].scene.root_ref;
                    tsc.watertight = sv[sc].scene.watertight;
                    gid = mine - sv[sc].pixel_begin;
                    rng.state = sv[sc].rng[gid];
                    acc = sv[sc].cp.current_iteration > 1.0f ? sv[sc].acc[gid] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    k = 0;
                    mode = start_samples();
                }
            }
        }
        if (exhausted && mode == B_IDLE) mode = B_DONE;
        if (__ballot_sync(kFull, mode == B_TRAVERSE || mode == B_SHADE) == 0u &&
            __ballot_sync(kFull, mode == B_IDLE) == 0u)
            break;

        if (mode == B_TRAVERSE) {
            const float t_min = sv[sc].cp.ray_cast_epsilon;
#pragma unroll 1
            for (int s = 0; s < kStepsPerIteration; ++s) {
                if (!walker_step<false, kSmemStack, FAST>(w, tsc, ro, rd, t_min, &h, stack, &vc, &err)) {
                    mode = B_SHADE;
                    break;
                }
            }
        }

        const unsigned ready = __ballot_sync(kFull, mode == B_SHADE);
        const unsigned busy = __ballot_sync(kFull, mode == B_TRAVERSE);
        if (ready != 0u && ((int)__popc(ready) >= shade_threshold || busy == 0u)) {
            if (mode == B_SHADE) {
                const BatchView& V = sv[sc];
                bool cont;
                if (!w.any) {
                    if (err) color = mk(0.0f, 0.0f, 0.0f);
                    else color = sky_color(color, rd);
                    cont = false;
                } else {
                    cont = shade_hit<SEM, MATH_PORTABLE, false>(V.scene, V.cp, rng, h, &ro, &rd, &color, &scn);
                }
                if (cont && ++bounce < V.cp.depth) {
                    walker_begin(w, tsc, ro, rd);
                    mode = B_TRAVERSE;
                } else {
                    add_sample(V.cp.current_iteration + (float)k);
                    ++k;
                    mode = start_samples();
                }
            }
        }
        __syncwarp();
    }
    if (err) atomicOr(error, err);
}

// SM count and resident blocks of one instantiation, queried once (the
// first query runs before any stream capture: launch_frame primes it).
template <int SEM, bool FAST, int BLOCK>
void occupancy(int* sms_out, int* maxb_out) {
    static int sms = 0, maxb = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, batch_kernel<SEM, FAST, BLOCK>, BLOCK, 0);
    }
    *sms_out = sms;
    *maxb_out = maxb;
}

template <int SEM, bool FAST, int BLOCK>
cudaError_t launch_tt(const BatchView* views, uint32_t nviews, uint32_t total_pixels, uint32_t* work_counter,
                      uint32_t* error, const BatchConfig& cfg, cudaStream_t s) {
    int sms = 0, maxb = 0;
    occupancy<SEM, FAST, BLOCK>(&sms, &maxb);
    const int per_sm = std::max(1, std::min(cfg.blocks_per_sm, std::max(maxb, 1)));
    uint32_t grid = (uint32_t)(per_sm * sms);
    const uint32_t need = (total_pixels + BLOCK - 1) / BLOCK;
    if (need < grid) grid = std::max<uint32_t>(need, 1u);
    batch_kernel<SEM, FAST, BLOCK><<<grid, BLOCK, 0, s>>>(views, nviews, total_pixels, work_counter, error,
                                                           cfg.shade_threshold);
    return cudaGetLastError();
}

template <int SEM, bool FAST>
cudaError_t launch_t(const BatchView* views, uint32_t nviews, uint32_t total_pixels, uint32_t* work_counter,
                     uint32_t* error, const BatchConfig& cfg, cudaStream_t s) {
    switch (cfg.block) {
        case 64: return launch_tt<SEM, FAST, 64>(views, nviews, total_pixels, work_counter, error, cfg, s);
        case 192: return launch_tt<SEM, FAST, 192>(views, nviews, total_pixels, work_counter, error, cfg, s);
        default: return launch_tt<SEM, FAST, 128>(views, nviews, total_pixels, work_counter, error, cfg, s);
    }
}

template <int SEM, bool FAST>
int max_blocks_t(int block) {
    int sms = 0, m = 0;
    if (block == 64) occupancy<SEM, FAST, 64>(&sms, &m);
    else if (block == 192) occupancy<SEM, FAST, 192>(&sms, &m);
    else occupancy<SEM, FAST, 128>(&sms, &m);
    return m;
}

}  // namespace

cudaError_t launch_batch(const BatchView* views, uint32_t nviews, uint32_t total_pixels, uint32_t* work_counter,
                         uint32_t* error, int semantics, bool fast, const BatchConfig& cfg, cudaStream_t s) {
    if (semantics == SEM_WGSL)
        return fast ? launch_t<SEM_WGSL, true>(views, nviews, total_pixels, work_counter, error, cfg, s)
                    : launch_t<SEM_WGSL, false>(views, nviews, total_pixels, work_counter, error, cfg, s);
    return fast ? launch_t<SEM_HIP, true>(views, nviews, total_pixels, work_counter, error, cfg, s)
                : launch_t<SEM_HIP, false>(views, nviews, total_pixels, work_counter, error, cfg, s);
}

int batch_max_blocks_per_sm(int block, int semantics, bool fast) {
    if (semantics == SEM_WGSL) return fast ? max_blocks_t<SEM_WGSL, true>(block) : max_blocks_t<SEM_WGSL, false>(block);
    return fast ? max_blocks_t<SEM_HIP, true>(block) : max_blocks_t<SEM_HIP, false>(block);
}

}  // namespace orn

// ---- host object ------------------------------------------------------------------------
struct orn_batch {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr, ev_done = nullptr;
    std::vector<orn_context*> contexts;
    orn::BatchView* h_views = nullptr;   // pinned
    orn::BatchView* d_views = nullptr;
    uint32_t* d_work = nullptr;
    uint32_t* d_error = nullptr;
    orn::BatchConfig config{128, 6, 8};
    bool tuned = false;
    // the captured frame and what it was captured for
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint32_t g_nviews = 0, g_pixels = 0, g_sem = 0;
    bool g_fast = false;
    orn::BatchConfig g_cfg{0, 0, 0};
    bool rendered = false;
    uint64_t frames = 0;
    std::string last_error;
};

namespace {

int bfail(orn_batch* b, int st, const std::string& msg) {
    if (b) b->last_error = msg;
    return st;
}

#define B_CUDA(b, call)                                                                                   \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return bfail((b), e_ == cudaErrorMemoryAllocation ? ORN_ERR_OUT_OF_MEMORY : ORN_ERR_CUDA,     \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                             \
    } while (0)

void drop_graph(orn_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// Host side of one frame: every context's orn_render bookkeeping, the view
// table (pinned) and the frame's pixel total.
int prepare_frame(orn_batch* b, uint32_t* total_pixels, uint32_t* semantics, bool* fast) {
    uint64_t total = 0;
    bool all_fast = true;
    uint32_t sem0 = 0;
    for (size_t i = 0; i < b->contexts.size(); ++i) {
        orn::BatchView v;
        bool f = false;
        uint32_t sem = 0;
        int dev = 0;
        int st = orn::batch_prepare(b->contexts[i], &v, &f, &sem, &dev, b->stream, true);
        if (st) return bfail(b, st, std::string("context ") + std::to_string(i) + ": " + orn_last_error(b->contexts[i]));
        if (dev != b->device) return bfail(b, ORN_ERR_INVALID_ARGUMENT, "contexts on different devices");
        if (i == 0) sem0 = sem;
        else if (sem != sem0) return bfail(b, ORN_ERR_INVALID_ARGUMENT, "contexts with different semantics");
        v.pixel_begin = (uint32_t)total;
        total += (uint64_t)v.cp.width * v.cp.height;
        if (total >= 0xFFFFFFFFull) return bfail(b, ORN_ERR_INVALID_ARGUMENT, "batch frame too large");
        all_fast = all_fast && f;
        b->h_views[i] = v;
    }
    *total_pixels = (uint32_t)total;
    *semantics = sem0;
    *fast = all_fast;
    return ORN_OK;
}

// Queues one frame: the view table, the work counter and the kernel, from a
// CUDA graph captured for this (view count, pixel total, semantics, slab
// mode, launch shape) and replayed afterwards.
int launch_frame(orn_batch* b, uint32_t nviews, uint32_t total, uint32_t sem, bool fast) {
    const orn::BatchConfig& c = b->config;
    const bool same = b->exec && b->g_nviews == nviews && b->g_pixels == total && b->g_sem == sem &&
                      b->g_fast == fast && b->g_cfg.block == c.block && b->g_cfg.blocks_per_sm == c.blocks_per_sm &&
                      b->g_cfg.shade_threshold == c.shade_threshold;
    if (!same) {
        drop_graph(b);
        // the launcher's device queries happen here, outside the capture
        orn::batch_max_blocks_per_sm(c.block, (int)sem, fast);
        B_CUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaMemcpyAsync(b->d_views, b->h_views, nviews * sizeof(orn::BatchView),
                                        cudaMemcpyHostToDevice, b->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(b->d_work, 0, 4, b->stream);
        if (e == cudaSuccess)
            e = orn::launch_batch(b->d_views, nviews, total, b->d_work, b->d_error, (int)sem, fast, c, b->stream);
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return bfail(b, ORN_ERR_CUDA, std::string("capturing the batch frame: ") +
                                              cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        b->graph = g;
        B_CUDA(b, cudaGraphInstantiate(&b->exec, b->graph, 0));
        b->g_nviews = nviews;
        b->g_pixels = total;
        b->g_sem = sem;
        b->g_fast = fast;
        b->g_cfg = c;
    }
    B_CUDA(b, cudaGraphLaunch(b->exec, b->stream));
    return ORN_OK;
}

// ---- autotuner cache: {"<key>": {"block": B, "blocks_per_sm": N, "shade_threshold": T, "ms": X}, ...}
// The launch configurations the batched kernel is compiled for.
bool valid_config(int block, int blocks_per_sm, int shade_threshold) {
    return (block == 64 || block == 128 || block == 192) && blocks_per_sm >= 1 && blocks_per_sm <= 32 &&
           shade_threshold >= 1 && shade_threshold <= 32;
}

// The file's entries that hold a launchable configuration (one outside the
// range, from a hand-edited or foreign file, is dropped: its workload is
// tuned again).
std::map<std::string, orn::BatchConfig> read_cache(const char* path) {
    std::map<std::string, orn::BatchConfig> out;
    for (const auto& kv : orn::read_tune_cache(path)) {
        const auto& f = kv.second.fields;
        auto b = f.find("block"), n = f.find("blocks_per_sm"), t = f.find("shade_threshold");
        if (b == f.end() || n == f.end() || t == f.end()) continue;
        orn::BatchConfig c{(int)b->second, (int)n->second, (int)t->second};
        if (valid_config(c.block, c.blocks_per_sm, c.shade_threshold)) out[kv.first] = c;
    }
    return out;
}

}  // namespace

extern "C" {

int orn_batch_create(orn_context* const* contexts, uint32_t count, orn_batch** out) {
    if (!out || !contexts || count == 0) return ORN_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (count > orn::kMaxBatch) return ORN_ERR_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < count; ++i)
        if (!contexts[i]) return ORN_ERR_INVALID_ARGUMENT;
    int dev = -1;
    int st = orn_get_device(contexts[0], &dev);
    if (st) return st;
    orn_batch* b = new orn_batch();
    b->contexts.assign(contexts, contexts + count);
    b->device = dev;
    auto bail = [&](int s) {
        orn_batch_destroy(b);
        return s;
    };
    for (uint32_t i = 0; i < count; ++i) {
        int d = -1;
        if (orn_get_device(contexts[i], &d) || d != dev) return bail(ORN_ERR_INVALID_ARGUMENT);
    }
    if (cudaSetDevice(dev) != cudaSuccess) return bail(ORN_ERR_CUDA);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev_start) != cudaSuccess || cudaEventCreate(&b->ev_stop) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming) != cudaSuccess)
        return bail(ORN_ERR_CUDA);
    if (cudaMallocHost(&b->h_views, orn::kMaxBatch * sizeof(orn::BatchView)) != cudaSuccess ||
        cudaMalloc(&b->d_views, orn::kMaxBatch * sizeof(orn::BatchView)) != cudaSuccess ||
        cudaMalloc(&b->d_work, 4) != cudaSuccess || cudaMalloc(&b->d_error, 4) != cudaSuccess ||
        cudaMemset(b->d_error, 0, 4) != cudaSuccess)
        return bail(ORN_ERR_OUT_OF_MEMORY);
    *out = b;
    return ORN_OK;
}

int orn_batch_destroy(orn_batch* b) {
    if (!b) return ORN_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    if (b->h_views) cudaFreeHost(b->h_views);
    if (b->d_views) cudaFree(b->d_views);
    if (b->d_work) cudaFree(b->d_work);
    if (b->d_error) cudaFree(b->d_error);
    if (b->ev_start) cudaEventDestroy(b->ev_start);
    if (b->ev_stop) cudaEventDestroy(b->ev_stop);
    if (b->ev_done) cudaEventDestroy(b->ev_done);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return ORN_OK;
}

int orn_batch_render(orn_batch* b) {
    if (!b) return ORN_ERR_INVALID_ARGUMENT;
    B_CUDA(b, cudaSetDevice(b->device));
    // the previous frame has read the pinned view table before it is rewritten
    B_CUDA(b, cudaEventSynchronize(b->ev_done));
    uint32_t total = 0, sem = 0;
    bool fast = false;
    int st = prepare_frame(b, &total, &sem, &fast);
    if (st) return st;
    B_CUDA(b, cudaEventRecord(b->ev_start, b->stream));
    st = launch_frame(b, (uint32_t)b->contexts.size(), total, sem, fast);
    if (st) return st;
    B_CUDA(b, cudaEventRecord(b->ev_stop, b->stream));
    B_CUDA(b, cudaEventRecord(b->ev_done, b->stream));
    for (orn_context* c : b->contexts) {
        st = orn::batch_finish(c, b->ev_done);
        if (st) return bfail(b, st, orn_last_error(c));
    }
    b->rendered = true;
    b->frames++;
    return ORN_OK;
}

int orn_batch_synchronize(orn_batch* b) {
    if (!b) return ORN_ERR_INVALID_ARGUMENT;
    B_CUDA(b, cudaSetDevice(b->device));
    B_CUDA(b, cudaStreamSynchronize(b->stream));
    uint32_t err = 0;
    B_CUDA(b, cudaMemcpy(&err, b->d_error, 4, cudaMemcpyDeviceToHost));
    if (err) {
        B_CUDA(b, cudaMemset(b->d_error, 0, 4));
        if (err & orn::ERR_STACK)
            return bfail(b, ORN_ERR_STACK_OVERFLOW, "a ray needed more than 64 traversal stack entries");
        return bfail(b, ORN_ERR_TIMEOUT, "a ray exceeded the per-ray node-visit limit");
    }
    return ORN_OK;
}

int orn_batch_last_render_ms(orn_batch* b, float* ms) {
    if (!b || !ms) return ORN_ERR_INVALID_ARGUMENT;
    if (!b->rendered) return bfail(b, ORN_ERR_INVALID_ARGUMENT, "nothing rendered yet");
    int st = orn_batch_synchronize(b);
    if (st) return st;
    B_CUDA(b, cudaEventElapsedTime(ms, b->ev_start, b->ev_stop));
    return ORN_OK;
}

int orn_batch_get_config(const orn_batch* b, orn_batch_config* out) {
    if (!b || !out) return ORN_ERR_INVALID_ARGUMENT;
    out->block = (uint32_t)b->config.block;
    out->blocks_per_sm = (uint32_t)b->config.blocks_per_sm;
    out->shade_threshold = (uint32_t)b->config.shade_threshold;
    out->tuned = b->tuned ? 1u : 0u;
    return ORN_OK;
}

int orn_batch_set_config(orn_batch* b, const orn_batch_config* c) {
    if (!b || !c) return ORN_ERR_INVALID_ARGUMENT;
    if (!valid_config((int)c->block, (int)c->blocks_per_sm, (int)c->shade_threshold))
        return bfail(b, ORN_ERR_INVALID_ARGUMENT, "invalid batch launch configuration");
    b->config = orn::BatchConfig{(int)c->block, (int)c->blocks_per_sm, (int)c->shade_threshold};
    return ORN_OK;
}

int orn_batch_tune(orn_batch* b, const char* cache_path, orn_batch_config* chosen) {
    if (!b) return ORN_ERR_INVALID_ARGUMENT;
    B_CUDA(b, cudaSetDevice(b->device));
    B_CUDA(b, cudaStreamSynchronize(b->stream));
    // The tuning frames render into scratch targets with at most 2 passes
    // per context: the contexts' own images and progress are untouched.
    std::vector<orn::BatchView> saved(b->contexts.size());
    uint64_t total64 = 0, samples = 0;
    bool fast = true;
    uint32_t sem = 0;
    for (size_t i = 0; i < b->contexts.size(); ++i) {
        bool f = false;
        uint32_t sm = 0;
        int dev = 0;
        int st = orn::batch_prepare(b->contexts[i], &saved[i], &f, &sm, &dev, b->stream, false);
        if (st) return bfail(b, st, orn_last_error(b->contexts[i]));
        fast = fast && f;
        sem = sm;
        const uint32_t px = saved[i].cp.width * saved[i].cp.height;
        saved[i].pixel_begin = (uint32_t)total64;
        total64 += px;
        samples += (uint64_t)px * saved[i].spp;
    }
    if (total64 >= 0xFFFFFFFFull) return bfail(b, ORN_ERR_INVALID_ARGUMENT, "batch frame too large");
    const uint32_t total = (uint32_t)total64;
    char dev_name[256] = {0};
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, b->device) == cudaSuccess)
        std::snprintf(dev_name, sizeof(dev_name), "%s", prop.name);
    char key[512];
    std::snprintf(key, sizeof(key), "%s|sm%d|scenes=%zu|pixels=%u|samples=%llu|sem=%u|fast=%d", dev_name, b->sms,
                  b->contexts.size(), total, (unsigned long long)samples, sem, fast ? 1 : 0);
    auto cache = read_cache(cache_path);
    auto hit = cache.find(key);
    if (hit != cache.end()) {
        b->config = hit->second;
        b->tuned = true;
        if (chosen) orn_batch_get_config(b, chosen);
        return ORN_OK;
    }
    // scratch targets
    float4 *acc = nullptr, *fb = nullptr;
    uint32_t* rng = nullptr;
    B_CUDA(b, cudaMalloc(&acc, (size_t)total * sizeof(float4)));
    if (cudaMalloc(&fb, (size_t)total * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&rng, (size_t)total * 4) != cudaSuccess) {
        cudaFree(acc);
        if (fb) cudaFree(fb);
        return bfail(b, ORN_ERR_OUT_OF_MEMORY, "tuning scratch targets");
    }
    cudaMemsetAsync(acc, 0, (size_t)total * sizeof(float4), b->stream);
    cudaMemsetAsync(rng, 0x5A, (size_t)total * 4, b->stream);
    for (size_t i = 0; i < saved.size(); ++i) {
        orn::BatchView v = saved[i];
        v.acc = acc + v.pixel_begin;
        v.fb = fb + v.pixel_begin;
        v.rng = rng + v.pixel_begin;
        v.spp = std::min<uint32_t>(v.spp, 2u);
        v.cp.current_iteration = 1.0f;
        b->h_views[i] = v;
    }
    cudaMemcpyAsync(b->d_views, b->h_views, saved.size() * sizeof(orn::BatchView), cudaMemcpyHostToDevice, b->stream);
    const int blocks[3] = {64, 128, 192};
    const int thresholds[3] = {4, 8, 16};
    orn::BatchConfig best = b->config;
    float best_ms = 3.0e38f;
    int st = ORN_OK;
    for (int bi = 0; bi < 3 && st == ORN_OK; ++bi) {
        const int maxb = orn::batch_max_blocks_per_sm(blocks[bi], (int)sem, fast);
        if (maxb < 1) continue;
        const int fracs[3] = {maxb, std::max(1, (3 * maxb) / 4), std::max(1, maxb / 2)};
        for (int fi = 0; fi < 3 && st == ORN_OK; ++fi) {
            if (fi > 0 && fracs[fi] == fracs[fi - 1]) continue;
            for (int ti = 0; ti < 3; ++ti) {
                orn::BatchConfig c{blocks[bi], fracs[fi], thresholds[ti]};
                float ms = 0.0f;
                cudaError_t e = cudaSuccess;
                for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {   // the first run warms the caches
                    e = cudaMemsetAsync(b->d_work, 0, 4, b->stream);
                    if (e == cudaSuccess) e = cudaEventRecord(b->ev_start, b->stream);
                    if (e == cudaSuccess)
                        e = orn::launch_batch(b->d_views, (uint32_t)saved.size(), total, b->d_work, b->d_error,
                                              (int)sem, fast, c, b->stream);
                    if (e == cudaSuccess) e = cudaEventRecord(b->ev_stop, b->stream);
                    if (e == cudaSuccess) e = cudaEventSynchronize(b->ev_stop);
                    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, b->ev_start, b->ev_stop);
                }
                if (e != cudaSuccess) {
                    st = bfail(b, ORN_ERR_CUDA, std::string("tuning launch: ") + cudaGetErrorString(e));
                    break;
                }
                if (ms < best_ms) {
                    best_ms = ms;
                    best = c;
                }
            }
        }
    }
    cudaStreamSynchronize(b->stream);
    cudaFree(acc);
    cudaFree(fb);
    cudaFree(rng);
    if (st) return st;
    st = orn_batch_synchronize(b);
    if (st) return st;
    b->config = best;
    b->tuned = true;
    if (cache_path) {
        auto entries = orn::read_tune_cache(cache_path);
        orn::TuneEntry e;
        e.fields["block"] = best.block;
        e.fields["blocks_per_sm"] = best.blocks_per_sm;
        e.fields["shade_threshold"] = best.shade_threshold;
        e.ms = best_ms;
        entries[key] = e;
        orn::write_tune_cache(cache_path, entries, {"block", "blocks_per_sm", "shade_threshold"});
    }
    if (chosen) orn_batch_get_config(b, chosen);
    return ORN_OK;
}

const char* orn_batch_last_error(const orn_batch* b) { return b ? b->last_error.c_str() : "batch is NULL"; }

}  // extern "C"
