// noalloc.cu — a wavefront render entry point that allocates nothing.
//
// orn_render_noalloc renders with the persistent wavefront (wavefront.cu)
// into device buffers the caller provides, for callers that cannot allocate
// device memory while they render: engines whose frame loop must not call
// cudaMalloc (an allocation can synchronise the device and stall the frame)
// and hosts that give a plug-in a fixed memory budget.  Its working memory
// — one path slot per pixel, the ray queue and the iteration counters —
// lives in the file-scope array `g_noalloc_scratch` below, sized for
// kNoAllocMaxPixels pixels; every GPU that loads the library holds that
// array (about 15 MiB) until the process exits.
//
// Host code cannot use the array's name as a device address, so the first
// call on each device looks the address up with cudaGetSymbolAddress (with
// that device current) and keeps it; that first call should come before
// any stream capture.  Every call shares the one array: the call clears the
// parts that must start at zero, and calls whose work overlaps on the GPU
// (different streams, or another thread) race on it.
//
// The call never waits for the GPU: device-side errors of one call are
// reported by the next (through a pinned copy of the context's error word
// that each call queues behind its work), and the caller's current device
// is restored before returning.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "ornament_cuda.h"
#include "pt_kernels.h"

namespace {

constexpr uint32_t kNoAllocMaxPixels = ORN_NOALLOC_MAX_PIXELS;

// Byte layout of the scratch array (each region 256-byte aligned).
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }
constexpr size_t kOffCounters = 0;                                            // pixel counter + qstat
constexpr size_t kOffQueue = align_up(kOffCounters + 20 * sizeof(uint32_t));
constexpr size_t kOffMode = align_up(kOffQueue + (size_t)kNoAllocMaxPixels * 4);
constexpr size_t kOffPixel = align_up(kOffMode + (size_t)kNoAllocMaxPixels * 4);
constexpr size_t kOffKb = align_up(kOffPixel + (size_t)kNoAllocMaxPixels * 4);
constexpr size_t kOffRngState = align_up(kOffKb + (size_t)kNoAllocMaxPixels * 8);
constexpr size_t kOffAccum = align_up(kOffRngState + (size_t)kNoAllocMaxPixels * 4);
constexpr size_t kOffColor = align_up(kOffAccum + (size_t)kNoAllocMaxPixels * 16);
constexpr size_t kOffRo = align_up(kOffColor + (size_t)kNoAllocMaxPixels * 16);
constexpr size_t kOffRd = align_up(kOffRo + (size_t)kNoAllocMaxPixels * 16);
constexpr size_t kOffHit = align_up(kOffRd + (size_t)kNoAllocMaxPixels * 16);
constexpr size_t kScratchBytes = align_up(kOffHit + (size_t)kNoAllocMaxPixels * 32);

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on `device` (looked up once, with the
// device current).
cudaError_t scratch_address(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[device] = (unsigned char*)ptr;
    }
    *out = g_scratch_addr[device];
    return cudaSuccess;
}

}  // namespace

namespace orn {
bool noalloc_link(const orn_context* ctx, const orn_camera* camera, NoAllocLink* out);
}

namespace {

// Restores the caller's current device when the call returns.
struct DeviceRestore {
    int device = -1;
    ~DeviceRestore() {
        if (device >= 0) cudaSetDevice(device);
    }
};

int status_of(uint32_t err) {
    return (err & orn::ERR_STACK) ? ORN_ERR_STACK_OVERFLOW : ORN_ERR_TIMEOUT;
}

}  // namespace

extern "C" int orn_render_noalloc(const orn_context* ctx, const orn_constant_params* params, uint32_t spp,
                                  float* accumulation, uint32_t* rng_state, float* framebuffer, void* stream) {
    if (!ctx || !params || !accumulation || !rng_state || !framebuffer || spp == 0) return ORN_ERR_INVALID_ARGUMENT;
    const uint64_t pixels = (uint64_t)params->width * params->height;
    if (pixels == 0 || pixels > kNoAllocMaxPixels) return ORN_ERR_INVALID_ARGUMENT;
    if (params->depth > ORN_NOALLOC_MAX_DEPTH) return ORN_ERR_INVALID_ARGUMENT;
    orn::NoAllocLink link;
    if (!orn::noalloc_link(ctx, &params->camera, &link) || link.device < 0 || link.device >= kMaxDevices)
        return ORN_ERR_INVALID_ARGUMENT;
    int caller_device = -1;
    if (cudaGetDevice(&caller_device) != cudaSuccess) return ORN_ERR_CUDA;
    DeviceRestore restore;
    if (caller_device != link.device) {
        if (cudaSetDevice(link.device) != cudaSuccess) return ORN_ERR_CUDA;
        restore.device = caller_device;
    }
    unsigned char* base = nullptr;
    if (scratch_address(link.device, &base) != cudaSuccess) return ORN_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;

    // A device-side limit hit by the previous call's work (or any other work
    // of the context): reported once the pinned copy queued after that work
    // has arrived, without waiting for it.
    if (*link.pending) {
        const cudaError_t q = cudaEventQuery(*link.done);
        if (q == cudaSuccess) {
            *link.pending = false;
            const uint32_t err = *link.host_error;
            if (err) {
                *link.host_error = 0;
                if (cudaMemsetAsync(link.error_word, 0, sizeof(uint32_t), s) != cudaSuccess) return ORN_ERR_CUDA;
                return status_of(err);
            }
        } else if (q != cudaErrorNotReady) {
            return ORN_ERR_CUDA;
        }
    }

    orn::WaveLaunch w;
    std::memset(&w, 0, sizeof(w));
    w.scene = *link.scene;
    w.cp = *params;
    w.spp = spp;
    w.do_post = 1;
    w.pixel_count = (uint32_t)pixels;
    w.slots = (uint32_t)pixels;
    w.acc = (float4*)accumulation;
    w.fb = (float4*)framebuffer;
    w.rng = rng_state;
    w.error = link.error_word;
    w.counters = nullptr;
    w.pixel_counter = (uint32_t*)(base + kOffCounters);
    w.qstat = (uint32_t*)(base + kOffCounters) + 4;
    w.queue = (uint32_t*)(base + kOffQueue);
    w.mode = (uint32_t*)(base + kOffMode);
    w.pixel = (uint32_t*)(base + kOffPixel);
    w.kb = (uint2*)(base + kOffKb);
    w.rng_state = (uint32_t*)(base + kOffRngState);
    w.accum = (float4*)(base + kOffAccum);
    w.color = (float4*)(base + kOffColor);
    w.ro = (float4*)(base + kOffRo);
    w.rd = (float4*)(base + kOffRd);
    w.hit = (float4*)(base + kOffHit);
    w.fetch_threshold = orn::kFetchThreshold;

    // What must start at zero: the counters and every slot's mode.
    if (cudaMemsetAsync(base + kOffCounters, 0, 20 * sizeof(uint32_t), s) != cudaSuccess) return ORN_ERR_CUDA;
    if (cudaMemsetAsync(w.mode, 0, (size_t)pixels * 4, s) != cudaSuccess) return ORN_ERR_CUDA;
    // One slot per pixel: every pixel starts in the first iteration and a
    // pixel casts at most spp * depth rays, one per iteration, so
    // spp * (depth + 1) + 2 iterations finish the render (iterations after
    // the last ray find an empty queue and return at once).  No readback.
    const uint64_t iterations = (uint64_t)spp * ((uint64_t)params->depth + 1) + 2;
    for (uint64_t it = 0; it < iterations; ++it) {
        if (orn::launch_wf_logic(w, (uint32_t)it, (int)link.semantics, orn::MATH_PORTABLE, false, s) != cudaSuccess)
            return ORN_ERR_CUDA;
        if (orn::launch_wf_extend(w, (uint32_t)it, false, link.fast_slabs, s) != cudaSuccess) return ORN_ERR_CUDA;
    }
    // the error word after this call's work, for the next call to report
    if (cudaMemcpyAsync(link.host_error, link.error_word, sizeof(uint32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return ORN_ERR_CUDA;
    if (cudaEventRecord(*link.done, s) != cudaSuccess) return ORN_ERR_CUDA;
    *link.pending = true;
    return ORN_OK;
}
