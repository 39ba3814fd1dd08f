// rc_host.h — the radiance cache object behind the orn_cache_* entry points,
// shared by cache_capi.cu (its own calls) and capi.cu (cached rendering).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "ornament_cuda.h"
#include "rc_kernels.h"

struct orn_cache {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;   // for the host-buffer calls
    orn_cache_config config{};
    uint64_t steps = 0;
    uint64_t frames = 0;

    // parameters and optimiser state
    float* params = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float* grads = nullptr;
    uint16_t* w_f16 = nullptr;
    uint16_t* w_bf16 = nullptr;
    float* d_loss = nullptr;
    uint32_t* d_status = nullptr;

    // per-sample training activations, grown on demand
    uint32_t cap = 0;
    uint16_t* h = nullptr;     // [5][cap][64]
    uint16_t* dz = nullptr;    // [5][cap][64]
    uint16_t* dz6 = nullptr;   // [cap][16]

    // staging for the host-buffer calls, grown on demand
    uint32_t io_cap = 0;
    float* io_in = nullptr;
    float* io_target = nullptr;
    float* io_out = nullptr;

    std::string last_error;
};

namespace orn {

// Queues one training step (forward, backward, weight gradients and, when
// `adam`, the optimiser) on n samples held in device memory.  *d_loss gets
// the summed loss of the step.  `status` receives ERR_MMA on a tensor-core
// timeout.
int cache_train_step(orn_cache* c, const float* d_in, const float* d_target, uint32_t n, bool adam,
                     uint32_t* status, cudaStream_t s);

// Queues inference for the queue of cache queries written by a cached
// megakernel launch (RcForward with pixel/throughput/acc set).
int cache_apply_queries(orn_cache* c, const uint32_t* d_count, uint32_t capacity, const float* d_in,
                        const uint32_t* d_pixel, const float4* d_thr, float4* acc, uint32_t* status,
                        cudaStream_t s);

}  // namespace orn
