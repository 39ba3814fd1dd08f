// cache_capi.cu — the orn_cache_* entry points: creation, weights, the
// host-buffer inference / gradient / training calls, and the training step
// and query pass the cached renderer queues (capi.cu).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "pt_scene.h"
#include "rc_host.h"

namespace {

int cfail(orn_cache* c, int status, const std::string& msg) {
    if (c) c->last_error = msg;
    return status;
}

int ccuda(orn_cache* c, cudaError_t e, const char* what) {
    std::string msg = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) return cfail(c, ORN_ERR_OUT_OF_MEMORY, msg);
    return cfail(c, ORN_ERR_CUDA, msg);
}

#define RC_CUDA(c, call)                                          \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return ccuda((c), e_, #call);      \
    } while (0)

bool valid_config(const orn_cache_config& k) {
    return k.batch >= 128 && k.batch % 128 == 0 && k.batch <= (1u << 20) && k.steps_per_frame <= 64 &&
           k.train_shift <= 10 && k.learning_rate > 0.0f && std::isfinite(k.learning_rate) && k.beta1 >= 0.0f &&
           k.beta1 < 1.0f && k.beta2 >= 0.0f && k.beta2 < 1.0f && k.epsilon > 0.0f;
}

// splitmix64: seeds the weight initialisation.
uint64_t splitmix(uint64_t& x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void free_buffers(orn_cache* c) {
    void* ptrs[] = {c->params, c->m,  c->v,     c->grads, c->w_f16,  c->w_bf16,    c->d_loss, c->d_status,
                    c->h,      c->dz, c->dz6,   c->io_in, c->io_target, c->io_out};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    c->params = c->m = c->v = c->grads = nullptr;
    c->w_f16 = c->w_bf16 = nullptr;
    c->d_loss = nullptr;
    c->d_status = nullptr;
    c->h = c->dz = c->dz6 = nullptr;
    c->io_in = c->io_target = c->io_out = nullptr;
    c->cap = c->io_cap = 0;
}

int ensure_cap(orn_cache* c, uint32_t n) {
    if (n <= c->cap) return ORN_OK;
    uint32_t cap = std::max<uint32_t>(n, 16384u);
    cap = (cap + 127u) & ~127u;
    RC_CUDA(c, cudaDeviceSynchronize());   // queued steps may still use the old buffers
    if (c->h) cudaFree(c->h);
    if (c->dz) cudaFree(c->dz);
    if (c->dz6) cudaFree(c->dz6);
    c->h = c->dz = c->dz6 = nullptr;
    c->cap = 0;
    RC_CUDA(c, cudaMalloc(&c->h, (size_t)5 * cap * orn::kHidden * 2));
    RC_CUDA(c, cudaMalloc(&c->dz, (size_t)5 * cap * orn::kHidden * 2));
    RC_CUDA(c, cudaMalloc(&c->dz6, (size_t)cap * orn::kOutPad * 2));
    c->cap = cap;
    return ORN_OK;
}

int ensure_io(orn_cache* c, uint32_t n) {
    if (n <= c->io_cap) return ORN_OK;
    uint32_t cap = (n + 127u) & ~127u;
    RC_CUDA(c, cudaDeviceSynchronize());
    if (c->io_in) cudaFree(c->io_in);
    if (c->io_target) cudaFree(c->io_target);
    if (c->io_out) cudaFree(c->io_out);
    c->io_in = c->io_target = c->io_out = nullptr;
    c->io_cap = 0;
    RC_CUDA(c, cudaMalloc(&c->io_in, (size_t)cap * orn::kInputs * 4));
    RC_CUDA(c, cudaMalloc(&c->io_target, (size_t)cap * orn::kOutputs * 4));
    RC_CUDA(c, cudaMalloc(&c->io_out, (size_t)cap * orn::kOutputs * 4));
    c->io_cap = cap;
    return ORN_OK;
}

// Rewrites the FP16/BF16 operand copies from the FP32 weights (no update).
int refresh_copies(orn_cache* c, cudaStream_t s) {
    orn::RcAdam a{};
    a.params = c->params;
    a.m = c->m;
    a.v = c->v;
    a.grads = c->grads;
    a.weights_f16 = c->w_f16;
    a.weights_bf16 = c->w_bf16;
    a.step = 0;
    RC_CUDA(c, orn::rc_launch_adam(a, s));
    return ORN_OK;
}

int finish(orn_cache* c) {
    RC_CUDA(c, cudaStreamSynchronize(c->stream));
    uint32_t st = 0;
    RC_CUDA(c, cudaMemcpy(&st, c->d_status, 4, cudaMemcpyDeviceToHost));
    if (st) {
        RC_CUDA(c, cudaMemset(c->d_status, 0, 4));
        return cfail(c, ORN_ERR_TIMEOUT, "a tensor-core wait timed out");
    }
    return ORN_OK;
}

}  // namespace

namespace orn {

int cache_train_step(orn_cache* c, const float* d_in, const float* d_target, uint32_t n, bool adam, uint32_t* status,
                     cudaStream_t s) {
    if (n == 0) return ORN_OK;
    int st = ensure_cap(c, n);
    if (st) return st;
    const uint32_t tiles = (n + 127) / 128;
    const int grid = (int)std::min<uint32_t>(tiles, (uint32_t)c->sms);
    RC_CUDA(c, cudaMemsetAsync(c->d_loss, 0, 4, s));
    RcForward f{};
    f.weights_f16 = c->w_f16;
    f.inputs = d_in;
    f.targets = d_target;
    f.h_out = c->h;
    f.dz_out = c->dz6;
    f.loss = c->d_loss;
    f.n = n;
    f.status = status;
    RC_CUDA(c, rc_launch_forward(f, true, grid, s));
    RcBackward b{};
    b.weights_bf16 = c->w_bf16;
    b.dz6 = c->dz6;
    b.h = c->h;
    b.dz = c->dz;
    b.n = n;
    b.status = status;
    RC_CUDA(c, rc_launch_backward(b, grid, s));
    RcWgrad g{};
    g.inputs = d_in;
    g.h = c->h;
    g.dz = c->dz;
    g.dz6 = c->dz6;
    g.grads = c->grads;
    g.n = n;
    g.splits = std::min<uint32_t>(tiles, 32u);
    g.status = status;
    RC_CUDA(c, rc_launch_wgrad(g, s));
    if (adam) {
        c->steps++;
        RcAdam a{};
        a.params = c->params;
        a.m = c->m;
        a.v = c->v;
        a.grads = c->grads;
        a.weights_f16 = c->w_f16;
        a.weights_bf16 = c->w_bf16;
        a.step = (uint32_t)std::min<uint64_t>(c->steps, 0xFFFFFFFFull);
        a.lr = c->config.learning_rate;
        a.beta1 = c->config.beta1;
        a.beta2 = c->config.beta2;
        a.eps = c->config.epsilon;
        a.beta1_pow = (float)std::pow((double)c->config.beta1, (double)c->steps);
        a.beta2_pow = (float)std::pow((double)c->config.beta2, (double)c->steps);
        a.grad_scale = 1.0f / (3.0f * (float)n);
        RC_CUDA(c, rc_launch_adam(a, s));
    }
    return ORN_OK;
}

int cache_apply_queries(orn_cache* c, const uint32_t* d_count, uint32_t capacity, const float* d_in,
                        const uint32_t* d_pixel, const float4* d_thr, float4* acc, uint32_t* status, cudaStream_t s) {
    if (capacity == 0) return ORN_OK;
    RcForward f{};
    f.weights_f16 = c->w_f16;
    f.inputs = d_in;
    f.pixel = d_pixel;
    f.throughput = d_thr;
    f.acc = acc;
    f.n_dev = d_count;
    f.n = capacity;
    f.status = status;
    const uint32_t tiles = (capacity + 127) / 128;
    const int grid = (int)std::min<uint32_t>(tiles, (uint32_t)c->sms);
    RC_CUDA(c, rc_launch_forward(f, false, grid, s));
    return ORN_OK;
}

}  // namespace orn

extern "C" {

int orn_cache_default_config(orn_cache_config* out) {
    if (!out) return ORN_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    out->batch = 16384;
    out->steps_per_frame = 4;
    out->train_shift = 4;
    out->learning_rate = 1e-3f;
    out->beta1 = 0.9f;
    out->beta2 = 0.99f;
    out->epsilon = 1e-8f;
    return ORN_OK;
}

int orn_cache_create(int device, uint64_t seed, const orn_cache_config* config, orn_cache** out) {
    if (!out) return ORN_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    orn_cache_config k;
    if (config) k = *config;
    else orn_cache_default_config(&k);
    if (!valid_config(k)) return ORN_ERR_INVALID_ARGUMENT;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return ORN_ERR_NO_DEVICE;
    if (device < 0) device = count - 1;
    if (device >= count) return ORN_ERR_INVALID_ARGUMENT;
    orn_cache* c = new orn_cache();
    c->device = device;
    c->config = k;
    auto bail = [&](int st) {
        free_buffers(c);
        if (c->stream) cudaStreamDestroy(c->stream);
        delete c;
        return st;
    };
    if (cudaSetDevice(device) != cudaSuccess) return bail(ORN_ERR_CUDA);
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
    if (major != 10) return bail(ORN_ERR_NO_DEVICE);   // tcgen05 needs an sm_10x device
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    const size_t pbytes = (size_t)orn::kWeightCount * 4;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&c->params, pbytes) != cudaSuccess || cudaMalloc(&c->m, pbytes) != cudaSuccess ||
        cudaMalloc(&c->v, pbytes) != cudaSuccess || cudaMalloc(&c->grads, pbytes) != cudaSuccess ||
        cudaMalloc(&c->w_f16, (size_t)orn::kWeightCount * 2) != cudaSuccess ||
        cudaMalloc(&c->w_bf16, (size_t)orn::kBackwardWeightCount * 2) != cudaSuccess ||
        cudaMalloc(&c->d_loss, 4) != cudaSuccess || cudaMalloc(&c->d_status, 4) != cudaSuccess)
        return bail(ORN_ERR_OUT_OF_MEMORY);
    // He-uniform weights: U(-sqrt(6 / fan_in), +sqrt(6 / fan_in)); padded
    // output rows zero.
    std::vector<float> w(orn::kWeightCount, 0.0f);
    uint64_t state = seed;
    for (int l = 0; l < orn::kLayers; ++l) {
        const uint32_t in = orn::rc_layer_in(l), outn = orn::rc_layer_out(l);
        const uint32_t real = l == orn::kLayers - 1 ? (uint32_t)orn::kOutputs : outn;
        const double a = std::sqrt(6.0 / (double)in);
        for (uint32_t o = 0; o < real; ++o)
            for (uint32_t i = 0; i < in; ++i) {
                double u = (double)(splitmix(state) >> 11) * (1.0 / 9007199254740992.0);
                w[orn::rc_layer_offset(l) + (size_t)o * in + i] = (float)((2.0 * u - 1.0) * a);
            }
    }
    if (cudaMemcpy(c->params, w.data(), pbytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(c->m, 0, pbytes) != cudaSuccess || cudaMemset(c->v, 0, pbytes) != cudaSuccess ||
        cudaMemset(c->grads, 0, pbytes) != cudaSuccess || cudaMemset(c->d_status, 0, 4) != cudaSuccess ||
        cudaMemset(c->d_loss, 0, 4) != cudaSuccess)
        return bail(ORN_ERR_CUDA);
    if (refresh_copies(c, c->stream) != ORN_OK || cudaStreamSynchronize(c->stream) != cudaSuccess)
        return bail(ORN_ERR_CUDA);
    *out = c;
    return ORN_OK;
}

int orn_cache_destroy(orn_cache* c) {
    if (!c) return ORN_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaDeviceSynchronize();   // a context may have queued cache work on its own stream
    free_buffers(c);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return ORN_OK;
}

int orn_cache_set_config(orn_cache* c, const orn_cache_config* config) {
    if (!c || !config) return ORN_ERR_INVALID_ARGUMENT;
    if (!valid_config(*config)) return cfail(c, ORN_ERR_INVALID_ARGUMENT, "invalid cache configuration");
    c->config = *config;
    return ORN_OK;
}

int orn_cache_get_params(orn_cache* c, float* dst, size_t count) {
    if (!c || !dst) return ORN_ERR_INVALID_ARGUMENT;
    if (count < orn::kWeightCount) return cfail(c, ORN_ERR_BUFFER_TOO_SMALL, "parameter buffer too small");
    RC_CUDA(c, cudaSetDevice(c->device));
    RC_CUDA(c, cudaDeviceSynchronize());
    RC_CUDA(c, cudaMemcpy(dst, c->params, (size_t)orn::kWeightCount * 4, cudaMemcpyDeviceToHost));
    return ORN_OK;
}

int orn_cache_set_params(orn_cache* c, const float* src, size_t count) {
    if (!c || !src || count != orn::kWeightCount) return ORN_ERR_INVALID_ARGUMENT;
    RC_CUDA(c, cudaSetDevice(c->device));
    RC_CUDA(c, cudaDeviceSynchronize());
    const size_t pbytes = (size_t)orn::kWeightCount * 4;
    RC_CUDA(c, cudaMemcpy(c->params, src, pbytes, cudaMemcpyHostToDevice));
    RC_CUDA(c, cudaMemset(c->m, 0, pbytes));
    RC_CUDA(c, cudaMemset(c->v, 0, pbytes));
    RC_CUDA(c, cudaMemset(c->grads, 0, pbytes));
    c->steps = 0;
    int st = refresh_copies(c, c->stream);
    if (st) return st;
    return finish(c);
}

int orn_cache_infer(orn_cache* c, const float* inputs, size_t n, float* outputs) {
    if (!c || (n && (!inputs || !outputs))) return ORN_ERR_INVALID_ARGUMENT;
    if (n > (1u << 24)) return cfail(c, ORN_ERR_INVALID_ARGUMENT, "at most 2^24 samples per call");
    if (n == 0) return ORN_OK;
    RC_CUDA(c, cudaSetDevice(c->device));
    int st = ensure_io(c, (uint32_t)n);
    if (st) return st;
    RC_CUDA(c, cudaMemcpyAsync(c->io_in, inputs, n * orn::kInputs * 4, cudaMemcpyHostToDevice, c->stream));
    orn::RcForward f{};
    f.weights_f16 = c->w_f16;
    f.inputs = c->io_in;
    f.outputs = c->io_out;
    f.n = (uint32_t)n;
    f.status = c->d_status;
    const uint32_t tiles = (uint32_t)((n + 127) / 128);
    RC_CUDA(c, orn::rc_launch_forward(f, false, (int)std::min<uint32_t>(tiles, (uint32_t)c->sms), c->stream));
    RC_CUDA(c, cudaMemcpyAsync(outputs, c->io_out, n * orn::kOutputs * 4, cudaMemcpyDeviceToHost, c->stream));
    return finish(c);
}

static int gradients_or_train(orn_cache* c, const float* inputs, const float* targets, size_t n, float* grads,
                              float* loss, bool adam) {
    if (!c || !inputs || !targets || n == 0) return ORN_ERR_INVALID_ARGUMENT;
    if (n > (1u << 20)) return cfail(c, ORN_ERR_INVALID_ARGUMENT, "at most 2^20 samples per step");
    RC_CUDA(c, cudaSetDevice(c->device));
    int st = ensure_io(c, (uint32_t)n);
    if (st) return st;
    RC_CUDA(c, cudaMemcpyAsync(c->io_in, inputs, n * orn::kInputs * 4, cudaMemcpyHostToDevice, c->stream));
    RC_CUDA(c, cudaMemcpyAsync(c->io_target, targets, n * orn::kOutputs * 4, cudaMemcpyHostToDevice, c->stream));
    st = orn::cache_train_step(c, c->io_in, c->io_target, (uint32_t)n, adam, c->d_status, c->stream);
    if (st) return st;
    if (grads) {
        RC_CUDA(c, cudaMemcpyAsync(grads, c->grads, (size_t)orn::kWeightCount * 4, cudaMemcpyDeviceToHost,
                                   c->stream));
        RC_CUDA(c, cudaMemsetAsync(c->grads, 0, (size_t)orn::kWeightCount * 4, c->stream));
    }
    float l = 0.0f;
    RC_CUDA(c, cudaMemcpyAsync(&l, c->d_loss, 4, cudaMemcpyDeviceToHost, c->stream));
    st = finish(c);
    if (st) return st;
    if (loss) *loss = l;
    return ORN_OK;
}

int orn_cache_gradients(orn_cache* c, const float* inputs, const float* targets, size_t n, float* grads, float* loss) {
    if (!grads) return ORN_ERR_INVALID_ARGUMENT;
    return gradients_or_train(c, inputs, targets, n, grads, loss, false);
}

int orn_cache_train(orn_cache* c, const float* inputs, const float* targets, size_t n, float* loss) {
    return gradients_or_train(c, inputs, targets, n, nullptr, loss, true);
}

int orn_cache_stats(orn_cache* c, uint64_t* steps, uint64_t* frames, float* last_loss) {
    if (!c) return ORN_ERR_INVALID_ARGUMENT;
    if (steps) *steps = c->steps;
    if (frames) *frames = c->frames;
    if (last_loss) {
        RC_CUDA(c, cudaSetDevice(c->device));
        RC_CUDA(c, cudaDeviceSynchronize());
        RC_CUDA(c, cudaMemcpy(last_loss, c->d_loss, 4, cudaMemcpyDeviceToHost));
    }
    return ORN_OK;
}

const char* orn_cache_last_error(const orn_cache* c) { return c ? c->last_error.c_str() : "cache is NULL"; }

}  // extern "C"
