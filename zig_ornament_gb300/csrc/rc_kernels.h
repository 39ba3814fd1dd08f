// rc_kernels.h — launch interface of the radiance-cache MLP kernels
// (radiance_cache.cu) and the shapes they share with the host.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace orn {

constexpr int kInputs = 10;                          // position 3, direction 3, normal 3, roughness 1
constexpr int kBands = 12;                           // frequency bands per input
constexpr int kEncoded = kInputs * 2 * kBands;       // 240 sin/cos features
constexpr int kFeatures = 256;                       // + 10 raw inputs, a constant 1, 5 zeros
constexpr int kHidden = 64;
constexpr int kLayers = 6;                           // 5 hidden layers + the output layer
constexpr int kOutputs = 3;
constexpr int kOutPad = 16;                          // output rows padded to the MMA's minimum N
constexpr uint32_t kWeightCount = kFeatures * kHidden + 4 * kHidden * kHidden + kHidden * kOutPad;   // 33,792
constexpr uint32_t kBackwardWeightCount = 4 * kHidden * kHidden + kHidden * kOutPad;                  // layers 2..6
constexpr uint32_t kTmemCols = 64;
constexpr int kWgradJobs = 7;                        // layer 1 in two 128-input blocks + layers 2..6
constexpr float kGradClamp = 1.0e4f;

// Forward pass over n samples.  Inference writes `outputs` (n x 3) or, when
// `pixel` is set, adds throughput x max(output, 0) to acc[pixel[i]].xyz;
// training stores the hidden activations (FP16, [5][n][64]) and the loss
// gradient of the output (BF16, [n][16]) and sums the loss into *loss.
// `n_dev`, when set, supplies n from device memory (a queue length).
struct RcForward {
    const uint16_t* weights_f16;    // forward operand copies, K-major per layer
    const float* inputs;            // [n][10]
    const float* targets;           // [n][3]; target.x < 0 marks a sample without a target
    float* outputs;                 // [n][3] or null
    const uint32_t* pixel;          // query pixel per sample (cache queries) or null
    const float4* throughput;       // path throughput per query
    float4* acc;                    // per-pixel accumulation the queries add to
    uint16_t* h_out;                // training: hidden activations
    uint16_t* dz_out;               // training: output gradients
    float* loss;
    const uint32_t* n_dev;
    uint32_t n;
    uint32_t* status;
};

// Backward pass through layers 6..2: dZ(l-1) = (dZ(l) · W(l)) ⊙ [H(l-1) > 0].
struct RcBackward {
    const uint16_t* weights_bf16;   // backward operand copies (W(l) with K = outputs)
    const uint16_t* dz6;            // [n][16]
    const uint16_t* h;              // [5][n][64] FP16
    uint16_t* dz;                   // [5][n][64] BF16 out
    uint32_t n;
    uint32_t* status;
};

// Weight gradients, added to `grads` (FP32, [layer][out][in] like the params).
struct RcWgrad {
    const float* inputs;            // layer 1's input features are re-encoded from these
    const uint16_t* h;
    const uint16_t* dz;
    const uint16_t* dz6;
    float* grads;
    uint32_t n;
    uint32_t splits;                // CTAs per job; each sums every splits-th sample tile
    uint32_t* status;
};

struct RcAdam {
    float* params;                  // FP32 master weights [layer][out][in]
    float* m;
    float* v;
    float* grads;                   // read and cleared
    uint16_t* weights_f16;
    uint16_t* weights_bf16;
    uint32_t step;                  // 0: only rewrite the operand copies
    float lr, beta1, beta2, eps, beta1_pow, beta2_pow, grad_scale;
};

// Number of FP32 parameters before layer l and its shape.
__host__ __device__ constexpr uint32_t rc_layer_in(int l) { return l == 0 ? kFeatures : kHidden; }
__host__ __device__ constexpr uint32_t rc_layer_out(int l) { return l == kLayers - 1 ? kOutPad : kHidden; }
__host__ __device__ constexpr uint32_t rc_layer_offset(int l) {
    uint32_t o = 0;
    for (int i = 0; i < l; ++i) o += rc_layer_in(i) * rc_layer_out(i);
    return o;
}

cudaError_t rc_launch_forward(const RcForward& p, bool train, int grid, cudaStream_t s);
cudaError_t rc_launch_backward(const RcBackward& p, int grid, cudaStream_t s);
cudaError_t rc_launch_wgrad(const RcWgrad& p, cudaStream_t s);
cudaError_t rc_launch_adam(const RcAdam& p, cudaStream_t s);

}  // namespace orn
