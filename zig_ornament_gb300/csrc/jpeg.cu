// jpeg.cu — the GPU stage of JPEG texture decoding (orn_jpeg_decode): the
// coefficient planes from the host entropy decoder (jpeg.cpp) are
// dequantised and inverse-transformed (one 64-thread group per 8x8 block,
// separable 8-point IDCT through shared memory), then one thread per output
// pixel upsamples the chroma planes by replication, converts YCbCr to RGB
// (JFIF equations) and writes RGBA8 with alpha 255, rows flipped when asked
// — what the reference's example app gets from zstbi with
// setFlipVerticallyOnLoad(true) and 4 forced components
// (glfw_example/app_no_interop.zig:17, glfw_example/examples.zig:492-503).
//
// The transform is the exact DCT-III in FP32 (no fixed-point approximation),
// rounded to nearest; stb_image's integer IDCT and upsampling filter are not
// reproduced, so results can differ from the reference's by a few levels.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "jpeg.h"
#include "ornament_cuda.h"

namespace orn {
namespace {

struct JpegPlanes {
    uint32_t ncomp, width, height, hmax, vmax, flip, ycbcr, total_blocks;
    uint32_t block_begin[3];
    uint32_t bw[3], h[3], v[3];
    unsigned long long plane_off[3];   // in samples
    float q[3][64];                    // dequantisation steps, natural order
    float basis[64];                   // basis[x * 8 + u] = C(u) / 2 * cos((2x + 1) u pi / 16)
};

__device__ __forceinline__ int clamp_level(float f) { return min(max(__float2int_rn(f), 0), 255); }

__global__ void __launch_bounds__(256) jpeg_idct_kernel(const int16_t* __restrict__ coef,
                                                        uint8_t* __restrict__ planes, const JpegPlanes d) {
    __shared__ float s[4][64];
    __shared__ float t[4][64];
    const uint32_t sub = threadIdx.x >> 6, e = threadIdx.x & 63;
    const uint32_t b = blockIdx.x * 4 + sub;
    const bool live = b < d.total_blocks;
    uint32_t c = 0;
    if (live) {
        c = (d.ncomp > 1 && b >= d.block_begin[1]) + (d.ncomp > 2 && b >= d.block_begin[2]);
        s[sub][e] = (float)coef[(size_t)b * 64 + e] * d.q[c][e];
    }
    __syncthreads();
    const uint32_t row = e >> 3, col = e & 7;
    if (live) {   // along each row: t[v][x] = sum_u basis[x][u] * F[v][u]
        float acc = 0.0f;
#pragma unroll
        for (int u = 0; u < 8; ++u) acc += d.basis[col * 8 + u] * s[sub][row * 8 + u];
        t[sub][row * 8 + col] = acc;
    }
    __syncthreads();
    if (live) {   // down each column: f[y][x] = sum_v basis[y][v] * t[v][x]
        float acc = 0.0f;
#pragma unroll
        for (int v = 0; v < 8; ++v) acc += d.basis[row * 8 + v] * t[sub][v * 8 + col];
        const uint32_t bi = b - d.block_begin[c];
        const uint32_t by = bi / d.bw[c], bx = bi % d.bw[c];
        const size_t stride = (size_t)d.bw[c] * 8;
        planes[d.plane_off[c] + (size_t)(by * 8 + row) * stride + bx * 8 + col] =
            (uint8_t)min(max(__float2int_rn(acc) + 128, 0), 255);
    }
}

__global__ void __launch_bounds__(256) jpeg_color_kernel(const uint8_t* __restrict__ planes,
                                                         uchar4* __restrict__ out, const JpegPlanes d) {
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (unsigned long long)d.width * d.height) return;
    const uint32_t x = (uint32_t)(i % d.width), y = (uint32_t)(i / d.width);
    const uint32_t sy = d.flip ? d.height - 1 - y : y;
    float comp[3] = {0.0f, 0.0f, 0.0f};
    for (uint32_t c = 0; c < d.ncomp; ++c) {
        const uint32_t cx = x * d.h[c] / d.hmax, cy = sy * d.v[c] / d.vmax;
        comp[c] = (float)planes[d.plane_off[c] + (size_t)cy * d.bw[c] * 8 + cx];
    }
    int r, g, b;
    if (d.ncomp == 1) {
        r = g = b = (int)comp[0];
    } else if (d.ycbcr) {
        const float cb = comp[1] - 128.0f, cr = comp[2] - 128.0f;
        r = clamp_level(comp[0] + 1.402f * cr);
        g = clamp_level(comp[0] - 0.344136f * cb - 0.714136f * cr);
        b = clamp_level(comp[0] + 1.772f * cb);
    } else {
        r = (int)comp[0];
        g = (int)comp[1];
        b = (int)comp[2];
    }
    out[i] = make_uchar4((unsigned char)r, (unsigned char)g, (unsigned char)b, 255);
}

}  // namespace
}  // namespace orn

extern "C" int orn_jpeg_decode(const void* data, size_t len, int device, uint32_t flip_y, uint8_t* rgba,
                               size_t rgba_len) {
    using namespace orn;
    using namespace orn::jpeg;
    if (!data || !rgba) return ORN_ERR_INVALID_ARGUMENT;
    last_error().clear();
    Image img;
    int st = parse((const uint8_t*)data, len, false, &img, &last_error());
    if (st != ORN_OK) return st;
    const size_t pixels = (size_t)img.width * img.height;
    if (rgba_len < pixels * 4) {
        last_error() = "RGBA buffer smaller than width * height * 4";
        return ORN_ERR_BUFFER_TOO_SMALL;
    }
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        last_error() = "no CUDA device";
        return ORN_ERR_NO_DEVICE;
    }
    int prev = 0;
    cudaGetDevice(&prev);
    if (device < 0) device = prev;
    if (device >= count) {
        last_error() = "device ordinal out of range";
        return ORN_ERR_NO_DEVICE;
    }

    JpegPlanes d{};
    d.ncomp = img.ncomp;
    d.width = img.width;
    d.height = img.height;
    d.hmax = img.hmax;
    d.vmax = img.vmax;
    d.flip = flip_y ? 1u : 0u;
    d.ycbcr = img.ycbcr ? 1u : 0u;
    uint32_t blocks = 0;
    unsigned long long samples = 0;
    for (uint32_t c = 0; c < img.ncomp; ++c) {
        const Component& k = img.comp[c];
        d.block_begin[c] = blocks;
        d.bw[c] = k.bw;
        d.h[c] = k.h;
        d.v[c] = k.v;
        d.plane_off[c] = samples;
        for (int e = 0; e < 64; ++e) d.q[c][e] = (float)img.quant[k.tq][e];
        blocks += k.bw * k.bh;
        samples += (unsigned long long)k.bw * k.bh * 64;
    }
    d.total_blocks = blocks;
    const double pi = 3.14159265358979323846;
    for (int x = 0; x < 8; ++x)
        for (int u = 0; u < 8; ++u)
            d.basis[x * 8 + u] = (float)(0.5 * (u == 0 ? std::sqrt(0.5) : 1.0) * std::cos((2 * x + 1) * u * pi / 16.0));

    int16_t* d_coef = nullptr;
    uint8_t* d_planes = nullptr;
    uchar4* d_out = nullptr;
    cudaStream_t s = nullptr;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess && st == ORN_OK) {
            st = e == cudaErrorMemoryAllocation ? ORN_ERR_OUT_OF_MEMORY : ORN_ERR_CUDA;
            last_error() = cudaGetErrorString(e);
        }
        return st == ORN_OK;
    };
    if (ok(cudaSetDevice(device)) && ok(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) &&
        ok(cudaMalloc(&d_coef, (size_t)blocks * 64 * sizeof(int16_t))) && ok(cudaMalloc(&d_planes, samples)) &&
        ok(cudaMalloc(&d_out, pixels * sizeof(uchar4)))) {
        for (uint32_t c = 0; c < img.ncomp; ++c)
            ok(cudaMemcpyAsync(d_coef + (size_t)d.block_begin[c] * 64, img.comp[c].coef.data(),
                               img.comp[c].coef.size() * sizeof(int16_t), cudaMemcpyHostToDevice, s));
        jpeg_idct_kernel<<<(blocks + 3) / 4, 256, 0, s>>>(d_coef, d_planes, d);
        ok(cudaGetLastError());
        jpeg_color_kernel<<<(unsigned)((pixels + 255) / 256), 256, 0, s>>>(d_planes, d_out, d);
        ok(cudaGetLastError());
        ok(cudaMemcpyAsync(rgba, d_out, pixels * sizeof(uchar4), cudaMemcpyDeviceToHost, s));
        ok(cudaStreamSynchronize(s));
    }
    if (d_coef) cudaFree(d_coef);
    if (d_planes) cudaFree(d_planes);
    if (d_out) cudaFree(d_out);
    if (s) cudaStreamDestroy(s);
    cudaSetDevice(prev);
    return st;
}
