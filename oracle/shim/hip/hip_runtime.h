// Test infrastructure (oracle): the smallest host stand-in for
// <hip/hip_runtime.h> that lets the unmodified reference kernels
// (src/hip_backend/kernels/pathtracer.hip.cpp and its headers) compile with a
// host C++ compiler.  Only the oracle build (oracle/build_oracle.py) uses it.
//
//  - __global__/__constant__/__device__/__host__ expand to nothing, so the
//    three extern "C" kernels become plain host functions and
//    `constant_params` a host global set before each pass.
//  - blockDim/blockIdx/threadIdx are thread_local globals that the driver sets
//    per pixel (defined in oracle/ref_driver.cpp).
//  - hipTextureObject_t points at a host texture; tex2D<float4> samples it
//    with point filtering and normalised coordinates, wrap addressing
//    (src/hip_backend/buffers.zig:136-140).
//  - Scalar min/max follow the HIP device builtins (fminf/fmaxf); the float
//    overloads of abs/pow/acos/atan2 are made visible as they are on the
//    device, where these calls take and return float.
//  - With ORN_SHIM_PORTABLE_MATH the four transcendentals resolve to the
//    project's portable implementations (zig_ornament_gb300/csrc/pmath.h)
//    instead of glibc, exactly as a different libm would be linked.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <cmath>
#include <hiprt/hiprt_vec.h>

#define __global__
#define __constant__
#define __device__
#define __host__
#define __forceinline__ inline

struct orn_shim_dim3 { uint32_t x, y, z; };
extern thread_local orn_shim_dim3 blockDim;
extern thread_local orn_shim_dim3 blockIdx;
extern thread_local orn_shim_dim3 threadIdx;

struct uint2 { uint32_t x, y; };
inline uint2 make_uint2(uint32_t x, uint32_t y) { return {x, y}; }

// A host texture: RGBA8 unorm or RGBA16F texels, rows `pitch` bytes apart.
struct orn_shim_texture {
    const unsigned char* data;
    uint32_t width, height, pitch, format;  // format 0 = RGBA8, 1 = RGBA16F
};
typedef const orn_shim_texture* hipTextureObject_t;

float orn_shim_half_to_float(uint16_t h);

// Point sampling, normalised coordinates, wrap addressing.
inline int orn_shim_wrap_index(float c, uint32_t n) {
    if (!(c == c)) c = 0.0f;
    float f = c - floorf(c);
    float x = floorf(f * (float)n);
    if (x > (float)(n - 1)) x = (float)(n - 1);
    if (x < 0.0f) x = 0.0f;
    return (int)x;
}

template <typename T> T tex2D(hipTextureObject_t tex, float u, float v);
template <> inline hiprtFloat4 tex2D<hiprtFloat4>(hipTextureObject_t tex, float u, float v) {
    int x = orn_shim_wrap_index(u, tex->width);
    int y = orn_shim_wrap_index(v, tex->height);
    const unsigned char* row = tex->data + (size_t)y * tex->pitch;
    if (tex->format == 0) {
        const unsigned char* p = row + (size_t)x * 4;
        return {p[0] / 255.0f, p[1] / 255.0f, p[2] / 255.0f, p[3] / 255.0f};
    }
    const uint16_t* p = (const uint16_t*)(row + (size_t)x * 8);
    return {orn_shim_half_to_float(p[0]), orn_shim_half_to_float(p[1]),
            orn_shim_half_to_float(p[2]), orn_shim_half_to_float(p[3])};
}

inline float min(float a, float b) { return fminf(a, b); }
inline float max(float a, float b) { return fmaxf(a, b); }
using std::abs;
using std::pow;
using std::acos;
using std::atan2;

#ifdef ORN_SHIM_PORTABLE_MATH
#include "pmath.h"
inline float orn_shim_pow(float a, float b) { return pm_powf(a, b); }
inline float orn_shim_acos(float a) { return pm_acosf(a); }
inline float orn_shim_atan2(float a, float b) { return pm_atan2f(a, b); }
inline void orn_shim_sincosf(float a, float* s, float* c) { pm_sincosf(a, s, c); }
#define pow orn_shim_pow
#define acos orn_shim_acos
#define atan2 orn_shim_atan2
#define sincosf orn_shim_sincosf
#endif
