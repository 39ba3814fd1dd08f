// Test infrastructure (oracle): host stand-in for the hiprt vector types that
// src/hip_backend/kernels/vec_math.hip.h:7-28 maps float2/3/4 and int2/3/4 to
// when it is not compiled by a GPU compiler.  Layouts match HIP's: 8/12/16-byte
// float vectors with 4-byte alignment (BvhNode stays 64 bytes).
#pragma once

struct hiprtFloat2 { float x, y; };
struct hiprtFloat3 { float x, y, z; };
struct hiprtFloat4 { float x, y, z, w; };
struct hiprtInt2 { int x, y; };
struct hiprtInt3 { int x, y, z; };
struct hiprtInt4 { int x, y, z, w; };

inline hiprtFloat2 make_hiprtFloat2(float x, float y) { return {x, y}; }
inline hiprtFloat3 make_hiprtFloat3(float x, float y, float z) { return {x, y, z}; }
inline hiprtFloat4 make_hiprtFloat4(float x, float y, float z, float w) { return {x, y, z, w}; }
inline hiprtInt2 make_hiprtInt2(int x, int y) { return {x, y}; }
inline hiprtInt3 make_hiprtInt3(int x, int y, int z) { return {x, y, z}; }
inline hiprtInt4 make_hiprtInt4(int x, int y, int z, int w) { return {x, y, z, w}; }
