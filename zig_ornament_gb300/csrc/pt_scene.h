// pt_scene.h — device-resident scene description shared by the host C ABI
// and the kernels.
//
// Node layout in HBM (one array, TLAS nodes [0, tlas_len), BLAS nodes
// after them with every BLAS id offset by tlas_len), four float4 per node:
//   internal  a=(left.min, left id)  b=(left.max, right id)
//             c=(right.min, type=0)  e=(right.max, 0)
//   triangle  a=(v0, triangle id)    b=(v1, e2.x)  c=(v2, e2.y)
//             e=(e1, e2.z)  with e1 = v1 - v0, e2 = v2 - v0
//   sphere    a,b=inverse rows 0,1   c=(inverse row 2 xyz, type=1)
//             e=(inverse row 2 w, material, transform id, 0)
//   mesh      as sphere with type=2 and e.w = BLAS root id
// (BvhNode, src/gpu_structs.zig:22-31, carries the same information; the
// leaf's own AABB, unused by traversal, is replaced by the transform rows.)
//
// Node references (child ids, the BLAS root of a mesh leaf, stack entries)
// carry the referenced node's type in their top two bits:
// ref = index | type << 30.  A warp therefore knows the type of every lane's
// next node before loading it and can process one node type at a time.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace orn {

enum { SEM_HIP = 0, SEM_WGSL = 1 };          // enum orn_semantics
enum { MATH_PORTABLE = 0, MATH_DEVICE = 1 };  // transcendental implementation
// Error bits written to the context's device error word.
// ERR_MMA: a tensor-core wait timed out; ERR_WAIT: a wavefront queue wait timed out
enum { ERR_STACK = 1u, ERR_VISITS = 2u, ERR_MMA = 4u, ERR_WAIT = 8u };
constexpr uint32_t kRefIndexMask = 0x3FFFFFFFu;

struct TexDesc {
    const unsigned char* data;
    uint32_t width, height, pitch, format;
};

struct SceneDev {
    const float4* nodes;        // 4 float4 per node, TLAS then BLAS
    uint32_t tlas_len;
    uint32_t node_count;
    uint32_t root_ref;          // reference of the TLAS root
    uint32_t exact_slabs;       // 1: some node bound is non-finite or >= 1e30 in magnitude
    const float4* xforms;       // 4 float4 per matrix, blob transforms as given
    const float4* normals;
    const uint32_t* normal_indices;
    const float2* uvs;
    const uint32_t* uv_indices;
    const float4* materials;    // 2 float4 per material
    const TexDesc* textures;
    uint32_t textures_len;
    uint32_t watertight;        // 1: watertight triangle test (orn_state.triangle_test), 0: the reference's
};

}  // namespace orn
