// lbvh.h — GPU BLAS construction (lbvh.cu), called by the host builder
// (bvh_build.cpp) for orn_scene_desc.builder = ORN_BVH_LBVH.
#pragma once

#include <stdint.h>

#include "ornament_cuda.h"

namespace orn {

// Builds the BLAS of one mesh on the current CUDA device: `tri_host` holds
// n triangles as 9 floats (v0, v1, v2, object space); writes 2n - 1 nodes to
// out_host in the reference's format (post-order, root last; child ids are
// node_offset + slot, triangle ids first_global + index).  Returns ORN_*.
int lbvh_build_blas(const float* tri_host, uint32_t n, uint32_t first_global, uint32_t node_offset,
                    orn_bvh_node* out_host);

}  // namespace orn
