// lbvh.cu — BLAS construction on the GPU (a non-parity builder mode,
// ORN_BVH_LBVH): linear BVH after Karras, "Maximizing Parallelism in the
// Construction of BVHs, Octrees, and k-d Trees" (HPG 2012).
//
//   1. 30-bit Morton code of each triangle's centroid in the mesh's bounds,
//      with the triangle index as the low 32 bits of a 64-bit key (distinct
//      keys, deterministic order); keys sorted with CUB's radix sort.
//   2. Karras' per-node range and split search over the sorted keys gives
//      the n-1 internal nodes, their children and parents.
//   3. Bounds bottom-up: each leaf walks towards the root; at every internal
//      node the second arriving thread (an atomic counter) forms the union of
//      the children's boxes and continues.
//   4. Post-order relabelling: the reference's node format wants children
//      before parents (root last).  A subtree over leaves [a, b] occupies
//      2(b - a + 1) - 1 consecutive slots ending with its root; a node's first
//      slot is the sum of the sizes of the left siblings on its path to the
//      root.
//   5. Nodes written in the reference's layout (one triangle per leaf, raw
//      vertices, child ids global) and copied back to the host arrays.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "lbvh.h"

namespace orn {
namespace {

constexpr uint32_t kLeafBit = 0x80000000u;

__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void morton_kernel(const float* __restrict__ tri, uint32_t n, float3 lo, float3 scale,
                              unsigned long long* __restrict__ keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* v = tri + (size_t)i * 9;
    float c[3];
    for (int k = 0; k < 3; ++k) {
        const float mn = fminf(fminf(v[k], v[3 + k]), v[6 + k]), mx = fmaxf(fmaxf(v[k], v[3 + k]), v[6 + k]);
        c[k] = 0.5f * (mn + mx);
    }
    const float fx = fminf(fmaxf((c[0] - lo.x) * scale.x, 0.0f), 1023.0f);
    const float fy = fminf(fmaxf((c[1] - lo.y) * scale.y, 0.0f), 1023.0f);
    const float fz = fminf(fmaxf((c[2] - lo.z) * scale.z, 0.0f), 1023.0f);
    const uint32_t m = (expand_bits((uint32_t)fx) << 2) | (expand_bits((uint32_t)fy) << 1) | expand_bits((uint32_t)fz);
    keys[i] = ((unsigned long long)m << 32) | i;
}

__device__ __forceinline__ int delta(const unsigned long long* keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    return __clzll(keys[i] ^ keys[j]);
}

// Karras 2012, section 4: node i's range, split and children.
__global__ void hierarchy_kernel(const unsigned long long* __restrict__ keys, int n, uint32_t* __restrict__ left,
                                 uint32_t* __restrict__ right, int* __restrict__ parent_int,
                                 int* __restrict__ parent_leaf, uint32_t* __restrict__ range_lo,
                                 uint32_t* __restrict__ range_hi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (lmax < n && delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;   // (the bound keeps i + lmax*d from overflowing)
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0;
    for (int div = 2;; div *= 2) {
        const int t = (l + div - 1) / div;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
        if (t <= 1) break;
    }
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const uint32_t lc = (lo == gamma) ? (kLeafBit | (uint32_t)gamma) : (uint32_t)gamma;
    const uint32_t rc = (hi == gamma + 1) ? (kLeafBit | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
    left[i] = lc;
    right[i] = rc;
    range_lo[i] = (uint32_t)lo;
    range_hi[i] = (uint32_t)hi;
    if (lc & kLeafBit) parent_leaf[lc & ~kLeafBit] = i;
    else parent_int[lc] = i;
    if (rc & kLeafBit) parent_leaf[rc & ~kLeafBit] = i;
    else parent_int[rc] = i;
}

__device__ __forceinline__ void tri_box(const float* tri, const unsigned long long* keys, uint32_t leaf, float* mn,
                                        float* mx) {
    const float* v = tri + (size_t)(uint32_t)(keys[leaf] & 0xFFFFFFFFull) * 9;
    for (int k = 0; k < 3; ++k) {
        mn[k] = fminf(fminf(v[k], v[3 + k]), v[6 + k]);
        mx[k] = fmaxf(fmaxf(v[k], v[3 + k]), v[6 + k]);
    }
}

__device__ __forceinline__ void child_box(uint32_t c, const float* tri, const unsigned long long* keys,
                                          const float* boxes, float* mn, float* mx) {
    if (c & kLeafBit) {
        tri_box(tri, keys, c & ~kLeafBit, mn, mx);
    } else {
        const volatile float* b = boxes + (size_t)c * 6;
        for (int k = 0; k < 3; ++k) {
            mn[k] = b[k];
            mx[k] = b[3 + k];
        }
    }
}

// Bounds bottom-up; the second thread to reach a node computes it.
__global__ void bounds_kernel(const float* __restrict__ tri, const unsigned long long* __restrict__ keys, int n,
                              const uint32_t* __restrict__ left, const uint32_t* __restrict__ right,
                              const int* __restrict__ parent_int, const int* __restrict__ parent_leaf,
                              uint32_t* __restrict__ arrivals, float* boxes) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int p = parent_leaf[k];
    while (p >= 0) {
        __threadfence();
        if (atomicAdd(&arrivals[p], 1u) == 0u) return;   // the sibling's thread finishes this node
        float lmn[3], lmx[3], rmn[3], rmx[3];
        child_box(left[p], tri, keys, boxes, lmn, lmx);
        child_box(right[p], tri, keys, boxes, rmn, rmx);
        volatile float* b = boxes + (size_t)p * 6;
        for (int c = 0; c < 3; ++c) {
            b[c] = fminf(lmn[c], rmn[c]);
            b[3 + c] = fmaxf(lmx[c], rmx[c]);
        }
        p = parent_int[p];
    }
}

__device__ __forceinline__ uint32_t subtree_size(uint32_t c, const uint32_t* range_lo, const uint32_t* range_hi) {
    if (c & kLeafBit) return 1u;
    return 2u * (range_hi[c] - range_lo[c] + 1u) - 1u;
}

// Post-order slot of every node: first slot of its block (left siblings on
// the path to the root) plus its block size minus one.
__global__ void postorder_kernel(int n, const uint32_t* __restrict__ left, const uint32_t* __restrict__ range_lo,
                                 const uint32_t* __restrict__ range_hi, const int* __restrict__ parent_int,
                                 const int* __restrict__ parent_leaf, uint32_t* __restrict__ slot_int,
                                 uint32_t* __restrict__ slot_leaf) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * n - 1) return;
    const bool leaf = t >= n - 1;
    const uint32_t self = leaf ? (kLeafBit | (uint32_t)(t - (n - 1))) : (uint32_t)t;
    uint32_t start = 0;
    uint32_t cur = self;
    int p = leaf ? parent_leaf[self & ~kLeafBit] : parent_int[self];
    while (p >= 0) {
        if (left[p] != cur) start += subtree_size(left[p], range_lo, range_hi);
        cur = (uint32_t)p;
        p = parent_int[p];
    }
    const uint32_t slot = start + subtree_size(self, range_lo, range_hi) - 1u;
    if (leaf) slot_leaf[self & ~kLeafBit] = slot;
    else slot_int[self] = slot;
}

__global__ void write_kernel(const float* __restrict__ tri, const unsigned long long* __restrict__ keys, int n,
                             const uint32_t* __restrict__ left, const uint32_t* __restrict__ right,
                             const float* __restrict__ boxes, const uint32_t* __restrict__ slot_int,
                             const uint32_t* __restrict__ slot_leaf, uint32_t first_global, uint32_t node_offset,
                             orn_bvh_node* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * n - 1) return;
    orn_bvh_node node;
    memset(&node, 0, sizeof(node));
    uint32_t slot;
    if (t >= n - 1) {
        const uint32_t k = (uint32_t)(t - (n - 1));
        const uint32_t tri_id = (uint32_t)(keys[k] & 0xFFFFFFFFull);
        const float* v = tri + (size_t)tri_id * 9;
        for (int c = 0; c < 3; ++c) {
            node.left_aabb_min_or_v0[c] = v[c];
            node.left_aabb_max_or_v1[c] = v[3 + c];
            node.right_aabb_min_or_v2[c] = v[6 + c];
        }
        node.left_or_custom_id = first_global + tri_id;
        node.node_type = ORN_NODE_TRIANGLE;
        slot = slot_leaf[k];
    } else {
        float mn[3], mx[3];
        child_box(left[t], tri, keys, boxes, mn, mx);
        for (int c = 0; c < 3; ++c) {
            node.left_aabb_min_or_v0[c] = mn[c];
            node.left_aabb_max_or_v1[c] = mx[c];
        }
        child_box(right[t], tri, keys, boxes, mn, mx);
        for (int c = 0; c < 3; ++c) {
            node.right_aabb_min_or_v2[c] = mn[c];
            node.right_aabb_max_or_v3[c] = mx[c];
        }
        const uint32_t l = left[t], r = right[t];
        node.left_or_custom_id = node_offset + ((l & kLeafBit) ? slot_leaf[l & ~kLeafBit] : slot_int[l]);
        node.right_or_material_index = node_offset + ((r & kLeafBit) ? slot_leaf[r & ~kLeafBit] : slot_int[r]);
        node.node_type = ORN_NODE_INTERNAL;
        slot = slot_int[t];
    }
    out[slot] = node;
}

}  // namespace

int lbvh_build_blas(const float* tri_host, uint32_t n, uint32_t first_global, uint32_t node_offset,
                    orn_bvh_node* out_host) {
    if (n == 0) return ORN_ERR_EMPTY_SCENE;
    if (n >= (1u << 31)) return ORN_ERR_INVALID_ARGUMENT;   // node and sort indices are int
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return ORN_ERR_NO_DEVICE;
    if (n == 1) {
        orn_bvh_node node;
        std::memset(&node, 0, sizeof(node));
        std::memcpy(node.left_aabb_min_or_v0, tri_host, 12);
        std::memcpy(node.left_aabb_max_or_v1, tri_host + 3, 12);
        std::memcpy(node.right_aabb_min_or_v2, tri_host + 6, 12);
        node.left_or_custom_id = first_global;
        node.node_type = ORN_NODE_TRIANGLE;
        out_host[0] = node;
        return ORN_OK;
    }
    // centroid bounds on the host (one pass)
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            const float* v = tri_host + (size_t)i * 9;
            const float c = 0.5f * (std::min(std::min(v[k], v[3 + k]), v[6 + k]) +
                                    std::max(std::max(v[k], v[3 + k]), v[6 + k]));
            lo[k] = std::min(lo[k], c);
            hi[k] = std::max(hi[k], c);
        }
    float3 flo = make_float3(lo[0], lo[1], lo[2]);
    float3 fscale;
    {
        float e[3];
        for (int k = 0; k < 3; ++k) e[k] = hi[k] - lo[k];
        fscale = make_float3(e[0] > 0 ? 1023.0f / e[0] : 0.0f, e[1] > 0 ? 1023.0f / e[1] : 0.0f,
                             e[2] > 0 ? 1023.0f / e[2] : 0.0f);
    }
    const size_t nn = n, ni = n - 1;
    float* d_tri = nullptr;
    unsigned long long *d_keys = nullptr, *d_keys2 = nullptr;
    uint32_t *d_left = nullptr, *d_right = nullptr, *d_lo = nullptr, *d_hi = nullptr, *d_arr = nullptr;
    uint32_t *d_slot_int = nullptr, *d_slot_leaf = nullptr;
    int *d_pint = nullptr, *d_pleaf = nullptr;
    float* d_boxes = nullptr;
    orn_bvh_node* d_out = nullptr;
    void* d_temp = nullptr;
    size_t temp_bytes = 0;
    int st = ORN_OK;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess && st == ORN_OK) st = e == cudaErrorMemoryAllocation ? ORN_ERR_OUT_OF_MEMORY : ORN_ERR_CUDA;
        return st == ORN_OK;
    };
    cudaStream_t s = nullptr;
    if (ok(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) && ok(cudaMalloc(&d_tri, nn * 9 * 4)) &&
        ok(cudaMalloc(&d_keys, nn * 8)) && ok(cudaMalloc(&d_keys2, nn * 8)) && ok(cudaMalloc(&d_left, ni * 4)) &&
        ok(cudaMalloc(&d_right, ni * 4)) && ok(cudaMalloc(&d_lo, ni * 4)) && ok(cudaMalloc(&d_hi, ni * 4)) &&
        ok(cudaMalloc(&d_arr, ni * 4)) && ok(cudaMalloc(&d_slot_int, ni * 4)) &&
        ok(cudaMalloc(&d_slot_leaf, nn * 4)) && ok(cudaMalloc(&d_pint, ni * 4)) && ok(cudaMalloc(&d_pleaf, nn * 4)) &&
        ok(cudaMalloc(&d_boxes, ni * 6 * 4)) && ok(cudaMalloc(&d_out, (2 * nn - 1) * sizeof(orn_bvh_node))) &&
        ok(cub::DeviceRadixSort::SortKeys(nullptr, temp_bytes, d_keys, d_keys2, (int)n, 0, 64, s)) &&
        ok(cudaMalloc(&d_temp, std::max<size_t>(temp_bytes, 16)))) {
        const int B = 256;
        const unsigned gn = (unsigned)((nn + B - 1) / B), gall = (unsigned)((2 * nn - 1 + B - 1) / B);
        ok(cudaMemcpyAsync(d_tri, tri_host, nn * 9 * 4, cudaMemcpyHostToDevice, s));
        ok(cudaMemsetAsync(d_arr, 0, ni * 4, s));
        ok(cudaMemsetAsync(d_pint, 0xFF, ni * 4, s));   // root's parent = -1
        morton_kernel<<<gn, B, 0, s>>>(d_tri, n, flo, fscale, d_keys);
        ok(cudaGetLastError());
        ok(cub::DeviceRadixSort::SortKeys(d_temp, temp_bytes, d_keys, d_keys2, (int)n, 0, 64, s));
        hierarchy_kernel<<<gn, B, 0, s>>>(d_keys2, (int)n, d_left, d_right, d_pint, d_pleaf, d_lo, d_hi);
        ok(cudaGetLastError());
        bounds_kernel<<<gn, B, 0, s>>>(d_tri, d_keys2, (int)n, d_left, d_right, d_pint, d_pleaf, d_arr, d_boxes);
        ok(cudaGetLastError());
        postorder_kernel<<<gall, B, 0, s>>>((int)n, d_left, d_lo, d_hi, d_pint, d_pleaf, d_slot_int, d_slot_leaf);
        ok(cudaGetLastError());
        write_kernel<<<gall, B, 0, s>>>(d_tri, d_keys2, (int)n, d_left, d_right, d_boxes, d_slot_int, d_slot_leaf,
                                        first_global, node_offset, d_out);
        ok(cudaGetLastError());
        ok(cudaMemcpyAsync(out_host, d_out, (2 * nn - 1) * sizeof(orn_bvh_node), cudaMemcpyDeviceToHost, s));
        ok(cudaStreamSynchronize(s));
    }
    void* ptrs[] = {d_tri, d_keys, d_keys2, d_left, d_right, d_lo, d_hi, d_arr, d_slot_int, d_slot_leaf,
                    d_pint, d_pleaf, d_boxes, d_out, d_temp};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (s) cudaStreamDestroy(s);
    return st;
}

}  // namespace orn
