// bvh_build.cpp — the scene → flat TLAS/BLAS arrays builder.
//
// Restates the rules of zig_ornament's Bvh.init (src/bvh.zig:33-78, build
// :92-108, buildMeshBvhRecursive :172-219, buildBvhBlasRecursive :221-270,
// buildBvhTlasRecursive :272-362, appendTransform :364-367,
// getMaterialIndex :369-383):
//   * TLAS leaf order: spheres, then mesh instances, then meshes.
//   * One BLAS per mesh, built in mesh order before the TLAS.  A mesh's
//     triangles get global ids (normal_indices.len / 3 before the mesh) + i;
//     its normal/uv indices are rebased onto the global arrays.
//   * Each internal node draws a split axis uniformly from {0,1,2}, orders
//     its leaves by aabb.min[axis] and splits at len/2.  Children are
//     appended before their parent (post-order), so every root is last.
//   * Each TLAS leaf appends {inverse(M), M} (transposed when
//     row_major_transforms, the HIP layout) and takes transform_id = pair
//     index; material indices are assigned at first use in leaf order, and a
//     textured material appends its texture at that moment.
//
// Differences from the Zig builder, all deterministic and platform
// independent: the axis PRNG is xoshiro256++ seeded through splitmix64
// (Blackman & Vigna) with Lemire's bounded draw, not Zig's DefaultPrng; the
// median split uses a selection on the total order (key, original position)
// instead of an unstable heap sort, so ties break by position; inverses are
// computed in double and rounded to float.  The trees therefore match the
// Zig builder's rules but not its bits; the parity tests feed the same flat
// arrays to every implementation.
//
// Because a subtree over n leaves always holds 2n-1 nodes and draws n-1
// axes in pre-order, every node's output slot and PRNG draw are known
// before it is built; BLAS subtrees are built on worker threads with
// output identical to a sequential build.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "ornament_cuda.h"
#include "lbvh.h"

static_assert(sizeof(orn_bvh_node) == 64, "BvhNode is 64 bytes");
static_assert(sizeof(orn_material) == 32, "Material is 32 bytes");
static_assert(sizeof(orn_camera) == 112, "Camera is 112 bytes");
static_assert(sizeof(orn_constant_params) == 144, "ConstantParams is 144 bytes");

struct orn_bvh {
    std::vector<orn_bvh_node> tlas, blas;
    std::vector<float> normals, uvs, transforms;
    std::vector<uint32_t> normal_indices, uv_indices;
    std::vector<orn_material> materials;
    std::vector<orn_texture> textures;
    uint32_t scene_textures_count = 0;
};

namespace {

// ---- PRNG: xoshiro256++ with splitmix64 seeding ------------------------
struct Xoshiro256pp {
    uint64_t s[4];
    explicit Xoshiro256pp(uint64_t seed) {
        uint64_t x = seed;
        for (int i = 0; i < 4; ++i) {
            x += 0x9e3779b97f4a7c15ull;
            uint64_t z = x;
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
            s[i] = z ^ (z >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        uint64_t result = rotl(s[0] + s[3], 23) + s[0];
        uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return result;
    }
    // Uniform integer in [0, bound) (Lemire's multiply-shift with rejection).
    uint32_t below(uint32_t bound) {
        uint32_t x = (uint32_t)(next() >> 32);
        uint64_t m = (uint64_t)x * bound;
        uint32_t l = (uint32_t)m;
        if (l < bound) {
            uint32_t t = (0u - bound) % bound;
            while (l < t) {
                x = (uint32_t)(next() >> 32);
                m = (uint64_t)x * bound;
                l = (uint32_t)m;
            }
        }
        return (uint32_t)(m >> 32);
    }
};

// ---- 4x4 helpers (zmath row-vector convention, row-major storage) -------
bool invert4(const float* m, float* out) {
    double a[16], inv[16];
    for (int i = 0; i < 16; ++i) a[i] = m[i];
    inv[0] = a[5]*a[10]*a[15] - a[5]*a[11]*a[14] - a[9]*a[6]*a[15] + a[9]*a[7]*a[14] + a[13]*a[6]*a[11] - a[13]*a[7]*a[10];
    inv[4] = -a[4]*a[10]*a[15] + a[4]*a[11]*a[14] + a[8]*a[6]*a[15] - a[8]*a[7]*a[14] - a[12]*a[6]*a[11] + a[12]*a[7]*a[10];
    inv[8] = a[4]*a[9]*a[15] - a[4]*a[11]*a[13] - a[8]*a[5]*a[15] + a[8]*a[7]*a[13] + a[12]*a[5]*a[11] - a[12]*a[7]*a[9];
    inv[12] = -a[4]*a[9]*a[14] + a[4]*a[10]*a[13] + a[8]*a[5]*a[14] - a[8]*a[6]*a[13] - a[12]*a[5]*a[10] + a[12]*a[6]*a[9];
    inv[1] = -a[1]*a[10]*a[15] + a[1]*a[11]*a[14] + a[9]*a[2]*a[15] - a[9]*a[3]*a[14] - a[13]*a[2]*a[11] + a[13]*a[3]*a[10];
    inv[5] = a[0]*a[10]*a[15] - a[0]*a[11]*a[14] - a[8]*a[2]*a[15] + a[8]*a[3]*a[14] + a[12]*a[2]*a[11] - a[12]*a[3]*a[10];
    inv[9] = -a[0]*a[9]*a[15] + a[0]*a[11]*a[13] + a[8]*a[1]*a[15] - a[8]*a[3]*a[13] - a[12]*a[1]*a[11] + a[12]*a[3]*a[9];
    inv[13] = a[0]*a[9]*a[14] - a[0]*a[10]*a[13] - a[8]*a[1]*a[14] + a[8]*a[2]*a[13] + a[12]*a[1]*a[10] - a[12]*a[2]*a[9];
    inv[2] = a[1]*a[6]*a[15] - a[1]*a[7]*a[14] - a[5]*a[2]*a[15] + a[5]*a[3]*a[14] + a[13]*a[2]*a[7] - a[13]*a[3]*a[6];
    inv[6] = -a[0]*a[6]*a[15] + a[0]*a[7]*a[14] + a[4]*a[2]*a[15] - a[4]*a[3]*a[14] - a[12]*a[2]*a[7] + a[12]*a[3]*a[6];
    inv[10] = a[0]*a[5]*a[15] - a[0]*a[7]*a[13] - a[4]*a[1]*a[15] + a[4]*a[3]*a[13] + a[12]*a[1]*a[7] - a[12]*a[3]*a[5];
    inv[14] = -a[0]*a[5]*a[14] + a[0]*a[6]*a[13] + a[4]*a[1]*a[14] - a[4]*a[2]*a[13] - a[12]*a[1]*a[6] + a[12]*a[2]*a[5];
    inv[3] = -a[1]*a[6]*a[11] + a[1]*a[7]*a[10] + a[5]*a[2]*a[11] - a[5]*a[3]*a[10] - a[9]*a[2]*a[7] + a[9]*a[3]*a[6];
    inv[7] = a[0]*a[6]*a[11] - a[0]*a[7]*a[10] - a[4]*a[2]*a[11] + a[4]*a[3]*a[10] + a[8]*a[2]*a[7] - a[8]*a[3]*a[6];
    inv[11] = -a[0]*a[5]*a[11] + a[0]*a[7]*a[9] + a[4]*a[1]*a[11] - a[4]*a[3]*a[9] - a[8]*a[1]*a[7] + a[8]*a[3]*a[5];
    inv[15] = a[0]*a[5]*a[10] - a[0]*a[6]*a[9] - a[4]*a[1]*a[10] + a[4]*a[2]*a[9] + a[8]*a[1]*a[6] - a[8]*a[2]*a[5];
    double det = a[0]*inv[0] + a[1]*inv[4] + a[2]*inv[8] + a[3]*inv[12];
    if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) return false;
    for (int i = 0; i < 16; ++i) out[i] = (float)(inv[i] / det);
    return true;
}

void append_transform(orn_bvh* b, const float* m, bool row_major) {
    size_t base = b->transforms.size();
    b->transforms.resize(base + 16);
    float* o = b->transforms.data() + base;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) o[r * 4 + c] = row_major ? m[c * 4 + r] : m[r * 4 + c];
}

bool finite3(const float* v) {
    return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]);
}

// ---- binned SAH split (the non-parity builder) -------------------------------
// Partitions items[0..n) in place into a left and a right part and returns
// the left count (1..n-1): centroids are binned (up to 32 bins) along each
// axis with a non-zero centroid extent, and the bin boundary minimising
// area(left) * count(left) + area(right) * count(right) is taken; items whose
// centroids coincide are split in half.  `box(item, mn, mx)` gives an item's
// bounds.
template <class T, class Box>
size_t sah_split(T* items, size_t n, Box box) {
    float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = 0; i < n; ++i) {
        float mn[3], mx[3];
        box(items[i], mn, mx);
        for (int k = 0; k < 3; ++k) {
            const float c = 0.5f * (mn[k] + mx[k]);
            cmin[k] = std::min(cmin[k], c);
            cmax[k] = std::max(cmax[k], c);
        }
    }
    constexpr int kBins = 32;
    const int bins = (int)std::min<size_t>(kBins, std::max<size_t>(n, 2));
    double best_cost = INFINITY;
    int best_axis = -1, best_bin = 0;
    auto area = [](const float* mn, const float* mx) {
        const double dx = (double)mx[0] - mn[0], dy = (double)mx[1] - mn[1], dz = (double)mx[2] - mn[2];
        return dx < 0 ? 0.0 : 2.0 * (dx * dy + dy * dz + dz * dx);
    };
    for (int axis = 0; axis < 3; ++axis) {
        const float ext = cmax[axis] - cmin[axis];
        if (!(ext > 0.0f) || !std::isfinite(ext)) continue;
        const float scale = (float)bins / ext;
        size_t cnt[kBins] = {};
        float bmn[kBins][3], bmx[kBins][3];
        for (int b = 0; b < bins; ++b)
            for (int k = 0; k < 3; ++k) { bmn[b][k] = INFINITY; bmx[b][k] = -INFINITY; }
        for (size_t i = 0; i < n; ++i) {
            float mn[3], mx[3];
            box(items[i], mn, mx);
            const float c = 0.5f * (mn[axis] + mx[axis]);
            const int b = std::min(bins - 1, std::max(0, (int)((c - cmin[axis]) * scale)));
            cnt[b]++;
            for (int k = 0; k < 3; ++k) {
                bmn[b][k] = std::min(bmn[b][k], mn[k]);
                bmx[b][k] = std::max(bmx[b][k], mx[k]);
            }
        }
        // right-to-left suffix areas, then a left-to-right sweep
        double rarea[kBins];
        size_t rcnt[kBins];
        float rmn[3] = {INFINITY, INFINITY, INFINITY}, rmx[3] = {-INFINITY, -INFINITY, -INFINITY};
        size_t rc = 0;
        for (int b = bins - 1; b >= 1; --b) {
            for (int k = 0; k < 3; ++k) { rmn[k] = std::min(rmn[k], bmn[b][k]); rmx[k] = std::max(rmx[k], bmx[b][k]); }
            rc += cnt[b];
            rarea[b] = area(rmn, rmx);
            rcnt[b] = rc;
        }
        float lmn[3] = {INFINITY, INFINITY, INFINITY}, lmx[3] = {-INFINITY, -INFINITY, -INFINITY};
        size_t lc = 0;
        for (int b = 1; b < bins; ++b) {   // left = bins [0, b)
            for (int k = 0; k < 3; ++k) { lmn[k] = std::min(lmn[k], bmn[b - 1][k]); lmx[k] = std::max(lmx[k], bmx[b - 1][k]); }
            lc += cnt[b - 1];
            if (lc == 0 || rcnt[b] == 0) continue;
            const double cost = area(lmn, lmx) * (double)lc + rarea[b] * (double)rcnt[b];
            if (cost < best_cost) {
                best_cost = cost;
                best_axis = axis;
                best_bin = b;
            }
        }
    }
    if (best_axis < 0) return n / 2;   // all centroids coincide: any split
    const float scale = (float)bins / (cmax[best_axis] - cmin[best_axis]);
    T* mid = std::partition(items, items + n, [&](const T& it) {
        float mn[3], mx[3];
        box(it, mn, mx);
        const float c = 0.5f * (mn[best_axis] + mx[best_axis]);
        return std::min(bins - 1, std::max(0, (int)((c - cmin[best_axis]) * scale))) < best_bin;
    });
    const size_t nl = (size_t)(mid - items);
    return (nl == 0 || nl == n) ? n / 2 : nl;
}

// ---- BLAS ------------------------------------------------------------------
struct MeshTris {
    std::vector<float> v;        // 9 floats per triangle (v0, v1, v2)
    std::vector<float> key;      // 3 floats per triangle: aabb.min
    uint32_t first_global = 0;   // global id of triangle 0
};

struct BlasJob {
    const MeshTris* tris;
    const uint8_t* axes;   // pre-drawn split axes of this mesh (pre-order)
    orn_bvh_node* out;     // this mesh's node slots (2n-1), post-order
    bool sah;              // binned-SAH splits instead of the reference's rule
};

void bbox(const MeshTris& t, const uint32_t* idx, size_t n, float* mn, float* mx) {
    mn[0] = mn[1] = mn[2] = INFINITY;
    mx[0] = mx[1] = mx[2] = -INFINITY;
    for (size_t i = 0; i < n; ++i) {
        const float* v = &t.v[(size_t)idx[i] * 9];
        for (int k = 0; k < 3; ++k) {
            float lo = std::min(std::min(v[k], v[3 + k]), v[6 + k]);
            float hi = std::max(std::max(v[k], v[3 + k]), v[6 + k]);
            mn[k] = std::min(mn[k], lo);
            mx[k] = std::max(mx[k], hi);
        }
    }
}

// Builds the subtree over idx[0..n) into out[0..2n-1) (root at out[2n-2]),
// drawing axes from axes[0..n-1).  `node_offset` is the global index of
// out[0] (children ids are global blas indices).
void build_blas(const BlasJob& job, uint32_t* idx, size_t n, size_t node_slot,
                size_t draw, uint32_t node_offset, int spawn_depth) {
    const MeshTris& t = *job.tris;
    orn_bvh_node* node = &job.out[node_slot + 2 * n - 2];
    std::memset(node, 0, sizeof(*node));
    if (n == 1) {
        const float* v = &t.v[(size_t)idx[0] * 9];
        std::memcpy(node->left_aabb_min_or_v0, v, 12);
        std::memcpy(node->left_aabb_max_or_v1, v + 3, 12);
        std::memcpy(node->right_aabb_min_or_v2, v + 6, 12);
        node->left_or_custom_id = t.first_global + idx[0];
        node->node_type = ORN_NODE_TRIANGLE;
        return;
    }
    size_t mid = n / 2;
    if (job.sah) {
        mid = sah_split(idx, n, [&t](uint32_t i, float* mn, float* mx) {
            const float* v = &t.v[(size_t)i * 9];
            for (int k = 0; k < 3; ++k) {
                mn[k] = std::min(std::min(v[k], v[3 + k]), v[6 + k]);
                mx[k] = std::max(std::max(v[k], v[3 + k]), v[6 + k]);
            }
        });
    } else {
        const int axis = job.axes[draw];
        const float* key = t.key.data();
        std::nth_element(idx, idx + mid, idx + n, [key, axis](uint32_t a, uint32_t b) {
            float ka = key[(size_t)a * 3 + axis], kb = key[(size_t)b * 3 + axis];
            return ka < kb || (ka == kb && a < b);
        });
    }
    const size_t nl = mid, nr = n - mid;
    const size_t left_slot = node_slot, right_slot = node_slot + 2 * nl - 1;
    const size_t left_draw = draw + 1, right_draw = draw + 1 + (nl - 1);
    float lmin[3], lmax[3], rmin[3], rmax[3];
    if (spawn_depth > 0 && n > 65536) {
        std::thread th([&] {
            build_blas(job, idx, nl, left_slot, left_draw, node_offset, spawn_depth - 1);
            bbox(t, idx, nl, lmin, lmax);
        });
        build_blas(job, idx + nl, nr, right_slot, right_draw, node_offset, spawn_depth - 1);
        bbox(t, idx + nl, nr, rmin, rmax);
        th.join();
    } else {
        build_blas(job, idx, nl, left_slot, left_draw, node_offset, 0);
        bbox(t, idx, nl, lmin, lmax);
        build_blas(job, idx + nl, nr, right_slot, right_draw, node_offset, 0);
        bbox(t, idx + nl, nr, rmin, rmax);
    }
    std::memcpy(node->left_aabb_min_or_v0, lmin, 12);
    std::memcpy(node->left_aabb_max_or_v1, lmax, 12);
    std::memcpy(node->right_aabb_min_or_v2, rmin, 12);
    std::memcpy(node->right_aabb_max_or_v3, rmax, 12);
    node->left_or_custom_id = node_offset + (uint32_t)(left_slot + 2 * nl - 2);
    node->right_or_material_index = node_offset + (uint32_t)(right_slot + 2 * nr - 2);
    node->node_type = ORN_NODE_INTERNAL;
}

// ---- TLAS ------------------------------------------------------------------
struct Leaf {
    int kind;        // 0 sphere, 1 mesh instance, 2 mesh
    uint32_t index;  // into the desc array of that kind
    float mn[3], mx[3];
};

struct TlasBuilder {
    const orn_scene_desc* desc;
    orn_bvh* out;
    const std::vector<uint32_t>* mesh_bvh_id;
    std::vector<uint32_t> material_index;  // per desc material, ~0u = unassigned
    const uint8_t* axes;
    size_t draw = 0;
    int status = ORN_OK;

    uint32_t get_material(uint32_t m) {
        if (material_index[m] != 0xFFFFFFFFu) return material_index[m];
        const orn_material_desc& md = desc->materials[m];
        orn_material gm;
        std::memset(&gm, 0, sizeof(gm));
        gm.albedo[0] = md.albedo[0];
        gm.albedo[1] = md.albedo[1];
        gm.albedo[2] = md.albedo[2];
        gm.albedo_texture_index = ORN_NO_TEXTURE;
        if (md.texture != ORN_NO_TEXTURE) {
            // Zig: Material.from keeps the default albedo (1, 0, 1) for
            // textured materials (src/gpu_structs.zig:42-49).
            gm.albedo[0] = 1.0f; gm.albedo[1] = 0.0f; gm.albedo[2] = 1.0f;
            out->textures.push_back(desc->textures[md.texture]);
            gm.albedo_texture_index = (uint32_t)(out->textures.size() - 1);
        }
        gm.fuzz = md.fuzz;
        gm.ior = md.ior;
        gm.type = md.type;
        out->materials.push_back(gm);
        material_index[m] = (uint32_t)(out->materials.size() - 1);
        return material_index[m];
    }

    orn_bvh_node make_leaf(const Leaf& l) {
        orn_bvh_node n;
        std::memset(&n, 0, sizeof(n));
        const float* transform = nullptr;
        uint32_t material = 0;
        if (l.kind == 0) {
            transform = desc->spheres[l.index].transform;
            material = desc->spheres[l.index].material;
            n.node_type = ORN_NODE_SPHERE;
        } else if (l.kind == 1) {
            const orn_mesh_instance_desc& mi = desc->mesh_instances[l.index];
            transform = mi.transform;
            material = mi.material;
            n.node_type = ORN_NODE_MESH;
            n.left_or_custom_id = (*mesh_bvh_id)[mi.mesh];
        } else {
            transform = desc->meshes[l.index].transform;
            material = desc->meshes[l.index].material;
            n.node_type = ORN_NODE_MESH;
            n.left_or_custom_id = (*mesh_bvh_id)[l.index];
        }
        float inv[16];
        if (!invert4(transform, inv)) { status = ORN_ERR_BAD_SCENE; return n; }
        bool row_major = desc->row_major_transforms != 0;
        append_transform(out, inv, row_major);
        append_transform(out, transform, row_major);
        n.transform_id = (uint32_t)(out->transforms.size() / 32 - 1);
        std::memcpy(n.left_aabb_min_or_v0, l.mn, 12);
        std::memcpy(n.left_aabb_max_or_v1, l.mx, 12);
        n.right_or_material_index = get_material(material);
        return n;
    }

    static void bounds(const Leaf* l, size_t n, float* mn, float* mx) {
        mn[0] = mn[1] = mn[2] = INFINITY;
        mx[0] = mx[1] = mx[2] = -INFINITY;
        for (size_t i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) {
                mn[k] = std::min(mn[k], l[i].mn[k]);
                mx[k] = std::max(mx[k], l[i].mx[k]);
            }
    }

    bool sah = false;

    // Returns the node for leaves[0..n); the caller appends it.
    orn_bvh_node build(Leaf* leaves, const uint32_t* order, size_t n) {
        if (n == 1) return make_leaf(leaves[0]);
        if (sah) return build_sah(leaves, n);
        const int axis = axes[draw++];
        const size_t mid = n / 2;
        // sort positions by (aabb.min[axis], original position)
        std::vector<size_t> p(n);
        for (size_t i = 0; i < n; ++i) p[i] = i;
        std::nth_element(p.begin(), p.begin() + mid, p.end(), [&](size_t a, size_t b) {
            float ka = leaves[a].mn[axis], kb = leaves[b].mn[axis];
            return ka < kb || (ka == kb && order[a] < order[b]);
        });
        // keep each half in original-position order so recursion is stable
        std::sort(p.begin(), p.begin() + mid, [&](size_t a, size_t b) { return order[a] < order[b]; });
        std::sort(p.begin() + mid, p.end(), [&](size_t a, size_t b) { return order[a] < order[b]; });
        std::vector<Leaf> tmp(n);
        std::vector<uint32_t> tord(n);
        for (size_t i = 0; i < n; ++i) { tmp[i] = leaves[p[i]]; tord[i] = order[p[i]]; }
        std::copy(tmp.begin(), tmp.end(), leaves);
        std::vector<uint32_t> ord2(tord);
        orn_bvh_node left = build(leaves, ord2.data(), mid);
        out->tlas.push_back(left);
        uint32_t left_id = (uint32_t)(out->tlas.size() - 1);
        float lmin[3], lmax[3];
        bounds(leaves, mid, lmin, lmax);
        orn_bvh_node right = build(leaves + mid, ord2.data() + mid, n - mid);
        out->tlas.push_back(right);
        uint32_t right_id = (uint32_t)(out->tlas.size() - 1);
        float rmin[3], rmax[3];
        bounds(leaves + mid, n - mid, rmin, rmax);
        orn_bvh_node node;
        std::memset(&node, 0, sizeof(node));
        std::memcpy(node.left_aabb_min_or_v0, lmin, 12);
        std::memcpy(node.left_aabb_max_or_v1, lmax, 12);
        std::memcpy(node.right_aabb_min_or_v2, rmin, 12);
        std::memcpy(node.right_aabb_max_or_v3, rmax, 12);
        node.left_or_custom_id = left_id;
        node.right_or_material_index = right_id;
        node.node_type = ORN_NODE_INTERNAL;
        return node;
    }

    // The non-parity builder: binned-SAH splits over the leaves' boxes.
    orn_bvh_node build_sah(Leaf* leaves, size_t n) {
        if (n == 1) return make_leaf(leaves[0]);
        const size_t mid = sah_split(leaves, n, [](const Leaf& l, float* mn, float* mx) {
            std::memcpy(mn, l.mn, 12);
            std::memcpy(mx, l.mx, 12);
        });
        orn_bvh_node node;
        std::memset(&node, 0, sizeof(node));
        orn_bvh_node left = build_sah(leaves, mid);
        out->tlas.push_back(left);
        node.left_or_custom_id = (uint32_t)(out->tlas.size() - 1);
        orn_bvh_node right = build_sah(leaves + mid, n - mid);
        out->tlas.push_back(right);
        node.right_or_material_index = (uint32_t)(out->tlas.size() - 1);
        float mn[3], mx[3];
        bounds(leaves, mid, mn, mx);
        std::memcpy(node.left_aabb_min_or_v0, mn, 12);
        std::memcpy(node.left_aabb_max_or_v1, mx, 12);
        bounds(leaves + mid, n - mid, mn, mx);
        std::memcpy(node.right_aabb_min_or_v2, mn, 12);
        std::memcpy(node.right_aabb_max_or_v3, mx, 12);
        node.node_type = ORN_NODE_INTERNAL;
        return node;
    }
};

int validate(const orn_scene_desc* d) {
    if (!d) return ORN_ERR_INVALID_ARGUMENT;
    uint64_t shapes = (uint64_t)d->spheres_len + d->meshes_len + d->mesh_instances_len;
    if (shapes == 0) return ORN_ERR_EMPTY_SCENE;
    if (d->builder > ORN_BVH_LBVH) return ORN_ERR_INVALID_ARGUMENT;
    if ((d->spheres_len && !d->spheres) || (d->meshes_len && !d->meshes) ||
        (d->mesh_instances_len && !d->mesh_instances) ||
        (d->materials_len && !d->materials) || (d->textures_len && !d->textures))
        return ORN_ERR_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < d->materials_len; ++i) {
        const orn_material_desc& m = d->materials[i];
        if (m.type > ORN_DIFFUSE_LIGHT) return ORN_ERR_BAD_SCENE;
        if (m.texture != ORN_NO_TEXTURE && m.texture >= d->textures_len) return ORN_ERR_BAD_SCENE;
    }
    for (uint32_t i = 0; i < d->textures_len; ++i) {
        const orn_texture& t = d->textures[i];
        if (!t.data || t.width == 0 || t.height == 0 || t.format > ORN_TEXEL_RGBA16F)
            return ORN_ERR_BAD_SCENE;
        uint32_t texel = t.format == ORN_TEXEL_RGBA8 ? 4u : 8u;
        if (t.bytes_per_row < t.width * texel) return ORN_ERR_BAD_SCENE;
    }
    for (uint32_t i = 0; i < d->spheres_len; ++i) {
        const orn_sphere_desc& s = d->spheres[i];
        if (s.material >= d->materials_len) return ORN_ERR_BAD_SCENE;
        if (!finite3(s.aabb_min) || !finite3(s.aabb_max)) return ORN_ERR_BAD_SCENE;
    }
    for (uint32_t i = 0; i < d->meshes_len; ++i) {
        const orn_mesh_desc& m = d->meshes[i];
        if (m.material >= d->materials_len) return ORN_ERR_BAD_SCENE;
        if (m.vertex_indices_len < 3) return ORN_ERR_EMPTY_SCENE;
        if (m.vertex_indices_len % 3 != 0) return ORN_ERR_BAD_SCENE;
        if (m.normal_indices_len != m.vertex_indices_len ||
            m.uv_indices_len != m.vertex_indices_len)
            return ORN_ERR_BAD_SCENE;
        if (!m.vertices || !m.vertex_indices || !m.normals || !m.normal_indices ||
            !m.uvs || !m.uv_indices)
            return ORN_ERR_INVALID_ARGUMENT;
        for (uint32_t k = 0; k < m.vertex_indices_len; ++k) {
            if (m.vertex_indices[k] >= m.vertices_len) return ORN_ERR_BAD_SCENE;
            if (m.normal_indices[k] >= m.normals_len) return ORN_ERR_BAD_SCENE;
            if (m.uv_indices[k] >= m.uvs_len) return ORN_ERR_BAD_SCENE;
        }
        if (!finite3(m.aabb_min) || !finite3(m.aabb_max)) return ORN_ERR_BAD_SCENE;
    }
    for (uint32_t i = 0; i < d->mesh_instances_len; ++i) {
        const orn_mesh_instance_desc& mi = d->mesh_instances[i];
        if (mi.mesh >= d->meshes_len || mi.material >= d->materials_len) return ORN_ERR_BAD_SCENE;
        if (!finite3(mi.aabb_min) || !finite3(mi.aabb_max)) return ORN_ERR_BAD_SCENE;
    }
    return ORN_OK;
}

int build_all(const orn_scene_desc* d, orn_bvh* b) {
    const uint32_t M = d->meshes_len;
    // Per-mesh triangle data and global offsets (src/bvh.zig:172-219).
    std::vector<MeshTris> tris(M);
    std::vector<size_t> blas_base(M + 1, 0), draw_base(M + 1, 0);
    size_t normals_total = 0, uvs_total = 0, idx_total = 0;
    for (uint32_t i = 0; i < M; ++i) {
        const orn_mesh_desc& m = d->meshes[i];
        size_t nt = m.vertex_indices_len / 3;
        blas_base[i + 1] = blas_base[i] + 2 * nt - 1;
        draw_base[i + 1] = draw_base[i] + nt - 1;
        normals_total += m.normals_len;
        uvs_total += m.uvs_len;
        idx_total += m.vertex_indices_len;
    }
    const size_t shapes = (size_t)d->spheres_len + d->meshes_len + d->mesh_instances_len;
    if (blas_base[M] > 0xFFFFFFFEull || shapes > 0x7FFFFFFFull) return ORN_ERR_BAD_SCENE;
    // All split axes, drawn in the reference's order: every BLAS (mesh
    // order, pre-order within a mesh), then the TLAS.
    std::vector<uint8_t> axes(draw_base[M] + (shapes - 1));
    {
        Xoshiro256pp rng(d->seed);
        for (size_t i = 0; i < axes.size(); ++i) axes[i] = (uint8_t)rng.below(3);
    }
    b->normals.reserve(normals_total * 4);
    b->uvs.reserve(uvs_total * 2);
    b->normal_indices.reserve(idx_total);
    b->uv_indices.reserve(idx_total);
    b->blas.resize(blas_base[M]);
    for (uint32_t i = 0; i < M; ++i) {
        const orn_mesh_desc& m = d->meshes[i];
        size_t nt = m.vertex_indices_len / 3;
        MeshTris& t = tris[i];
        t.first_global = (uint32_t)(b->normal_indices.size() / 3);
        t.v.resize(nt * 9);
        t.key.resize(nt * 3);
        for (size_t k = 0; k < nt; ++k)
            for (int c = 0; c < 3; ++c) {
                const float* v = m.vertices + (size_t)m.vertex_indices[k * 3 + c] * 4;
                t.v[k * 9 + c * 3 + 0] = v[0];
                t.v[k * 9 + c * 3 + 1] = v[1];
                t.v[k * 9 + c * 3 + 2] = v[2];
            }
        for (size_t k = 0; k < nt; ++k)
            for (int a = 0; a < 3; ++a)
                t.key[k * 3 + a] = std::min(std::min(t.v[k * 9 + a], t.v[k * 9 + 3 + a]), t.v[k * 9 + 6 + a]);
        uint32_t nbase = (uint32_t)(b->normals.size() / 4);
        for (uint32_t k = 0; k < m.normal_indices_len; ++k) b->normal_indices.push_back(m.normal_indices[k] + nbase);
        b->normals.insert(b->normals.end(), m.normals, m.normals + (size_t)m.normals_len * 4);
        uint32_t ubase = (uint32_t)(b->uvs.size() / 2);
        for (uint32_t k = 0; k < m.uv_indices_len; ++k) b->uv_indices.push_back(m.uv_indices[k] + ubase);
        b->uvs.insert(b->uvs.end(), m.uvs, m.uvs + (size_t)m.uvs_len * 2);
    }
    // Build the BLASes on worker threads (output slots are precomputed).
    std::vector<uint32_t> mesh_bvh_id(M);
    {
        unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        std::vector<std::thread> pool;
        std::vector<uint32_t> next(1, 0);
        auto work = [&](uint32_t i) {
            size_t nt = d->meshes[i].vertex_indices_len / 3;
            std::vector<uint32_t> idx(nt);
            for (size_t k = 0; k < nt; ++k) idx[k] = (uint32_t)k;
            BlasJob job{&tris[i], axes.data() + draw_base[i], b->blas.data() + blas_base[i], d->builder == ORN_BVH_SAH};
            int spawn = nt > 262144 ? 3 : 0;
            build_blas(job, idx.data(), nt, 0, 0, (uint32_t)blas_base[i], spawn);
        };
        std::vector<uint32_t> order(M);
        for (uint32_t i = 0; i < M; ++i) { order[i] = i; mesh_bvh_id[i] = (uint32_t)(blas_base[i + 1] - 1); }
        std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t c) {
            return d->meshes[a].vertex_indices_len > d->meshes[c].vertex_indices_len;
        });
        if (d->builder == ORN_BVH_LBVH) {
            // on the GPU, one mesh after another
            for (uint32_t i = 0; i < M; ++i) {
                const size_t nt = d->meshes[i].vertex_indices_len / 3;
                int st = orn::lbvh_build_blas(tris[i].v.data(), (uint32_t)nt, tris[i].first_global,
                                              (uint32_t)blas_base[i], b->blas.data() + blas_base[i]);
                if (st != ORN_OK) return st;
            }
            order.clear();
        }
        std::atomic_size_t cursor{0};
        unsigned nthreads = std::min<unsigned>(hw, std::max<uint32_t>(1, M));
        for (unsigned w = 0; w < nthreads; ++w)
            pool.emplace_back([&] {
                for (;;) {
                    size_t k = cursor.fetch_add(1);
                    if (k >= order.size()) break;
                    work(order[k]);
                }
            });
        for (auto& th : pool) th.join();
    }
    tris.clear();
    // TLAS (src/bvh.zig:92-108, 272-362).
    std::vector<Leaf> leaves;
    leaves.reserve(shapes);
    for (uint32_t i = 0; i < d->spheres_len; ++i) {
        Leaf l{0, i, {}, {}};
        std::memcpy(l.mn, d->spheres[i].aabb_min, 12);
        std::memcpy(l.mx, d->spheres[i].aabb_max, 12);
        leaves.push_back(l);
    }
    for (uint32_t i = 0; i < d->mesh_instances_len; ++i) {
        Leaf l{1, i, {}, {}};
        std::memcpy(l.mn, d->mesh_instances[i].aabb_min, 12);
        std::memcpy(l.mx, d->mesh_instances[i].aabb_max, 12);
        leaves.push_back(l);
    }
    for (uint32_t i = 0; i < M; ++i) {
        Leaf l{2, i, {}, {}};
        std::memcpy(l.mn, d->meshes[i].aabb_min, 12);
        std::memcpy(l.mx, d->meshes[i].aabb_max, 12);
        leaves.push_back(l);
    }
    std::vector<uint32_t> order(shapes);
    for (size_t i = 0; i < shapes; ++i) order[i] = (uint32_t)i;
    TlasBuilder tb;
    tb.desc = d;
    tb.out = b;
    tb.mesh_bvh_id = &mesh_bvh_id;
    tb.material_index.assign(d->materials_len, 0xFFFFFFFFu);
    tb.axes = axes.data() + draw_base[M];
    tb.sah = d->builder == ORN_BVH_SAH || d->builder == ORN_BVH_LBVH;
    b->tlas.reserve(2 * shapes - 1);
    orn_bvh_node root = tb.build(leaves.data(), order.data(), shapes);
    if (tb.status != ORN_OK) return tb.status;
    b->tlas.push_back(root);
    b->scene_textures_count = d->textures_len;
    return ORN_OK;
}

}  // namespace

extern "C" {

int orn_bvh_build(const orn_scene_desc* desc, orn_bvh** out) {
    if (!out) return ORN_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int st = validate(desc);
    if (st != ORN_OK) return st;
    orn_bvh* b = new (std::nothrow) orn_bvh();
    if (!b) return ORN_ERR_OUT_OF_MEMORY;
    try {
        st = build_all(desc, b);
    } catch (const std::bad_alloc&) {
        st = ORN_ERR_OUT_OF_MEMORY;
    } catch (...) {
        st = ORN_ERR_BAD_SCENE;
    }
    if (st != ORN_OK) { delete b; return st; }
    *out = b;
    return ORN_OK;
}

int orn_bvh_get_blob(const orn_bvh* b, orn_scene_blob* blob) {
    if (!b || !blob) return ORN_ERR_INVALID_ARGUMENT;
    std::memset(blob, 0, sizeof(*blob));
    blob->tlas_nodes = b->tlas.data();
    blob->tlas_nodes_len = (uint32_t)b->tlas.size();
    blob->blas_nodes = b->blas.data();
    blob->blas_nodes_len = (uint32_t)b->blas.size();
    blob->normals = b->normals.data();
    blob->normals_len = (uint32_t)(b->normals.size() / 4);
    blob->normal_indices = b->normal_indices.data();
    blob->normal_indices_len = (uint32_t)b->normal_indices.size();
    blob->uvs = b->uvs.data();
    blob->uvs_len = (uint32_t)(b->uvs.size() / 2);
    blob->uv_indices = b->uv_indices.data();
    blob->uv_indices_len = (uint32_t)b->uv_indices.size();
    blob->transforms = b->transforms.data();
    blob->transforms_len = (uint32_t)(b->transforms.size() / 16);
    blob->materials = b->materials.data();
    blob->materials_len = (uint32_t)b->materials.size();
    blob->textures = b->textures.data();
    blob->textures_len = (uint32_t)b->textures.size();
    blob->scene_textures_count = b->scene_textures_count;
    return ORN_OK;
}

int orn_bvh_free(orn_bvh* b) {
    delete b;
    return ORN_OK;
}

}  // extern "C"
