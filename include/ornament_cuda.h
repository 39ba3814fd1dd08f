/*
 * ornament_cuda.h — C ABI of libornament_cuda, a GB300 (sm_103a) path-tracing
 * backend for the zig_ornament scene model.
 *
 * The library replaces the two GPU backends of zig_ornament
 * (src/wgpu_backend/path_tracer.zig, src/hip_backend/path_tracer.zig) behind
 * the same duck-typed PathTracer surface: init / deinit / setResolution /
 * render / getFrameBuffer, with the public `state` and `scene.camera` fields
 * mapped to orn_set_state / orn_set_camera.  Every entry point below names
 * the reference function it replaces as `file:line` (paths inside the
 * zig_ornament project).
 *
 * Conventions
 *   - Plain C types only; every call returns an int status (ORN_OK = 0).
 *     The library never aborts; orn_last_error() gives a message.
 *   - One context per host thread.  orn_render() is asynchronous on the
 *     context's own CUDA stream; every orn_get_* call synchronises.
 *   - Struct layouts are byte-identical to src/gpu_structs.zig (checked by
 *     static asserts in the library and by the Python binding).
 */
#ifndef ORNAMENT_CUDA_H
#define ORNAMENT_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORN_ABI_VERSION 1u

/* ---- status codes ------------------------------------------------------ */
enum orn_status {
    ORN_OK = 0,
    ORN_ERR_INVALID_ARGUMENT = 1, /* null pointer, zero size, bad enum      */
    ORN_ERR_EMPTY_SCENE = 2,      /* src/bvh.zig:35-37 panics; we return    */
    ORN_ERR_OUT_OF_MEMORY = 3,    /* host or device allocation failed       */
    ORN_ERR_CUDA = 4,             /* a CUDA runtime call failed             */
    ORN_ERR_NO_DEVICE = 5,        /* no CUDA device / bad device ordinal    */
    ORN_ERR_BAD_SCENE = 6,        /* an index in the scene is out of range  */
    ORN_ERR_STACK_OVERFLOW = 7,   /* a ray needed more than 64 stack slots  */
    ORN_ERR_BUFFER_TOO_SMALL = 8, /* destination smaller than the target    */
    ORN_ERR_TIMEOUT = 9,          /* a bounded device-side wait gave up     */
    ORN_ERR_UNSUPPORTED = 10,     /* valid input of a kind not handled      */
    ORN_ERR_BAD_IMAGE = 11        /* a corrupt or truncated image stream    */
};

/* ---- GPU data layouts (src/gpu_structs.zig) ---------------------------- */

/* BvhNodeType, src/gpu_structs.zig:15-20 */
enum orn_node_type {
    ORN_NODE_INTERNAL = 0,
    ORN_NODE_SPHERE = 1,
    ORN_NODE_MESH = 2,
    ORN_NODE_TRIANGLE = 3
};

/* BvhNode, src/gpu_structs.zig:22-31 — 64 bytes. */
typedef struct orn_bvh_node {
    float left_aabb_min_or_v0[3];
    uint32_t left_or_custom_id;
    float left_aabb_max_or_v1[3];
    uint32_t right_or_material_index;
    float right_aabb_min_or_v2[3];
    uint32_t node_type;
    float right_aabb_max_or_v3[3];
    uint32_t transform_id;
} orn_bvh_node;

/* MaterialType, src/material.zig:4-9 */
enum orn_material_type {
    ORN_LAMBERTIAN = 0,
    ORN_METAL = 1,
    ORN_DIELECTRIC = 2,
    ORN_DIFFUSE_LIGHT = 3
};

#define ORN_NO_TEXTURE 0xFFFFFFFFu

/* Material, src/gpu_structs.zig:33-59 — 32 bytes. */
typedef struct orn_material {
    float albedo[3];
    uint32_t albedo_texture_index; /* ORN_NO_TEXTURE = plain albedo */
    float fuzz;
    float ior;
    uint32_t type; /* enum orn_material_type */
    uint32_t _padding;
} orn_material;

/* Camera, src/gpu_structs.zig:88-117 — 112 bytes. */
typedef struct orn_camera {
    float origin[3];
    float lens_radius;
    float lower_left_corner[3];
    uint32_t _padding0;
    float horizontal[3];
    uint32_t _padding1;
    float vertical[3];
    uint32_t _padding2;
    float u[3];
    uint32_t _padding3;
    float v[3];
    uint32_t _padding4;
    float w[3];
    uint32_t _padding5;
} orn_camera;

/* ConstantParams, src/gpu_structs.zig:61-86 — 144 bytes. */
typedef struct orn_constant_params {
    orn_camera camera;
    uint32_t depth;
    uint32_t width;
    uint32_t height;
    uint32_t flip_y;
    float inverted_gamma;
    float ray_cast_epsilon;
    uint32_t textures_count;
    float current_iteration;
} orn_constant_params;

/* Texture texel formats.  RGBA8 unorm is the LDR path of both backends
 * (src/hip_backend/buffers.zig:106, src/wgpu_backend/buffers.zig:305-319);
 * RGBA16F is the wgpu HDR path (rgba16_float). */
enum orn_texel_format { ORN_TEXEL_RGBA8 = 0, ORN_TEXEL_RGBA16F = 1 };

/* One texture (src/texture.zig:3-14).  Rows are `bytes_per_row` apart;
 * the data is copied at orn_create time. */
typedef struct orn_texture {
    const void* data;
    uint32_t width;
    uint32_t height;
    uint32_t bytes_per_row;
    uint32_t format; /* enum orn_texel_format */
} orn_texture;

/* The flat arrays that Bvh.init returns (src/bvh.zig:22-31), in the HIP
 * layout: `transforms` hold the TRANSPOSE of each zmath matrix
 * (row_major_transforms = true, src/bvh.zig:364-367), pairs
 * {inverse, forward} indexed transform_id*2 and transform_id*2+1. */
typedef struct orn_scene_blob {
    const orn_bvh_node* tlas_nodes;  uint32_t tlas_nodes_len;
    const orn_bvh_node* blas_nodes;  uint32_t blas_nodes_len;
    const float* normals;            uint32_t normals_len;        /* 4 floats each */
    const uint32_t* normal_indices;  uint32_t normal_indices_len;
    const float* uvs;                uint32_t uvs_len;            /* 2 floats each */
    const uint32_t* uv_indices;      uint32_t uv_indices_len;
    const float* transforms;         uint32_t transforms_len;     /* 16 floats each */
    const orn_material* materials;   uint32_t materials_len;
    const orn_texture* textures;     uint32_t textures_len;
    /* scene.textures.items.len (src/hip_backend/path_tracer.zig:165): the
     * value written to ConstantParams.textures_count. */
    uint32_t scene_textures_count;
} orn_scene_blob;

/* Which backend's semantics to reproduce where the two differ:
 * metal absorption (src/wgpu_backend/shaders/material.wgsl:22-27 vs
 * src/hip_backend/kernels/material.hip.h:58-64) and the texture address
 * mode (clamp-to-edge for wgpu's default sampler, wrap for HIP). */
enum orn_semantics { ORN_SEMANTICS_HIP = 0, ORN_SEMANTICS_WGSL = 1 };

/* Kernel variant used by orn_render. */
enum orn_kernel {
    ORN_KERNEL_MEGA = 0,        /* persistent warp-synchronous megakernel, a pixel's
                                   samples looped in one lane */
    ORN_KERNEL_WAVEFRONT = 1,   /* persistent wavefront: per-block path pools, ray and
                                   hit queues in shared memory, warps that traverse
                                   or shade (same bits as MEGA) */
    ORN_KERNEL_CACHED = 2,      /* learned radiance cache (orn_attach_cache) on the
                                   megakernel; biased, not bit-exact with the
                                   reference */
    ORN_KERNEL_CACHED_WAVEFRONT = 3  /* the same cached renderer on the persistent
                                        wavefront (the same estimator, path for
                                        path) */
};

/* State, src/state.zig:3-23 (resolution set by orn_set_resolution). */
typedef struct orn_state {
    uint32_t depth;           /* default 10   */
    uint32_t flip_y;          /* default 0    */
    float inverted_gamma;     /* default 1    */
    uint32_t iterations;      /* default 1    */
    float ray_cast_epsilon;   /* default 1e-3 */
    uint32_t semantics;       /* enum orn_semantics, default HIP */
    uint32_t kernel;          /* enum orn_kernel, default MEGA   */
    uint32_t spp_per_launch;  /* MEGA/WAVEFRONT: passes per launch, 0 = library
                                 chooses.  CACHED: sample streams per pixel in each
                                 frame's launch (0 = 1, at most 64), each with its
                                 own RNG state; more than one fills the GPU at low
                                 resolutions and adds samples atomically */
    uint32_t triangle_test;   /* enum orn_triangle_test, default MOLLER_TRUMBORE */
    uint32_t pixel_order;     /* enum orn_pixel_order, default COST */
    uint32_t sampler;         /* enum orn_sampler, default PCG */
} orn_state;

/* Random numbers of the cached kernel (no counterpart in the reference).
 * PCG: the reference's per-pixel stream (random.hip.h:14-30), as every other
 * kernel always uses.  SOBOL: each pixel's jitter, lens, first-bounce
 * direction and first light sample come from 2-D Owen-scrambled Sobol
 * points (Burley 2020), stratified over the pixel's samples since the last
 * camera change; the rest from the stream.  Unbiased; fewer samples to a
 * given error where pixel footprint and first-bounce visibility dominate. */
enum orn_sampler { ORN_SAMPLER_PCG = 0, ORN_SAMPLER_SOBOL = 1 };

/* Order in which a plain megakernel launch (ORN_KERNEL_MEGA, and
 * orn_render_f64) hands pixels to lanes (no counterpart in the reference,
 * whose grid is one thread per pixel).  Results are the same either way.
 * COST: from the second launch of a context on, tiles of 32 pixels go out
 * costliest first, by the traversal steps they took in the previous launch,
 * so that the launch does not end with a few lanes finishing expensive
 * pixels; RASTER: pixel index order.  The cached kernel (one sample per
 * pixel per launch, costs too noisy to predict) always uses raster order. */
enum orn_pixel_order { ORN_PIXEL_ORDER_COST = 0, ORN_PIXEL_ORDER_RASTER = 1 };

/* Ray/triangle test.  MOLLER_TRUMBORE is the reference's (bvh.hip.h:72-117),
 * the one every parity claim is made on.  WATERTIGHT (no counterpart in the
 * reference) is Woop, Benthin and Wald's watertight test: a ray through an
 * edge or vertex shared by two triangles of a mesh always hits one of them;
 * results can differ from the reference's at such edges. */
enum orn_triangle_test { ORN_TRIANGLE_MOLLER_TRUMBORE = 0, ORN_TRIANGLE_WATERTIGHT = 1 };

/* A ray for orn_trace_rays (src/hip_backend/kernels/ray.hip.h:7-18). */
typedef struct orn_ray {
    float origin[3];
    float direction[3];
} orn_ray;

/* The closest hit that Bvh::hit reports through its out-parameters
 * (src/hip_backend/kernels/bvh.hip.h:145-152).  Fields other than `hit`
 * keep the value 0 when hit == 0; tri_id and uv keep 0 for sphere hits. */
typedef struct orn_hit {
    uint32_t hit;
    float t;
    uint32_t material_index;
    uint32_t node_type;             /* ORN_NODE_SPHERE or ORN_NODE_MESH */
    uint32_t inverted_transform_id; /* identifies the instance          */
    uint32_t tri_id;                /* 3 * global triangle index        */
    float uv[2];
} orn_hit;

typedef struct orn_context orn_context;

/* ---- context life cycle ------------------------------------------------- */

/* PathTracer.init — src/hip_backend/path_tracer.zig:36-86.  Copies every
 * blob array to device `device` (-1 = the last device, as the HIP backend
 * picks, src/hip_backend/path_tracer.zig:40).  The caller keeps ownership
 * of the blob.  Validates every index in the blob. */
int orn_create(const orn_scene_blob* blob, int device, orn_context** out);

/* PathTracer.deinit — src/hip_backend/path_tracer.zig:88-101. */
int orn_destroy(orn_context* ctx);

/* State setters (src/state.zig:25-71).  Returns the defaults of
 * State.init (src/state.zig:13-23) before the first set. */
int orn_set_state(orn_context* ctx, const orn_state* state);
int orn_get_state(const orn_context* ctx, orn_state* out);

/* Assigning scene.camera / Camera.setLookAt / setAspectRatio sets the
 * camera dirty flag (src/camera.zig:66,70-80,98-113); the next render
 * restarts accumulation (src/hip_backend/path_tracer.zig:150-158). */
int orn_set_camera(orn_context* ctx, const orn_camera* camera);

/* PathTracer.setResolution — src/hip_backend/path_tracer.zig:103-109.
 * Drops the target buffers; the next render re-creates them and reseeds
 * every pixel's RNG state with its pixel index. */
int orn_set_resolution(orn_context* ctx, uint32_t width, uint32_t height);
int orn_get_resolution(const orn_context* ctx, uint32_t* width, uint32_t* height);

/* PathTracer.render — src/hip_backend/path_tracer.zig:121-133:
 * `iterations` sample passes then post-processing.  Asynchronous. */
int orn_render(orn_context* ctx);

/* Blocks until all work queued on the context has finished. */
int orn_synchronize(orn_context* ctx);

/* Launch parameters of ORN_KERNEL_WAVEFRONT (no counterpart in the
 * reference, whose launch shape is fixed by its grid).  Every configuration
 * renders the same bits; only the speed differs.  Counting renders
 * (orn_enable_counters) always run shape 0. */
typedef struct orn_wave_config {
    uint32_t shape;   /* block shape: 0 = 10 warps (9 traversing, 1 shading),
                         320 path slots, 2 blocks per SM (default);
                         1 = 8 warps (7 + 1), 256 slots, 3 blocks per SM;
                         2 = 12 warps (11 + 1), 384 slots, 2 blocks per SM;
                         3 = 11 warps (10 + 1), 352 slots, 2 blocks per SM */
    uint32_t fetch;   /* idle lanes a traversing warp gathers before it takes
                         new rays: 1..32 (default 4) */
    uint32_t steps;   /* node visits per traversal round: 32 (default) or 64 */
    uint32_t tuned;   /* out: 1 when chosen by orn_wave_tune */
} orn_wave_config;
int orn_wave_get_config(const orn_context* ctx, orn_wave_config* out);
/* ORN_ERR_INVALID_ARGUMENT outside the ranges above. */
int orn_wave_set_config(orn_context* ctx, orn_wave_config const* config);
/* Autotuner: renders one launch (the passes orn_render would put in one
 * launch, at most 8 and at most ~16 M samples) of the context's current
 * scene, camera, resolution and state with every candidate (4 shapes x
 * fetch 2/4/8 x steps 32/64) into scratch targets — the context's image,
 * RNG states and pixel order are not touched — and keeps the fastest.  With `cache_path`, a JSON file keyed by
 * device and workload (pixels, passes, depth, semantics, tree sizes) is
 * read first and updated after tuning.  `chosen` may be NULL.
 * Synchronous. */
int orn_wave_tune(orn_context* ctx, const char* cache_path, orn_wave_config* chosen);

/* PathTracer.getFrameBuffer — src/hip_backend/path_tracer.zig:111-119.
 * `dst` holds pixel_count RGBA float4 values (16 bytes each). */
int orn_get_framebuffer(orn_context* ctx, float* dst, size_t pixel_count);

/* The FP32 RGBA accumulation buffer (not exposed by the reference; used
 * for checkpointing and parity tests). */
int orn_get_accumulation(orn_context* ctx, float* dst, size_t pixel_count);

/* Checkpoint / resume of the progressive state: accumulation buffer,
 * per-pixel RNG states and State.current_iteration. */
int orn_get_progress(orn_context* ctx, float* accumulation, uint32_t* rng_state,
                     size_t pixel_count, float* current_iteration);
int orn_set_progress(orn_context* ctx, const float* accumulation,
                     const uint32_t* rng_state, size_t pixel_count,
                     float current_iteration);

/* The ConstantParams the next sample pass would use (after applying the
 * camera dirty flag), for parity checks.  Does not change the state. */
int orn_peek_constant_params(const orn_context* ctx, orn_constant_params* out);

/* ---- parity / debugging ------------------------------------------------- */

/* Bvh::hit on a list of rays — src/hip_backend/kernels/bvh.hip.h:145-276.
 * Writes one orn_hit per ray and, if `visits` is not NULL, the number of
 * traversal-loop iterations (node visits) each ray took.  Synchronous. */
int orn_trace_rays(orn_context* ctx, const orn_ray* rays, size_t count,
                   orn_hit* hits, uint32_t* visits);

/* Work counters of the last orn_render (zeros unless enabled with
 * orn_enable_counters): [0] samples, [1] extension rays, [2] node visits,
 * [3] internal-node visits, [4] sphere-leaf visits, [5] mesh-entry visits,
 * [6] triangle visits, [7] sphere hits, [8] mesh hits, [9] textured hits. */
#define ORN_COUNTER_COUNT 10
int orn_enable_counters(orn_context* ctx, int enable);
int orn_get_counters(orn_context* ctx, uint64_t* out, size_t count);

/* Device-side kernel time of the last orn_render in milliseconds (CUDA
 * events on the context stream). */
int orn_last_render_ms(orn_context* ctx, float* ms);

/* The context's CUDA stream (a cudaStream_t), so a caller can order its own
 * work and CUDA events with the library's. */
int orn_get_stream(const orn_context* ctx, void** stream);

/* Number of kernel launches the context has issued since creation. */
int orn_launch_count(const orn_context* ctx, uint64_t* launches);

/* ---- FP64 reference and error -------------------------------------------
 * The image-quality oracle of the time-to-relMSE measurements (an
 * extension: the reference has no error metric): `spp` passes from a
 * fresh start (RNG seeded with the pixel index, current_iteration 1..spp)
 * with the context's resolution, State and camera, accumulated in FP64 on
 * the GPU (the only FP64 in the renderer besides the error reduction);
 * writes the per-pixel FP64 mean RGBA (4 doubles per pixel) to host memory.
 * The context's own progressive target is not touched.  Synchronous. */
int orn_render_f64(orn_context* ctx, uint32_t spp, double* mean_rgba, size_t pixel_count);

/* relMSE of the context's current accumulation (per-pixel mean = sum / count)
 * against a reference mean (host, 4 doubles per pixel, e.g. from
 * orn_render_f64): mean over pixels and RGB of (x - r)^2 / (r^2 + 1e-2),
 * reduced in FP64 on the GPU.  Pixels whose estimate or reference is not
 * finite are left out of the mean and counted in *skipped_pixels (may be
 * NULL): the reference's own sampling occasionally yields a NaN sample,
 * which stays in that pixel's accumulation.  Synchronous. */
int orn_relmse(orn_context* ctx, const double* reference_mean_rgba, size_t pixel_count, double* relmse,
               uint64_t* skipped_pixels);

/* One-tile tensor-core GEMM self-test (no counterpart in the reference):
 * D[128 x N] = A[128 x K] · B[N x K]^T with 16-bit A, B (F16, or BF16 when
 * `bf16`), row-major host arrays, FP32 result.  K a multiple of 16 up to
 * 256, N a multiple of 16 from 16 to 128.  `mode` bit 1 stages both
 * operands MN-major instead of K-major (the layout of the weight-gradient
 * GEMMs); bit 0 exchanges the two operand-descriptor byte offsets (a
 * deliberately wrong encoding, to show the test can tell them apart).
 * Checks the tcgen05 encodings the radiance cache relies on.  Synchronous;
 * uses device 0. */
int orn_tc_selftest(uint32_t K, uint32_t N, int bf16, int mode, const uint16_t* A, const uint16_t* B,
                    float* D);

/* ---- rendering without allocation -----------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory while they render — a frame loop that must never call cudaMalloc
 * (an allocation can synchronise the device and stall the frame), or a host
 * that gives the renderer a fixed memory budget — this renders with the
 * wavefront kernels into device buffers the caller owns and allocates
 * nothing: its working memory is a fixed array inside the library, sized for
 * ORN_NOALLOC_MAX_PIXELS pixels (about 15 MiB, held on every GPU that loads
 * the library until the process exits).
 *
 * `ctx` supplies the scene (uploaded by orn_create) and the semantics;
 * `params` is the complete ConstantParams of the first pass (camera,
 * resolution, depth, flip_y, inverted_gamma, epsilon, textures_count and
 * current_iteration, as PathTracer.update() would upload it); `spp` passes
 * run with current_iteration, current_iteration + 1, …, then
 * post-processing.  `accumulation` (float4 per pixel) and `rng_state` (u32
 * per pixel) are device buffers read and updated in place (seed a fresh
 * render with rng_state[i] = i); `framebuffer` (float4 per pixel) is a
 * device buffer written.  Work is queued on `stream` (a cudaStream_t; NULL
 * is the default stream) and the call returns without waiting, so a frame
 * loop is never blocked by it.  A device-side limit hit by a render (a ray
 * needing more than 64 stack entries or 2^24 node visits) is recorded in
 * the context's error word; each call queues a copy of that word into
 * pinned host memory (allocated by orn_create) behind its work, and the next
 * call, once that copy has arrived, returns ORN_ERR_STACK_OVERFLOW /
 * ORN_ERR_TIMEOUT without queuing anything and clears the word.
 * orn_synchronize(ctx) reports it too (and waits).  Results are
 * bit-identical to orn_render with the same state.  The work runs on the
 * context's device; the caller's current device is restored on return.
 *
 * Returns ORN_ERR_INVALID_ARGUMENT when width * height exceeds
 * ORN_NOALLOC_MAX_PIXELS, depth exceeds ORN_NOALLOC_MAX_DEPTH (the call
 * queues spp * (depth + 1) + 2 kernel pairs, bounded by these limits) or a
 * pointer is NULL.  The first call on each device looks up the array's
 * device address (cudaGetSymbolAddress); make that first call before any
 * stream capture.  All calls share the one array, so calls whose GPU work
 * overlaps (other streams, other threads) race. */
#define ORN_NOALLOC_MAX_PIXELS 131072u
#define ORN_NOALLOC_MAX_DEPTH 64u
int orn_render_noalloc(const orn_context* ctx, const orn_constant_params* params, uint32_t spp,
                       float* accumulation, uint32_t* rng_state, float* framebuffer, void* stream);

/* ---- learned radiance cache ----------------------------------------------
 * No counterpart in the reference (an extension of the renderer).  A small
 * MLP, trained online on the renderer's own path samples, predicts the
 * radiance leaving a surface point; with state.kernel = ORN_KERNEL_CACHED,
 * orn_render ends regular paths at their cache vertex — the first rough
 * surface hit (lambertian, or metal with fuzz >= 0.25) from the second
 * vertex on — and adds throughput x surface colour x cache(vertex) instead
 * of tracing the rest of the path.  Emission, sky and smooth metal/glass
 * before that vertex are traced as usual, and the cached renderer samples
 * emissive mesh triangles directly (next-event estimation with multiple
 * importance sampling, also at the cache vertex), so the network carries
 * only the light arriving after the cache vertex's scatter.  The estimate
 * is biased by the cache's error; without the cache (every pixel a training
 * pixel, train_shift 0) it is unbiased.
 *
 * Network: inputs (ORN_CACHE_INPUTS floats, each in [0, 1]) = hit position
 * normalised to the scene bounds (3), (incoming direction + 1) / 2 (3),
 * (normal + 1) / 2 (3), roughness (1: lambertian 1, metal fuzz, dielectric
 * 0); 12-band sin/cos frequency encoding of every input (240 features) plus
 * the raw inputs, a constant 1 and 5 zeros (256 features); 5 hidden layers
 * of 64 with ReLU, no biases; 3 outputs (RGB).  Forward in FP16, backward in
 * BF16, FP32 accumulation (tensor cores), FP32 master weights and Adam.
 * Loss: relative L2, per channel (y - r)^2 / (y^2 + 0.01) with y held
 * constant in the denominator; samples whose target r[0] < 0 (or NaN) are
 * ignored.
 *
 * Parameters (ORN_CACHE_PARAM_COUNT FP32 values): the six weight matrices
 * in order, each row-major [outputs][inputs]: 64 x 256, 4 x (64 x 64), and
 * the output layer as 16 x 64 whose rows 3..15 are padding (kept zero).
 *
 * A cache belongs to one device.  Calls are not thread-safe, and a cache
 * attached to a context must not be used from another thread while that
 * context renders.  The host-buffer calls below are synchronous. */
#define ORN_CACHE_INPUTS 10u
#define ORN_CACHE_OUTPUTS 3u
#define ORN_CACHE_PARAM_COUNT 33792u

typedef struct orn_cache orn_cache;

typedef struct orn_cache_config {
    uint32_t batch;            /* samples per training step, multiple of 128 (default 16384) */
    uint32_t steps_per_frame;  /* training steps after each cached frame, at most 64 and at
                                  most the batches the frame's slots fill (default 4)         */
    uint32_t train_shift;      /* training samples per frame: pixels / 2^train_shift per
                                  sample stream (default 4).  Paths become training paths
                                  at their cache vertex, with the probability that fills
                                  those slots given the previous frame's vertex count; a
                                  training path runs to its end, the others stop at the
                                  vertex and query the cache.  0: every path trains (no
                                  queries: light sampling alone, unbiased)                    */
    float learning_rate;       /* Adam (default 1e-3) */
    float beta1;               /* default 0.9   */
    float beta2;               /* default 0.99  */
    float epsilon;             /* default 1e-8  */
    uint32_t reserved;         /* 0 */
} orn_cache_config;

int orn_cache_default_config(orn_cache_config* out);
/* Creates a cache on `device` (-1: the last device) with weights drawn from
 * `seed` (He-uniform); `config` may be NULL for the defaults. */
int orn_cache_create(int device, uint64_t seed, const orn_cache_config* config, orn_cache** out);
int orn_cache_destroy(orn_cache* cache);
int orn_cache_set_config(orn_cache* cache, const orn_cache_config* config);
int orn_cache_get_params(orn_cache* cache, float* dst, size_t count);
/* Replaces the weights and resets the Adam moments and step count. */
int orn_cache_set_params(orn_cache* cache, const float* src, size_t count);
/* outputs[n][3] = network(inputs[n][10]). */
int orn_cache_infer(orn_cache* cache, const float* inputs, size_t n, float* outputs);
/* Gradient of the summed loss over the n samples with respect to every
 * parameter (grads[ORN_CACHE_PARAM_COUNT]) and the summed loss; the weights
 * are not changed. */
int orn_cache_gradients(orn_cache* cache, const float* inputs, const float* targets, size_t n, float* grads,
                        float* loss);
/* One Adam step on the mean loss over the n samples (n <= 2^20); returns
 * the summed loss before the step. */
int orn_cache_train(orn_cache* cache, const float* inputs, const float* targets, size_t n, float* loss);
/* Adam steps taken and cached frames rendered so far; loss summed over the
 * last training step (synchronises with the cache's work). */
int orn_cache_stats(orn_cache* cache, uint64_t* steps, uint64_t* frames, float* last_loss);
const char* orn_cache_last_error(const orn_cache* cache);
/* Attaches `cache` (same device; NULL detaches) for ORN_KERNEL_CACHED.
 * Detach a cache (or destroy the context) before destroying the cache. */
int orn_attach_cache(orn_context* ctx, orn_cache* cache);

/* ---- batched rendering ------------------------------------------------------
 * No counterpart in the reference (which renders one scene per PathTracer).
 * A batch groups up to ORN_BATCH_MAX contexts of one device (any scenes,
 * resolutions and `iterations`) and renders one orn_render() of every one of
 * them in a single persistent launch: each context's accumulation, RNG
 * states, framebuffer and progress end exactly as orn_render would leave
 * them (bit for bit), and the contexts' own calls (orn_get_framebuffer, …)
 * are ordered after the batch's work.  The frame is captured as a CUDA graph
 * on first use and replayed while the contexts' sizes and the launch shape
 * stay the same.  All contexts must use the same semantics.
 * orn_last_render_ms of a context does not cover batched frames; use
 * orn_batch_last_render_ms. */
#define ORN_BATCH_MAX 64u
typedef struct orn_batch orn_batch;

typedef struct orn_batch_config {
    uint32_t block;            /* threads per block: 64, 128 or 192 (default 128) */
    uint32_t blocks_per_sm;    /* resident blocks per SM the grid is sized for (default 6) */
    uint32_t shade_threshold;  /* ready lanes a warp waits for before shading (default 8) */
    uint32_t tuned;            /* out: 1 when chosen by orn_batch_tune */
} orn_batch_config;

int orn_get_device(const orn_context* ctx, int* device);
int orn_batch_create(orn_context* const* contexts, uint32_t count, orn_batch** out);
int orn_batch_destroy(orn_batch* batch);
int orn_batch_render(orn_batch* batch);
int orn_batch_synchronize(orn_batch* batch);
int orn_batch_last_render_ms(orn_batch* batch, float* ms);
int orn_batch_get_config(const orn_batch* batch, orn_batch_config* out);
int orn_batch_set_config(orn_batch* batch, const orn_batch_config* config);
/* Autotuner: times the candidate launch shapes (block size x resident
 * blocks x shade threshold) on scratch targets — the contexts are not
 * touched — and keeps the fastest; with `cache_path`, a JSON file keyed by
 * device and workload (scene count, pixels, samples) is read first and
 * updated after tuning.  `chosen` may be NULL. */
int orn_batch_tune(orn_batch* batch, const char* cache_path, orn_batch_config* chosen);
const char* orn_batch_last_error(const orn_batch* batch);

/* ---- errors ------------------------------------------------------------- */
const char* orn_last_error(const orn_context* ctx);
const char* orn_status_string(int status);
uint32_t orn_abi_version(void);

/* ---- BVH builder (src/bvh.zig:33-78 Bvh.init) ----------------------------
 * Builds the flat TLAS/BLAS arrays from a scene description with the rules
 * of src/bvh.zig: leaf order spheres → mesh instances → meshes; random split
 * axis per node, sort by aabb.min[axis], median split; children appended
 * before the parent so each root is last; {inverse, forward} transform
 * pairs per TLAS leaf; material and texture indices assigned in order of
 * first use.  Matrices are zmath row-vector matrices (v' = v · M). */

typedef struct orn_material_desc {
    float albedo[3];
    uint32_t texture;   /* index into orn_scene_desc.textures or ORN_NO_TEXTURE */
    float fuzz;
    float ior;
    uint32_t type;      /* enum orn_material_type */
} orn_material_desc;

typedef struct orn_sphere_desc {       /* src/sphere.zig, src/scene.zig:124-134 */
    float transform[16];
    float aabb_min[3];
    float aabb_max[3];
    uint32_t material;
} orn_sphere_desc;

typedef struct orn_mesh_desc {         /* src/mesh.zig, src/scene.zig:263-316 */
    const float* vertices;       uint32_t vertices_len;       /* 4 floats each */
    const uint32_t* vertex_indices; uint32_t vertex_indices_len;
    const float* normals;        uint32_t normals_len;        /* 4 floats each */
    const uint32_t* normal_indices; uint32_t normal_indices_len;
    const float* uvs;            uint32_t uvs_len;            /* 2 floats each */
    const uint32_t* uv_indices;  uint32_t uv_indices_len;
    float transform[16];
    float aabb_min[3];
    float aabb_max[3];
    uint32_t material;
} orn_mesh_desc;

typedef struct orn_mesh_instance_desc { /* src/mesh_instance.zig */
    uint32_t mesh;
    float transform[16];
    float aabb_min[3];
    float aabb_max[3];
    uint32_t material;
} orn_mesh_instance_desc;

typedef struct orn_scene_desc {
    const orn_sphere_desc* spheres;               uint32_t spheres_len;
    const orn_mesh_desc* meshes;                  uint32_t meshes_len;
    const orn_mesh_instance_desc* mesh_instances; uint32_t mesh_instances_len;
    const orn_material_desc* materials;           uint32_t materials_len;
    const orn_texture* textures;                  uint32_t textures_len;
    uint64_t seed;                /* split-axis PRNG seed (bvh.zig uses 1244) */
    uint32_t row_major_transforms;/* 1 = HIP layout (transposed), 0 = wgpu   */
    uint32_t builder;             /* enum orn_bvh_builder, default REFERENCE */
} orn_scene_desc;

/* Tree builder.  REFERENCE follows bvh.zig's rules (random split axis,
 * median of aabb.min): the tree every parity claim is made on.  SAH is a
 * non-parity mode with no counterpart in the reference: binned
 * surface-area-heuristic splits over the same node format (one primitive
 * per leaf, 2n-1 nodes, children before parents), so the kernels run it
 * unchanged with fewer node visits; images agree with the reference's in
 * expectation, not bit for bit (equal-distance hits may resolve to another
 * primitive and visit counts differ). */
enum orn_bvh_builder { ORN_BVH_REFERENCE = 0, ORN_BVH_SAH = 1, ORN_BVH_LBVH = 2 };
/* LBVH (no counterpart in the reference): the BLASes are built on the GPU
 * (device 0 or the current device) as linear BVHs — Morton-code sort and
 * Karras' hierarchy, far faster to build than the CPU builders, fewer visits
 * than the reference's tree, more than SAH — and the TLAS with SAH on the
 * CPU.  Needs a CUDA device; non-parity like SAH. */

typedef struct orn_bvh orn_bvh;

/* Bvh.init — src/bvh.zig:33-78.  Returns ORN_ERR_EMPTY_SCENE for a scene
 * without shapes or a mesh without triangles (the reference panics). */
int orn_bvh_build(const orn_scene_desc* desc, orn_bvh** out);
/* Fills `blob` with pointers into the builder's arrays (valid until
 * orn_bvh_free).  Texture pointers refer to the caller's desc textures. */
int orn_bvh_get_blob(const orn_bvh* bvh, orn_scene_blob* blob);
/* Bvh.deinit — src/bvh.zig:80-90. */
int orn_bvh_free(orn_bvh* bvh);

/* Parity / debugging (host only): points of the cached kernel's Sobol
 * sampler (orn_state.sampler = ORN_SAMPLER_SOBOL) — `count` 2-D points of
 * use `pair` (0 pixel jitter, 1 lens, 2 first-bounce direction, 3 first
 * light sample) for the pixel with index `pixel`, sample indices `first` ..
 * first + count - 1, exactly as the kernel computes them (the same inline
 * code); `out` receives 2 * count floats in [0, 1). */
int orn_qmc_points(uint32_t pixel, uint32_t pair, uint32_t first, uint32_t count, float* out);

/* ---- JPEG textures -------------------------------------------------------
 * The example app loads its textures with zstbi (stb_image) as 4-component
 * RGBA8 images flipped vertically on load (glfw_example/examples.zig:492-503
 * loadTexture(..., 4); glfw_example/app_no_interop.zig:17
 * setFlipVerticallyOnLoad(true)) and passes them to Scene.createTexture
 * (src/scene.zig:339-351).  These calls replace that loader for JPEG files:
 * sequential Huffman JPEG (SOF0/SOF1, 8-bit, 1 or 3 components, any 1..4
 * sampling factors, restart intervals); progressive, arithmetic-coded,
 * lossless, 12-bit and CMYK streams return ORN_ERR_UNSUPPORTED, corrupt
 * ones ORN_ERR_BAD_IMAGE.  Entropy decoding runs on the host; dequantisation,
 * the inverse DCT (exact, FP32), chroma replication, YCbCr->RGB and the flip
 * run on the GPU.  Outputs may differ from stb_image's by a few levels (its
 * integer IDCT and chroma filter are not reproduced). */

/* Width, height and component count from the frame header (host only). */
int orn_jpeg_info(const void* data, size_t len, uint32_t* width, uint32_t* height, uint32_t* components);
/* Decodes into `rgba` (width * height * 4 bytes, row-major, alpha 255) on
 * `device` (-1: the current device); flip_y = 1 puts the last image row
 * first, like stb_image's flip-on-load.  Synchronous. */
int orn_jpeg_decode(const void* data, size_t len, int device, uint32_t flip_y, uint8_t* rgba, size_t rgba_len);
/* Parity / debugging (host only): the quantised coefficients of one
 * component as entropy-decoded, [blocks_h][blocks_w][64] in natural
 * (row-major) order, the planes padded to whole MCUs, and the component's
 * quantisation table (64 values, natural order).  `out` may be null to query
 * the plane size; any of blocks_w, blocks_h and quant may be null. */
int orn_jpeg_coefficients(const void* data, size_t len, uint32_t component, int16_t* out, size_t out_len,
                          uint32_t* blocks_w, uint32_t* blocks_h, uint16_t* quant);
/* Message of the calling thread's last failed orn_jpeg_* call. */
const char* orn_jpeg_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* ORNAMENT_CUDA_H */
