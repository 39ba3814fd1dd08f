/* orn_headless.c — a headless frame loop over libornament_cuda's C ABI, in
 * plain C: what the reference's example app does each frame
 * (glfw_example/app_no_interop.zig:163-184: update(), PathTracer.render(),
 * getFrameBuffer(), show) with the window replaced by a file, on the fixed
 * part of its sphere scene (glfw_example/examples.zig:94-175: the ground
 * sphere and three unit spheres — glass, a planet texture loaded like
 * loadTexture(name, 4) with setFlipVerticallyOnLoad(true), metal).  The
 * Zig backend glue makes the same calls in the same order.
 *
 *   orn_headless [-w W] [-h H] [-frames N] [-iterations K] [-depth D]
 *                [-gamma G] [-texture planet.jpg] [-move-at F] [-out PREFIX]
 *
 * At frame F (if given) the eye orbits the target a little, as the app's
 * A/D keys do (app_no_interop.zig:140-158), which restarts accumulation.
 * Writes PREFIX.fb (the last framebuffer, float32 RGBA) and PREFIX.cam (the
 * orn_camera of each camera set, in order); prints one line per frame.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "ornament_cuda.h"

static orn_context* g_ctx = NULL;

static void check(int status, const char* what) {
    if (status == ORN_OK) return;
    const char* msg = g_ctx ? orn_last_error(g_ctx) : orn_status_string(status);
    if (!msg || !*msg) msg = orn_status_string(status);
    fprintf(stderr, "orn_headless: %s failed: %s (%d)\n", what, msg, status);
    exit(1);
}

static void cross3(const float a[3], const float b[3], float out[3]) {
    out[0] = a[1] * b[2] - a[2] * b[1];
    out[1] = a[2] * b[0] - a[0] * b[2];
    out[2] = a[0] * b[1] - a[1] * b[0];
}

static void normalize3(float v[3]) {
    const float len = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int i = 0; i < 3; ++i) v[i] /= len;
}

/* Camera.init (src/camera.zig:24-68) into the kernel layout. */
static orn_camera make_camera(const float from[3], const float at[3], const float vup[3], float aspect, float vfov,
                              float aperture, float focus) {
    orn_camera c;
    memset(&c, 0, sizeof(c));
    const float theta = vfov * 3.14159265358979f / 180.0f;
    const float vh = 2.0f * tanf(theta / 2.0f), vw = aspect * vh;
    float w[3] = {from[0] - at[0], from[1] - at[1], from[2] - at[2]}, u[3], v[3];
    normalize3(w);
    cross3(vup, w, u);
    normalize3(u);
    cross3(w, u, v);
    for (int i = 0; i < 3; ++i) {
        c.origin[i] = from[i];
        c.horizontal[i] = focus * vw * u[i];
        c.vertical[i] = focus * vh * v[i];
        c.lower_left_corner[i] = from[i] - c.horizontal[i] / 2.0f - c.vertical[i] / 2.0f - focus * w[i];
        c.u[i] = u[i];
        c.v[i] = v[i];
        c.w[i] = w[i];
    }
    c.lens_radius = aperture / 2.0f;
    return c;
}

/* Scene.createSphere (src/scene.zig:124-134): scaling(r) * translation(c). */
static orn_sphere_desc make_sphere(float x, float y, float z, float r, uint32_t material) {
    orn_sphere_desc s;
    memset(&s, 0, sizeof(s));
    s.transform[0] = r;
    s.transform[5] = r;
    s.transform[10] = r;
    s.transform[12] = x;
    s.transform[13] = y;
    s.transform[14] = z;
    s.transform[15] = 1.0f;
    const float c[3] = {x, y, z};
    for (int i = 0; i < 3; ++i) {
        s.aabb_min[i] = c[i] - r;
        s.aabb_max[i] = c[i] + r;
    }
    s.material = material;
    return s;
}

static unsigned char* read_file(const char* path, size_t* len) {
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    unsigned char* buf = (unsigned char*)malloc(n > 0 ? (size_t)n : 1);
    if (buf && n > 0 && fread(buf, 1, (size_t)n, f) != (size_t)n) {
        free(buf);
        buf = NULL;
    }
    fclose(f);
    *len = n > 0 ? (size_t)n : 0;
    return buf;
}

static double now_ms(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec * 1e3 + ts.tv_nsec / 1e6;
}

int main(int argc, char** argv) {
    uint32_t width = 320, height = 180, frames = 8, iterations = 4, depth = 10;
    float gamma = 2.2f;
    const char* texture_path = NULL;
    const char* out = "orn_headless";
    int move_at = -1;
    for (int i = 1; i < argc; ++i) {
        const char* a = argv[i];
        const char* v = i + 1 < argc ? argv[i + 1] : NULL;
        if (!v) {
            fprintf(stderr, "orn_headless: %s needs a value\n", a);
            return 2;
        }
        if (!strcmp(a, "-w")) width = (uint32_t)atoi(v);
        else if (!strcmp(a, "-h")) height = (uint32_t)atoi(v);
        else if (!strcmp(a, "-frames")) frames = (uint32_t)atoi(v);
        else if (!strcmp(a, "-iterations")) iterations = (uint32_t)atoi(v);
        else if (!strcmp(a, "-depth")) depth = (uint32_t)atoi(v);
        else if (!strcmp(a, "-gamma")) gamma = (float)atof(v);
        else if (!strcmp(a, "-texture")) texture_path = v;
        else if (!strcmp(a, "-move-at")) move_at = atoi(v);
        else if (!strcmp(a, "-out")) out = v;
        else {
            fprintf(stderr, "orn_headless: unknown option %s\n", a);
            return 2;
        }
        ++i;
    }
    if (width == 0 || height == 0 || frames == 0) {
        fprintf(stderr, "orn_headless: width, height and frames must be positive\n");
        return 2;
    }

    /* materials in creation order: ground, glass, left sphere, metal */
    orn_material_desc mats[4];
    memset(mats, 0, sizeof(mats));
    mats[0].albedo[0] = mats[0].albedo[1] = mats[0].albedo[2] = 0.5f;
    mats[0].texture = ORN_NO_TEXTURE;
    mats[0].type = ORN_LAMBERTIAN;
    mats[1].texture = ORN_NO_TEXTURE;
    mats[1].ior = 1.5f;
    mats[1].type = ORN_DIELECTRIC;
    mats[2].albedo[0] = 0.4f;
    mats[2].albedo[1] = 0.2f;
    mats[2].albedo[2] = 0.1f;
    mats[2].texture = ORN_NO_TEXTURE;
    mats[2].type = ORN_LAMBERTIAN;
    mats[3].albedo[0] = 0.7f;
    mats[3].albedo[1] = 0.6f;
    mats[3].albedo[2] = 0.5f;
    mats[3].texture = ORN_NO_TEXTURE;
    mats[3].type = ORN_METAL;

    orn_texture tex;
    memset(&tex, 0, sizeof(tex));
    uint8_t* texels = NULL;
    uint32_t textures = 0;
    if (texture_path) {
        size_t len = 0;
        unsigned char* jpg = read_file(texture_path, &len);
        if (!jpg) {
            fprintf(stderr, "orn_headless: cannot read %s\n", texture_path);
            return 1;
        }
        uint32_t tw = 0, th = 0, tc = 0;
        check(orn_jpeg_info(jpg, len, &tw, &th, &tc), "orn_jpeg_info");
        texels = (uint8_t*)malloc((size_t)tw * th * 4);
        if (!texels) return 1;
        check(orn_jpeg_decode(jpg, len, -1, 1, texels, (size_t)tw * th * 4), "orn_jpeg_decode");
        free(jpg);
        tex.data = texels;
        tex.width = tw;
        tex.height = th;
        tex.bytes_per_row = tw * 4;
        tex.format = ORN_TEXEL_RGBA8;
        textures = 1;
        mats[2].albedo[0] = 1.0f;   /* a textured material's albedo is unused */
        mats[2].albedo[1] = 0.0f;
        mats[2].albedo[2] = 1.0f;
        mats[2].texture = 0;
    }
    orn_sphere_desc spheres[4] = {
        make_sphere(0.0f, -1000.0f, 0.0f, 1000.0f, 0),
        make_sphere(0.0f, 1.0f, 0.0f, 1.0f, 1),
        make_sphere(-4.0f, 1.0f, 0.0f, 1.0f, 2),
        make_sphere(4.0f, 1.0f, 0.0f, 1.0f, 3),
    };
    orn_scene_desc desc;
    memset(&desc, 0, sizeof(desc));
    desc.spheres = spheres;
    desc.spheres_len = 4;
    desc.materials = mats;
    desc.materials_len = 4;
    desc.textures = textures ? &tex : NULL;
    desc.textures_len = textures;
    desc.seed = 1244;                /* Bvh.init's split-axis seed (src/bvh.zig:12) */
    desc.row_major_transforms = 1;   /* the HIP backend's layout */
    desc.builder = ORN_BVH_REFERENCE;

    /* HipPathTracer.init (src/hip_backend/path_tracer.zig:36-86) */
    orn_bvh* bvh = NULL;
    check(orn_bvh_build(&desc, &bvh), "orn_bvh_build");
    orn_scene_blob blob;
    check(orn_bvh_get_blob(bvh, &blob), "orn_bvh_get_blob");
    check(orn_create(&blob, -1, &g_ctx), "orn_create");

    orn_state state;
    check(orn_get_state(g_ctx, &state), "orn_get_state");
    state.depth = depth;
    state.inverted_gamma = 1.0f / gamma;
    state.iterations = iterations;
    check(orn_set_state(g_ctx, &state), "orn_set_state");
    check(orn_set_resolution(g_ctx, width, height), "orn_set_resolution");

    const float vup[3] = {0.0f, 1.0f, 0.0f}, target[3] = {0.0f, 0.0f, 0.0f};
    float eye[3] = {13.0f, 2.0f, 3.0f};
    const float aspect = (float)width / (float)height;
    char path[4096];
    snprintf(path, sizeof(path), "%s.cam", out);
    FILE* cams = fopen(path, "wb");
    if (!cams) {
        fprintf(stderr, "orn_headless: cannot write %s\n", path);
        return 1;
    }
    orn_camera cam = make_camera(eye, target, vup, aspect, 20.0f, 0.1f, 10.0f);
    check(orn_set_camera(g_ctx, &cam), "orn_set_camera");
    fwrite(&cam, sizeof(cam), 1, cams);

    const size_t pixels = (size_t)width * height;
    float* fb = (float*)malloc(pixels * 4 * sizeof(float));
    if (!fb) return 1;
    for (uint32_t f = 0; f < frames; ++f) {
        if ((int)f == move_at) {   /* update(): the eye orbits the target */
            const float a = 0.05f, x = eye[0], z = eye[2];
            eye[0] = x * cosf(a) - z * sinf(a);
            eye[2] = x * sinf(a) + z * cosf(a);
            cam = make_camera(eye, target, vup, aspect, 20.0f, 0.1f, 10.0f);
            check(orn_set_camera(g_ctx, &cam), "orn_set_camera");
            fwrite(&cam, sizeof(cam), 1, cams);
        }
        const double t0 = now_ms();
        check(orn_render(g_ctx), "orn_render");
        check(orn_get_framebuffer(g_ctx, fb, pixels), "orn_get_framebuffer");
        float gpu_ms = 0.0f;
        check(orn_last_render_ms(g_ctx, &gpu_ms), "orn_last_render_ms");
        printf("frame %u: %.3f ms wall, %.3f ms device, %.1f Msamples/s\n", f, now_ms() - t0, gpu_ms,
               (double)pixels * iterations / (gpu_ms * 1e3));
    }
    fclose(cams);
    snprintf(path, sizeof(path), "%s.fb", out);
    FILE* fo = fopen(path, "wb");
    if (!fo || fwrite(fb, sizeof(float) * 4, pixels, fo) != pixels) {
        fprintf(stderr, "orn_headless: cannot write %s\n", path);
        return 1;
    }
    fclose(fo);

    /* deinit (src/hip_backend/path_tracer.zig:88-101) */
    check(orn_destroy(g_ctx), "orn_destroy");
    g_ctx = NULL;
    check(orn_bvh_free(bvh), "orn_bvh_free");
    free(fb);
    free(texels);
    return 0;
}
