/*
 * abi_driver.c - a plain C11 program that drives the library through
 * include/radiantium.h alone (no Python, no C++): what a native host binding
 * does.  It builds a small room (floor, back wall, ceiling light quad) with its
 * own camera matrices, renders it with the path integrator and the light
 * tracer, traces a ray batch, reads the counters and checks the error paths.
 *
 *   abi_driver            full run on CUDA device 0
 *   abi_driver --no-gpu   only the calls that need no device
 *
 * Prints "abi ok" and exits 0 when every check holds.
 */
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "radiantium.h"

#define W 48
#define H 36

static int failures = 0;
#define CHECK(cond, ...)                                           \
    do {                                                           \
        if (!(cond)) {                                             \
            fprintf(stderr, "check failed (%s:%d): ", __FILE__, __LINE__); \
            fprintf(stderr, __VA_ARGS__);                          \
            fprintf(stderr, "\n");                                 \
            failures++;                                            \
        }                                                          \
    } while (0)

/* row-vector 4x4 matrices (System.Numerics.Matrix4x4 layout, M11..M44) */
static void mat_mul(const float a[16], const float b[16], float r[16]) {
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            float acc = 0.0f;
            for (int k = 0; k < 4; k++) acc += a[4 * i + k] * b[4 * k + j];
            r[4 * i + j] = acc;
        }
}

/* general inverse by Gauss-Jordan elimination with partial pivoting (double) */
static int mat_inv(const float m[16], float r[16]) {
    double a[4][8];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 8; j++) a[i][j] = j < 4 ? m[4 * i + j] : (j - 4 == i ? 1.0 : 0.0);
    for (int c = 0; c < 4; c++) {
        int piv = c;
        for (int i = c + 1; i < 4; i++)
            if (fabs(a[i][c]) > fabs(a[piv][c])) piv = i;
        if (fabs(a[piv][c]) < 1e-12) return 0;
        for (int j = 0; j < 8; j++) { double t = a[c][j]; a[c][j] = a[piv][j]; a[piv][j] = t; }
        const double d = a[c][c];
        for (int j = 0; j < 8; j++) a[c][j] /= d;
        for (int i = 0; i < 4; i++)
            if (i != c) {
                const double f = a[i][c];
                for (int j = 0; j < 8; j++) a[i][j] -= f * a[c][j];
            }
    }
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r[4 * i + j] = (float)a[i][j + 4];
    return 1;
}

static void normalize3(float v[3]) {
    const float l = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= l; v[1] /= l; v[2] /= l;
}
static void cross3(const float a[3], const float b[3], float r[3]) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}

/* camera->world of a left-handed look-at (rows: left, up, forward, origin) */
static void look_at(const float o[3], const float t[3], const float up_in[3], float m[16]) {
    float d[3] = {t[0] - o[0], t[1] - o[1], t[2] - o[2]}, up[3] = {up_in[0], up_in[1], up_in[2]}, left[3], u[3];
    normalize3(d);
    normalize3(up);
    cross3(up, d, left);
    normalize3(left);
    cross3(d, left, u);
    normalize3(u);
    const float r[16] = {left[0], left[1], left[2], 0, u[0], u[1], u[2], 0, d[0], d[1], d[2], 0, o[0], o[1], o[2], 1};
    memcpy(m, r, sizeof(r));
}

/* the four matrices of PerspectiveCamera.Update for fov (degrees), near, far */
static int make_camera(float fov, float nz, float fz, const float c2w[16], rt_camera_desc* cam) {
    const float aspect = (float)W / (float)H, recip = 1.0f / (fz - nz);
    const float cot = 1.0f / tanf(fov / 2.0f * (3.14159265f / 180.0f));
    const float persp[16] = {cot, 0, 0, 0, 0, cot, 0, 0, 0, 0, fz * recip, 1, 0, 0, -nz * fz * recip, 0};
    const float scale[16] = {-0.5f, 0, 0, 0, 0, -0.5f * aspect, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    const float trans[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, -1, -1.0f / aspect, 0, 1};
    float pt[16];
    mat_mul(persp, trans, pt);
    mat_mul(pt, scale, cam->camera_to_clip);
    memcpy(cam->camera_to_world, c2w, 16 * sizeof(float));
    cam->width = W;
    cam->height = H;
    cam->near_z = nz;
    cam->far_z = fz;
    return mat_inv(cam->camera_to_clip, cam->clip_to_camera) && mat_inv(c2w, cam->world_to_camera);
}

static double film_mean(const float* f, int n, int* finite) {
    double s = 0.0;
    *finite = 1;
    for (int i = 0; i < n; i++) {
        if (!isfinite(f[i])) *finite = 0;
        s += f[i];
    }
    return s / n;
}

int main(int argc, char** argv) {
    const int gpu = !(argc > 1 && strcmp(argv[1], "--no-gpu") == 0);
    CHECK(rt_abi_version() == RT_ABI_VERSION, "ABI version %d, header %d", rt_abi_version(), RT_ABI_VERSION);
    CHECK(rt_create(0, NULL) == RT_ERR_INVALID_ARG, "rt_create(NULL)");
    CHECK(rt_cancel(NULL) != RT_OK, "rt_cancel(NULL)");
    void* ctx = NULL;
    int rc = rt_create(0, &ctx);
    if (!gpu) {
        /* without a device the context cannot be made: an error code, never a crash */
        if (rc == RT_OK) rt_destroy(ctx);
        else CHECK(ctx == NULL, "context set on failure");
        if (failures) return 1;
        printf("abi ok (no gpu): rt_create -> %d\n", rc);
        return 0;
    }
    CHECK(rc == RT_OK && ctx, "rt_create: %d", rc);
    if (rc != RT_OK) return 1;

    float* film = (float*)malloc((size_t)W * H * 3 * sizeof(float));
    rt_render_params p;
    memset(&p, 0, sizeof(p));
    p.integrator = RT_INTEGRATOR_PATH;
    p.method = RT_METHOD_MIS;
    p.strategy = RT_STRATEGY_UNIFORM;
    p.max_depth = 5;
    p.min_depth = 3;
    p.rr_threshold = 0.99f;
    p.spp = 16;
    p.seed = 7;
    CHECK(rt_render(ctx, &p, film) == RT_ERR_NO_SCENE, "render before upload");
    CHECK(rt_render(ctx, NULL, film) == RT_ERR_INVALID_ARG || rt_render(ctx, NULL, film) == RT_ERR_NO_SCENE,
          "render with null params");

    /* the room: floor, back wall (inward-facing quads), ceiling light facing down */
    const float pos[] = {-1, -1, -1, -1, -1, 1, 1, -1, 1, 1, -1, -1,         /* floor */
                         -1, -1, -1, 1, -1, -1, 1, 1, -1, -1, 1, -1,         /* back wall */
                         -0.3f, 0.99f, -0.3f, 0.3f, 0.99f, -0.3f, 0.3f, 0.99f, 0.3f, -0.3f, 0.99f, 0.3f};
    const int32_t room_idx[] = {0, 1, 2, 0, 2, 3, 4, 5, 6, 4, 6, 7};
    const int32_t light_idx[] = {0, 1, 2, 0, 2, 3};
    rt_mesh_desc meshes[2];
    memset(meshes, 0, sizeof(meshes));
    meshes[0].vertex_count = 8; meshes[0].triangle_count = 4; meshes[0].positions = pos; meshes[0].indices = room_idx;
    meshes[1].vertex_count = 4; meshes[1].triangle_count = 2; meshes[1].positions = pos + 24; meshes[1].indices = light_idx;
    const float white[3] = {0.7f, 0.7f, 0.7f}, grey[3] = {0.5f, 0.5f, 0.5f};
    rt_texture_desc tex[2];
    memset(tex, 0, sizeof(tex));
    tex[0].width = tex[0].height = 1; tex[0].data = white;
    tex[1].width = tex[1].height = 1; tex[1].data = grey;
    rt_material_desc mats[2];
    memset(mats, 0, sizeof(mats));
    for (int i = 0; i < 2; i++) {
        mats[i].type = RT_MAT_DIFFUSE;
        mats[i].tex_r = i; mats[i].tex_t = mats[i].tex_roughness = mats[i].tex_anisotropic = -1;
    }
    rt_group_desc groups[2];
    memset(groups, 0, sizeof(groups));
    for (int i = 0; i < 2; i++) {
        groups[i].kind = RT_GROUP_MESH; groups[i].ref = i; groups[i].material = i;
        groups[i].medium_inside = groups[i].medium_outside = -1;
    }
    groups[1].emissive = 1;
    groups[1].le[0] = groups[1].le[1] = groups[1].le[2] = 12.0f;
    rt_scene_desc d;
    memset(&d, 0, sizeof(d));
    d.abi_version = RT_ABI_VERSION;
    d.mesh_count = 2; d.meshes = meshes;
    d.texture_count = 2; d.textures = tex;
    d.material_count = 2; d.materials = mats;
    d.group_count = 2; d.groups = groups;
    d.global_medium = -1;
    d.bvh_max_prims = 1;
    const float eye[3] = {0, 0, 3.5f}, at[3] = {0, 0, 0}, up[3] = {0, 1, 0};
    float c2w[16];
    look_at(eye, at, up, c2w);
    CHECK(make_camera(50.0f, 0.001f, 1000.0f, c2w, &d.camera), "camera matrices");
    rc = rt_upload_scene(ctx, &d);
    CHECK(rc == RT_OK, "rt_upload_scene: %d %s", rc, rt_last_error(ctx));

    /* path integrator, then the counters of that call */
    rc = rt_render(ctx, &p, film);
    CHECK(rc == RT_OK, "rt_render: %d %s", rc, rt_last_error(ctx));
    int finite = 0;
    double mean = film_mean(film, W * H * 3, &finite);
    CHECK(finite && mean > 0.01 && mean < 10.0, "path film mean %g finite %d", mean, finite);
    rt_stats st;
    CHECK(rt_get_stats(ctx, &st) == RT_OK && st.samples == (uint64_t)W * H * 16, "stats samples %llu",
          (unsigned long long)st.samples);

    /* a ray batch: down to the floor, and one that leaves the room */
    rt_ray rays[2];
    memset(rays, 0, sizeof(rays));
    float dn[3] = {0.0f, -1.0f, -3.5f};                  /* towards the floor's centre */
    normalize3(dn);
    memcpy(rays[0].o, eye, sizeof(eye)); memcpy(rays[0].d, dn, sizeof(dn));
    rays[1].o[2] = 3.5f; rays[1].d[2] = 1.0f;
    for (int i = 0; i < 2; i++) { rays[i].min_t = 1e-4f; rays[i].max_t = FLT_MAX; }
    rt_hit hits[2];
    uint8_t occ[2];
    CHECK(rt_trace_closest(ctx, rays, 2, hits) == RT_OK, "rt_trace_closest");
    CHECK(hits[0].prim >= 0 && hits[0].t > 0 && hits[1].prim == -1, "hits %d %g %d", hits[0].prim, hits[0].t,
          hits[1].prim);
    CHECK(rt_trace_any(ctx, rays, 2, occ) == RT_OK && occ[0] == 1 && occ[1] == 0, "occlusion %d %d", occ[0], occ[1]);

    /* the light tracer over the whole film */
    p.integrator = RT_INTEGRATOR_PARTICLE;
    p.max_depth = -1;
    rc = rt_render_particles(ctx, &p, 0, 200000, film);
    CHECK(rc == RT_OK, "rt_render_particles: %d %s", rc, rt_last_error(ctx));
    mean = film_mean(film, W * H * 3, &finite);
    CHECK(finite && mean > 0.01 && mean < 10.0, "particle film mean %g finite %d", mean, finite);
    p.x0 = 1;
    CHECK(rt_render_particles(ctx, &p, 0, 1000, film) == RT_ERR_INVALID_ARG, "particles with a crop");
    CHECK(strlen(rt_last_error(ctx)) > 0, "an error message after a failed call");
    p.x0 = 0;
    CHECK(rt_render_particles(ctx, &p, 0, 0, film) == RT_ERR_INVALID_ARG, "zero particles");

    rt_destroy(ctx);
    free(film);
    if (failures) return 1;
    printf("abi ok\n");
    return 0;
}
