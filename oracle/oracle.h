/*
 * oracle.h - C entry points of the CPU oracle (liboracle.so).
 *
 * TEST INFRASTRUCTURE ONLY: the reference restatement the CUDA library is compared with.
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg load it.
 * It consumes the same rt_scene_desc as the library (include/radiantium.h).
 */
#ifndef RT_ORACLE_H
#define RT_ORACLE_H
#include "../include/radiantium.h"
#ifdef __cplusplus
extern "C" {
#endif

/* builds the restated Scene; NULL on error (message in err) */
void* or_scene_create(const rt_scene_desc* scene, char* err, int errlen);
void or_scene_destroy(void* s);

/* Scene.Intersect / Scene.Intersect(ray) over a batch (threads <= 0: all cores);
 * stats (nullable) receives the summed node, primitive and instance visits */
int or_trace_closest(void* s, const rt_ray* rays, int64_t n, rt_hit* hits, int threads, rt_stats* stats);
int or_trace_any(void* s, const rt_ray* rays, int64_t n, uint8_t* occluded, int threads, rt_stats* stats);

/* BlockBasedRenderer over the crop; out_rgb in ColorBuffer layout of the crop.
 * stats (nullable) receives the summed counters. */
int or_render(void* s, const rt_render_params* p, float* out_rgb, int threads, rt_stats* stats);

/* AdjointParticleRenderer: particles [first, first + count) -> the whole film
 * (ColorBuffer layout).  Each thread splats a fixed share into its own film;
 * the films are summed in thread order. */
int or_render_particles(void* s, const rt_render_params* p, int64_t first, int64_t count, float* out_rgb,
                        int threads, rt_stats* stats);

/* camera connections of particles [first, first + count): n[i] of particle
 * first + i; the first max_per at pix[i * max_per + k] (x * ScreenY + y, -1
 * beyond n[i]) and rgb[(i * max_per + k) * 3 + c] */
int or_particle_splats(void* s, const rt_render_params* p, int64_t first, int64_t count, int max_per,
                       int32_t* n, int32_t* pix, float* rgb, int threads);

/* per-sample radiance (no averaging): out[((x*h + y) * spp + k) * 3 + c] */
int or_render_samples(void* s, const rt_render_params* p, float* out, int threads);

/* PerspectiveCamera.SampleRay for n screen positions (2 floats each) */
int or_camera_rays(void* s, const float* screen_pos, int64_t n, rt_ray* out);

/* flattened reference BVH: which = -1 top level, k >= 0 instanced prototype k.
 * bounds: 6 floats per node, idx: PrimitivesIndex/SecondChildIndex,
 * count: PrimitiveCount, axis: Axis, prim_order: primitive id per ordered slot.
 * Call with NULL arrays to query sizes. */
int or_bvh(void* s, int which, int64_t* node_count, int64_t* prim_count,
           float* bounds, int32_t* idx, int32_t* count, int32_t* axis, int32_t* prim_order);

/* Scene.Lights in order: kind 0 = DiffuseAreaLight (prim = id of the
 * aggregate primitive that carries it, le = its radiance), 1 = infinite light
 * (prim -1, le 0).  Call with NULL arrays to query the count. */
int or_scene_lights(void* s, int64_t* count, int32_t* kind, int32_t* prim, float* le);

/* deterministic math and RNG known-answer hooks */
int or_detmath(int fn, const float* a, const float* b, float* out, int64_t n);
int or_philox_raw(const uint32_t* ctr, const uint32_t* key, uint32_t* out);
int or_philox(uint64_t seed, uint32_t x, uint32_t y, uint32_t s, int count, uint32_t* out);

#ifdef __cplusplus
}
#endif
#endif
