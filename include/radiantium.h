/*
 * radiantium.h - C ABI of the GB300 path-tracing library (libradiantium_gb300.so).
 *
 * The library replaces the CPU render loop of Radiantium (ksgfk/Radiantium,
 * C#/.NET 6): BlockBasedRenderer -> PathTracer / VolumetricPathTracer ->
 * Scene -> Bvh -> shapes / materials / lights / media.  A host binding (the
 * C# P/Invoke shim, or the Python ctypes module in radiantium_gb300/native.py)
 * walks the reference's built Scene once, flattens it into rt_scene_desc and
 * hands it to rt_upload_scene; rt_render then produces the RenderTarget.
 *
 * Conventions
 *  - Every entry point returns RT_OK (0) or a negative RT_ERR_* status; the
 *    message is available from rt_last_error(ctx).  Nothing aborts or throws
 *    across the ABI.
 *  - Host pointers passed in are caller-owned and only read during the call.
 *    Device memory is owned by the context and freed by rt_destroy.
 *  - Calls on one context are serialised by the caller (one context owns one
 *    CUDA stream); different contexts may be used from different threads.
 *  - Matrices are 16 floats in System.Numerics.Matrix4x4 field order
 *    (M11, M12, ..., M44), used with row vectors: p' = p * M.
 *  - Images/textures use the reference ColorBuffer layout: element (x, y, c)
 *    at ((x * height) + y) * 3 + c  (Radiantium.Core/ColorBuffer.cs:25-36).
 *  - Random numbers: both this library and its CPU oracle draw from
 *    Philox4x32-10 (Salmon et al., SC'11) keyed by the render seed and
 *    counted by (pixel x, pixel y, sample index, block); the stream is
 *    consumed in the same order as the reference consumes System.Random.
 */
#ifndef RADIANTIUM_H
#define RADIANTIUM_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RT_ABI_VERSION 2

/* ---- status codes ---------------------------------------------------- */
#define RT_OK 0
#define RT_ERR_INVALID_ARG (-1)
#define RT_ERR_OOM (-2)
#define RT_ERR_CUDA (-3)
#define RT_ERR_ITER_CAP (-4)   /* a device loop hit its iteration cap */
#define RT_ERR_CANCELLED (-5)
#define RT_ERR_NO_SCENE (-6)
#define RT_ERR_UNSUPPORTED (-7)
#define RT_ERR_STACK (-8)      /* BVH traversal stack (64 entries, Bvh.cs:16) overflowed */
#define RT_ERR_BOUNDS (-9)     /* debug-bounds builds only: a device index left its buffer */

/* ---- enums (values mirror the reference enums) -------------------------- */
#define RT_WRAP_CLAMP 0        /* TextureSampler.cs:5-9 WrapMode */
#define RT_WRAP_REPEAT 1
#define RT_FILTER_NEAREST 0    /* TextureSampler.cs:11-15 FilterMode */
#define RT_FILTER_LINEAR 1

#define RT_MAT_DIFFUSE 0        /* Materials/Diffuse.cs */
#define RT_MAT_ROUGH_METAL 1    /* Materials/RoughMetal.cs */
#define RT_MAT_ROUGH_GLASS 2    /* Materials/RoughGlass.cs */
#define RT_MAT_ROUGH_PLASTIC 3  /* Materials/RoughPlastic.cs */
#define RT_MAT_PERFECT_MIRROR 4 /* Materials/PerfectMirror.cs */
#define RT_MAT_PERFECT_GLASS 5  /* Materials/PerfectGlass.cs */

#define RT_DIST_BECKMANN 0      /* Bxdf/Microfacet.cs:8-12 */
#define RT_DIST_GGX 1

#define RT_GROUP_MESH 0           /* every triangle of a mesh becomes a GeometricPrimitive */
#define RT_GROUP_SPHERE 1         /* Shapes/Sphere.cs */
#define RT_GROUP_INSTANCE 2       /* InstancedPrimitive (Primitive.cs:144-189) */
#define RT_GROUP_INFINITE_LIGHT 3 /* InfiniteAreaLight (Lights/InfiniteAreaLight.cs) */

#define RT_INTEGRATOR_PATH 0      /* Integrators/PathTracer.cs */
#define RT_INTEGRATOR_VOL_PATH 1  /* Integrators/VolumetricPathTracer.cs */
#define RT_INTEGRATOR_PARTICLE 2  /* Integrators/AdjointParticleIntegrator.cs ("adjoint_particle") */
#define RT_METHOD_BXDF 0          /* PathTracer.cs:12-17 PathSampleMethod */
#define RT_METHOD_NEE 1
#define RT_METHOD_MIS 2
#define RT_STRATEGY_UNIFORM 0     /* PathTracer.cs:19-23 LightSampleStrategy */
#define RT_STRATEGY_ALL 1

#define RT_HIT_TIE 1u             /* a candidate with exactly the same t was rejected (Bvh.cs:199) */

/* ---- scene description ---------------------------------------------------- */

/* Texture2D: ConstColorTexture2D is a 1x1 texture; ImageTexture2D carries its
 * ColorBuffer.  Textures/ConstColorTexture2D.cs, Textures/ImageTexture2D.cs,
 * TextureSampler.cs:28-72. */
typedef struct rt_texture_desc {
    int32_t width, height;
    int32_t wrap, filter;
    const float* data;        /* width * height * 3 floats, ColorBuffer layout */
} rt_texture_desc;

/* Material parameters, one record for all material plugins.
 * Texture fields are indices into the texture table (-1 where unused).
 * RendererBuilder.cs:93-169 lists the defaults the host binding applies. */
typedef struct rt_material_desc {
    int32_t type;             /* RT_MAT_* */
    int32_t dist;             /* RT_DIST_* (rough_*) */
    int32_t two_sided;        /* is_two_side */
    int32_t tex_r;            /* diffuse kd, plastic/glass/mirror r */
    int32_t tex_t;            /* glass t */
    int32_t tex_roughness;
    int32_t tex_anisotropic;
    float eta_a, eta_b;       /* glass etaA/etaB, plastic etaI/etaT */
    float kd, ks;             /* plastic lobe weights */
    float eta[3], k[3];       /* rough_metal conductor eta, k */
} rt_material_desc;

/* Mediums/Homogeneous.cs:15-21 (sigma values before `scale`). */
typedef struct rt_medium_desc {
    float sigma_a[3];
    float sigma_s[3];
    float g;
    float scale;
} rt_medium_desc;

/* A triangle mesh whose positions are already in the space of its owner
 * (world space for scene entities, instance space for instanced prototypes),
 * exactly as TriangleMesh stores them (Shapes/Triangle.cs:15-51). */
typedef struct rt_mesh_desc {
    int32_t vertex_count, triangle_count;
    const float* positions;   /* vertex_count * 3 */
    const float* normals;     /* nullable: vertex_count * 3 */
    const float* uvs;         /* nullable: vertex_count * 2 */
    const int32_t* indices;   /* triangle_count * 3 */
} rt_mesh_desc;

/* Shapes/Sphere.cs: center already transformed by the shape builder
 * (RendererBuilder.cs:52-57). */
typedef struct rt_sphere_desc {
    float center[3];
    float radius;
    float model_to_world[16];
    float world_to_model[16];
} rt_sphere_desc;

/* One scene entity contribution, in the order RendererBuilder.Build visits
 * them (RendererBuilder.cs:942-1000): per entity its spheres, then its mesh
 * triangles, then its instances; an entity with neither material nor medium
 * but with a light is an infinite light.  The library expands groups into the
 * reference's primitive list and light list in that order. */
typedef struct rt_group_desc {
    int32_t kind;             /* RT_GROUP_* */
    int32_t ref;              /* mesh, sphere, blas or texture (env map) index */
    int32_t material;         /* -1: no material (medium boundary) */
    int32_t medium_inside;    /* -1: none */
    int32_t medium_outside;   /* -1: none */
    int32_t emissive;         /* 1: one DiffuseAreaLight per primitive */
    float le[3];              /* diffuse_area "le" */
    float model_to_world[16]; /* INSTANCE, INFINITE_LIGHT */
    float world_to_model[16]; /* INSTANCE, INFINITE_LIGHT (Matrix4x4.Invert of the above) */
} rt_group_desc;

/* PerspectiveCamera (Camera.cs:81-241); the matrices are the ones Update()
 * derives (Camera.cs:128-180): camera->clip is perspective*translate*scale,
 * clip->camera its Matrix4x4.Invert, world->camera the Invert of
 * camera->world.  The light tracer (SampleWi, Camera.cs:221-241) reads the
 * camera->clip and world->camera matrices; the camera rays read the other two. */
typedef struct rt_camera_desc {
    int32_t width, height;    /* ScreenX, ScreenY */
    float near_z, far_z;
    float clip_to_camera[16];
    float camera_to_world[16];
    float camera_to_clip[16];
    float world_to_camera[16];
} rt_camera_desc;

typedef struct rt_scene_desc {
    int32_t abi_version;              /* RT_ABI_VERSION */
    int32_t mesh_count;
    const rt_mesh_desc* meshes;
    int32_t sphere_count;
    const rt_sphere_desc* spheres;
    int32_t texture_count;
    const rt_texture_desc* textures;
    int32_t material_count;
    const rt_material_desc* materials;
    int32_t medium_count;
    const rt_medium_desc* media;
    /* instanced prototypes ("instanced" section, RendererBuilder.cs:895-921):
     * blas_ranges[2*i], blas_ranges[2*i+1] = first group, group count in
     * blas_groups (kinds MESH / SPHERE only; other fields ignored). */
    int32_t blas_group_count;
    const rt_group_desc* blas_groups;
    int32_t blas_count;
    const int32_t* blas_ranges;
    int32_t group_count;
    const rt_group_desc* groups;
    int32_t global_medium;            /* camera "medium" (-1: none) */
    rt_camera_desc camera;
    int32_t bvh_max_prims;            /* accel "max_prim" (Bvh.cs:89, default 1) */
} rt_scene_desc;

/* ---- rays / hits (parity interface of Scene.Intersect / IsOccluded) ---- */
typedef struct rt_ray {
    float o[3];
    float d[3];
    float min_t, max_t;       /* Ray3F.MinT / MaxT; InvD = 1/d is derived */
} rt_ray;

typedef struct rt_hit {
    float t;                  /* Intersection.T (world distance for instances) */
    float u, v;               /* SurfacePoint barycentrics of the hit triangle */
    int32_t prim;             /* index in the reference primitive list, -1: miss */
    int32_t sub;              /* triangle index inside the instanced prototype, else -1 */
    uint32_t flags;           /* RT_HIT_TIE */
} rt_hit;

/* ---- render parameters ------------------------------------------------- */
typedef struct rt_render_params {
    int32_t integrator;       /* RT_INTEGRATOR_* */
    int32_t method;           /* RT_METHOD_* (path) */
    int32_t strategy;         /* RT_STRATEGY_* */
    int32_t max_depth;        /* -1: unbounded (RendererBuilder.cs:56-72 defaults) */
    int32_t min_depth;        /* default 3 */
    float rr_threshold;       /* default 0.99 */
    int32_t spp;              /* renderer "spp" */
    int32_t sample_begin;     /* index of the first sample (progressive resume) */
    uint64_t seed;
    int32_t x0, y0;           /* crop origin; width/height 0 = whole film */
    int32_t width, height;
} rt_render_params;

typedef struct rt_stats {
    uint64_t samples;
    uint64_t rays_closest;    /* Scene.Intersect calls */
    uint64_t rays_shadow;     /* Scene.IsOccluded calls */
    uint64_t node_visits;     /* LinearBVHNode boxes tested, reference traversal order */
    uint64_t prim_tests;      /* primitive intersection tests */
    uint64_t instance_visits; /* instanced-prototype traversals */
    uint64_t invalid_samples; /* Color3F.IsValid == false, zeroed (BlockBasedRenderer.cs:141-145) */
    uint64_t kernel_launches; /* kernels this library launched for the call */
    uint64_t render_launches; /* of which path-tracing launches */
    double render_kernel_ms;  /* summed duration of the path-tracing launches (CUDA events on their stream):
                                 the megakernel, or the wavefront traversal kernel */
    double shade_kernel_ms;   /* wavefront shading kernel (0 for the megakernel) */
    uint64_t h2d_bytes;       /* bytes the call copied from host memory to the device: wavefront job
                                 tables and queue counters, rays, dL/dI (kernel arguments not counted) */
} rt_stats;

/* ---- entry points ------------------------------------------------------ */

/* Library version of this header, for binding checks. */
int rt_abi_version(void);

/* Creates a context on CUDA device `device` (one stream, no scene).
 * Replaces constructing BlockBasedRenderer (Renderers/BlockBasedRenderer.cs:36-54). */
int rt_create(int device, void** out_ctx);

/* Frees every device buffer of the context. */
void rt_destroy(void* ctx);

/* Message of the last failed call on this context ("" if none). */
const char* rt_last_error(const void* ctx);

/* Flattens the scene, builds the SAH BVHs of the reference
 * (Accelerators/Bvh.cs:89-124, RendererBuilder.cs:895-921,1002) and uploads
 * everything.  Replaces RendererBuilder.Build's accelerator/scene steps. */
int rt_upload_scene(void* ctx, const rt_scene_desc* scene);

/* Closest hit of n rays from host memory into host memory.
 * Scene.Intersect(ray, out inct) (Scene.cs:32-35 -> Bvh.cs:174-232). */
int rt_trace_closest(void* ctx, const rt_ray* rays, int64_t n, rt_hit* hits);

/* Any hit: occluded[i] = 1 if ray i hits anything in [min_t, max_t].
 * Scene.Intersect(ray) (Scene.cs:27-30 -> Bvh.cs:126-172). */
int rt_trace_any(void* ctx, const rt_ray* rays, int64_t n, uint8_t* occluded);

/* Device-pointer variants of the two calls above on a caller stream
 * (cudaStream_t passed as void*; NULL = the context stream). */
int rt_trace_closest_device(void* ctx, const rt_ray* d_rays, int64_t n, rt_hit* d_hits, void* stream);
int rt_trace_any_device(void* ctx, const rt_ray* d_rays, int64_t n, uint8_t* d_occluded, void* stream);

/* Renders params->spp samples per pixel of the crop and writes the averaged
 * film (ColorBuffer layout over the crop) to host memory `out_rgb`.
 * BlockBasedRenderer.RenderTask (BlockBasedRenderer.cs:107-179) with
 * MonteCarloIntegrator.Li (PathTracer.cs:402-411, VolumetricPathTracer.cs:28-119). */
int rt_render(void* ctx, const rt_render_params* params, float* out_rgb);

/* Same, film written to device memory on `stream` (no host copies). */
int rt_render_device(void* ctx, const rt_render_params* params, float* d_out_rgb, void* stream);

/* Size of the fixed device scratch behind rt_render_device_noalloc. */
#define RT_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)

/* rt_render_device without any device allocation.  No counterpart in the
 * reference: it exists for hosts that cannot let a library allocate device
 * memory while they render (an engine whose pool allocator owns the whole
 * GPU, a frame loop that cannot take cudaFree's device-wide synchronisation).
 * It always runs the megakernel renderer, whatever rt_set_renderer chose, out
 * of one static device array of RT_NOALLOC_SCRATCH_BYTES.  The first call on
 * a device sets that array up (looks up its device address; under lazy module
 * loading, the CUDA 12.2+ default, this is also when the runtime loads its
 * module and reserves the array - with CUDA_MODULE_LOADING=EAGER it is
 * reserved when the context is created), so make one call before any stream
 * capture or allocation-free phase begins.  Every call waits for its stream
 * to drain before it returns (it reads the render's status word).
 * The film sums and one sample plane must fit:
 * 512 + 2 * 12 * width * height <= RT_NOALLOC_SCRATCH_BYTES (crop size; a
 * 1024 x 1024 crop fits), else RT_ERR_INVALID_ARG.  Counters are not
 * gathered.  Every context on a device shares that one array, so calls that
 * overlap in time on one device race and must be serialised by the caller.
 * The film is the same as rt_render_device's, bit for bit. */
int rt_render_device_noalloc(void* ctx, const rt_render_params* params, float* d_out_rgb, void* stream);

/* ---- gradients (no counterpart in the reference) ----------------------------
 * The reference renders only; these entry points differentiate its `path`
 * integrator with MIS (PathTracer.Mis, Integrators/PathTracer.cs:192-270) with
 * respect to material parameters, for inverse rendering on top of the same
 * scenes.  The parameters are the texels of one albedo texture (the `r`
 * texture of diffuse and rough_plastic materials) and the GGX / Beckmann
 * alpha = roughness^2 of chosen rough_plastic / rough_metal materials. */
#define RT_ADJ_MAX_ALPHA 1024
typedef struct rt_adjoint_desc {
    int32_t albedo_texture;          /* texture index, or -1 for no albedo parameters */
    int32_t alpha_count;             /* 0 .. RT_ADJ_MAX_ALPHA */
    const int32_t* alpha_materials;  /* material indices whose alpha is a parameter */
} rt_adjoint_desc;

/* The film the gradients refer to (same as rt_render). */
int rt_adjoint_forward(void* ctx, const rt_render_params* params, float* out_rgb);

/* Gradient of sum over the crop of dL_dimage * I with respect to the
 * parameters, I the film of `params` (crop layout like rt_render's output):
 * path replay with detached sampling, the same random numbers as the
 * forward film.  grad_albedo: the albedo texture's width * height * 3 floats
 * in its ColorBuffer layout; grad_alpha: alpha_count floats, d/d alpha in the
 * order of alpha_materials.  Gradients are float sums of atomic adds, so the
 * last bits vary between runs. */
int rt_adjoint_backward(void* ctx, const rt_render_params* params, const rt_adjoint_desc* desc,
                        const float* dL_dimage, float* grad_albedo, float* grad_alpha);

/* Replaces the texels (width * height * 3 floats, ColorBuffer layout) of one
 * texture of the uploaded scene without rebuilding anything else: an albedo
 * map, or the 1x1 roughness texture that sets a material's alpha.  Textures
 * of infinite lights are rejected (their sampling tables would go stale). */
int rt_update_texture(void* ctx, int texture, const float* texels);

/* Counters of the last render / trace call (Stopwatch/Logger counterpart). */
int rt_get_stats(void* ctx, rt_stats* out);

/* Enables per-ray counters (node visits, primitive tests) in later calls:
 * the counting build of the kernels, used for the roofline's algorithmic bytes. */
int rt_set_counting(void* ctx, int enabled);

/* Selects the render pipeline: RT_RENDERER_AUTO (wavefront where it applies,
 * i.e. the `path` integrator with either light strategy and `vol_path` with
 * the Uniform one, megakernel otherwise; vol_path and the light tracer drive their
 * wavefront loop as a CUDA graph), RT_RENDERER_MEGAKERNEL, RT_RENDERER_WAVEFRONT (bounce loop
 * driven by the host, with per-phase timings in rt_stats) or
 * RT_RENDERER_WAVEFRONT_GRAPH (bounce loop as one CUDA graph launch per
 * round of samples).  All produce identical camera-path films (light-tracer
 * films differ only in the order of their float splat additions); this is
 * the GpuWavefrontRenderer "renderer" option. */
#define RT_RENDERER_AUTO 0
#define RT_RENDERER_MEGAKERNEL 1
#define RT_RENDERER_WAVEFRONT 2
#define RT_RENDERER_WAVEFRONT_GRAPH 3
int rt_set_renderer(void* ctx, int mode);

/* ---- traversal mode (no counterpart in the reference) ------------------------
 * RT_TRAVERSAL_EXACT (default): the reference's binary tree, visited in the
 * order Bvh.Intersect visits it (Accelerators/Bvh.cs:126-232); hits, films
 * and traversal counters equal the reference's restatement bit for bit.
 * RT_TRAVERSAL_WIDE: an opt-in fast traversal for the wavefront renderers,
 * batches and the ray-batch calls (the megakernel always runs the exact one):
 * the same trees collapsed 8-wide with quantised child boxes read as six
 * 16-byte loads per node, children visited near to far.  It finds the same
 * closest primitive except where two candidates have exactly the same t
 * (flagged RT_HIT_TIE by either traversal) or where the reference's own slab
 * test misses a box at rounding scale; node-visit counters count wide nodes.
 * A scene whose wide trees could overflow the 64-entry stack (or whose binary
 * trees are deeper than 65 levels) renders with the exact traversal;
 * rt_get_traversal reports what the next call will use. */
#define RT_TRAVERSAL_EXACT 0
#define RT_TRAVERSAL_WIDE 1
int rt_set_traversal(void* ctx, int mode);
int rt_get_traversal(void* ctx, int* effective);

/* ---- environment-light sampling (no counterpart in the reference) ----------
 * How an infinite light's Distribution2D (Distribution2D.cs:9-61) picks a
 * texel in SampleLi and SampleEmit (Lights/InfiniteAreaLight.cs:92-133).
 * RT_LIGHT_SAMPLING_CDF (default): the reference's binary search over the
 * marginal and conditional CDFs (Distribution1D.cs:51-85); films equal the
 * reference's restatement bit for bit.
 * RT_LIGHT_SAMPLING_ALIAS: an opt-in O(1) alias-table pick from the same two
 * uniforms.  Over the renderer's uniforms (k / 2^24) it draws every texel for
 * exactly as many values of k as the CDF search does, so both modes sample
 * the same texel pmf and report the same pdf; only which uniform maps to
 * which texel differs, so films agree statistically, not bit for bit.  A light
 * whose table is not a non-decreasing CDF (negative or non-finite texels)
 * keeps the search.  The mode belongs to the context's scene: it applies to
 * every render of that scene, in a batch too, and may be set before or after
 * rt_upload_scene (not while a call on the context is running). */
#define RT_LIGHT_SAMPLING_CDF 0
#define RT_LIGHT_SAMPLING_ALIAS 1
int rt_set_light_sampling(void* ctx, int mode);
int rt_get_light_sampling(void* ctx, int* mode);

/* One render of a batch: the context holding its uploaded scene (may be the
 * batch context itself), its parameters and its host output film (crop,
 * ColorBuffer layout, width * height * 3 floats). */
typedef struct rt_batch_item {
    void* scene_ctx;
    rt_render_params params;
    float* out_rgb;
} rt_batch_item;

/* Renders n (1..256) scenes as one wavefront: their paths share one pool of
 * path slots and every trace / shade launch, so small scenes do not leave
 * the GPU idle and the launch overhead is paid once per bounce for the whole
 * batch.  Each film equals what rt_render gives for the same item, bit for
 * bit.  All items must use the same integrator (`path`, either light
 * strategy, or `vol_path` with the Uniform one), and all scene contexts must
 * be on the batch context's device.
 * The bounce loop is driven from the host, or runs as a CUDA graph when
 * rt_set_renderer selected RT_RENDERER_WAVEFRONT_GRAPH.  No counterpart in
 * the reference, which renders one scene per process
 * (Radiantium.Cli/Program.cs). */
int rt_render_batch(void* ctx, const rt_batch_item* items, int n);

/* Same, every out_rgb a device pointer written on `stream` (NULL = the
 * context stream); returns once the films are written. */
int rt_render_batch_device(void* ctx, const rt_batch_item* items, int n, void* stream);

/* ---- light tracing ----------------------------------------------------------
 * The "adjoint_particle" renderer + integrator (Renderers/AdjointParticleRenderer.cs,
 * Integrators/AdjointParticleIntegrator.cs): particles leave the lights
 * (Light.SampleEmit), and every surface vertex is connected to the camera
 * (PerspectiveCamera.SampleWi) and splatted into the film when visible.  The
 * film is then scaled by ScreenX * ScreenY / particle_count
 * (AdjointParticleRenderer.cs:156-164) and each pixel (x, y) gains
 * CameraTraceLight of the camera ray through screen position (x, y)
 * (AdjointParticleRenderer.cs:166-172).
 *
 * Particle i (0 <= i < 2^63) draws its random numbers from the Philox
 * stream with counter (i mod 2^32, i / 2^32, RT_PARTICLE_STREAM) and key
 * params->seed, so a range of particles renders the same on any number of
 * calls or devices; films of disjoint ranges combine as their
 * particle-count-weighted mean.  Splats are added with float atomics, so the
 * film's low bits depend on their order (as under the reference's lock).
 * A splat whose screen position is NaN (the reference's ColorBuffer throws
 * there) is dropped. */
#define RT_PARTICLE_STREAM 0x80000000u

/* Traces particles [first_particle, first_particle + particle_count) and
 * writes the whole film (ScreenX * ScreenY * 3 floats, ColorBuffer layout) to
 * host memory.  params: integrator RT_INTEGRATOR_PARTICLE, max_depth,
 * min_depth, rr_threshold ("max_depth", "min_depth", "rr_threshold",
 * RendererBuilder.cs:73-79), seed; the crop fields must be 0 (whole film).
 * particle_count >= 1 ("particle_count", RendererBuilder.cs:36-41). */
int rt_render_particles(void* ctx, const rt_render_params* params, int64_t first_particle,
                        int64_t particle_count, float* out_rgb);

/* Same, film written to device memory on `stream` (NULL = the context stream). */
int rt_render_particles_device(void* ctx, const rt_render_params* params, int64_t first_particle,
                               int64_t particle_count, float* d_out_rgb, void* stream);

/* Settings chosen by rt_autotune. */
typedef struct rt_tune_result {
    int32_t capacity;      /* path slots in flight */
    int32_t refill;        /* idle lanes of a trace warp before it fetches new rays */
    int32_t renderer;      /* RT_RENDERER_WAVEFRONT or RT_RENDERER_WAVEFRONT_GRAPH */
    float ms;              /* probe time of the chosen settings */
    float ms_default;      /* probe time of the defaults (2 Mi slots, refill 8, host-driven loop) */
} rt_tune_result;

/* Renders the batch (rt_render_batch, films into the items' outputs) under
 * each combination of the wavefront settings that do not change a film -
 * path slots in flight (2 Mi, 1 Mi, 512 Ki), trace-warp refill threshold
 * (4, 8, 16 idle lanes) and host- or graph-driven bounce loop - and keeps
 * the fastest on this context for later renders and batches (the loop
 * driver applies under RT_RENDERER_AUTO).  Probe with a representative,
 * short batch (a few spp).  No counterpart in the reference. */
int rt_autotune(void* ctx, const rt_batch_item* items, int n, rt_tune_result* out);

/* Requests cancellation of a running render (Renderer.Stop, BlockBasedRenderer.cs:85-88). */
int rt_cancel(void* ctx);

#ifdef __cplusplus
}
#endif

#endif /* RADIANTIUM_H */
