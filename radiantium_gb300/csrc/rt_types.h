/*
 * rt_types.h - device-resident scene layout of the GB300 path tracer.
 *
 * Plain-old-data records shared by the host builder (rt_host.cpp, rt_bvh.cpp)
 * and the kernels (rt_kernels.cu).  All arrays live in HBM and are read with
 * 16-byte loads:
 *
 *  - BVH nodes: the reference's binary SAH tree (Accelerators/Bvh.cs) stored
 *    as interior nodes only, each holding BOTH children's boxes (64 bytes =
 *    4 x float4).  A traversal step therefore tests two boxes from one node
 *    fetch; leaves are referenced from their parent and never fetched.
 *  - primitive slots: 48 bytes (3 x float4) per primitive in BVH leaf order,
 *    with the triangle's first vertex and both edges pre-subtracted (the
 *    Moller-Trumbore operands, bit-identical to computing them per test).
 *  - everything the shading stages need is indexed by the reference's
 *    primitive id.
 */
#ifndef RT_TYPES_H
#define RT_TYPES_H

#include <stdint.h>

#define RT_KIND_TRI 0
#define RT_KIND_SPHERE 1
#define RT_KIND_INSTANCE 2
#define RT_KIND_SHIFT 29
#define RT_REF_MASK ((1u << RT_KIND_SHIFT) - 1u)

#define RT_STACK_SIZE 64            /* Bvh.StackSize (Accelerators/Bvh.cs:16) */

/* device status bits (rt_status) */
#define RT_STATUS_STACK 1u
#define RT_STATUS_ITER 2u
#define RT_STATUS_BADREF 4u
#define RT_STATUS_BOUNDS 8u         /* debug-bounds builds: an index left its buffer, the access was skipped */
#define RT_STATUS_TRAV 16u          /* a traversal reached RT_TRAVERSAL_CAP steps */
#define RT_STATUS_WALK 32u          /* a null-boundary walk reached RT_WALK_CAP segments */
#define RT_STATUS_WFITER 64u        /* a graph-driven wavefront round reached WF_ITER_CAP iterations */

#define RT_LIGHT_AREA_TRI 0
#define RT_LIGHT_AREA_SPHERE 1
#define RT_LIGHT_INFINITE 2

/* one BVH (top level or an instanced prototype) */
struct RtBvh {
    float root_min[3];
    float root_max[3];
    int32_t root_ref;   /* >= 0: interior node (absolute), < 0: ~first slot of a root leaf, INT32_MIN: empty */
    int32_t wide_root;  /* the same tree collapsed 8-wide: >= 0 wide node, < 0 as root_ref */
};

/* a wide node (the opt-in fast traversal; rtb::WideNode): float4 w0..w5
 *   w0 = (p.x, p.y, p.z, uint e.x | e.y << 8 | e.z << 16 | nchild << 24)
 *   w1 = (qlo.x of children 0-3, 4-7, qhi.x of 0-3, 4-7)   one byte per child
 *   w2, w3: the same for y and z
 *   w4 = (int ref 0..3), w5 = (int ref 4..7)   refs as in the binary tree
 * the quantised child box of axis a is [p + qlo * s, p + qhi * s], s = 2^(e - 127) */
#define RT_WIDE_F4 6

/* an interior node: float4 n0..n3
 *   n0 = (L.min.x, L.min.y, L.min.z, L.max.x)
 *   n1 = (L.max.y, L.max.z, R.min.x, R.min.y)
 *   n2 = (R.min.z, R.max.x, R.max.y, R.max.z)
 *   n3 = (int Lref, int Rref, int axis, 0)   refs: >= 0 node, < 0 ~first slot
 * a primitive slot: float4 s0..s2
 *   s0 = (Pa.xyz, int prim_id)            prim_id: index in the owner's primitive list
 *   s1 = (e1.xyz, int kind << 29 | ref)   ref: global triangle / sphere / instance index
 *   s2 = (e2.xyz, int leaf_count)         leaf_count valid on a leaf's first slot
 */

struct RtPrim {          /* shading data of a top-level primitive, by prim id */
    int32_t kind, ref;   /* RT_KIND_*, global triangle / sphere / instance index */
    int32_t material, light;
    int32_t med_in, med_out;
    int32_t pad0, pad1;
};

struct RtTri {           /* global triangle: vertex indices into the global vertex arrays */
    int32_t v0, v1, v2;
    int32_t flags;       /* bit0 normals, bit1 uvs */
};

struct RtSphere {
    float center[3];
    float radius;
    float w2m[12];       /* rows of WorldToModel (3x3 part + translation) */
};

struct RtInstance {
    float m2w[12];       /* ModelToWorld rows 1..4, first three columns */
    float w2m[12];
    int32_t blas;
    int32_t pad[3];
};

struct RtTexture {
    int32_t width, height, wrap, filter;
    int64_t offset;      /* float offset into the texel pool (ColorBuffer layout) */
};

struct RtMaterial {
    int32_t type, dist, two_sided;
    int32_t tex_r, tex_t, tex_rough, tex_anis;
    float eta_a, eta_b, kd, ks;
    float eta[3], k[3];
};

struct RtMedium {
    float sig_a[3], sig_s[3], sig_t[3];
    float g;
};

struct RtLight {
    int32_t kind;        /* RT_LIGHT_* */
    int32_t ref;         /* triangle / sphere index, or texture index (infinite) */
    float le[3];
    float area;          /* Shape.SurfaceArea at construction */
    /* infinite light */
    float m2w[12], w2m[12];
    float world_center[3];
    float world_radius;
    int32_t dist;        /* index of its Distribution2D */
    int32_t pad;
};

/* Distribution2D (Distribution2D.cs): nv conditional Distribution1D of nu
 * entries plus the marginal; cdfs have n + 1 entries. */
struct RtDist2D {
    int32_t nu, nv;
    int64_t cond_pdf;    /* float offsets into the distribution pool */
    int64_t cond_cdf;
    int64_t cond_int;
    int64_t marg_pdf;
    int64_t marg_cdf;
    int64_t marg_alias;  /* int2 offsets into the alias pool: the marginal's table (nv */
    int64_t cond_alias;  /* entries), then nv conditional tables of nu; -1 if none */
    float marg_int;
    int32_t pad;
};

struct RtCamera {
    int32_t width, height;
    float near_z, far_z;
    float inv_res_x, inv_res_y;
    float clip_to_camera[16];
    float camera_to_world[16];
    float camera_to_clip[16];       /* light tracing (PerspectiveCamera.SampleWi) */
    float world_to_camera[16];
    float min_x, min_y, max_x, max_y; /* _min, _max of the z = 1 image plane (Camera.cs:172-177) */
    float normalization;            /* _normalization = 1 / its area (Camera.cs:178-179) */
};

/* pointers handed to the kernels by value */
struct RtSceneView {
    const float4* nodes;
    const float4* slots;
    const RtBvh* bvhs;          /* [0] top level, [1 + k] instanced prototype k */
    const RtPrim* prims;        /* top-level primitives by prim id */
    const RtTri* tris;
    const float4* pos;          /* global vertex positions */
    const float4* nrm;
    const float2* uv;
    const RtSphere* spheres;
    const RtInstance* instances;
    const RtMaterial* materials;
    const RtTexture* textures;
    const float* texels;
    const RtMedium* media;
    const RtLight* lights;
    const int32_t* infinite_lights;
    const RtDist2D* dists;
    const float* dist_pool;
    const int2* alias_pool;     /* {threshold, alias} per entry of every Distribution1D */
    int32_t light_count;
    int32_t infinite_count;
    int32_t global_medium;
    int32_t deep_trees;         /* a tree is taller than RT_STACK_SIZE + 1 levels: its
                                 * traversal may overflow the stack, so every far child
                                 * is pushed exactly as the reference pushes it */
    const float4* wnodes;       /* wide nodes of every tree (RT_WIDE_F4 float4 each) */
    int32_t wide_ok;            /* every wide traversal fits the stack: the fast mode may run */
    int32_t env_alias;          /* infinite lights pick texels from their alias tables */
    RtCamera camera;
};

/* integrator parameters */
struct RtParams {
    int32_t integrator, method, strategy;
    int32_t max_depth, min_depth;
    float rr;
    uint64_t seed;
    int32_t x0, y0, w, h;        /* crop */
    int32_t spp, sample_begin;
    int32_t chunk_begin, chunk_len; /* samples of this launch: [chunk_begin, chunk_begin + chunk_len) */
};

#endif
