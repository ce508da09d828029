/*
 * rt_wavefront.h - device state of the wavefront renderer (rt_wavefront.cu).
 */
#ifndef RT_WAVEFRONT_H
#define RT_WAVEFRONT_H
#include <cuda_runtime.h>
#include <stdint.h>
#include "rt_types.h"

enum { WF_RAY_EXT = 0, WF_RAY_SHADOW = 1, WF_RAY_MIS = 2 };

/* structure-of-arrays path state; every array has one entry per path slot
 * except the ray queue (3 entries per slot) */
struct WfState {
    /* ray queue: origin + MinT, direction + MaxT, (slot << 2) | kind.
     * Closest-hit rays (extension, MIS) fill [0, 2 * slots), shadow rays
     * [shadow_base, shadow_base + slots): the two ray kinds never share a warp. */
    float4* q_o; float4* q_d; int32_t* q_meta;
    int32_t* n_rays_next;
    int32_t* n_shadow_next;
    int32_t shadow_base;
    int32_t* fetch;              /* [0] closest, [1] shadow: next queue entry to hand out */
    /* active slot lists (read by the shade kernel / written for the next one) */
    int32_t* active; int32_t* active_next;
    /* the active list regrouped by shade key before shading (see shade_key) */
    int32_t* sorted; uint8_t* sort_key;
    int32_t* key_count;      /* [0, 16) entries per key, [16, 32) scatter cursors */
    int32_t* n_active; int32_t* n_active_next;
    unsigned long long* next_sample;
    /* path state */
    int4* pix;               /* crop x, crop y, sample index in chunk, sample index t */
    uint32_t* rng_n;         /* draws consumed from the path's Philox stream */
    float4* coeff; float4* rad;
    int2* bounce;            /* bounces, loop guard */
    uint32_t* flags;
    float4* ray_o; float4* ray_d;
    /* direct-lighting term waiting for its shadow / MIS rays */
    float4* pd_coeff;        /* coeff at the bounce, light selection pdf */
    float4* pd_l1;           /* light-sample term (NEE: the whole estimate) */
    float4* pd_fr;           /* BSDF-sample f*cos, MIS weight */
    float4* pd_mis;          /* BSDF pdf, light index */
    float4* pd_w;            /* direction passed to the light's L() */
    float4* pd_ray_o; float4* pd_ray_d;
    /* ray results */
    float4* ext_hit; int32_t* ext_sub;
    float4* mis_hit; int32_t* mis_sub;
    uint8_t* occluded;
    float* samples;          /* per-sample radiance, [k][crop pixel][rgb] */
};

cudaError_t rt_wf_start(const RtSceneView* S, const RtParams& P, const WfState& W, int slots, cudaStream_t s);
cudaError_t rt_wf_trace(const RtSceneView* S, const WfState& W, int n_closest, int n_shadow, uint32_t* status,
                        unsigned long long* stats, bool counting, cudaStream_t s);
/* Shades the n active paths; launches += the kernels it started. */
cudaError_t rt_wf_shade(const RtSceneView* S, const RtParams& P, const WfState& W, int n, uint32_t* status,
                        unsigned long long* stats, bool counting, bool regenerate, cudaStream_t s, uint64_t* launches);

#endif
