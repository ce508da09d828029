/*
 * rt_wavefront.h - device state of the wavefront renderer (rt_wavefront.cu).
 *
 * One wavefront run renders a batch of jobs (a job = one scene, its render
 * parameters and its sample buffer) with one pool of path slots: paths of
 * different jobs share the ray queues and the trace / shade launches.  A
 * single render is a batch of one.  Everything a launch needs to know about
 * the current round (job table, sample counts, queue lengths) lives in device
 * memory, so the per-bounce launch sequence is the same every time and can
 * be captured once into a CUDA graph whose while-loop runs until no path is
 * left.
 */
#ifndef RT_WAVEFRONT_H
#define RT_WAVEFRONT_H
#include <cuda_runtime.h>
#include <stdint.h>
#include "rt_types.h"

/* ray kinds: extension, shadow (any hit), MIS / IntersectTr-walk segment,
 * Transmittance-walk segment (the last three closest hit except shadow).
 * In the shadow queue, WF_RAY_SPLAT marks a light-tracer camera connection:
 * the trace kernel adds its pending splat to the film when the way is clear. */
enum { WF_RAY_EXT = 0, WF_RAY_SHADOW = 1, WF_RAY_MIS = 2, WF_RAY_TRW = 3 };
enum { WF_RAY_SPLAT = 2 };

#define WF_MAX_JOBS 256            /* job index is 8 bits in the ray-queue meta word */
#define WF_MAX_SLOTS (1 << 21)     /* slot index is 21 bits in the ray-queue meta word */
#define WF_SHADE_KEYS 1024         /* shade key: (job mod 64) * 16 + the path's code key (0..15) */
#ifndef WF_ITER_CAP
#define WF_ITER_CAP (1 << 20)      /* bounce iterations of one round before a run gives up */
#endif

/* one render of a batch, for the current round of samples (light tracing:
 * `samples` is the film sums, one float4 per pixel, `first` the first
 * particle index, `count` the particles of the round) */
struct WfJob {
    const RtSceneView* view;       /* the job's scene (device) */
    RtParams P;                    /* chunk_begin / chunk_len: this round's sample indices */
    float* samples;                /* per-sample radiance, [k][crop pixel][rgb] */
    long long first;               /* first batch-wide sample id of this job's round */
    long long count;               /* P.w * P.h * P.chunk_len */
};

/* the adjoint replay pass (rt_adjoint.cuh): parameters and gradient sums */
struct WfAdjoint {
    int albedo_tex;          /* texture whose texels are parameters, or -1 */
    int n_alpha;
    const int* alpha_slot;   /* per material: alpha parameter index or -1 */
    float* grad_albedo;
    float* grad_alpha;
    const float* dLdI;       /* crop film layout, already divided by spp */
};
/* shade pass of a run: a render, the adjoint's forward pass (per-sample
 * radiance kept raw, invalid values included), or the adjoint's replay */
enum { WF_PASS_RENDER = 0, WF_PASS_FORWARD_RAW = 1, WF_PASS_REPLAY = 2 };

/* device counters of a run; iteration i reads active[i & 1] and fills active[(i + 1) & 1] */
struct WfCounters {
    long long total;               /* samples of the round, all jobs */
    unsigned long long next_sample;/* next batch-wide sample id to start */
    int32_t n_jobs;
    int32_t iter;
    int32_t n_closest, n_shadow;   /* rays queued for the next trace */
    int32_t n_active[2];
    int32_t fetch[2];              /* next closest / shadow queue entry to hand out */
    int32_t shade_fetch;           /* next sorted entry to shade (resident-grid shading) */
    int32_t pad;
};

/* structure-of-arrays path state; every array has one entry per path slot
 * except the ray queue (3 entries per slot) */
struct WfState {
    /* ray queue: origin + MinT, direction + MaxT, (slot << 10) | (job << 2) | kind.
     * Closest-hit rays (extension, MIS) fill [0, 2 * slots), shadow rays
     * [shadow_base, shadow_base + slots): the two ray kinds never share a warp. */
    float4* q_o; float4* q_d; int32_t* q_meta;
    int32_t shadow_base;
    int32_t slots;
    uint32_t* status;        /* the context's status word (RT_STATUS_*) */
    int32_t refill;          /* idle lanes of a trace warp before it fetches new rays */
    int32_t iter_cap;        /* bounce iterations of one round before the run gives up (WF_ITER_CAP) */
    int32_t dense_sort;      /* the shade-key sort may walk the slots in index order (not for vol_path) */
    WfCounters* ctr;
    const WfJob* jobs;
    /* active slot lists by iteration parity, and the list regrouped by shade key */
    int32_t* active[2];
    int32_t* sorted; uint16_t* sort_key;
    int32_t* key_count;      /* per shade key: entries, then scatter cursors (2 * WF_SHADE_KEYS) */
    uint8_t* mark;           /* per slot: 1 + the active list (iteration parity) it is on, 0 if none */
    /* path state */
    uint8_t* job;            /* job of the slot's path */
    int4* pix;               /* crop x, crop y, sample index in chunk, sample index t */
    uint32_t* rng_n;         /* draws consumed from the path's Philox stream */
    float4* coeff; float4* rad;
    int2* bounce;            /* bounces, loop guard */
    uint32_t* flags;
    float4* ray_o; float4* ray_d;
    /* direct-lighting term waiting for its shadow / MIS rays */
    float4* pd_coeff;        /* coeff at the bounce, light selection pdf */
    float4* pd_l1;           /* light-sample term (NEE: the whole estimate; light tracing:
                                the splat's colour and film pixel) */
    float4* pd_fr;           /* BSDF-sample f*cos, MIS weight */
    float4* pd_mis;          /* BSDF pdf, light index */
    float4* pd_w;            /* direction passed to the light's L() */
    float4* pd_ray_o; float4* pd_ray_d;
    float4* pd_acc;          /* All light strategy: the vertex's summed direct terms, light index (int bits) */
    /* ray results */
    float4* ext_hit; int32_t* ext_sub;
    float4* mis_hit; int32_t* mis_sub;
    uint8_t* occluded;
    /* adjoint replay: d ln (f w) / d alpha of the pending light and BSDF terms,
     * d ln f / d alpha of the continuation, alpha slot of the pending vertex */
    float4* adj_rho;
    /* vol_path: the ray's medium, and the two boundary walks of a pending
     * direct term - Scene.Transmittance towards the light sample (start +
     * medium, end + segment count, direction, throughput) and
     * Scene.IntersectTr along the phase / BSDF sample (ray + medium, throughput
     * + segment count) - with the raw light-sample radiance */
    int32_t* vol_env;
    float4* trw_start; float4* trw_end; float4* trw_dir; float4* trw_tr;
    float4* itw_o; float4* itw_d; float4* itw_tr;
    float4* vol_li;
    float4* trw_hit; int32_t* trw_sub;
};

/* Starts the round: every slot takes a camera sample (or, `particle`, a light
 * particle of job 0), the first active list is built.  The counters must hold
 * the round's total / n_jobs and zeros. */
cudaError_t rt_wf_start(const WfState& W, cudaStream_t s, bool particle = false);
/* Traces the queued closest-hit and shadow rays (lengths read on the device);
 * `deep`: a tree of the scene has RT_DEEP_TREE levels or more, the kernels
 * keep the bottom of the traversal stack in shared memory.  `wide`: the
 * opt-in fast traversal over the scenes' wide nodes. */
#ifndef RT_DEEP_TREE
#define RT_DEEP_TREE 16
#endif
/* With `fork`, the shadow-ray kernel runs on fork->side, joined back into `s`
 * before the call returns (in stream order): its blocks take the SM slots the
 * closest-hit kernel's blocks free as its queue runs dry, so neither kernel's
 * tail leaves the GPU idle. */
struct WfFork {
    cudaStream_t side;
    cudaEvent_t fork, join;
};
cudaError_t rt_wf_trace(const WfState& W, uint32_t* status, unsigned long long* stats, bool counting, cudaStream_t s,
                        bool deep = false, bool wide = false, const WfFork* fork = nullptr);
/* Shades the active paths (`particle`: light-tracer particles) - regrouped by
 * shade key first with `sort` - then advances the iteration; with `loop` set
 * (inside a captured while-loop), also sets the loop's condition to "paths
 * remain".  n_hint: the active count when the host knows it (grids sized to
 * it), -1 inside a graph (grids cover every slot, surplus blocks return).
 * Kernel launches are added to *launches. */
cudaError_t rt_wf_shade(const WfState& W, int n_hint, uint32_t* status, unsigned long long* stats, bool counting,
                        cudaGraphConditionalHandle loop, bool has_loop, cudaStream_t s, uint64_t* launches,
                        int pass = WF_PASS_RENDER, const WfAdjoint* adj = nullptr, bool vol = false,
                        bool particle = false, bool sort = true);

#endif
