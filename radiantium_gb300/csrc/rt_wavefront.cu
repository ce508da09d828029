/*
 * rt_wavefront.cu - wavefront renderer for the `path` integrator.
 *
 * The megakernel runs PathTracer.Li (Integrators/PathTracer.cs) as one loop
 * per thread.  Here the loop is cut at its ray casts and the pieces run as
 * separate kernels over compacted queues:
 *
 *   k_wf_trace_closest / k_wf_trace_shadow   the queued rays: extension and
 *                MIS rays (closest hit), shadow rays (any hit), each kind in
 *                its own persistent kernel with dynamic ray fetch;
 *   k_wf_sort_count / k_wf_sort_scatter   regroup the active list by shade
 *                key (finished, missed, material type) so that a warp runs
 *                one material's code instead of the union of several;
 *   k_wf_shade   per path: first adds the direct-lighting term scheduled in
 *                the previous shade (its shadow / MIS rays are now resolved),
 *                then runs one bounce of the reference loop on the new
 *                extension hit and enqueues the next rays.
 *
 * All random numbers of a bounce are drawn in k_wf_shade in the reference's
 * order, and the radiance of a path is accumulated in the reference's order
 * (the deferred direct term of bounce b is added before the emission of
 * bounce b+1), so every sample is bit-identical to the megakernel and to the
 * CPU oracle.  Path slots whose path has finished are refilled with the next
 * camera sample, which keeps the queues full to the end of a render.
 *
 * A run renders a batch of jobs (rt_wavefront.h): a path slot records its
 * job, and the scene view and parameters of that job drive its traversal and
 * shading, so paths of every scene of a batch share one set of launches.
 * Every launch reads its work count from device memory and the active lists
 * alternate by iteration parity, so the launch sequence of one bounce never
 * changes and can be captured into a CUDA graph loop.
 */
#include <cuda_runtime.h>
#include <algorithm>
#include "rt_integrators.cuh"
#include "rt_adjoint.cuh"
#include "rt_wavefront.h"

using namespace rtd;

namespace {

enum : uint32_t {
    F_ALIVE = 1u,        /* the slot holds a path */
    F_SPECULAR = 2u,     /* isSpecularPath */
    F_PENDING = 4u,      /* a direct-lighting term waits for its rays */
    F_L1 = 8u,           /* pending light-sample term (gated by the shadow ray) */
    F_L2 = 16u,          /* pending BSDF-sample term (resolved by the MIS ray) */
    F_DZERO = 32u,       /* pending direct term is exactly zero (no light / no estimate) */
    F_DONE = 64u,        /* the path ends once its pending term is added */
    F_EXT = 128u,        /* an extension ray was enqueued */
    F_WTR = 256u,        /* vol_path: a Transmittance-walk segment is being traced */
    F_WIT = 512u,        /* vol_path: an IntersectTr-walk segment is being traced */
    F_CONT = 1024u,      /* vol_path: the next extension ray waits for the pending term */
    F_ALL = 2048u,       /* path, All light strategy: the vertex's lights are estimated one per iteration */
};

DF void warp_add64(unsigned long long* dst, uint32_t v) {
    unsigned mask = __activemask();
    uint32_t s = __reduce_add_sync(mask, v);
    if ((threadIdx.x & 31) == (unsigned)(__ffs(mask) - 1) && s) atomicAdd(dst, (unsigned long long)s);
}

/* warp-aggregated append to a queue counter */
DF int warp_append(int* counter, bool want) {
    unsigned mask = __ballot_sync(__activemask(), want);
    if (!want) return -1;
    int leader = __ffs(mask) - 1;
    int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

/* Appends a shade's rays and its slot for the next iteration in one pass:
 * the shadow queue, the closest-hit queue (the warp's MIS rays, then its
 * extension rays) and the next active list `next`.  kBlock: one atomic per
 * counter per block, every thread of the block calls it (blockDim.x a
 * multiple of 32); else one per warp, every lane of the warp calls it.  The
 * three counters' atomics are in flight together.  Outputs are queue
 * positions (the shadow one including shadow_base), -1 where not wanted. */
template <bool kBlock>
DF void queue_append(const WfState& W, int next, bool shadow, bool mis, bool ext, bool keep,
                     int* qs, int* qm, int* qe, int* qa) {
    const unsigned full = 0xffffffffu;
    const unsigned bs = __ballot_sync(full, shadow), bm = __ballot_sync(full, mis),
                   be = __ballot_sync(full, ext), ba = __ballot_sync(full, keep);
    const int lane = threadIdx.x & 31;
    int b0, b1, b2;
    if (kBlock) {
        __shared__ int s_cnt[3][32];
        __shared__ int s_base[3];
        const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
        if (lane == 0) { s_cnt[0][w] = __popc(bs); s_cnt[1][w] = __popc(bm) + __popc(be); s_cnt[2][w] = __popc(ba); }
        __syncthreads();
        if (threadIdx.x < 3) {
            int* c = threadIdx.x == 0 ? &W.ctr->n_shadow : (threadIdx.x == 1 ? &W.ctr->n_closest : &W.ctr->n_active[next]);
            int t = 0;
            for (int k = 0; k < nw; k++) { const int v = s_cnt[threadIdx.x][k]; s_cnt[threadIdx.x][k] = t; t += v; }
            s_base[threadIdx.x] = t ? atomicAdd(c, t) : 0;
        }
        __syncthreads();
        b0 = s_base[0] + s_cnt[0][w]; b1 = s_base[1] + s_cnt[1][w]; b2 = s_base[2] + s_cnt[2][w];
        __syncthreads();
    } else {
        int v = 0;
        if (lane < 3) {
            const int t = lane == 0 ? __popc(bs) : (lane == 1 ? __popc(bm) + __popc(be) : __popc(ba));
            int* c = lane == 0 ? &W.ctr->n_shadow : (lane == 1 ? &W.ctr->n_closest : &W.ctr->n_active[next]);
            if (t) v = atomicAdd(c, t);
        }
        b0 = __shfl_sync(full, v, 0); b1 = __shfl_sync(full, v, 1); b2 = __shfl_sync(full, v, 2);
    }
    const unsigned lt = (1u << lane) - 1u;
    *qs = shadow ? W.shadow_base + b0 + __popc(bs & lt) : -1;
    *qm = mis ? b1 + __popc(bm & lt) : -1;
    *qe = ext ? b1 + __popc(bm) + __popc(be & lt) : -1;
    *qa = keep ? b2 + __popc(ba & lt) : -1;
}

/* Debug-bounds builds (-DRT_DEBUG_BOUNDS) check every computed index into a
 * path-state buffer: one outside its buffer sets RT_STATUS_BOUNDS and the
 * access is skipped (no trap), so the host reports RT_ERR_BOUNDS. */
#ifdef RT_DEBUG_BOUNDS
DF bool in_bounds(const WfState& W, long long i, long long n) {
    if (i >= 0 && i < n) return true;
    atomicOr(W.status, RT_STATUS_BOUNDS);
    return false;
}
#else
DF bool in_bounds(const WfState&, long long, long long) { return true; }
#endif
DF void set_active(const WfState& W, int list, int a, int slot) {
    if (in_bounds(W, a, W.slots)) W.active[list][a] = slot;
    if (in_bounds(W, slot, W.slots)) W.mark[slot] = (uint8_t)(list + 1);
}
/* a shaded slot that leaves the active lists */
DF void clear_active(const WfState& W, int slot) {
    if (slot >= 0 && in_bounds(W, slot, W.slots)) W.mark[slot] = 0;
}

DF void push_ray4(const WfState& W, int q, int path, int kind, float4 o, float4 d) {
    if (!in_bounds(W, q, 3LL * W.slots)) return;
    W.q_o[q] = o;
    W.q_d[q] = d;
    W.q_meta[q] = (path << 10) | ((int)W.job[path] << 2) | kind;
}

DF void ray4(const Ray& r, float4* o, float4* d) {
    *o = make_float4(r.O.x, r.O.y, r.O.z, r.MinT);
    *d = make_float4(r.D.x, r.D.y, r.D.z, r.MaxT);
}

DF int meta_path(int meta) { return meta >> 10; }
DF int meta_job(int meta) { return (meta >> 2) & (WF_MAX_JOBS - 1); }
DF int meta_kind(int meta) { return meta & 3; }

/* job of a batch-wide sample id (jobs are ordered by their first id) */
DF int job_of(const WfState& W, long long sid) {
    int lo = 0, hi = W.ctr->n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (W.jobs[mid].first <= sid) lo = mid; else hi = mid - 1;
    }
    return lo;
}

/* Rng resumed at draw n of its stream */
DF void rng_resume(Rng& r, uint64_t seed, uint32_t x, uint32_t y, uint32_t s, uint32_t n) {
    rng_init(r, seed, x, y, s);
    r.n = n;
    if (n & 3u) philox(r.c0, r.c1, r.c2, n >> 2, r.k0, r.k1, r.buf);
}

/* sample id -> (crop pixel, sample index in chunk): ids are dense over the
 * crop; within a sample index the pixels run through bands of four rows,
 * column by column, so 32 consecutive ids cover an 8x4 pixel tile */
DF void sample_pixel(const RtParams& P, int64_t sid, int* lx, int* ly, int* k) {
    const int64_t npix = (int64_t)P.w * P.h;
    *k = (int)(sid / npix);
    const int r = (int)(sid - (int64_t)(*k) * npix);
    const int band = r / (4 * P.w);
    const int bh = min(4, P.h - band * 4);
    const int rr = r - band * 4 * P.w;
    *lx = rr / bh;
    *ly = band * 4 + rr % bh;
}

/* The lanes of `active` with `want` claim consecutive sample ids with one
 * atomic; -1 for the others and for ids past the round's end.  Every lane of
 * `active` calls it. */
DF long long claim_sample(const WfState& W, unsigned active, bool want) {
    const unsigned m = __ballot_sync(active, want);
    if (!want) return -1;
    const int leader = __ffs(m) - 1, lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(&W.ctr->next_sample, (unsigned long long)__popc(m));
    base = __shfl_sync(m, base, leader);
    const long long id = (long long)base + __popc(m & ((1u << lane) - 1u));
    return id < W.ctr->total ? id : -1;
}

/* Initialises camera sample `sid` in `slot`; its first ray goes to W.ray_o /
 * ray_d and to (o, d).  sid < 0 empties the slot.  Returns whether a path
 * started. */
DF bool init_path(const WfState& W, int slot, long long sid, float4* o, float4* d) {
    if (sid < 0) { W.flags[slot] = 0; return false; }
    const int j = job_of(W, sid);
    const WfJob& J = W.jobs[j];
    const RtParams P = J.P;
    W.job[slot] = (uint8_t)j;
    int lx, ly, k;
    sample_pixel(P, sid - J.first, &lx, &ly, &k);
    int px = P.x0 + lx, py = P.y0 + ly, t = P.sample_begin + P.chunk_begin + k;
    Rng rand;
    rng_init(rand, P.seed, (uint32_t)px, (uint32_t)py, (uint32_t)t);
    V2 jit = NextVec2(rand);
    Ray ray = CameraRay(J.view->camera, v2((float)px + jit.x, (float)py + jit.y));
    W.pix[slot] = make_int4(lx, ly, k, t);
    W.rng_n[slot] = rand.n;
    W.coeff[slot] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    W.rad[slot] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    W.bounce[slot] = make_int2(0, 0);
    W.flags[slot] = F_ALIVE | F_SPECULAR | F_EXT;
    W.vol_env[slot] = J.view->global_medium;
    ray4(ray, o, d);
    W.ray_o[slot] = *o;
    W.ray_d[slot] = *d;
    return true;
}

__global__ void __launch_bounds__(256) k_wf_start(WfState W) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = slot < W.slots;
    const long long sid = claim_sample(W, 0xffffffffu, in);
    float4 o, d;
    const bool ok = in && init_path(W, slot, sid, &o, &d);
    int qs, qm, qe, qa;
    queue_append<true>(W, 0, false, false, ok, false, &qs, &qm, &qe, &qa);
    if (ok) push_ray4(W, qe, slot, WF_RAY_EXT, o, d);
}

/* Persistent traversal with dynamic ray fetch (Aila & Laine 2009): each warp
 * keeps its lanes busy by handing a new queue entry to every lane whose ray
 * has finished, as soon as W.refill lanes are idle, instead of idling until
 * the warp's longest ray is done.  The traversal is the step machine of
 * TravClosest / TravAny, so a lane can take a new ray between any two steps
 * and the per-ray results are the same as a one-ray-per-thread launch. */
constexpr unsigned kFullWarp = 0xffffffffu;

/* resident blocks of 128 threads per SM the trace kernels are compiled for
 * (the register budget: 65536 / (128 * blocks)) */
#ifndef RT_CLOSEST_BLOCKS
#define RT_CLOSEST_BLOCKS 6
#endif
#ifndef RT_SHADOW_BLOCKS
#define RT_SHADOW_BLOCKS 7
#endif
/* the same for the shade kernels of `path` (the host-driven render pass; the
 * graph-driven and adjoint-replay variants keep 5, where 6 spills far more)
 * and of the light tracer.  Path shade, M samples/s C2 / C1 / C4: 157.2 /
 * 444.3 / 443.2 at 6, 158.8 / 445.6 / 443.4 at 7; at 8, C2 159.9 but C1 440.1. */
#ifndef RT_SHADE_BLOCKS
#define RT_SHADE_BLOCKS 7
#endif
#ifndef RT_PSHADE_BLOCKS
#define RT_PSHADE_BLOCKS 6
#endif
#ifndef RT_VSHADE_BLOCKS
#define RT_VSHADE_BLOCKS 5       /* C3 M samples/s: 124.7 at 4, 126.1 at 5, 126.0 at 6 */
#endif

/* One warp-wide fetch: returns this lane's queue entry (>= n: none) and sets
 * `exhausted` (warp-uniform) once the queue has been handed out. */
DF int fetch_entry(int32_t* counter, int n, unsigned idle, bool* exhausted) {
    const unsigned lane = threadIdx.x & 31;
    int first = 0;
    if (lane == 0) first = atomicAdd(counter, __popc(idle));
    first = __shfl_sync(kFullWarp, first, 0);
    *exhausted = first + __popc(idle) >= n;
    return first + __popc(idle & ((1u << lane) - 1u));
}

DF Ray queued_ray(const WfState& W, int q) {
    const float4 o = W.q_o[q], d = W.q_d[q];
    return mkray(v3(o.x, o.y, o.z), v3(d.x, d.y, d.z), o.w, d.w);
}

DF void closest_done(const WfState& W, int meta, const TravClosest& T) {
    const int path = meta_path(meta);
    const float4 h = make_float4(T.best.t, T.best.u, T.best.v, __int_as_float(T.any ? T.best.slot : -1));
    const int kind = meta_kind(meta);
    if (kind == WF_RAY_EXT) { W.ext_hit[path] = h; W.ext_sub[path] = T.best.sub; }
    else if (kind == WF_RAY_MIS) { W.mis_hit[path] = h; W.mis_sub[path] = T.best.sub; }
    else { W.trw_hit[path] = h; W.trw_sub[path] = T.best.sub; }
}

/* interior nodes per traversal step in scenes with tall trees (C2 / C3 trace ms per step:
 * 85.7 / 24.3 at 3, 83.7 / 23.8 at 4, 83.5 / 23.7 at 5, 87.5 / 23.2 at 6) */
#ifndef RT_DESCEND_DEEP
#define RT_DESCEND_DEEP 5
#endif

/* The traversal stack of a trace kernel: with kSh (scenes with tall trees)
 * its bottom RT_SH_STACK entries live in shared memory, which keeps the stack
 * of a deep traversal out of the L1 lines the node data needs; shallow trees
 * keep the whole stack in local memory, where it stays in a few hot lines. */
template <bool kSh> struct TraceStack;
template <> struct TraceStack<false> {
    int2 a[2 * RT_STACK_SIZE];
    DF int2* get() { return a; }
};
template <> struct TraceStack<true> {
    int2 a[2 * RT_STACK_SIZE];
    DF SplitStack get() {
        __shared__ int2 sh[RT_SH_STACK * RT_TRACE_BLOCK];
        return SplitStack{sh + threadIdx.x, a};
    }
};

/* wide nodes per traversal step of the fast traversal (kWide) */
#ifndef RT_DESCEND_WIDE
#define RT_DESCEND_WIDE 1        /* C2 M samples/s: 154.7 at 1, 134.9 at 2, 120.5 at 3 */
#endif

/* closest-hit rays: extension and MIS rays (queue [0, n_closest)); kWide: the
 * opt-in fast traversal over the wide nodes */
template <bool kSh, bool kWide>
__global__ void __launch_bounds__(RT_TRACE_BLOCK, RT_CLOSEST_BLOCKS) k_wf_trace_closest(WfState W, uint32_t* status, unsigned long long* stats,
                                                            bool counting) {
    const int n = min(W.ctr->n_closest, 2 * W.slots);
    TraceStack<kSh> stk;
    const auto stack = stk.get();
    TravStats st = {0, 0, 0};
    TravStats* pst = counting ? &st : nullptr;
    uint32_t done = 0;
    TravClosest T;
    const RtSceneView* S = nullptr;
    int item = -1, meta = 0;
    bool exhausted = false;
    while (true) {
        const unsigned idle = __ballot_sync(kFullWarp, item < 0);
        if (exhausted) {
            if (idle == kFullWarp) break;
        } else if (__popc(idle) >= W.refill) {
            const int q = fetch_entry(&W.ctr->fetch[0], n, idle, &exhausted);
            if (item < 0 && q < n) {
                meta = W.q_meta[q];
                S = W.jobs[meta_job(meta)].view;
                if (ClosestBegin<kWide>(S, queued_ray(W, q), T, pst)) { closest_done(W, meta, T); done++; }
                else item = q;
            }
        }
        if (item >= 0 && ClosestStep<decltype(stack), kWide ? RT_DESCEND_WIDE : (kSh ? RT_DESCEND_DEEP : RT_DESCEND), kWide>(
                             S, T, stack, status, pst)) {
            closest_done(W, meta, T);
            done++;
            item = -1;
        }
    }
    if (counting) {
        warp_add64(stats + 1, done);
        warp_add64(stats + 3, st.nodes);
        warp_add64(stats + 4, st.prims);
        warp_add64(stats + 5, st.insts);
    }
}

/* a shadow ray's answer: the path's occlusion flag, or for a light-tracer
 * camera connection its splat, added to the film sums when nothing is in the
 * way (the reference's `lock (renderTarget)` add, AdjointParticleIntegrator.cs:53-66) */
DF void shadow_done(const WfState& W, int meta, bool hit) {
    const int path = meta_path(meta);
    if (meta_kind(meta) != WF_RAY_SPLAT) { W.occluded[path] = hit ? 1 : 0; return; }
    if (hit) return;
    const float4 sp = W.pd_l1[path];
    const int pix = __float_as_int(sp.w);
    const WfJob& J = W.jobs[meta_job(meta)];
    if (pix >= 0 && in_bounds(W, pix, (long long)J.P.w * J.P.h))
        atomicAdd(reinterpret_cast<float4*>(J.samples) + pix, make_float4(sp.x, sp.y, sp.z, 0.0f));
}

/* shadow rays: any-hit (queue [shadow_base, shadow_base + n_shadow)) */
template <bool kSh, bool kWide>
__global__ void __launch_bounds__(RT_TRACE_BLOCK, RT_SHADOW_BLOCKS) k_wf_trace_shadow(WfState W, uint32_t* status, unsigned long long* stats,
                                                           bool counting) {
    const int n = min(W.ctr->n_shadow, W.slots);
    TraceStack<kSh> stk;
    const auto stack = stk.get();
    TravStats st = {0, 0, 0};
    TravStats* pst = counting ? &st : nullptr;
    uint32_t done = 0;
    TravAny T;
    const RtSceneView* S = nullptr;
    int item = -1, meta = 0;
    bool exhausted = false;
    while (true) {
        const unsigned idle = __ballot_sync(kFullWarp, item < 0);
        if (exhausted) {
            if (idle == kFullWarp) break;
        } else if (__popc(idle) >= W.refill) {
            const int e = fetch_entry(&W.ctr->fetch[1], n, idle, &exhausted);
            if (item < 0 && e < n) {
                const int q = W.shadow_base + e;
                meta = W.q_meta[q];
                S = W.jobs[meta_job(meta)].view;
                if (AnyBegin<kWide>(S, queued_ray(W, q), T, pst)) { shadow_done(W, meta, false); done++; }
                else item = q;
            }
        }
        if (item >= 0 && AnyStep<decltype(stack), kWide ? RT_DESCEND_WIDE : (kSh ? RT_DESCEND_DEEP : RT_DESCEND), kWide>(
                             S, T, stack, status, pst)) {
            shadow_done(W, meta, T.hit);
            done++;
            item = -1;
        }
    }
    if (counting) {
        warp_add64(stats + 2, done);
        warp_add64(stats + 3, st.nodes);
        warp_add64(stats + 4, st.prims);
        warp_add64(stats + 5, st.insts);
    }
}

DF bool load_hit(const RtSceneView* S, const Ray& ray, float4 h, int sub, Isect* it) {
    int slot = __float_as_int(h.w);
    if (slot < 0) return false;
    Best b;
    b.t = h.x; b.u = h.y; b.v = h.z; b.slot = slot; b.sub = sub; b.flags = 0;
    b.pw = v3s(0);
    /* instance hits: the world point is recomputed exactly as during traversal */
    float4 s1 = __ldg(S->slots + 3 * (int64_t)slot + 1);
    uint32_t kr = __float_as_uint(s1.w);
    if ((kr >> RT_KIND_SHIFT) == RT_KIND_INSTANCE) {
        const RtInstance& I = S->instances[kr & RT_REF_MASK];
        float w2m[12], m2w[12];
        for (int q = 0; q < 12; q++) { w2m[q] = I.w2m[q]; m2w[q] = I.m2w[q]; }
        float4 p1 = __ldg(S->slots + 3 * (int64_t)sub + 1);
        uint32_t pkr = __float_as_uint(p1.w);
        V3 pm;
        if ((pkr >> RT_KIND_SHIFT) == RT_KIND_TRI) {
            V3 bary = v3(1 - (b.u + b.v), b.u, b.v);
            RtTri t = S->tris[pkr & RT_REF_MASK];
            pm = bary.x * f4xyz(S->pos[t.v0]) + bary.y * f4xyz(S->pos[t.v1]) + bary.z * f4xyz(S->pos[t.v2]);
        } else {
            RtSphere sph = S->spheres[pkr & RT_REF_MASK];
            V3 c = v3(sph.center[0], sph.center[1], sph.center[2]);
            Ray mr = XfRay(ray, w2m);
            float tm = 0;
            SphereTest(c, sph.radius, mr, &tm);
            V3 n = Normalize(At(mr, tm) - c);
            pm = n * sph.radius + c;
        }
        b.pw = Xf12(pm, m2w);
    }
    Finish(S, ray, b, it);
    return true;
}

DF void finish_path(const WfJob& J, const WfState& W, int slot, C3 rad, unsigned long long* stats, int pass) {
    if (pass == WF_PASS_REPLAY) return;
    bool invalid = !IsValid(rad);
    if (invalid && pass == WF_PASS_RENDER) { rad = c3s(0.0f); atomicAdd(stats + 6, 1ull); }
    int4 px = W.pix[slot];
    const RtParams& P = J.P;
    const int64_t npix = (int64_t)P.w * P.h;
    const int64_t sample = (int64_t)px.z * npix + (int64_t)px.x * P.h + px.y;
    if (!in_bounds(W, sample, J.count)) return;
    float* o = J.samples + sample * 3;
    o[0] = rad.r; o[1] = rad.g; o[2] = rad.b;
}

/* one bounce of PathTracer.Mis / NextEventEstimation / OnlySampleBxdf after the
 * extension hit is known (PathTracer.cs:43-270) */
/* What a path shade leaves for the queues: its shadow ray, whether it
 * queued a MIS ray (in pd_ray_o / pd_ray_d) or an extension ray (in ray_o /
 * ray_d), whether the slot stays active, and whether the path is over (the
 * caller starts the next camera sample in the slot). */
struct PathOut {
    float4 so, sd;
    bool shadow, mis, ext, keep, restart;
};

/* Schedules one light's direct term at vertex `it` (PathTracer.cs:309-399
 * for Mis, :95-190 for Nee): draws its light sample and, for Mis, its BSDF
 * sample, stores the term's parts and queues its shadow / MIS rays; the next
 * shade adds it once they are traced.  lightPdf: SampleLight's pdf (Uniform)
 * or 1 (All). */
template <bool kAdj>
DF void schedule_direct(PathOut* o, const WfState& W, const RtSceneView* S, int slot, const Isect& it, V3 wo, int mat,
                        int light, float lightPdf, C3 coeff, int method, Rng& rand, uint32_t& fl, float4& rho) {
    if (method == RT_METHOD_MIS) {
        fl |= F_PENDING;
        W.pd_coeff[slot] = make_float4(coeff.r, coeff.g, coeff.b, lightPdf);
        if (lightPdf > 0.0f) {
            V3 wod = it.Wr;
            LSample ls = LightSampleLi(S, light, it.P, rand);
            if (ls.Pdf > 0.0f && !IsBlack(ls.Li)) {
                C3 fr = MatFr(S, mat, Lo(it, wod), Lo(it, ls.Wi), it.UV);
                float scatteringPdf = MatPdf(S, mat, Lo(it, wod), Lo(it, ls.Wi), it.UV);
                if (!IsBlack(fr)) {
                    /* IsOccluded(it.P, ls.P) */
                    V3 vec = ls.P - it.P;
                    float dis = Length(vec);
                    if (!(dis < 0.001f)) {
                        fr = fr * AbsCosTheta(Lo(it, ls.Wi));
                        float weight = PowerHeuristic(ls.Pdf, scatteringPdf);
                        if (kAdj && __float_as_int(rho.w) >= 0)
                            rho.x = DirectDln(S, mat, Lo(it, wod), Lo(it, ls.Wi), weight, true, it.UV);
                        C3 l1 = fr * ls.Li * weight / ls.Pdf;
                        W.pd_l1[slot] = make_float4(l1.r, l1.g, l1.b, 0);
                        fl |= F_L1;
                        ray4(mkray(it.P, Normalize(vec), 0.0001f, dis - 0.0001f), &o->so, &o->sd);
                        o->shadow = true;
                    }
                }
            }
            BSample sample = MatSample(S, mat, Lo(it, wod), it.UV, rand);
            C3 fr = sample.Fr * AbsCosTheta(sample.Wi);
            float scatteringPdf = sample.Pdf;
            bool sampledSpecular = (sample.Type & BX_SPECULAR) != 0;
            if (!IsBlack(fr) && scatteringPdf > 0) {
                float weight = 1;
                bool go = true;
                if (!sampledSpecular) {
                    float bxdfToLightPdf = LightPdfLi(S, light, it.P, Wo(it, sample.Wi));
                    if (bxdfToLightPdf == 0.0f) go = false;
                    else weight = PowerHeuristic(scatteringPdf, bxdfToLightPdf);
                }
                if (go) {
                    if (kAdj && __float_as_int(rho.w) >= 0)
                        rho.y = DirectDln(S, mat, Lo(it, wod), sample.Wi, sampledSpecular ? 2.0f : weight, false,
                                          it.UV);
                    Ray toLight = Spawn(it, Wo(it, sample.Wi));
                    V3 wle = Wo(it, -sample.Wi);
                    W.pd_fr[slot] = make_float4(fr.r, fr.g, fr.b, weight);
                    W.pd_mis[slot] = make_float4(scatteringPdf, __int_as_float(light), 0, 0);
                    W.pd_w[slot] = make_float4(wle.x, wle.y, wle.z, 0);
                    W.pd_ray_o[slot] = make_float4(toLight.O.x, toLight.O.y, toLight.O.z, toLight.MinT);
                    W.pd_ray_d[slot] = make_float4(toLight.D.x, toLight.D.y, toLight.D.z, toLight.MaxT);
                    fl |= F_L2;
                    o->mis = true;
                }
            }
        } else {
            fl |= F_DZERO;
        }
    } else { /* NEE: NeeEstimateLight */
        if (lightPdf > 0.0f) {
            fl |= F_PENDING;
            W.pd_coeff[slot] = make_float4(coeff.r, coeff.g, coeff.b, lightPdf);
            LSample r = LightSampleLi(S, light, it.P, rand);
            bool zero = true;
            if (r.Pdf > 0.0f) {
                V3 vec = r.P - it.P;
                float dis = Length(vec);
                if (!(dis < 0.001f)) {
                    C3 fr = MatFr(S, mat, Lo(it, wo), Lo(it, r.Wi), it.UV);
                    C3 e = fr * r.Li * AbsCosTheta(Lo(it, r.Wi)) / r.Pdf;
                    W.pd_l1[slot] = make_float4(e.r, e.g, e.b, 0);
                    zero = false;
                    ray4(mkray(it.P, Normalize(vec), 0.0001f, dis - 0.0001f), &o->so, &o->sd);
                    o->shadow = true;
                }
            }
            if (zero) fl |= F_DZERO;
        }
    }
}

template <bool kAdj>
DF void shade_path(PathOut* o, const WfState& W, int slot, uint32_t* status, unsigned long long* stats, bool counting,
                   int pass, const WfAdjoint& A, float* s_alpha) {
    const WfJob& J = W.jobs[W.job[slot]];
    const RtSceneView* S = J.view;
    const RtParams P = J.P;                  /* registers: the path-state stores below cannot alias it */
    uint32_t fl = W.flags[slot];
    float4 cf = W.coeff[slot], rd = W.rad[slot];
    C3 coeff = c3(cf.x, cf.y, cf.z), radiance = c3(rd.x, rd.y, rd.z);
    /* replay: the sample's radiance from the forward pass and its pixel's dL/dI */
    C3 Ltot = c3s(0.0f), dL = c3s(0.0f);
    bool grad = false;
    if (kAdj) {
        const int4 q = W.pix[slot];
        const int64_t pix = (int64_t)q.x * P.h + q.y;
        const float* ls = J.samples + ((int64_t)q.z * P.w * P.h + pix) * 3;
        Ltot = c3(ls[0], ls[1], ls[2]);
        dL = c3(A.dLdI[pix * 3], A.dLdI[pix * 3 + 1], A.dLdI[pix * 3 + 2]);
        grad = IsValid(Ltot) && (dL.r != 0.0f || dL.g != 0.0f || dL.b != 0.0f);
    }

    /* 1. the direct term scheduled by the previous bounce (or, All strategy,
     * the term of one light of this vertex) */
    bool resume = false;                     /* All: the vertex's last light is in, its continuation runs below */
    if (fl & F_PENDING) {
        float4 pc = W.pd_coeff[slot];
        C3 coeffb = c3(pc.x, pc.y, pc.z);
        float lightPdf = pc.w;
        const bool all = (fl & F_ALL) != 0;
        if (P.method == RT_METHOD_MIS) {
            C3 direct = c3s(0);
            C3 tl = c3s(0.0f), tb = c3s(0.0f);
            C3 le = c3s(0.0f);
            if (!(fl & F_DZERO)) {
                if ((fl & F_L1) && !W.occluded[slot]) {
                    float4 l1 = W.pd_l1[slot];
                    tl = c3(l1.x, l1.y, l1.z);
                    le = le + tl;
                }
                if (fl & F_L2) {
                    float4 fr2 = W.pd_fr[slot];
                    float4 mi = W.pd_mis[slot];
                    float4 wl = W.pd_w[slot];
                    const int light = __float_as_int(mi.y);
                    C3 li = c3s(0);
                    Isect lit;
                    float4 mo = W.pd_ray_o[slot], md = W.pd_ray_d[slot];
                    Ray mr = mkray(v3(mo.x, mo.y, mo.z), v3(md.x, md.y, md.z), mo.w, md.w);
                    if (load_hit(S, mr, W.mis_hit[slot], W.mis_sub[slot], &lit)) {
                        if (LightOf(S, lit) >= 0 && LightOf(S, lit) == light) li = IsectLe(S, lit, v3(wl.x, wl.y, wl.z));
                    } else {
                        li = EvalAllInfinite(S, mr.D);
                    }
                    if (!IsBlack(li)) { tb = c3(fr2.x, fr2.y, fr2.z) * li * fr2.w / mi.x; le = le + tb; }
                }
                if (!all) direct = direct + le / lightPdf;
            }
            if (all) {
                /* PathTracer.cs:297-304: result += EstimateDirect(light) over Scene.Lights */
                const float4 ac = W.pd_acc[slot];
                const C3 acc = c3(ac.x, ac.y, ac.z) + le;
                W.pd_acc[slot] = make_float4(acc.r, acc.g, acc.b, ac.w);
            } else {
                radiance = radiance + coeffb * direct;
            }
            if (kAdj && grad && !all) {
                /* alpha terms of the pending vertex: its two direct terms, then its
                 * continuation, which carries everything after its direct light */
                const float4 ar = W.adj_rho[slot];
                const int aslot = __float_as_int(ar.w);
                if (aslot >= 0) {
                    float g = ar.z * Dot3(dL, Ltot - radiance);
                    if (!IsBlack(tl)) g += ar.x * Dot3(dL, coeffb * tl) / lightPdf;
                    if (!IsBlack(tb)) g += ar.y * Dot3(dL, coeffb * tb) / lightPdf;
                    if (g != 0.0f) atomicAdd(s_alpha + aslot, g);
                }
            }
        } else { /* NEE */
            C3 e = c3s(0);
            if (!(fl & F_DZERO) && !W.occluded[slot]) { float4 l1 = W.pd_l1[slot]; e = c3(l1.x, l1.y, l1.z); }
            radiance = all ? radiance + coeffb * e : radiance + coeffb * e / lightPdf;
        }
        fl &= ~(F_PENDING | F_L1 | F_L2 | F_DZERO);
        if (all) {
            const float4 ac = W.pd_acc[slot];
            const int next = __float_as_int(ac.w) + 1;
            if (next < S->light_count) {
                /* the next light at the same vertex: its draws follow the previous light's */
                const float4 ro = W.ray_o[slot], rdd = W.ray_d[slot];
                const Ray ray = mkray(v3(ro.x, ro.y, ro.z), v3(rdd.x, rdd.y, rdd.z), ro.w, rdd.w);
                Isect it;
                load_hit(S, ray, W.ext_hit[slot], W.ext_sub[slot], &it);
                const int4 px = W.pix[slot];
                Rng rand;
                rng_resume(rand, P.seed, (uint32_t)(P.x0 + px.x), (uint32_t)(P.y0 + px.y), (uint32_t)px.w, W.rng_n[slot]);
                float4 rho = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
                schedule_direct<kAdj>(o, W, S, slot, it, -ray.D, PrimOf(S, it).material, next, 1.0f, coeffb, P.method,
                                      rand, fl, rho);
                W.pd_acc[slot] = make_float4(ac.x, ac.y, ac.z, __int_as_float(next));
                W.rng_n[slot] = rand.n;
                W.flags[slot] = fl;
                W.rad[slot] = make_float4(radiance.r, radiance.g, radiance.b, 0);
                o->keep = true;
                return;
            }
            if (P.method == RT_METHOD_MIS) radiance = radiance + coeffb * c3(ac.x, ac.y, ac.z);
            fl &= ~F_ALL;
            resume = true;
        }
    }

    bool done = (fl & F_DONE) != 0;
    if (!done) {
        /* 2. the bounce itself */
        int2 bc = W.bounce[slot];
        int bounces = bc.x, guard = bc.y;
        float4 ro = W.ray_o[slot], rdd = W.ray_d[slot];
        Ray ray = mkray(v3(ro.x, ro.y, ro.z), v3(rdd.x, rdd.y, rdd.z), ro.w, rdd.w);
        int4 px = W.pix[slot];
        Rng rand;
        rng_resume(rand, P.seed, (uint32_t)(P.x0 + px.x), (uint32_t)(P.y0 + px.y), (uint32_t)px.w, W.rng_n[slot]);
        bool isSpecularPath = (fl & F_SPECULAR) != 0;
        Ray nray = ray;
        bool ext = false;
        do {
            if (!resume && ++guard > RT_LOOP_CAP) { atomicOr(status, RT_STATUS_ITER); done = true; break; }
            Isect it;
            bool isHit = load_hit(S, ray, W.ext_hit[slot], W.ext_sub[slot], &it);
            V3 wo = -ray.D;
            if (resume) {
                /* All: emission and the lights of this vertex are in; its continuation follows */
            } else if (P.method == RT_METHOD_BXDF) {
                if (!isHit) { radiance = radiance + coeff * EvalAllInfinite(S, ray.D); done = true; break; }
                if (P.max_depth != -1 && bounces >= P.max_depth) { done = true; break; }
                if (!HasSurface(S, it)) { nray = mkray(it.P, ray.D, ray.MinT); ext = true; break; }
                if (LightOf(S, it) >= 0) radiance = radiance + coeff * IsectLe(S, it, wo);
            } else {
                if (bounces == 0 || isSpecularPath) {
                    if (isHit) radiance = radiance + coeff * IsectLe(S, it, wo);
                    else radiance = radiance + coeff * EvalAllInfinite(S, ray.D);
                }
                if (!isHit) { done = true; break; }
                if (P.max_depth != -1 && bounces >= P.max_depth) { done = true; break; }
                if (!HasSurface(S, it)) { nray = mkray(it.P, ray.D, ray.MinT); ext = true; break; }
                /* direct lighting: everything but the two ray casts */
                const int mat = PrimOf(S, it).material;
                float4 rho = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
                if (kAdj && grad) {
                    if (UsesAlbedo(S, A.albedo_tex, mat)) {
                        const C3 R = TexSample(S, A.albedo_tex, it.UV);
                        const C3 rest = Ltot - radiance;
                        ScatterAlbedo(S, A.albedo_tex, A.grad_albedo, it.UV,
                                      c3(R.r > 0 ? dL.r * rest.r / R.r : 0.0f, R.g > 0 ? dL.g * rest.g / R.g : 0.0f,
                                         R.b > 0 ? dL.b * rest.b / R.b : 0.0f));
                    }
                    if (A.alpha_slot) rho.w = __int_as_float(A.alpha_slot[mat]);
                }
                if (P.strategy == RT_STRATEGY_ALL) {
                    if (S->light_count > 0) {
                        /* light 0 now, the others one per iteration; the continuation waits */
                        fl |= F_ALL;
                        W.pd_acc[slot] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(0));
                        schedule_direct<kAdj>(o, W, S, slot, it, wo, mat, 0, 1.0f, coeff, P.method, rand, fl, rho);
                        break;
                    }
                    if (P.method == RT_METHOD_MIS) radiance = radiance + coeff * c3s(0.0f);
                } else {
                    int light;
                    float lightPdf = SampleLight(S, rand, &light);
                    schedule_direct<kAdj>(o, W, S, slot, it, wo, mat, light, lightPdf, coeff, P.method, rand, fl, rho);
                }
                if (kAdj) W.adj_rho[slot] = rho;
            }
            /* continuation */
            BSample s = MatSample(S, PrimOf(S, it).material, Lo(it, wo), it.UV, rand);
            if (kAdj && P.method == RT_METHOD_MIS && (fl & F_PENDING)) {
                float4 rho = W.adj_rho[slot];
                float rc = 0.0f, rcp;
                if (__float_as_int(rho.w) >= 0 && s.Pdf > 0.0f)
                    DlnAlpha(S, PrimOf(S, it).material, Lo(it, wo), s.Wi, it.UV, &rc, &rcp);
                rho.z = rc;
                W.adj_rho[slot] = rho;
            }
            if (P.method != RT_METHOD_BXDF) isSpecularPath = (s.Type & BX_SPECULAR) != 0;
            if (s.Pdf > 0.0f) coeff = coeff * (s.Fr * AbsCosTheta(s.Wi) / s.Pdf);
            else { done = true; break; }
            nray = Spawn(it, Wo(it, s.Wi));
            if (bounces > P.min_depth) {
                float q = nmin(MaxElement(coeff), P.rr);
                if (NextFloat(rand) > q) { done = true; break; }
                coeff = coeff / q;
            }
            bounces++;
            ext = true;
        } while (false);
        if (ext) {
            W.ray_o[slot] = make_float4(nray.O.x, nray.O.y, nray.O.z, nray.MinT);
            W.ray_d[slot] = make_float4(nray.D.x, nray.D.y, nray.D.z, nray.MaxT);
            o->ext = true;
        }
        W.bounce[slot] = make_int2(bounces, guard);
        W.rng_n[slot] = rand.n;
        fl = (fl & ~F_SPECULAR) | (isSpecularPath ? F_SPECULAR : 0u);
        if (done) fl |= F_DONE;
    }
    W.coeff[slot] = make_float4(coeff.r, coeff.g, coeff.b, 0);
    W.rad[slot] = make_float4(radiance.r, radiance.g, radiance.b, 0);
    /* the slot stays active while it waits for rays */
    if ((fl & F_PENDING) || !(fl & F_DONE)) {
        W.flags[slot] = fl;
        o->keep = true;
        return;
    }
    finish_path(J, W, slot, radiance, stats, pass);
    if (counting) warp_add64(stats + 0, 1u);
    o->restart = true;
}

/* The shade's queue appends, for the block (kBlock) or the warp: a finished
 * path's slot takes the next camera sample at once. */
template <bool kBlock>
DF void path_queues(const WfState& W, int slot, int next, PathOut& o) {
    const long long sid = claim_sample(W, 0xffffffffu, o.restart);
    float4 ro, rd;
    if (o.restart && init_path(W, slot, sid, &ro, &rd)) { o.ext = true; o.keep = true; }
    int qs, qm, qe, qa;
    queue_append<kBlock>(W, next, o.shadow, o.mis, o.ext, o.keep, &qs, &qm, &qe, &qa);
    if (o.shadow) push_ray4(W, qs, slot, WF_RAY_SHADOW, o.so, o.sd);
    if (o.mis) push_ray4(W, qm, slot, WF_RAY_MIS, W.pd_ray_o[slot], W.pd_ray_d[slot]);
    if (o.ext) {
        if (!o.restart) { ro = W.ray_o[slot]; rd = W.ray_d[slot]; }
        push_ray4(W, qe, slot, WF_RAY_EXT, ro, rd);
    }
    if (o.keep) set_active(W, next, qa, slot);
    else clear_active(W, slot);
}

/* ---- vol_path (VolumetricPathTracer.Li, Integrators/VolumetricPathTracer.cs) ----
 * A bounce draws all of its random numbers in one shade, in the reference's
 * order: medium distance, light choice and sample, phase / BSDF sample of
 * the direct term, continuation, Russian roulette.  The boundary walks of
 * the direct term (Scene.Transmittance towards the light sample,
 * Scene.IntersectTr along the phase / BSDF sample) draw none; each of their
 * segments is one closest-hit ray, traced in later iterations while the
 * path waits.  When both walks are done the direct term is added, then the
 * continuation ray (already sampled) is enqueued, so radiance accumulates
 * in the reference's order. */

DF int pack_env(int env, int count) { return (count << 16) | ((env + 1) & 0xFFFF); }
DF int env_of(int packed) { return (packed & 0xFFFF) - 1; }
DF int count_of(int packed) { return packed >> 16; }

/* the next Transmittance segment from the walk's current start (o, d); false: the walk is over */
DF bool trw_ray(const WfState& W, int slot, float4* o, float4* d) {
    const float4 st = W.trw_start[slot], en = W.trw_end[slot], dr = W.trw_dir[slot];
    const V3 start = v3(st.x, st.y, st.z), to = v3(en.x, en.y, en.z);
    const float dis = Length(to - start);
    if (dis < 0.0001f) return false;
    ray4(mkray(start, v3(dr.x, dr.y, dr.z), 0.0001f, dis - 0.0001f), o, d);
    return true;
}
DF bool trw_next(const WfState& W, int slot) {
    float4 o, d;
    return trw_ray(W, slot, &o, &d);
}
/* Scene.Transmittance (Scene.cs:72-103), one traced segment; true: continues */
DF bool trw_step(const RtSceneView* S, const WfState& W, int slot) {
    float4 st = W.trw_start[slot], en = W.trw_end[slot];
    const float4 dr = W.trw_dir[slot], trv = W.trw_tr[slot];
    V3 start = v3(st.x, st.y, st.z);
    const V3 to = v3(en.x, en.y, en.z), dir = v3(dr.x, dr.y, dr.z);
    int env = __float_as_int(st.w), count = __float_as_int(en.w);
    const float dis = Length(to - start);
    const Ray ray = mkray(start, dir, 0.0001f, dis - 0.0001f);
    Isect inct;
    const bool anyHit = load_hit(S, ray, W.trw_hit[slot], W.trw_sub[slot], &inct);
    C3 tr = c3(trv.x, trv.y, trv.z);
    bool more = true;
    if (anyHit && HasSurface(S, inct)) { tr = c3s(0.0f); more = false; }
    else {
        if (env >= 0) tr = tr * MedTr(S->media[env], ray);
        if (!anyHit) more = false;
        else {
            start = inct.P;
            env = GetMedium(S, inct, dir);
            if (++count >= RT_WALK_CAP) { more = false; atomicOr(W.status, RT_STATUS_WALK); }
        }
    }
    W.trw_tr[slot] = make_float4(tr.r, tr.g, tr.b, 0.0f);
    if (!more) return false;
    W.trw_start[slot] = make_float4(start.x, start.y, start.z, __int_as_float(env));
    W.trw_end[slot] = make_float4(to.x, to.y, to.z, __int_as_float(count));
    return trw_next(W, slot);
}
/* Scene.IntersectTr (Scene.cs:105-131), one traced segment; true: continues.
 * When over, itw_o holds the radiance found (light-identity check of
 * EstimateDirect, or the environment on a miss) and itw_tr the throughput. */
DF bool itw_step(const RtSceneView* S, const WfState& W, int slot, int light, V3 wle) {
    const float4 o = W.itw_o[slot], d = W.itw_d[slot], trv = W.itw_tr[slot];
    Ray ray = mkray(v3(o.x, o.y, o.z), v3(d.x, d.y, d.z), o.w);
    const int packed = __float_as_int(trv.w);
    int env = env_of(packed), count = count_of(packed);
    C3 tr = c3(trv.x, trv.y, trv.z);
    Isect inct;
    const bool anyHit = load_hit(S, ray, W.mis_hit[slot], W.mis_sub[slot], &inct);
    C3 li = c3s(0.0f);
    bool more = false;
    if (!anyHit) {
        if (env >= 0) tr = tr * MedTr(S->media[env], ray);
        li = EvalAllInfinite(S, ray.D);
    } else {
        if (env >= 0) {
            const Ray realPath = mkray(ray.O, ray.D, ray.MinT, Length(At(ray, inct.T)));
            tr = tr * MedTr(S->media[env], realPath);
        }
        if (HasSurface(S, inct)) {
            if (LightOf(S, inct) >= 0 && LightOf(S, inct) == light) li = IsectLe(S, inct, wle);
        } else if (++count >= RT_WALK_CAP) {
            li = EvalAllInfinite(S, ray.D);             /* the walk gives up: a miss */
            atomicOr(W.status, RT_STATUS_WALK);
        } else {
            ray = mkray(inct.P, ray.D, 0.001f);
            env = GetMedium(S, inct, ray.D);
            more = true;
        }
    }
    if (more) {
        W.itw_o[slot] = make_float4(ray.O.x, ray.O.y, ray.O.z, ray.MinT);
        W.itw_tr[slot] = make_float4(tr.r, tr.g, tr.b, __int_as_float(pack_env(env, count)));
        return true;
    }
    W.itw_o[slot] = make_float4(li.r, li.g, li.b, 0.0f);
    W.itw_tr[slot] = make_float4(tr.r, tr.g, tr.b, 0.0f);
    return false;
}

/* What a vol_path shade leaves for the queues: a Transmittance segment
 * (its ray rebuilt from trw_*), an IntersectTr segment (from itw_*) or the
 * extension ray (ray_o / ray_d), whether the slot stays active, whether the
 * path is over.  A shade starts walk segments or an extension ray, never both. */
struct VolOut {
    bool trw, itw, ext, keep, restart;
};

/* one shade of a vol_path slot */
DF void shade_vol_path(VolOut* o, const WfState& W, int slot, uint32_t* status, unsigned long long* stats,
                       bool counting) {
    const WfJob& J = W.jobs[W.job[slot]];
    const RtSceneView* S = J.view;
    const RtParams P = J.P;
    uint32_t fl = W.flags[slot];
    /* 1. the boundary walks of a pending direct term */
    if (fl & (F_WTR | F_WIT)) {
        if ((fl & F_WTR) && !trw_step(S, W, slot)) fl &= ~F_WTR;
        if (fl & F_WIT) {
            const float4 mi = W.pd_mis[slot], wl = W.pd_w[slot];
            if (!itw_step(S, W, slot, __float_as_int(mi.y), v3(wl.x, wl.y, wl.z))) fl &= ~F_WIT;
        }
        if (fl & (F_WTR | F_WIT)) {
            W.flags[slot] = fl;
            o->trw = (fl & F_WTR) != 0;
            o->itw = (fl & F_WIT) != 0;
            o->keep = true;
            return;
        }
    }
    float4 cf = W.coeff[slot], rdv = W.rad[slot];
    C3 coeff = c3(cf.x, cf.y, cf.z), radiance = c3(rdv.x, rdv.y, rdv.z);
    bool ext = false;
    for (int pass = 0; pass < 2; pass++) {
        /* 2. the direct term, now that its walks are done (EstimateDirectSurface / Medium) */
        if (fl & F_PENDING) {
            const float4 pc = W.pd_coeff[slot];
            C3 direct = c3s(0.0f);
            if (!(fl & F_DZERO)) {
                C3 le = c3s(0.0f);
                if (fl & F_L1) {
                    const float4 l1 = W.pd_l1[slot], lr = W.vol_li[slot], t = W.trw_tr[slot];
                    const C3 lightLi = c3(lr.x, lr.y, lr.z) * c3(t.x, t.y, t.z);
                    if (!IsBlack(lightLi)) le = le + c3(l1.x, l1.y, l1.z) * lightLi * l1.w / W.pd_mis[slot].z;
                }
                if (fl & F_L2) {
                    const float4 fr2 = W.pd_fr[slot], mi = W.pd_mis[slot], li = W.itw_o[slot], t = W.itw_tr[slot];
                    const C3 L = c3(li.x, li.y, li.z);
                    if (!IsBlack(L)) le = le + c3(fr2.x, fr2.y, fr2.z) * L * c3(t.x, t.y, t.z) * fr2.w / mi.x;
                }
                direct = direct + le / pc.w;
            }
            radiance = radiance + c3(pc.x, pc.y, pc.z) * direct;
            fl &= ~(F_PENDING | F_L1 | F_L2 | F_DZERO);
        }
        if (fl & F_DONE) break;
        if (fl & F_CONT) {                       /* 3. the continuation sampled with the term */
            fl &= ~F_CONT;
            ext = true;
            break;
        }
        if (pass == 1) break;
        /* 4. one iteration of the Li loop on the extension hit */
        int2 bc = W.bounce[slot];
        int bounces = bc.x, guard = bc.y;
        float4 ro = W.ray_o[slot], rd = W.ray_d[slot];
        Ray ray = mkray(v3(ro.x, ro.y, ro.z), v3(rd.x, rd.y, rd.z), ro.w, rd.w);
        int env = W.vol_env[slot];
        const int4 px = W.pix[slot];
        Rng rand;
        rng_resume(rand, P.seed, (uint32_t)(P.x0 + px.x), (uint32_t)(P.y0 + px.y), (uint32_t)px.w, W.rng_n[slot]);
        bool isSpecularPath = (fl & F_SPECULAR) != 0;
        bool done = false, rr = true;
        do {
            if (++guard > RT_LOOP_CAP) { atomicOr(status, RT_STATUS_ITER); done = true; break; }
            const V3 wo = -ray.D;
            if (ray.MaxT <= ray.MinT) { done = true; break; }
            Isect it;
            const bool isHit = load_hit(S, ray, W.ext_hit[slot], W.ext_sub[slot], &it);
            MedSample msr; msr.sampled = false;
            if (env >= 0) {
                const Ray realRay = mkray(ray.O, ray.D, ray.MinT, isHit ? it.T : kFMax);
                msr = MedSampleDist(S->media[env], realRay, rand);
                coeff = coeff * msr.Tr;
            }
            if (IsBlack(coeff)) { done = true; break; }
            if (msr.sampled) {
                if (bounces >= P.max_depth) { done = true; break; }   /* VolumetricPathTracer.cs:55 */
                const RtMedium& M = S->media[env];
                int light;
                const float lightPdf = SampleLight(S, rand, &light);
                fl |= F_PENDING;
                W.pd_coeff[slot] = make_float4(coeff.r, coeff.g, coeff.b, lightPdf);
                if (lightPdf > 0.0f) {
                    const LSample ls = LightSampleLi(S, light, msr.P, rand);
                    if (ls.Pdf > 0.0f && !IsBlack(ls.Li)) {
                        const float p = MedP(M, msr.Wo, ls.Wi);
                        if (p != 0.0f) {
                            fl |= F_L1 | F_WTR;
                            const float weight = PowerHeuristic(ls.Pdf, p);
                            W.pd_l1[slot] = make_float4(p, p, p, weight);
                            W.vol_li[slot] = make_float4(ls.Li.r, ls.Li.g, ls.Li.b, 0.0f);
                            const V3 dir = Normalize(ls.P - msr.P);
                            W.trw_start[slot] = make_float4(msr.P.x, msr.P.y, msr.P.z, __int_as_float(env));
                            W.trw_end[slot] = make_float4(ls.P.x, ls.P.y, ls.P.z, __int_as_float(0));
                            W.trw_dir[slot] = make_float4(dir.x, dir.y, dir.z, 0.0f);
                            W.trw_tr[slot] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
                        }
                    }
                    V3 swi;
                    const float sp = MedSampleWi(M, msr.Wo, rand, &swi);
                    if (sp > 0) {
                        const float b2l = LightPdfLi(S, light, msr.P, swi);
                        if (b2l != 0.0f) {
                            fl |= F_L2 | F_WIT;
                            const float weight = PowerHeuristic(sp, b2l);
                            const Ray toLight = mkray(msr.P, swi);
                            W.pd_fr[slot] = make_float4(sp, sp, sp, weight);
                            W.pd_mis[slot] = make_float4(sp, __int_as_float(light), ls.Pdf, 0.0f);
                            W.pd_w[slot] = make_float4(-swi.x, -swi.y, -swi.z, 0.0f);
                            W.itw_o[slot] = make_float4(toLight.O.x, toLight.O.y, toLight.O.z, toLight.MinT);
                            W.itw_d[slot] = make_float4(toLight.D.x, toLight.D.y, toLight.D.z, 0.0f);
                            W.itw_tr[slot] = make_float4(1.0f, 1.0f, 1.0f, __int_as_float(pack_env(env, 0)));
                        } else {
                            W.pd_mis[slot] = make_float4(sp, __int_as_float(light), ls.Pdf, 0.0f);
                        }
                    } else {
                        W.pd_mis[slot] = make_float4(0.0f, __int_as_float(light), ls.Pdf, 0.0f);
                    }
                } else {
                    fl |= F_DZERO;
                }
                V3 swi;
                MedSampleWi(M, wo, rand, &swi);
                ray = mkray(msr.P, swi, ray.MinT);
                isSpecularPath = false;
            } else {
                if (bounces == 0 || isSpecularPath) {
                    if (isHit) radiance = radiance + coeff * IsectLe(S, it, wo);
                    else radiance = radiance + coeff * EvalAllInfinite(S, ray.D);
                }
                if (!isHit) { done = true; break; }
                if (P.max_depth != -1 && bounces >= P.max_depth) { done = true; break; }
                if (!HasSurface(S, it)) {
                    ray = mkray(it.P, ray.D, ray.MinT);
                    env = GetMedium(S, it, ray.D);
                    bounces--;
                    rr = false;                  /* `continue`: no Russian roulette this iteration */
                    break;
                }
                const int mat = PrimOf(S, it).material;
                int light;
                const float lightPdf = SampleLight(S, rand, &light);
                fl |= F_PENDING;
                W.pd_coeff[slot] = make_float4(coeff.r, coeff.g, coeff.b, lightPdf);
                if (lightPdf > 0.0f) {
                    const V3 wod = it.Wr;
                    const LSample ls = LightSampleLi(S, light, it.P, rand);
                    if (ls.Pdf > 0.0f && !IsBlack(ls.Li)) {
                        C3 fr = MatFr(S, mat, Lo(it, wod), Lo(it, ls.Wi), it.UV);
                        const float scatteringPdf = MatPdf(S, mat, Lo(it, wod), Lo(it, ls.Wi), it.UV);
                        if (!IsBlack(fr)) {
                            fl |= F_L1 | F_WTR;
                            fr = fr * AbsCosTheta(Lo(it, ls.Wi));
                            const float weight = PowerHeuristic(ls.Pdf, scatteringPdf);
                            W.pd_l1[slot] = make_float4(fr.r, fr.g, fr.b, weight);
                            W.vol_li[slot] = make_float4(ls.Li.r, ls.Li.g, ls.Li.b, 0.0f);
                            const V3 dir = Normalize(ls.P - it.P);
                            W.trw_start[slot] = make_float4(it.P.x, it.P.y, it.P.z, __int_as_float(env));
                            W.trw_end[slot] = make_float4(ls.P.x, ls.P.y, ls.P.z, __int_as_float(0));
                            W.trw_dir[slot] = make_float4(dir.x, dir.y, dir.z, 0.0f);
                            W.trw_tr[slot] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
                        }
                    }
                    const BSample sample = MatSample(S, mat, Lo(it, wod), it.UV, rand);
                    const C3 fr = sample.Fr * AbsCosTheta(sample.Wi);
                    const float scatteringPdf = sample.Pdf;
                    const bool sampledSpecular = (sample.Type & BX_SPECULAR) != 0;
                    float mis_pdf = 0.0f;
                    if (!IsBlack(fr) && scatteringPdf > 0) {
                        float weight = 1;
                        bool go = true;
                        if (!sampledSpecular) {
                            const float b2l = LightPdfLi(S, light, it.P, Wo(it, sample.Wi));
                            if (b2l == 0.0f) go = false;
                            else weight = PowerHeuristic(scatteringPdf, b2l);
                        }
                        if (go) {
                            fl |= F_L2 | F_WIT;
                            mis_pdf = scatteringPdf;
                            const Ray toLight = Spawn(it, Wo(it, sample.Wi));
                            const V3 wle = Wo(it, -sample.Wi);
                            W.pd_fr[slot] = make_float4(fr.r, fr.g, fr.b, weight);
                            W.pd_w[slot] = make_float4(wle.x, wle.y, wle.z, 0.0f);
                            W.itw_o[slot] = make_float4(toLight.O.x, toLight.O.y, toLight.O.z, toLight.MinT);
                            W.itw_d[slot] = make_float4(toLight.D.x, toLight.D.y, toLight.D.z, 0.0f);
                            W.itw_tr[slot] = make_float4(1.0f, 1.0f, 1.0f, __int_as_float(pack_env(env, 0)));
                        }
                    }
                    W.pd_mis[slot] = make_float4(mis_pdf, __int_as_float(light), ls.Pdf, 0.0f);
                } else {
                    fl |= F_DZERO;
                }
                const BSample sample = MatSample(S, mat, Lo(it, wo), it.UV, rand);
                isSpecularPath = (sample.Type & BX_SPECULAR) != 0;
                if (sample.Pdf > 0.0f) coeff = coeff * (sample.Fr * AbsCosTheta(sample.Wi) / sample.Pdf);
                else { done = true; break; }
                const V3 nextDir = Wo(it, sample.Wi);
                ray = mkray(it.P, nextDir, ray.MinT);
                env = GetMedium(S, it, nextDir);
            }
        } while (false);
        if (!done && rr && bounces > P.min_depth) {
            const float q = nmin(MaxElement(coeff), P.rr);
            if (NextFloat(rand) > q) done = true;
            else coeff = coeff / q;
        }
        if (!done) {
            bounces++;
            fl |= F_CONT;
            W.ray_o[slot] = make_float4(ray.O.x, ray.O.y, ray.O.z, ray.MinT);
            W.ray_d[slot] = make_float4(ray.D.x, ray.D.y, ray.D.z, ray.MaxT);
            W.vol_env[slot] = env;
        } else {
            fl |= F_DONE;
        }
        W.bounce[slot] = make_int2(bounces, guard);
        W.rng_n[slot] = rand.n;
        fl = (fl & ~F_SPECULAR) | (isSpecularPath ? F_SPECULAR : 0u);
        /* start the walks of the new direct term; if there are none, resolve it now */
        if (fl & F_WTR) {
            if (!trw_next(W, slot)) fl &= ~F_WTR;
        }
        if (fl & (F_WTR | F_WIT)) break;
    }
    W.coeff[slot] = make_float4(coeff.r, coeff.g, coeff.b, 0.0f);
    W.rad[slot] = make_float4(radiance.r, radiance.g, radiance.b, 0.0f);
    if (ext || (fl & (F_WTR | F_WIT))) {
        W.flags[slot] = fl;
        o->trw = (fl & F_WTR) != 0;
        o->itw = (fl & F_WIT) != 0;
        o->ext = ext;
        o->keep = true;
        return;
    }
    /* the path is over */
    finish_path(J, W, slot, radiance, stats, WF_PASS_RENDER);
    if (counting) warp_add64(stats + 0, 1u);
    o->restart = true;
}

/* The vol_path shade's queue appends for the block: a Transmittance segment
 * takes the first closest-hit position of the lane, an IntersectTr segment or
 * the extension ray the second; a finished path's slot takes the next camera
 * sample at once. */
DF void vol_queues(const WfState& W, int slot, int next, VolOut& o) {
    const long long sid = claim_sample(W, 0xffffffffu, o.restart);
    float4 ro, rd;
    if (o.restart && init_path(W, slot, sid, &ro, &rd)) { o.ext = true; o.keep = true; }
    int qs, qt, qe, qa;
    queue_append<true>(W, next, false, o.trw, o.itw || o.ext, o.keep, &qs, &qt, &qe, &qa);
    if (o.trw) {
        float4 to, td;
        trw_ray(W, slot, &to, &td);
        push_ray4(W, qt, slot, WF_RAY_TRW, to, td);
    }
    if (o.itw) {
        const float4 io = W.itw_o[slot], id = W.itw_d[slot];
        push_ray4(W, qe, slot, WF_RAY_MIS, io, make_float4(id.x, id.y, id.z, kFMax));
    } else if (o.ext) {
        if (!o.restart) { ro = W.ray_o[slot]; rd = W.ray_d[slot]; }
        push_ray4(W, qe, slot, WF_RAY_EXT, ro, rd);
    }
    if (o.keep) set_active(W, next, qa, slot);
    else clear_active(W, slot);
}

__global__ void __launch_bounds__(128, RT_VSHADE_BLOCKS) k_wf_shade_vol(WfState W, uint32_t* status, unsigned long long* stats,
                                                         bool counting, bool sorted) {
    const int cur = W.ctr->iter & 1;
    const int n = min(W.ctr->n_active[cur], W.slots);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int slot = -1;
    VolOut o;
    o.trw = o.itw = o.ext = o.keep = o.restart = false;
    if (i < n) { slot = sorted ? W.sorted[i] : W.active[cur][i]; shade_vol_path(&o, W, slot, status, stats, counting); }
    vol_queues(W, slot, cur ^ 1, o);
}

/* the active paths of this iteration, one thread each over the sorted list
 * (or, `sorted` false, the active list as built): either a grid sized to the
 * active count, or (kDynamic, inside a graph where the count is unknown at
 * launch) a resident grid whose warps take the next 32 entries from a
 * counter until the list is done.  The replay pass of the adjoint (kAdj)
 * sums its alpha gradients per block in shared memory. */
template <bool kAdj, bool kDynamic>
__global__ void __launch_bounds__(128, (kAdj || kDynamic) ? 5 : RT_SHADE_BLOCKS) k_wf_shade(WfState W, uint32_t* status, unsigned long long* stats, bool counting,
                                                       int pass, WfAdjoint A, bool sorted) {
    const int32_t* list;
    __shared__ float s_alpha[kAdj ? RT_ADJ_MAX_ALPHA : 1];
    if (kAdj) {
        for (int i = threadIdx.x; i < A.n_alpha; i += blockDim.x) s_alpha[i] = 0.0f;
        __syncthreads();
    }
    const int cur = W.ctr->iter & 1;
    const int n = min(W.ctr->n_active[cur], W.slots);
    list = sorted ? W.sorted : W.active[cur];
    if (!kDynamic) {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        int slot = -1;
        PathOut o;
        o.shadow = o.mis = o.ext = o.keep = o.restart = false;
        if (i < n) { slot = list[i]; shade_path<kAdj>(&o, W, slot, status, stats, counting, pass, A, s_alpha); }
        path_queues<true>(W, slot, cur ^ 1, o);
    } else {
        const int lane = threadIdx.x & 31;
        while (true) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&W.ctr->shade_fetch, 32);
            base = __shfl_sync(kFullWarp, base, 0);
            if (base >= n) break;
            const int i = base + lane;
            int slot = -1;
            PathOut o;
            o.shadow = o.mis = o.ext = o.keep = o.restart = false;
            if (i < n) { slot = list[i]; shade_path<kAdj>(&o, W, slot, status, stats, counting, pass, A, s_alpha); }
            __syncwarp();
            path_queues<false>(W, slot, cur ^ 1, o);
        }
    }
    if (kAdj) {
        __syncthreads();
        for (int i = threadIdx.x; i < A.n_alpha; i += blockDim.x)
            if (s_alpha[i] != 0.0f) atomicAdd(A.grad_alpha + i, s_alpha[i]);
    }
}

/* ---- light tracing (AdjointParticleIntegrator.EmitParticle, AdjointParticleIntegrator.cs:24-79) ----
 * A slot holds one particle; the job's `samples` is the film sums (float4 per
 * pixel) and its `first` the index of the round's first particle.  The loop
 * is cut at its two ray casts: the extension ray (Scene.Intersect) and the
 * camera connection's shadow ray (Scene.IsOccluded), both traced in the next
 * trace phase.  A shade runs one vertex: camera connection (its splat waits
 * in pd_l1 and the shadow-ray kernel adds it when the way is clear),
 * importance-mode BSDF sample, and the top of the reference's loop (depth
 * limit, Russian roulette) before the next extension ray, so the random
 * numbers are drawn in the reference's order.  A finished particle's slot
 * takes the next particle at once: the new particle writes no splat before
 * the pending shadow ray has been traced. */

/* top of the bounce loop (AdjointParticleIntegrator.cs:34-42); false ends the particle */
DF bool particle_continue(const RtParams& P, int bounces, C3* coeff, Rng& rand) {
    if (P.max_depth != -1 && bounces >= P.max_depth) return false;
    if (bounces > P.min_depth) {
        if (NextFloat(rand) > P.rr) return false;
        *coeff = *coeff / P.rr;
    }
    return true;
}

/* What a light-tracer shade leaves for the queues: the camera connection's
 * splat ray, the next extension ray, and whether the slot holds a particle
 * for the next iteration.  The kernel appends them for the whole block. */
struct PartOut {
    float4 so, sd, eo, ed;
    bool splat, ext, keep;
};

/* Claims particles for `slot`, the first one `sid` (claimed by the caller),
 * until one has an extension ray to trace (a particle can end before its
 * first ray: no light, black emission, depth limit or roulette).  The ray
 * goes to `o`; o->keep is false once every particle of the round is claimed. */
DF void start_particle(const WfState& W, int slot, long long sid, PartOut* o) {
    const WfJob& J = W.jobs[0];
    const RtSceneView* S = J.view;
    const RtParams P = J.P;
    for (bool first = true;; first = false) {
        if (!first) sid = (long long)atomicAdd(&W.ctr->next_sample, 1ull);
        if (sid >= W.ctr->total) { W.flags[slot] = 0; o->keep = false; return; }
        const long long i = J.first + sid;
        Rng rand;
        rng_init(rand, P.seed, (uint32_t)(uint64_t)i, (uint32_t)((uint64_t)i >> 32), RT_PARTICLE_STREAM);
        int light;
        const float selectPdf = SampleLight(S, rand, &light);
        if (selectPdf == 0.0f) continue;
        const Emit e = LightSampleEmit(S, light, rand);
        if (IsBlack(e.le)) continue;
        C3 coeff = e.le * AbsDot(e.dir, e.n) / (selectPdf * e.pdf_pos * e.pdf_dir);
        const Ray ray = mkray(e.pos, e.dir, 0.0001f);
        if (!particle_continue(P, 1, &coeff, rand)) continue;
        W.job[slot] = 0;
        W.pix[slot] = make_int4((int)(uint32_t)(uint64_t)i, (int)(uint32_t)((uint64_t)i >> 32), 0, 0);
        W.rng_n[slot] = rand.n;
        W.coeff[slot] = make_float4(coeff.r, coeff.g, coeff.b, 0.0f);
        W.bounce[slot] = make_int2(1, 1);
        W.flags[slot] = F_ALIVE | F_EXT;
        ray4(ray, &o->eo, &o->ed);
        W.ray_o[slot] = o->eo;
        W.ray_d[slot] = o->ed;
        o->ext = true;
        o->keep = true;
        return;
    }
}

/* The warp's lanes with `want` claim consecutive particle ids with one atomic;
 * -1 for the others.  Every lane of the warp calls it. */
DF long long claim_particle(const WfState& W, bool want) {
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if (!m) return -1;
    const int leader = __ffs(m) - 1, lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(&W.ctr->next_sample, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    return want ? (long long)base + __popc(m & ((1u << lane) - 1u)) : -1;
}

/* queue the block's splat and extension rays and its next active slots */
DF void particle_queues(const WfState& W, int slot, int next, const PartOut& o) {
    int qs, qm, qe, a;
    queue_append<true>(W, next, o.splat, false, o.ext, o.keep, &qs, &qm, &qe, &a);
    if (o.splat) push_ray4(W, qs, slot, WF_RAY_SPLAT, o.so, o.sd);
    if (o.ext) push_ray4(W, qe, slot, WF_RAY_EXT, o.eo, o.ed);
    if (o.keep) set_active(W, next, a, slot);
    else clear_active(W, slot);
}

__global__ void __launch_bounds__(256) k_wf_start_particles(WfState W) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    PartOut o;
    o.splat = o.ext = o.keep = false;
    const bool in = slot < W.slots;
    const long long sid = claim_particle(W, in);
    if (in) start_particle(W, slot, sid, &o);
    /* the first active list is built from the slots' flags afterwards */
    int qs, qm, qe, a;
    queue_append<true>(W, 0, false, false, o.ext, false, &qs, &qm, &qe, &a);
    if (o.ext) push_ray4(W, qe, slot, WF_RAY_EXT, o.eo, o.ed);
}

/* One vertex of the slot's particle; its rays go to `o`.  Returns true when
 * the particle is over (the caller starts the next one in the slot). */
DF bool shade_particle(const WfState& W, int slot, uint32_t* status, PartOut* o) {
    const WfJob& J = W.jobs[0];
    const RtSceneView* S = J.view;
    const RtParams P = J.P;
    uint32_t fl = W.flags[slot];
    bool done = (fl & F_DONE) != 0;
    if (!done) {
        /* 1. the vertex at the extension hit */
        int2 bc = W.bounce[slot];
        int bounces = bc.x, guard = bc.y;
        const float4 cf = W.coeff[slot];
        C3 coeff = c3(cf.x, cf.y, cf.z);
        const float4 ro = W.ray_o[slot], rdd = W.ray_d[slot];
        const Ray ray = mkray(v3(ro.x, ro.y, ro.z), v3(rdd.x, rdd.y, rdd.z), ro.w, rdd.w);
        const int4 id = W.pix[slot];
        Rng rand;
        rng_resume(rand, P.seed, (uint32_t)id.x, (uint32_t)id.y, RT_PARTICLE_STREAM, W.rng_n[slot]);
        Ray nray = ray;
        bool ext = false;
        do {
            Isect it;
            if (!load_hit(S, ray, W.ext_hit[slot], W.ext_sub[slot], &it)) { done = true; break; }
            if (HasSurface(S, it)) {
                const int mat = PrimOf(S, it).material;
                const V3 wo = Lo(it, it.Wr);
                CamWi cw;
                if (CameraSampleWi(S->camera, it.P, &cw) && cw.we != 0.0f) {
                    /* Scene.IsOccluded(camera, it.P): closer than 0.001 counts as occluded, no ray */
                    const V3 vec = it.P - cw.pos;
                    const float dis = Length(vec);
                    if (!(dis < 0.001f)) {
                        const V3 wi = Lo(it, cw.dir);
                        const C3 f = MatFr<true>(S, mat, wo, wi, it.UV);
                        const C3 color = coeff * f * cw.we * AbsCosTheta(wi);
                        int pix = -1;   /* a NaN position (the reference throws) splats nothing */
                        if (cw.sx == cw.sx && cw.sy == cw.sy) {
                            const int x = (int)floorf(cw.sx), y = (int)floorf(cw.sy);
                            if (x >= 0 && x < S->camera.width && y >= 0 && y < S->camera.height)
                                pix = x * S->camera.height + y;
                        }
                        W.pd_l1[slot] = make_float4(color.r, color.g, color.b, __int_as_float(pix));
                        ray4(mkray(cw.pos, Normalize(vec), 0.0001f, dis - 0.0001f), &o->so, &o->sd);
                        o->splat = true;
                    }
                }
                const BSample bs = MatSample<true>(S, mat, wo, it.UV, rand);
                if (bs.Pdf > 0.0f) coeff = coeff * (bs.Fr * AbsCosTheta(bs.Wi) / bs.Pdf);
                else { done = true; break; }
                nray = Spawn(it, Wo(it, bs.Wi));
                bounces++;
            } else {
                nray = mkray(it.P, ray.D, ray.MinT);   /* bounces-- and continue: the same depth again */
            }
            /* 2. the top of the next loop iteration */
            if (++guard > RT_LOOP_CAP) { atomicOr(status, RT_STATUS_ITER); done = true; break; }
            if (!particle_continue(P, bounces, &coeff, rand)) { done = true; break; }
            ext = true;
        } while (false);
        if (ext) {
            ray4(nray, &o->eo, &o->ed);
            o->ext = true;
            W.ray_o[slot] = o->eo;
            W.ray_d[slot] = o->ed;
        }
        W.bounce[slot] = make_int2(bounces, guard);
        W.rng_n[slot] = rand.n;
        W.coeff[slot] = make_float4(coeff.r, coeff.g, coeff.b, 0.0f);
        if (done) fl |= F_DONE;
    }
    if (!(fl & F_DONE)) {
        W.flags[slot] = fl;
        o->keep = true;
        return false;
    }
    return true;
}

/* `sorted`: the list regrouped by shade key, else the active list as built
 * (scenes of one material type gain nothing from the regrouping) */
__global__ void __launch_bounds__(128, RT_PSHADE_BLOCKS) k_wf_shade_particle(WfState W, uint32_t* status, bool sorted) {
    const int cur = W.ctr->iter & 1;
    const int n = min(W.ctr->n_active[cur], W.slots);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int slot = -1;
    PartOut o;
    o.splat = o.ext = o.keep = false;
    bool restart = false;
    if (i < n) { slot = sorted ? W.sorted[i] : W.active[cur][i]; restart = shade_particle(W, slot, status, &o); }
    /* a finished particle's slot takes the next particle at once */
    const long long sid = claim_particle(W, restart);
    if (restart) start_particle(W, slot, sid, &o);
    particle_queues(W, slot, cur ^ 1, o);
}

__global__ void k_wf_active_init(WfState W) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W.slots) return;
    bool alive = (W.flags[i] & F_ALIVE) != 0;
    int a = warp_append(&W.ctr->n_active[0], alive);
    if (alive) set_active(W, 0, a, i);
    else W.mark[i] = 0;
}

/* Code key of an active path: which code the shade kernel will run for it.
 * 0 finished (pending term, then a new sample), 1 missed the scene, 2 hit a
 * medium boundary without a surface, 3 + RT_MAT_* hit that material type,
 * 15 vol_path boundary walks.  The shade key puts the job (mod 64) above it,
 * so a batch shades - and then traces - one scene's paths together. */
DF int shade_key(const WfState& W, int slot) {
    const uint32_t fl = W.flags[slot];
    const int job = W.job[slot];
    const int jk = (job & 63) << 4;
    if (fl & (F_WTR | F_WIT)) return jk | 15;
    if (fl & F_DONE) return jk;
    const int hs = __float_as_int(W.ext_hit[slot].w);
    if (hs < 0) return jk | 1;
    const RtSceneView* S = W.jobs[job].view;
    const int prim = __float_as_int(__ldg(S->slots + 3 * (int64_t)hs).w);
    const int m = S->prims[prim].material;
    if (m < 0) return jk | 2;
    return jk | min(3 + S->materials[m].type, 14);
}

/* between trace and shade: the queues are consumed, reset their counters */
__global__ void k_wf_phase(WfState W) {
    if (threadIdx.x == 0) {
        WfCounters* c = W.ctr;
        c->n_closest = 0; c->n_shadow = 0; c->fetch[0] = 0; c->fetch[1] = 0; c->shade_fetch = 0;
        c->n_active[(c->iter & 1) ^ 1] = 0;
    }
    for (int k = threadIdx.x; k < 2 * WF_SHADE_KEYS; k += blockDim.x) W.key_count[k] = 0;
}

/* The sort's input order.  While at least one slot in WF_DENSE_SORT is active
 * (and the run allows it: W.dense_sort),
 * the sort walks the slots in index order (their marks say which are on this
 * iteration's list): a warp's entries of one key then land together in slot
 * order, so the shade's warps read path state of nearby slots - fewer sectors
 * per field than the appended list's scattered order.  Below that it walks the
 * active list itself.  Both kernels take the same decision from the same count. */
#ifndef WF_DENSE_SORT
#define WF_DENSE_SORT 8
#endif
DF bool sort_dense(const WfState& W, int n) { return W.dense_sort && n * WF_DENSE_SORT >= W.slots; }
DF int sort_span(const WfState& W, int n) { return sort_dense(W, n) ? W.slots : n; }
/* entry i of the sort's input: a slot, or -1 (a slot not on the list) */
DF int sort_input(const WfState& W, int cur, int n, int i) {
    if (!sort_dense(W, n)) return W.active[cur][i];
    return W.mark[i] == cur + 1 ? i : -1;
}

/* both sort kernels are grid-stride loops: one pass with a grid sized to the
 * active count, several with a resident grid inside a graph */
__global__ void __launch_bounds__(256) k_wf_sort_count(WfState W) {
    const int cur = W.ctr->iter & 1;
    const int n = min(W.ctr->n_active[cur], W.slots);
    const int span = sort_span(W, n);
    for (int i0 = blockIdx.x * blockDim.x; i0 < span; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + threadIdx.x;
        if (i >= span) break;
        const int slot = sort_input(W, cur, n, i);
        if (slot < 0) continue;
        const int key = shade_key(W, slot);
        W.sort_key[i] = (uint16_t)key;
        const unsigned peers = __match_any_sync(__activemask(), key);
        if ((threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1)) atomicAdd(W.key_count + key, __popc(peers));
    }
}

/* counting-sort scatter: entries of one key stay together, in any order
 * (every path's result is independent of the order paths are shaded in).
 * Each block turns the key counts into bases with a shared-memory scan. */
#define WF_KEYS_PER_THREAD (WF_SHADE_KEYS / 256)
static_assert(WF_SHADE_KEYS % 256 == 0, "the scatter's scan gives each of 256 threads the same number of keys");
__global__ void __launch_bounds__(256) k_wf_sort_scatter(WfState W) {
    __shared__ int base[WF_SHADE_KEYS];
    __shared__ int part[256];
    const int cur = W.ctr->iter & 1;
    const int n = min(W.ctr->n_active[cur], W.slots);
    const int span = sort_span(W, n);
    if ((int)(blockIdx.x * blockDim.x) >= span) return;
    const int t = threadIdx.x;
    /* exclusive scan of the key counts: each thread sums its run of keys,
     * the 256 sums are scanned (Hillis-Steele), then each run is filled in */
    int v[WF_KEYS_PER_THREAD], sum = 0;
#pragma unroll
    for (int j = 0; j < WF_KEYS_PER_THREAD; j++) { v[j] = W.key_count[t * WF_KEYS_PER_THREAD + j]; sum += v[j]; }
    part[t] = sum;
    __syncthreads();
    for (int off = 1; off < 256; off <<= 1) {
        const int add = t >= off ? part[t - off] : 0;
        __syncthreads();
        part[t] += add;
        __syncthreads();
    }
    int run = part[t] - sum;
#pragma unroll
    for (int j = 0; j < WF_KEYS_PER_THREAD; j++) { base[t * WF_KEYS_PER_THREAD + j] = run; run += v[j]; }
    __syncthreads();
    const unsigned lane = threadIdx.x & 31;
    for (int i0 = blockIdx.x * blockDim.x; i0 < span; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + threadIdx.x;
        if (i >= span) break;
        const int slot = sort_input(W, cur, n, i);
        if (slot < 0) continue;
        const int key = W.sort_key[i];
        const unsigned peers = __match_any_sync(__activemask(), key);
        const int leader = __ffs(peers) - 1;
        int first = 0;
        if ((int)lane == leader) first = atomicAdd(W.key_count + WF_SHADE_KEYS + key, __popc(peers));
        first = __shfl_sync(peers, first, leader);
        const int dst = base[key] + first + __popc(peers & ((1u << lane) - 1u));
        if (in_bounds(W, dst, W.slots)) W.sorted[dst] = slot;
    }
}

/* end of an iteration: the next active list becomes current */
__global__ void k_wf_tail(WfState W) {
    if (threadIdx.x == 0) W.ctr->iter++;
}
__global__ void k_wf_tail_loop(WfState W, cudaGraphConditionalHandle loop, uint32_t* status) {
    if (threadIdx.x == 0) {
        const int next = (W.ctr->iter & 1) ^ 1;
        W.ctr->iter++;
        /* queued shadow rays keep the loop going: a finished light-tracer
         * particle leaves its last splat in the queue without an active slot */
        bool more = W.ctr->n_active[next] > 0 || W.ctr->n_shadow > 0;
        if (more && W.ctr->iter >= W.iter_cap) { atomicOr(status, RT_STATUS_WFITER); more = false; }
        cudaGraphSetConditional(loop, more ? 1u : 0u);
    }
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

/* resident blocks of a grid-stride kernel: every SM filled once */
template <typename K>
int resident_blocks(K kernel, int block) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess || per_sm <= 0)
        per_sm = 1, sms = sms > 0 ? sms : 1;
    return sms * per_sm;
}

}  // namespace

cudaError_t rt_wf_start(const WfState& W, cudaStream_t s, bool particle) {
    if (particle) k_wf_start_particles<<<grid_for(W.slots, 256), 256, 0, s>>>(W);
    else k_wf_start<<<grid_for(W.slots, 256), 256, 0, s>>>(W);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_wf_active_init<<<grid_for(W.slots, 256), 256, 0, s>>>(W);
    return cudaGetLastError();
}

cudaError_t rt_wf_trace(const WfState& W, uint32_t* status, unsigned long long* stats, bool counting, cudaStream_t s,
                        bool deep, bool wide, const WfFork* fork) {
    static const int closest_blocks[4] = {resident_blocks(k_wf_trace_closest<false, false>, RT_TRACE_BLOCK),
                                          resident_blocks(k_wf_trace_closest<true, false>, RT_TRACE_BLOCK),
                                          resident_blocks(k_wf_trace_closest<false, true>, RT_TRACE_BLOCK),
                                          resident_blocks(k_wf_trace_closest<true, true>, RT_TRACE_BLOCK)};
    static const int shadow_blocks[4] = {resident_blocks(k_wf_trace_shadow<false, false>, RT_TRACE_BLOCK),
                                         resident_blocks(k_wf_trace_shadow<true, false>, RT_TRACE_BLOCK),
                                         resident_blocks(k_wf_trace_shadow<false, true>, RT_TRACE_BLOCK),
                                         resident_blocks(k_wf_trace_shadow<true, true>, RT_TRACE_BLOCK)};
    const int v = (deep ? 1 : 0) + (wide ? 2 : 0);
    cudaError_t e = cudaSuccess;
    if (fork) {
        e = cudaEventRecord(fork->fork, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(fork->side, fork->fork, 0);
        if (e != cudaSuccess) return e;
    }
    switch (v) {
    case 0: k_wf_trace_closest<false, false><<<closest_blocks[0], RT_TRACE_BLOCK, 0, s>>>(W, status, stats, counting); break;
    case 1: k_wf_trace_closest<true, false><<<closest_blocks[1], RT_TRACE_BLOCK, 0, s>>>(W, status, stats, counting); break;
    case 2: k_wf_trace_closest<false, true><<<closest_blocks[2], RT_TRACE_BLOCK, 0, s>>>(W, status, stats, counting); break;
    default: k_wf_trace_closest<true, true><<<closest_blocks[3], RT_TRACE_BLOCK, 0, s>>>(W, status, stats, counting); break;
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const cudaStream_t ss = fork ? fork->side : s;
    switch (v) {
    case 0: k_wf_trace_shadow<false, false><<<shadow_blocks[0], RT_TRACE_BLOCK, 0, ss>>>(W, status, stats, counting); break;
    case 1: k_wf_trace_shadow<true, false><<<shadow_blocks[1], RT_TRACE_BLOCK, 0, ss>>>(W, status, stats, counting); break;
    case 2: k_wf_trace_shadow<false, true><<<shadow_blocks[2], RT_TRACE_BLOCK, 0, ss>>>(W, status, stats, counting); break;
    default: k_wf_trace_shadow<true, true><<<shadow_blocks[3], RT_TRACE_BLOCK, 0, ss>>>(W, status, stats, counting); break;
    }
    e = cudaGetLastError();
    if (e != cudaSuccess || !fork) return e;
    e = cudaEventRecord(fork->join, fork->side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, fork->join, 0);
    return e;
}

cudaError_t rt_wf_shade(const WfState& W, int n_hint, uint32_t* status, unsigned long long* stats, bool counting,
                        cudaGraphConditionalHandle loop, bool has_loop, cudaStream_t s, uint64_t* launches,
                        int pass, const WfAdjoint* adj, bool vol, bool particle, bool sort) {
    static const int sort_blocks = resident_blocks(k_wf_sort_scatter, 256);
    static const int shade_blocks = resident_blocks(k_wf_shade<false, true>, 128);
    const WfAdjoint A = adj ? *adj : WfAdjoint{-1, 0, nullptr, nullptr, nullptr, nullptr};
    const bool known = n_hint >= 0;
    const int n = known ? std::min(n_hint, W.slots) : W.slots;
    k_wf_phase<<<1, 256, 0, s>>>(W);
    if (n > 0) {
        const unsigned sb = known ? grid_for(n, 256) : (unsigned)sort_blocks;
        if (sort) {
            k_wf_sort_count<<<sb, 256, 0, s>>>(W);
            k_wf_sort_scatter<<<sb, 256, 0, s>>>(W);
        } else {
            *launches -= 2;
        }
        if (particle) k_wf_shade_particle<<<grid_for(n, 128), 128, 0, s>>>(W, status, sort);
        else if (vol) k_wf_shade_vol<<<grid_for(n, 128), 128, 0, s>>>(W, status, stats, counting, sort);
        else if (!known) k_wf_shade<false, true><<<shade_blocks, 128, 0, s>>>(W, status, stats, counting, pass, A, sort);
        else if (pass == WF_PASS_REPLAY) k_wf_shade<true, false><<<grid_for(n, 128), 128, 0, s>>>(W, status, stats, counting, pass, A, sort);
        else k_wf_shade<false, false><<<grid_for(n, 128), 128, 0, s>>>(W, status, stats, counting, pass, A, sort);
        *launches += 3;
    }
    if (has_loop) k_wf_tail_loop<<<1, 32, 0, s>>>(W, loop, status);
    else k_wf_tail<<<1, 32, 0, s>>>(W);
    *launches += 2;
    return cudaGetLastError();
}
