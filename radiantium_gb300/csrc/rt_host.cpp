/*
 * rt_host.cpp - host runtime of the GB300 path tracer and the C ABI
 * (include/radiantium.h).
 *
 * rt_upload_scene flattens the scene description exactly as
 * RendererBuilder.Build orders it (RendererBuilder.cs:942-1004): primitives per
 * entity (spheres, mesh triangles, instances), one DiffuseAreaLight per
 * emissive primitive, infinite lights in entity order; builds the reference's
 * SAH trees (rt_bvh.cpp) for every instanced prototype and the top level;
 * and uploads the device layout of rt_types.h.  Compiled with
 * -ffp-contract=off so derived values (edges, areas, centroids, CDFs) round
 * exactly like the reference's single-precision code.
 */
#include <cuda_runtime.h>
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits.h>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/radiantium.h"
#include "../../include/rt_detmath.h"
#include "rt_bvh.h"
#include "rt_bvh_gpu.h"
#include "rt_launch.h"
#include "rt_types.h"
#include <nvtx3/nvToolsExt.h>
#include "rt_wavefront.h"

static std::atomic<unsigned long long> g_device_allocs{0};

cudaError_t rt_dev_malloc(void** p, size_t bytes) {
    g_device_allocs.fetch_add(1, std::memory_order_relaxed);
    return cudaMalloc(p, bytes);
}

namespace {

/* NVTX range over a scope: calls and wavefront phases show up named in
 * Nsight timelines; without a tool attached a push/pop is a no-op call */
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

struct RtFail : std::runtime_error {
    int code;
    RtFail(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CK(x)                                                                                   \
    do {                                                                                        \
        cudaError_t e_ = (x);                                                                   \
        if (e_ != cudaSuccess) throw RtFail(e_ == cudaErrorMemoryAllocation ? RT_ERR_OOM : RT_ERR_CUDA, \
                                            std::string(#x) + ": " + cudaGetErrorString(e_));   \
    } while (0)

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

#ifndef RT_WF_REFILL
#define RT_WF_REFILL 8                     /* default refill threshold of the trace warps */
#endif

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    std::vector<DevBuf> scene_bufs;
    RtSceneView view{};
    RtSceneView* d_view = nullptr;             /* device copy of `view` handed to the kernels */
    bool has_scene = false;
    int width = 0, height = 0;
    std::vector<RtTexture> h_textures;         /* host copies for the adjoint / texture updates */
    std::vector<RtMaterial> h_materials;
    int mat_types = 0;                         /* distinct material types of the scene */
    int tallest = 0;                           /* levels of the scene's tallest tree */
    std::vector<uint8_t> env_texture;          /* texture feeds an infinite light's sampling table */
    /* adjoint scratch */
    float* adj_dldi = nullptr; size_t adj_dldi_bytes = 0;
    float* adj_galb = nullptr; size_t adj_galb_bytes = 0;
    float* adj_galpha = nullptr; size_t adj_galpha_bytes = 0;
    int* adj_slot = nullptr; size_t adj_slot_bytes = 0;
    /* render scratch */
    float* samples = nullptr; size_t samples_bytes = 0;
    float* film = nullptr; size_t film_bytes = 0;
    float* out = nullptr; size_t out_bytes = 0;
    unsigned char* noalloc = nullptr;          /* this device's fixed scratch (rt_noalloc.cu) */
    uint32_t* status = nullptr;
    unsigned long long* stats = nullptr;
    void* io = nullptr; size_t io_bytes = 0;   /* device staging for host-pointer calls */
    bool counting = false;
    rt_stats last{};
    uint64_t h2d = 0;                          /* host -> device bytes copied by the current call */
    std::atomic<int> cancel{0};
    int64_t sample_budget = 1 << 24;          /* samples per launch (sample buffer = 12 B each) */
    std::vector<cudaEvent_t> events;           /* per-launch timing of the path-tracing kernel */
    int renderer = RT_RENDERER_AUTO;
    WfFork fork{};                             /* side stream for the shadow-ray kernel (rt_wf_trace) */
    int traversal = RT_TRAVERSAL_EXACT;        /* rt_set_traversal */
    int light_sampling = RT_LIGHT_SAMPLING_CDF; /* rt_set_light_sampling */
    int wf_iter_cap = WF_ITER_CAP;             /* bounce iterations of one wavefront round (test hook) */
    /* wavefront path state */
    WfState wf{};
    std::vector<DevBuf> wf_bufs;
    int wf_slots = 0;
    WfCounters* d_ctr = nullptr;               /* device counters of a wavefront run */
    WfCounters* h_ctr = nullptr;               /* pinned staging / mirror of d_ctr */
    WfJob* d_jobs = nullptr;                   /* device job table (WF_MAX_JOBS entries) */
    WfJob* h_jobs = nullptr;                   /* pinned staging of the job table */
    int wf_capacity = WF_MAX_SLOTS;            /* path slots in flight */
    int wf_refill = RT_WF_REFILL;              /* idle lanes before a trace warp fetches (1..32) */
    bool wf_graph_pref = false;                /* RT_RENDERER_AUTO drives the wavefront as a graph */
    int gpu_build_min = 1 << 15;               /* trees of at least this many primitives build on the GPU */
    uint64_t wf_generation = 0;                /* bumped whenever the path-state buffers move */
    /* the bounce loop captured as a CUDA graph while-loop */
    cudaGraph_t wf_graph = nullptr;
    cudaGraphExec_t wf_exec = nullptr;
    uint64_t wf_graph_key = 0;                 /* generation, slots and counting it was built for */
};

/* Host -> device copy on `s`, counted in the call's rt_stats.h2d_bytes. */
void h2d(Ctx* c, void* dst, const void* src, size_t bytes, cudaStream_t s) {
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
    c->h2d += bytes;
}

void ensure_events(Ctx* c, size_t n) {
    while (c->events.size() < n) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        c->events.push_back(e);
    }
}

template <class T>
T* upload(Ctx* c, const std::vector<T>& v) {
    DevBuf b;
    b.bytes = std::max<size_t>(sizeof(T), v.size() * sizeof(T));
    CK(rt_dev_malloc(&b.p, b.bytes));
    c->scene_bufs.push_back(b);
    if (!v.empty()) CK(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
    return (T*)b.p;
}

void free_scene(Ctx* c) {
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (DevBuf& b : c->scene_bufs) cudaFree(b.p);
    c->scene_bufs.clear();
    c->has_scene = false;
    c->view = RtSceneView{};
    c->d_view = nullptr;
}

template <class T>
void ensure(T** p, size_t* have, size_t need) {
    if (*have >= need && *p) return;
    if (*p) cudaFree(*p);
    *p = nullptr; *have = 0;
    CK(rt_dev_malloc((void**)p, need));
    *have = need;
}

template <class T>
T* wf_alloc(Ctx* c, size_t n) {
    DevBuf b;
    b.bytes = std::max<size_t>(sizeof(T), n * sizeof(T));
    CK(rt_dev_malloc(&b.p, b.bytes));
    c->wf_bufs.push_back(b);
    return (T*)b.p;
}

void free_wf(Ctx* c) {
    for (DevBuf& b : c->wf_bufs) cudaFree(b.p);
    c->wf_bufs.clear();
    c->wf = WfState{};
    c->wf_slots = 0;
}

/* path-state arrays for `slots` paths in flight (about 560 bytes per slot: 1.1 GiB at 2 Mi slots) */
void ensure_wf(Ctx* c, int slots) {
    if (c->wf_slots >= slots) return;
    free_wf(c);
    WfState& W = c->wf;
    const size_t n = (size_t)slots, q = 3 * (size_t)slots;
    W.q_o = wf_alloc<float4>(c, q); W.q_d = wf_alloc<float4>(c, q); W.q_meta = wf_alloc<int32_t>(c, q);
    W.active[0] = wf_alloc<int32_t>(c, n); W.active[1] = wf_alloc<int32_t>(c, n);
    W.sorted = wf_alloc<int32_t>(c, n); W.sort_key = wf_alloc<uint16_t>(c, n); W.mark = wf_alloc<uint8_t>(c, n);
    W.key_count = wf_alloc<int32_t>(c, 2 * WF_SHADE_KEYS);
    W.job = wf_alloc<uint8_t>(c, n);
    W.pix = wf_alloc<int4>(c, n); W.rng_n = wf_alloc<uint32_t>(c, n);
    W.coeff = wf_alloc<float4>(c, n); W.rad = wf_alloc<float4>(c, n);
    W.bounce = wf_alloc<int2>(c, n); W.flags = wf_alloc<uint32_t>(c, n);
    W.ray_o = wf_alloc<float4>(c, n); W.ray_d = wf_alloc<float4>(c, n);
    W.pd_coeff = wf_alloc<float4>(c, n); W.pd_l1 = wf_alloc<float4>(c, n); W.pd_fr = wf_alloc<float4>(c, n);
    W.pd_mis = wf_alloc<float4>(c, n); W.pd_w = wf_alloc<float4>(c, n);
    W.pd_ray_o = wf_alloc<float4>(c, n); W.pd_ray_d = wf_alloc<float4>(c, n);
    W.pd_acc = wf_alloc<float4>(c, n);
    W.ext_hit = wf_alloc<float4>(c, n); W.ext_sub = wf_alloc<int32_t>(c, n);
    W.mis_hit = wf_alloc<float4>(c, n); W.mis_sub = wf_alloc<int32_t>(c, n);
    W.occluded = wf_alloc<uint8_t>(c, n);
    W.adj_rho = wf_alloc<float4>(c, n);
    W.vol_env = wf_alloc<int32_t>(c, n);
    W.trw_start = wf_alloc<float4>(c, n); W.trw_end = wf_alloc<float4>(c, n);
    W.trw_dir = wf_alloc<float4>(c, n); W.trw_tr = wf_alloc<float4>(c, n);
    W.itw_o = wf_alloc<float4>(c, n); W.itw_d = wf_alloc<float4>(c, n); W.itw_tr = wf_alloc<float4>(c, n);
    W.vol_li = wf_alloc<float4>(c, n);
    W.trw_hit = wf_alloc<float4>(c, n); W.trw_sub = wf_alloc<int32_t>(c, n);
    if (!c->d_ctr) CK(rt_dev_malloc((void**)&c->d_ctr, sizeof(WfCounters)));
    if (!c->h_ctr) CK(cudaMallocHost((void**)&c->h_ctr, sizeof(WfCounters)));
    if (!c->d_jobs) CK(rt_dev_malloc((void**)&c->d_jobs, WF_MAX_JOBS * sizeof(WfJob)));
    if (!c->h_jobs) CK(cudaMallocHost((void**)&c->h_jobs, WF_MAX_JOBS * sizeof(WfJob)));
    W.ctr = c->d_ctr;
    W.jobs = c->d_jobs;
    W.status = c->status;
    c->wf_slots = slots;
    c->wf_generation++;
}

/* ---- host float helpers with the kernels' operation order --------------- */
struct F3 { float x, y, z; };
inline F3 f3(float x, float y, float z) { F3 r{x, y, z}; return r; }
inline F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline F3 cross(F3 a, F3 b) { return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline float length(F3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline F3 xform(F3 p, const float* m /* 16 */) {
    return f3(p.x * m[0] + p.y * m[4] + p.z * m[8] + m[12],
              p.x * m[1] + p.y * m[5] + p.z * m[9] + m[13],
              p.x * m[2] + p.y * m[6] + p.z * m[10] + m[14]);
}
inline void rows12(const float* m16, float* m12) {
    const int src[12] = {0, 1, 2, 4, 5, 6, 8, 9, 10, 12, 13, 14};
    for (int i = 0; i < 12; i++) m12[i] = m16[src[i]];
}
inline F3 vertex(const rt_mesh_desc& m, int i) { return f3(m.positions[3 * i], m.positions[3 * i + 1], m.positions[3 * i + 2]); }

/* TextureSampler.Sample on the host (environment luminance table) */
inline int host_f2i(float f) {
    if (f != f || f >= 2147483648.0f || f < -2147483648.0f) return INT_MIN;
    return (int)f;
}
inline float hclamp(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }
inline int hclampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
inline float hmin(float a, float b) {
    if (a != b) { if (a == a) return a < b ? a : b; return a; }
    return std::signbit(a) ? a : b;
}
void tex_sample(const rt_texture_desc& t, float x, float y, float* rgb) {
    auto wrap = [&](float a) { return t.wrap == RT_WRAP_CLAMP ? hclamp(a, 0, 1) : hclamp(a - std::floor(a), 0, 1); };
    auto rd = [&](int px, int py, float* o) {
        px = hclampi(px, 0, t.width - 1); py = hclampi(py, 0, t.height - 1);
        const float* p = t.data + ((size_t)px * t.height + py) * 3;
        o[0] = p[0]; o[1] = p[1]; o[2] = p[2];
    };
    float u = wrap(x), v = wrap(y);
    float fu = u * (float)(t.width - 1), fv = v * (float)(t.height - 1);
    int pu = host_f2i(fu), pv = host_f2i(fv);
    if (t.filter == RT_FILTER_LINEAR) {
        int dpu = (fu > (float)pu + 0.5f) ? 1 : -1, dpv = (fv > (float)pv + 0.5f) ? 1 : -1;
        int apu = hclampi(pu + dpu, 0, t.width - 1), apv = hclampi(pv + dpv, 0, t.height - 1);
        float du = hmin(std::fabs(fu - (float)pu - 0.5f), 1), dv = hmin(std::fabs(fv - (float)pv - 0.5f), 1);
        float a[3], b[3], c[3], d[3];
        rd(pu, pv, a); rd(apu, pv, b); rd(pu, apv, c); rd(apu, apv, d);
        for (int k = 0; k < 3; k++) rgb[k] = (a[k] * (1 - du) + b[k] * du) * (1 - dv) + (c[k] * (1 - du) + d[k] * du) * dv;
        return;
    }
    rd(pu, pv, rgb);
}

/* Distribution1D (Distribution1D.cs:19-49) appended to the pool */
void dist1d(std::vector<float>& pool, const float* f, int n, int64_t* pdf_off, int64_t* cdf_off, float* integ) {
    *pdf_off = (int64_t)pool.size();
    pool.insert(pool.end(), f, f + n);
    *cdf_off = (int64_t)pool.size();
    std::vector<float> cdf(n + 1);
    cdf[0] = 0;
    for (int i = 1; i < n + 1; ++i) cdf[i] = cdf[i - 1] + f[i - 1] / (float)n;
    float in = cdf[n];
    if (in == 0) { for (int i = 1; i < n + 1; i++) cdf[i] = (float)i / (float)n; }
    else { for (int i = 1; i < n + 1; i++) cdf[i] /= in; }
    pool.insert(pool.end(), cdf.begin(), cdf.end());
    *integ = in;
}

/* Walker's alias table for the pmf that the CDF search of a Distribution1D
 * (Distribution1D.cs:51-85) samples on the renderer's uniforms u = k / 2^24,
 * k in [0, 2^24).  FindInterval picks entry i for exactly
 *     c_i = ceil(cdf[i+1] 2^24) - ceil(cdf[i] 2^24)
 * values of k.  The alias pick (AliasPick, rt_shading.cuh) sends k to bucket
 * i = floor(k n / 2^24), which holds the B_i = ceil((i+1) 2^24 / n) -
 * ceil(i 2^24 / n) values of k from k0_i = ceil(i 2^24 / n) up, in increasing
 * order of rem = k n - i 2^24; it keeps i for the first own_i of them (rem <
 * threshold_i = (k0_i + own_i) n - i 2^24) and hands the rest to alias_i.
 * Vose's pairing, run on these integer counts, makes own_i plus what the other
 * buckets hand to i equal c_i for every i, so the alias pick and the search
 * draw every entry for the same number of k: the same pmf, exactly.  (A
 * bucket short of B_i takes the rest from one with more; buckets differ in
 * size by at most one, so a donor never goes below zero.)  Appends n
 * {threshold, alias} pairs; returns false, appending nothing, when the table is
 * not a non-decreasing CDF from 0 to 1 (negative or non-finite inputs). */
bool alias_from_cdf(const float* cdf, int n, std::vector<int2>& out) {
    const int64_t K = int64_t(1) << 24;
    if (n <= 0 || n > (1 << 24) || !(cdf[0] == 0.0f) || !(cdf[n] == 1.0f)) return false;
    auto kceil = [](float x) { return (int64_t)std::ceil((double)x * 16777216.0); };
    std::vector<int64_t> c(n), B(n), k0(n + 1);
    for (int i = 0; i <= n; i++) k0[i] = ((int64_t)i * K + n - 1) / n;
    for (int i = 0; i < n; i++) {
        if (!std::isfinite(cdf[i + 1]) || cdf[i + 1] < cdf[i]) return false;
        c[i] = kceil(cdf[i + 1]) - kceil(cdf[i]);
        B[i] = k0[i + 1] - k0[i];
    }
    std::vector<int> alias(n), small, large;
    for (int i = 0; i < n; i++) {
        alias[i] = i;
        if (c[i] < B[i]) small.push_back(i);
        else if (c[i] > B[i]) large.push_back(i);
    }
    while (!small.empty()) {
        const int s = small.back();
        small.pop_back();
        if (large.empty()) return false;   /* unreachable: deficits and surpluses both sum to the same */
        const int l = large.back();
        alias[s] = l;
        c[l] -= B[s] - c[s];
        if (c[l] <= B[l]) {
            large.pop_back();
            if (c[l] < B[l]) small.push_back(l);
        }
    }
    for (int i = 0; i < n; i++)
        out.push_back(make_int2((int32_t)((k0[i] + c[i]) * n - (int64_t)i * K), alias[i]));
    return true;
}

struct TopPrim {
    int kind, ref, material, light, med_in, med_out;
};

void check_index(int i, int n, const char* what) {
    if (i < 0 || i >= n) throw RtFail(RT_ERR_INVALID_ARG, std::string("scene: bad ") + what + " index " + std::to_string(i));
}

/* builds one BVH; appends nodes and slots; fills the header */
/* The reference's SAH tree: on the GPU for large primitive counts (the same
 * tree, rt_bvh_gpu.cu), on the host threads otherwise. */
rtb::BuildResult build_tree(Ctx* c, const std::vector<rtb::Box>& boxes, int maxp, int threads) {
    if ((int64_t)boxes.size() >= c->gpu_build_min) {
        rtb::BuildResult r;
        CK(rt_gpu_build_sah(boxes, maxp, &r, c->stream));
        return r;
    }
    return rtb::build_sah(boxes, maxp, threads);
}

/* the wide form of a tree (rtb::build_wide) for the fast traversal; leaf refs
 * are the binary tree's (first slot, count in that slot).  Returns the most
 * stack entries a wide traversal of the tree can hold below a node. */
int emit_wide(const rtb::BuildResult& br, int slot_base, std::vector<float4>& wnodes, RtBvh* hdr) {
    const std::vector<rtb::FlatNode>& fn = br.nodes;
    if (fn.empty()) { hdr->wide_root = INT_MIN; return 0; }
    if (fn[0].count != 0) { hdr->wide_root = hdr->root_ref; return 0; }
    const rtb::WideResult w = rtb::build_wide(br);
    const int base = (int)(wnodes.size() / RT_WIDE_F4);
    hdr->wide_root = base;
    for (const rtb::WideNode& n : w.nodes) {
        uint32_t meta = (uint32_t)n.e[0] | ((uint32_t)n.e[1] << 8) | ((uint32_t)n.e[2] << 16) | ((uint32_t)n.nchild << 24);
        float4 f[RT_WIDE_F4];
        f[0] = make_float4(n.p[0], n.p[1], n.p[2], 0.0f);
        std::memcpy(&f[0].w, &meta, 4);
        for (int a = 0; a < 3; a++) {
            std::memcpy(&f[1 + a].x, n.qlo[a], 8);
            std::memcpy(&f[1 + a].z, n.qhi[a], 8);
        }
        int32_t ref[8];
        for (int k = 0; k < 8; k++) {
            if (k >= n.nchild) ref[k] = INT_MIN;
            else if (n.wchild[k] >= 0) ref[k] = base + n.wchild[k];
            else ref[k] = ~(slot_base + fn[n.child[k]].second);
        }
        std::memcpy(&f[4], ref, 16);
        std::memcpy(&f[5], ref + 4, 16);
        for (int q = 0; q < RT_WIDE_F4; q++) wnodes.push_back(f[q]);
    }
    return w.max_push;
}

void emit_bvh(const rtb::BuildResult& br, const std::vector<std::array<float4, 3>>& recs, std::vector<float4>& nodes,
              std::vector<float4>& slots, RtBvh* hdr) {
    const int slot_base = (int)(slots.size() / 3);
    for (size_t i = 0; i < br.order.size(); i++) {
        const std::array<float4, 3>& r = recs[br.order[i]];
        slots.push_back(r[0]); slots.push_back(r[1]); slots.push_back(r[2]);
    }
    const std::vector<rtb::FlatNode>& fn = br.nodes;
    if (fn.empty()) {
        for (int k = 0; k < 3; k++) { hdr->root_min[k] = 0; hdr->root_max[k] = 0; }
        hdr->root_ref = INT_MIN;
        return;
    }
    /* interior nodes get consecutive device indices in depth-first order */
    std::vector<int> dev(fn.size(), -1);
    int node_base = (int)(nodes.size() / 4), nint = 0;
    for (size_t i = 0; i < fn.size(); i++) if (fn[i].count == 0) dev[i] = node_base + nint++;
    auto ref_of = [&](int i) -> int {
        if (fn[i].count == 0) return dev[i];
        int first = slot_base + fn[i].second;
        if (fn[i].count > 65535) throw RtFail(RT_ERR_UNSUPPORTED, "BVH leaf with more than 65535 primitives");
        float4& s2 = slots[3 * (size_t)first + 2];
        int c = fn[i].count;
        std::memcpy(&s2.w, &c, 4);
        return ~first;
    };
    for (int k = 0; k < 3; k++) { hdr->root_min[k] = fn[0].bounds.mn[k]; hdr->root_max[k] = fn[0].bounds.mx[k]; }
    hdr->root_ref = ref_of(0);
    for (size_t i = 0; i < fn.size(); i++) {
        if (fn[i].count != 0) { ref_of((int)i); continue; }
        const rtb::Box& L = fn[i + 1].bounds;
        const rtb::Box& R = fn[fn[i].second].bounds;
        int lref = ref_of((int)i + 1), rref = ref_of(fn[i].second), axis = fn[i].axis;
        float4 n0 = make_float4(L.mn[0], L.mn[1], L.mn[2], L.mx[0]);
        float4 n1 = make_float4(L.mx[1], L.mx[2], R.mn[0], R.mn[1]);
        float4 n2 = make_float4(R.mn[2], R.mx[0], R.mx[1], R.mx[2]);
        float4 n3;
        std::memcpy(&n3.x, &lref, 4); std::memcpy(&n3.y, &rref, 4); std::memcpy(&n3.z, &axis, 4); n3.w = 0;
        nodes.push_back(n0); nodes.push_back(n1); nodes.push_back(n2); nodes.push_back(n3);
    }
}

inline float4 f4bits(float x, float y, float z, int w) { float4 r = make_float4(x, y, z, 0); std::memcpy(&r.w, &w, 4); return r; }
inline float4 f4bitsu(float x, float y, float z, uint32_t w) { float4 r = make_float4(x, y, z, 0); std::memcpy(&r.w, &w, 4); return r; }

std::array<float4, 3> tri_rec(const rt_mesh_desc& m, int t, int prim_id, int global_tri) {
    const int* ix = m.indices + 3 * (size_t)t;
    F3 pa = vertex(m, ix[0]), pb = vertex(m, ix[1]), pc = vertex(m, ix[2]);
    F3 e1 = sub(pb, pa), e2 = sub(pc, pa);
    uint32_t kr = ((uint32_t)RT_KIND_TRI << RT_KIND_SHIFT) | (uint32_t)global_tri;
    return {f4bits(pa.x, pa.y, pa.z, prim_id), f4bitsu(e1.x, e1.y, e1.z, kr), f4bits(e2.x, e2.y, e2.z, 0)};
}
std::array<float4, 3> other_rec(int kind, int ref, int prim_id) {
    uint32_t kr = ((uint32_t)kind << RT_KIND_SHIFT) | (uint32_t)ref;
    return {f4bits(0, 0, 0, prim_id), f4bitsu(0, 0, 0, kr), f4bits(0, 0, 0, 0)};
}
rtb::Box tri_box(const rt_mesh_desc& m, int t) {
    const int* ix = m.indices + 3 * (size_t)t;
    F3 pa = vertex(m, ix[0]), pb = vertex(m, ix[1]), pc = vertex(m, ix[2]);
    rtb::Box b;
    b.mn[0] = b.mx[0] = pa.x; b.mn[1] = b.mx[1] = pa.y; b.mn[2] = b.mx[2] = pa.z;
    float q[3] = {pb.x, pb.y, pb.z}; rtb::box_expand(b, q);
    float r[3] = {pc.x, pc.y, pc.z}; rtb::box_expand(b, r);
    return b;
}
rtb::Box sphere_box(const rt_sphere_desc& s) {
    rtb::Box b;
    for (int k = 0; k < 3; k++) { b.mn[k] = s.center[k] - s.radius; b.mx[k] = s.center[k] + s.radius; }
    return b;
}
/* BoundingBox3F.Transform (BoundingBox3F.cs:232-244) */
rtb::Box xform_box(const rtb::Box& b, const float* m) {
    const float* mn = b.mn; const float* mx = b.mx;
    F3 c[8] = {f3(mn[0], mn[1], mn[2]), f3(mx[0], mn[1], mn[2]), f3(mn[0], mx[1], mn[2]), f3(mn[0], mn[1], mx[2]),
               f3(mn[0], mx[1], mx[2]), f3(mx[0], mx[1], mn[2]), f3(mx[0], mn[1], mx[2]), f3(mx[0], mx[1], mx[2])};
    F3 p = xform(c[0], m);
    rtb::Box r;
    r.mn[0] = r.mx[0] = p.x; r.mn[1] = r.mx[1] = p.y; r.mn[2] = r.mx[2] = p.z;
    for (int i = 1; i < 8; i++) { F3 q = xform(c[i], m); float v[3] = {q.x, q.y, q.z}; rtb::box_expand(r, v); }
    return r;
}

void upload_scene(Ctx* c, const rt_scene_desc* d) {
    NvtxRange nvtx_("rt.upload_scene");
    if (!d || d->abi_version != RT_ABI_VERSION) throw RtFail(RT_ERR_INVALID_ARG, "scene: null descriptor or ABI version mismatch");
    if (d->camera.width <= 0 || d->camera.height <= 0) throw RtFail(RT_ERR_INVALID_ARG, "scene: camera resolution must be positive");
    const int threads = std::max(1u, std::thread::hardware_concurrency());
    const int maxp = d->bvh_max_prims < 1 ? 1 : d->bvh_max_prims;
    int tallest = 0;                           /* levels of the tallest tree */

    /* global vertex / triangle tables: every mesh, in mesh order */
    std::vector<float4> pos, nrm;
    std::vector<float2> uvs;
    std::vector<RtTri> tris;
    std::vector<int> mesh_tri_base(d->mesh_count), mesh_vtx_base(d->mesh_count);
    for (int m = 0; m < d->mesh_count; m++) {
        const rt_mesh_desc& md = d->meshes[m];
        if (md.vertex_count < 0 || md.triangle_count < 0 || (md.triangle_count > 0 && (!md.positions || !md.indices)))
            throw RtFail(RT_ERR_INVALID_ARG, "scene: mesh " + std::to_string(m) + " has no positions / indices");
        mesh_vtx_base[m] = (int)pos.size();
        mesh_tri_base[m] = (int)tris.size();
        for (int i = 0; i < md.vertex_count; i++) {
            pos.push_back(make_float4(md.positions[3 * i], md.positions[3 * i + 1], md.positions[3 * i + 2], 0));
            nrm.push_back(md.normals ? make_float4(md.normals[3 * i], md.normals[3 * i + 1], md.normals[3 * i + 2], 0) : make_float4(0, 0, 0, 0));
            uvs.push_back(md.uvs ? make_float2(md.uvs[2 * i], md.uvs[2 * i + 1]) : make_float2(0, 0));
        }
        for (int t = 0; t < md.triangle_count; t++) {
            RtTri tr;
            for (int k = 0; k < 3; k++) {
                int vi = md.indices[3 * t + k];
                if (vi < 0 || vi >= md.vertex_count) throw RtFail(RT_ERR_INVALID_ARG, "scene: mesh " + std::to_string(m) + " index out of range");
            }
            tr.v0 = mesh_vtx_base[m] + md.indices[3 * t];
            tr.v1 = mesh_vtx_base[m] + md.indices[3 * t + 1];
            tr.v2 = mesh_vtx_base[m] + md.indices[3 * t + 2];
            tr.flags = (md.normals ? 1 : 0) | (md.uvs ? 2 : 0);
            tris.push_back(tr);
        }
    }
    std::vector<RtSphere> spheres(d->sphere_count);
    for (int i = 0; i < d->sphere_count; i++) {
        const rt_sphere_desc& s = d->spheres[i];
        for (int k = 0; k < 3; k++) spheres[i].center[k] = s.center[k];
        spheres[i].radius = s.radius;
        rows12(s.world_to_model, spheres[i].w2m);
    }
    for (int i = 0; i < d->material_count; i++) {
        const rt_material_desc& m = d->materials[i];
        bool needR = m.type != RT_MAT_ROUGH_METAL, needT = m.type == RT_MAT_ROUGH_GLASS || m.type == RT_MAT_PERFECT_GLASS;
        bool needRough = m.type == RT_MAT_ROUGH_METAL || m.type == RT_MAT_ROUGH_GLASS || m.type == RT_MAT_ROUGH_PLASTIC;
        auto ok = [&](int t) { return t >= 0 && t < d->texture_count; };
        if (m.type < 0 || m.type > RT_MAT_PERFECT_GLASS || (needR && !ok(m.tex_r)) || (needT && !ok(m.tex_t)) ||
            (needRough && (!ok(m.tex_roughness) || !ok(m.tex_anisotropic))))
            throw RtFail(RT_ERR_INVALID_ARG, "scene: material " + std::to_string(i) + " is missing a texture or has an unknown type");
    }

    std::vector<float4> nodes, slots, wnodes;
    int wide_push = 0;
    std::vector<RtBvh> bvhs(1 + d->blas_count);
    /* instanced prototypes: ShapeWrapperPrimitive per shape (RendererBuilder.cs:895-921) */
    std::vector<rtb::Box> blas_root(d->blas_count);
    for (int b = 0; b < d->blas_count; b++) {
        int first = d->blas_ranges[2 * b], count = d->blas_ranges[2 * b + 1];
        if (first < 0 || count < 0 || first + count > d->blas_group_count) throw RtFail(RT_ERR_INVALID_ARG, "scene: bad prototype range");
        std::vector<rtb::Box> boxes;
        std::vector<std::array<float4, 3>> recs;
        for (int g = first; g < first + count; g++) {
            const rt_group_desc& gd = d->blas_groups[g];
            if (gd.kind == RT_GROUP_SPHERE) {
                check_index(gd.ref, d->sphere_count, "sphere");
                boxes.push_back(sphere_box(d->spheres[gd.ref]));
                recs.push_back(other_rec(RT_KIND_SPHERE, gd.ref, (int)recs.size()));
            } else if (gd.kind == RT_GROUP_MESH) {
                check_index(gd.ref, d->mesh_count, "mesh");
                const rt_mesh_desc& md = d->meshes[gd.ref];
                for (int t = 0; t < md.triangle_count; t++) {
                    boxes.push_back(tri_box(md, t));
                    recs.push_back(tri_rec(md, t, (int)recs.size(), mesh_tri_base[gd.ref] + t));
                }
            } else {
                throw RtFail(RT_ERR_INVALID_ARG, "scene: instanced prototype groups must be meshes or spheres");
            }
        }
        rtb::BuildResult br = build_tree(c, boxes, maxp, threads);
        tallest = std::max(tallest, br.max_depth);
        const int blas_slots = (int)(slots.size() / 3);
        emit_bvh(br, recs, nodes, slots, &bvhs[1 + b]);
        wide_push = std::max(wide_push, emit_wide(br, blas_slots, wnodes, &bvhs[1 + b]));
        if (!br.nodes.empty()) blas_root[b] = br.nodes[0].bounds;
        else blas_root[b] = rtb::empty_box();
    }

    /* top level, lights, infinite lights */
    std::vector<rtb::Box> boxes;
    std::vector<std::array<float4, 3>> recs;
    std::vector<RtPrim> prims;
    std::vector<RtLight> lights;
    std::vector<int32_t> infinite;
    std::vector<RtInstance> insts;
    auto area_light = [&](int kind, int ref, const rt_group_desc& gd, float area) {
        RtLight L{};
        L.kind = kind; L.ref = ref; L.le[0] = gd.le[0]; L.le[1] = gd.le[1]; L.le[2] = gd.le[2]; L.area = area;
        L.dist = -1;
        lights.push_back(L);
        return (int)lights.size() - 1;
    };
    for (int g = 0; g < d->group_count; g++) {
        const rt_group_desc& gd = d->groups[g];
        if (gd.material >= d->material_count || gd.medium_inside >= d->medium_count || gd.medium_outside >= d->medium_count)
            throw RtFail(RT_ERR_INVALID_ARG, "scene: group " + std::to_string(g) + " references a missing material / medium");
        TopPrim tp{0, 0, gd.material < 0 ? -1 : gd.material, -1, gd.medium_inside < 0 ? -1 : gd.medium_inside,
                   gd.medium_outside < 0 ? -1 : gd.medium_outside};
        switch (gd.kind) {
        case RT_GROUP_INFINITE_LIGHT: {
            check_index(gd.ref, d->texture_count, "texture");
            RtLight L{};
            L.kind = RT_LIGHT_INFINITE; L.ref = gd.ref;
            rows12(gd.model_to_world, L.m2w); rows12(gd.world_to_model, L.w2m);
            L.dist = -1;
            infinite.push_back((int)lights.size());
            lights.push_back(L);
            break;
        }
        case RT_GROUP_SPHERE: {
            check_index(gd.ref, d->sphere_count, "sphere");
            const rt_sphere_desc& s = d->spheres[gd.ref];
            int id = (int)prims.size();
            int li = -1;
            if (gd.emissive) li = area_light(RT_LIGHT_AREA_SPHERE, gd.ref, gd, 4 * s.radius * s.radius * 3.14159265f);
            prims.push_back(RtPrim{RT_KIND_SPHERE, gd.ref, tp.material, li, tp.med_in, tp.med_out, 0, 0});
            boxes.push_back(sphere_box(s));
            recs.push_back(other_rec(RT_KIND_SPHERE, gd.ref, id));
            break;
        }
        case RT_GROUP_MESH: {
            check_index(gd.ref, d->mesh_count, "mesh");
            const rt_mesh_desc& md = d->meshes[gd.ref];
            for (int t = 0; t < md.triangle_count; t++) {
                int id = (int)prims.size();
                int gt = mesh_tri_base[gd.ref] + t;
                int li = -1;
                if (gd.emissive) {
                    const int* ix = md.indices + 3 * (size_t)t;
                    F3 pa = vertex(md, ix[0]), pb = vertex(md, ix[1]), pc = vertex(md, ix[2]);
                    float area = 0.5f * length(cross(sub(pb, pa), sub(pc, pa)));
                    li = area_light(RT_LIGHT_AREA_TRI, gt, gd, area);
                }
                prims.push_back(RtPrim{RT_KIND_TRI, gt, tp.material, li, tp.med_in, tp.med_out, 0, 0});
                boxes.push_back(tri_box(md, t));
                recs.push_back(tri_rec(md, t, id, gt));
            }
            break;
        }
        case RT_GROUP_INSTANCE: {
            check_index(gd.ref, d->blas_count, "instanced prototype");
            RtInstance I{};
            rows12(gd.model_to_world, I.m2w); rows12(gd.world_to_model, I.w2m);
            I.blas = gd.ref;
            int id = (int)prims.size();
            prims.push_back(RtPrim{RT_KIND_INSTANCE, (int)insts.size(), tp.material, -1, tp.med_in, tp.med_out, 0, 0});
            boxes.push_back(xform_box(blas_root[gd.ref], gd.model_to_world));
            recs.push_back(other_rec(RT_KIND_INSTANCE, (int)insts.size(), id));
            insts.push_back(I);
            break;
        }
        default:
            throw RtFail(RT_ERR_INVALID_ARG, "scene: unknown group kind " + std::to_string(gd.kind));
        }
    }
    if (prims.empty()) throw RtFail(RT_ERR_INVALID_ARG, "scene: no primitives");
    rtb::BuildResult top = build_tree(c, boxes, maxp, threads);
    tallest = std::max(tallest, top.max_depth);
    const int top_slots = (int)(slots.size() / 3);
    emit_bvh(top, recs, nodes, slots, &bvhs[0]);
    wide_push = std::max(wide_push, emit_wide(top, top_slots, wnodes, &bvhs[0]));

    /* textures */
    std::vector<RtTexture> texs(d->texture_count);
    std::vector<float> texels;
    for (int i = 0; i < d->texture_count; i++) {
        const rt_texture_desc& t = d->textures[i];
        if (t.width <= 0 || t.height <= 0 || !t.data) throw RtFail(RT_ERR_INVALID_ARG, "scene: bad texture " + std::to_string(i));
        texs[i].width = t.width; texs[i].height = t.height; texs[i].wrap = t.wrap; texs[i].filter = t.filter;
        texs[i].offset = (int64_t)texels.size();
        texels.insert(texels.end(), t.data, t.data + (size_t)t.width * t.height * 3);
    }
    /* infinite lights: luminance * sin(theta) table and Distribution2D (InfiniteAreaLight.cs:21-54),
     * world sphere from the top-level bounds (Light.cs:181-187) */
    std::vector<RtDist2D> dists;
    std::vector<float> pool;
    std::vector<int2> alias;
    const rtb::Box& wb = top.nodes[0].bounds;
    for (int li : infinite) {
        RtLight& L = lights[li];
        const rt_texture_desc& t = d->textures[L.ref];
        const int W = t.width, H = t.height;
        std::vector<float> lum((size_t)W * H);
        for (int y = 0; y < H; y++) {
            float sinTheta = rt_sinf(((float)y + 0.5f) / (float)H * 3.14159265f);
            float v = (float)y / (float)H;
            for (int x = 0; x < W; x++) {
                float u = (float)x / (float)W;
                float rgb[3];
                tex_sample(t, u, v, rgb);
                lum[(size_t)y * W + x] = (rgb[0] * 0.212671f + rgb[1] * 0.715160f + rgb[2] * 0.072169f) * sinTheta;
            }
        }
        RtDist2D D{};
        D.nu = W; D.nv = H;
        std::vector<float> cond_int(H);
        std::vector<float> cond_pdf_cdf;
        D.cond_pdf = (int64_t)pool.size();
        pool.insert(pool.end(), lum.begin(), lum.end());
        D.cond_cdf = (int64_t)pool.size();
        for (int y = 0; y < H; y++) {
            const float* f = lum.data() + (size_t)y * W;
            std::vector<float> cdf(W + 1);
            cdf[0] = 0;
            for (int i = 1; i < W + 1; ++i) cdf[i] = cdf[i - 1] + f[i - 1] / (float)W;
            float in = cdf[W];
            if (in == 0) { for (int i = 1; i < W + 1; i++) cdf[i] = (float)i / (float)W; }
            else { for (int i = 1; i < W + 1; i++) cdf[i] /= in; }
            pool.insert(pool.end(), cdf.begin(), cdf.end());
            cond_int[y] = in;
        }
        D.cond_int = (int64_t)pool.size();
        pool.insert(pool.end(), cond_int.begin(), cond_int.end());
        dist1d(pool, cond_int.data(), H, &D.marg_pdf, &D.marg_cdf, &D.marg_int);
        {   /* the alias tables of the same CDFs (RT_LIGHT_SAMPLING_ALIAS) */
            const size_t at = alias.size();
            bool ok = alias_from_cdf(pool.data() + D.marg_cdf, H, alias);
            for (int y = 0; ok && y < H; y++) ok = alias_from_cdf(pool.data() + D.cond_cdf + (int64_t)y * (W + 1), W, alias);
            if (ok) { D.marg_alias = (int64_t)at; D.cond_alias = (int64_t)at + H; }
            else { alias.resize(at); D.marg_alias = D.cond_alias = -1; }
        }
        L.dist = (int)dists.size();
        dists.push_back(D);
        float cx = (wb.mx[0] + wb.mn[0]) * 0.5f, cy = (wb.mx[1] + wb.mn[1]) * 0.5f, cz = (wb.mx[2] + wb.mn[2]) * 0.5f;
        L.world_center[0] = cx; L.world_center[1] = cy; L.world_center[2] = cz;
        F3 dg = f3(wb.mx[0] - wb.mn[0], wb.mx[1] - wb.mn[1], wb.mx[2] - wb.mn[2]);
        L.world_radius = length(dg) / 2.0f;
    }
    std::vector<RtMaterial> mats(d->material_count);
    for (int i = 0; i < d->material_count; i++) {
        const rt_material_desc& m = d->materials[i];
        RtMaterial& o = mats[i];
        o.type = m.type; o.dist = m.dist; o.two_sided = m.two_sided;
        o.tex_r = m.tex_r; o.tex_t = m.tex_t; o.tex_rough = m.tex_roughness; o.tex_anis = m.tex_anisotropic;
        o.eta_a = m.eta_a; o.eta_b = m.eta_b; o.kd = m.kd; o.ks = m.ks;
        for (int k = 0; k < 3; k++) { o.eta[k] = m.eta[k]; o.k[k] = m.k[k]; }
    }
    std::vector<RtMedium> meds(d->medium_count);
    for (int i = 0; i < d->medium_count; i++) {
        const rt_medium_desc& m = d->media[i];
        for (int k = 0; k < 3; k++) {
            meds[i].sig_a[k] = m.sigma_a[k] * m.scale;
            meds[i].sig_s[k] = m.sigma_s[k] * m.scale;
            meds[i].sig_t[k] = meds[i].sig_a[k] + meds[i].sig_s[k];
        }
        meds[i].g = m.g;
    }
    if (d->global_medium >= d->medium_count) throw RtFail(RT_ERR_INVALID_ARG, "scene: bad global medium");

    free_scene(c);
    RtSceneView& v = c->view;
    v.nodes = upload(c, nodes);
    v.slots = upload(c, slots);
    v.bvhs = upload(c, bvhs);
    v.prims = upload(c, prims);
    v.tris = upload(c, tris);
    v.pos = upload(c, pos);
    v.nrm = upload(c, nrm);
    v.uv = upload(c, uvs);
    v.spheres = upload(c, spheres);
    v.instances = upload(c, insts);
    v.materials = upload(c, mats);
    v.textures = upload(c, texs);
    c->h_textures = texs;
    c->h_materials = mats;
    {
        uint32_t seen = 0;
        for (const RtMaterial& m : mats) seen |= 1u << (m.type & 31);
        c->mat_types = __builtin_popcount(seen);
    }
    c->env_texture.assign(texs.size(), 0);
    for (int li : infinite) c->env_texture[lights[li].ref] = 1;
    v.texels = upload(c, texels);
    v.media = upload(c, meds);
    v.lights = upload(c, lights);
    v.infinite_lights = upload(c, infinite);
    v.dists = upload(c, dists);
    v.dist_pool = upload(c, pool);
    v.alias_pool = upload(c, alias);
    v.env_alias = c->light_sampling == RT_LIGHT_SAMPLING_ALIAS ? 1 : 0;
    v.light_count = (int)lights.size();
    v.infinite_count = (int)infinite.size();
    v.global_medium = d->global_medium < 0 ? -1 : d->global_medium;
    v.deep_trees = tallest > RT_STACK_SIZE + 1 ? 1 : 0;
    c->tallest = tallest;
    if (wnodes.empty()) wnodes.push_back(make_float4(0, 0, 0, 0));
    v.wnodes = upload(c, wnodes);
    /* a wide visit pushes at most 7 entries on top of what is below it */
    v.wide_ok = (!v.deep_trees && wide_push + 7 <= RT_STACK_SIZE) ? 1 : 0;
    RtCamera& cam = v.camera;
    cam.width = d->camera.width; cam.height = d->camera.height;
    cam.near_z = d->camera.near_z; cam.far_z = d->camera.far_z;
    cam.inv_res_x = 1.0f / (float)cam.width; cam.inv_res_y = 1.0f / (float)cam.height;
    std::memcpy(cam.clip_to_camera, d->camera.clip_to_camera, sizeof(cam.clip_to_camera));
    std::memcpy(cam.camera_to_world, d->camera.camera_to_world, sizeof(cam.camera_to_world));
    std::memcpy(cam.camera_to_clip, d->camera.camera_to_clip, sizeof(cam.camera_to_clip));
    std::memcpy(cam.world_to_camera, d->camera.world_to_camera, sizeof(cam.world_to_camera));
    {   /* PerspectiveCamera.Update (Camera.cs:172-179): the image plane at z = 1 */
        const float* m = cam.clip_to_camera;
        auto xf = [m](float x, float y, float z, float* o) {
            for (int k = 0; k < 3; k++) o[k] = x * m[k] + y * m[4 + k] + z * m[8 + k] + m[12 + k];
        };
        float pmin[3], pmax[3];
        xf(0, 0, 0, pmin);
        xf(1, 1, 0, pmax);
        const float zmin = pmin[2], zmax = pmax[2];
        for (int k = 0; k < 3; k++) { pmin[k] = pmin[k] / zmin; pmax[k] = pmax[k] / zmax; }
        cam.min_x = pmax[0]; cam.min_y = pmax[1];
        cam.max_x = pmin[0]; cam.max_y = pmin[1];
        const float area = std::fabs((cam.max_x - cam.min_x) * (cam.max_y - cam.min_y));
        cam.normalization = 1 / area;
    }
    c->d_view = upload(c, std::vector<RtSceneView>{v});
    CK(cudaStreamSynchronize(c->stream));
    c->has_scene = true;
    c->width = cam.width; c->height = cam.height;
}

/* the call's error for a device status word (rt_types.h RT_STATUS_*) */
void throw_status(uint32_t st) {
    if (st & RT_STATUS_STACK) throw RtFail(RT_ERR_STACK, "BVH traversal stack (64 entries) overflowed");
    if (st & RT_STATUS_TRAV) throw RtFail(RT_ERR_ITER_CAP, "a BVH traversal reached its step cap (RT_TRAVERSAL_CAP)");
    if (st & RT_STATUS_WALK) throw RtFail(RT_ERR_ITER_CAP, "a null-boundary walk reached its segment cap (RT_WALK_CAP)");
    if (st & RT_STATUS_WFITER) throw RtFail(RT_ERR_ITER_CAP, "wavefront: bounce iteration cap reached (WF_ITER_CAP)");
    if (st & RT_STATUS_ITER) throw RtFail(RT_ERR_ITER_CAP, "a path reached its bounce cap (RT_LOOP_CAP)");
    if (st & RT_STATUS_BADREF) throw RtFail(RT_ERR_INVALID_ARG, "an instanced prototype contains an instance");
    if (st & RT_STATUS_BOUNDS) throw RtFail(RT_ERR_BOUNDS, "a device index left its buffer (debug-bounds build)");
}

void check_status(Ctx* c) {
    uint32_t st = 0;
    CK(cudaMemcpyAsync(&st, c->status, 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    throw_status(st);
}

void read_stats(Ctx* c) {
    unsigned long long s[8];
    CK(cudaMemcpyAsync(s, c->stats, sizeof(s), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->last.rays_closest = s[1]; c->last.rays_shadow = s[2]; c->last.node_visits = s[3];
    c->last.prim_tests = s[4]; c->last.instance_visits = s[5]; c->last.invalid_samples = s[6];
}

void render_megakernel(Ctx* c, RtParams P, int chunk, int64_t npix, cudaStream_t s);
void render_wavefront(Ctx* c, RtParams P, int chunk, int64_t npix, cudaStream_t s);

void render(Ctx* c, const rt_render_params* p, float* dst, bool dst_host, cudaStream_t user) {
    NvtxRange nvtx_("rt.render");
    if (!c->has_scene) throw RtFail(RT_ERR_NO_SCENE, "no scene uploaded");
    if (!p || !dst || p->spp <= 0) throw RtFail(RT_ERR_INVALID_ARG, "render: null params/output or spp <= 0");
    if (p->integrator != RT_INTEGRATOR_PATH && p->integrator != RT_INTEGRATOR_VOL_PATH) throw RtFail(RT_ERR_INVALID_ARG, "render: unknown integrator");
    RtParams P{};
    P.integrator = p->integrator; P.method = p->method; P.strategy = p->strategy;
    P.max_depth = p->max_depth; P.min_depth = p->min_depth; P.rr = p->rr_threshold;
    P.seed = p->seed; P.x0 = p->x0; P.y0 = p->y0;
    P.w = p->width > 0 ? p->width : c->width - p->x0;
    P.h = p->height > 0 ? p->height : c->height - p->y0;
    if (P.x0 < 0 || P.y0 < 0 || P.w <= 0 || P.h <= 0 || P.x0 + P.w > c->width || P.y0 + P.h > c->height)
        throw RtFail(RT_ERR_INVALID_ARG, "render: crop outside the film");
    P.spp = p->spp; P.sample_begin = p->sample_begin;
    cudaStream_t s = user ? user : c->stream;
    const int64_t npix = (int64_t)P.w * P.h;
    int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(P.spp, c->sample_budget / std::max<int64_t>(1, npix)));
    ensure(&c->samples, &c->samples_bytes, (size_t)npix * chunk * 12);
    ensure(&c->film, &c->film_bytes, (size_t)npix * 12);
    CK(cudaMemsetAsync(c->film, 0, (size_t)npix * 12, s));
    CK(cudaMemsetAsync(c->status, 0, 4, s));
    CK(cudaMemsetAsync(c->stats, 0, 8 * sizeof(unsigned long long), s));
    c->cancel.store(0);
    /* the wavefront runs path with either light strategy, vol_path with Uniform */
    const bool wf_ok = P.strategy == RT_STRATEGY_UNIFORM || P.integrator == RT_INTEGRATOR_PATH;
    const bool wavefront = c->renderer == RT_RENDERER_WAVEFRONT || c->renderer == RT_RENDERER_WAVEFRONT_GRAPH;
    if (wavefront && !wf_ok)
        throw RtFail(RT_ERR_UNSUPPORTED, "the wavefront renderer runs vol_path with the Uniform light strategy");
    if (wavefront || (c->renderer == RT_RENDERER_AUTO && wf_ok)) {
        render_wavefront(c, P, chunk, npix, s);
    } else {
        render_megakernel(c, P, chunk, npix, s);
    }
    float* out = dst;
    if (dst_host) {
        ensure(&c->out, &c->out_bytes, (size_t)npix * 12);
        out = c->out;
    }
    CK(rt_launch_finalize(out, c->film, npix, (float)P.spp, s));
    if (dst_host) CK(cudaMemcpyAsync(dst, out, (size_t)npix * 12, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    check_status(c);
    double rms = c->last.render_kernel_ms, sms = c->last.shade_kernel_ms;
    uint64_t launches = c->last.kernel_launches, rl = c->last.render_launches;
    std::memset(&c->last, 0, sizeof(c->last));
    c->last.h2d_bytes = c->h2d;
    read_stats(c);
    c->last.samples = (uint64_t)npix * P.spp;
    c->last.render_kernel_ms = rms;
    c->last.shade_kernel_ms = sms;
    c->last.render_launches = rl;
    c->last.kernel_launches = launches + 1;
}

void render_megakernel(Ctx* c, RtParams P, int chunk, int64_t npix, cudaStream_t s) {
    const int nchunks = (P.spp + chunk - 1) / chunk;
    ensure_events(c, 2 * (size_t)nchunks);
    uint64_t launches = 0;
    for (int b = 0, ci = 0; b < P.spp; b += chunk, ci++) {
        /* at most two chunks queued, so a cancel from another thread takes
         * effect within a chunk or two (Renderer.Stop) */
        if (ci >= 2) CK(cudaEventSynchronize(c->events[2 * (ci - 2) + 1]));
        if (c->cancel.load()) {
            cudaStreamSynchronize(s);
            throw RtFail(RT_ERR_CANCELLED, "render cancelled");
        }
        P.chunk_begin = b;
        P.chunk_len = std::min(chunk, P.spp - b);
        CK(cudaEventRecord(c->events[2 * ci], s));
        CK(rt_launch_render(c->d_view, P, c->samples, c->status, c->stats, c->counting, s));
        CK(cudaEventRecord(c->events[2 * ci + 1], s));
        CK(rt_launch_accumulate(c->film, c->samples, npix, P.chunk_len, s));
        launches += 2;
    }
    CK(cudaStreamSynchronize(s));
    double ms = 0;
    for (int ci = 0; ci < nchunks; ci++) {
        float t = 0;
        CK(cudaEventElapsedTime(&t, c->events[2 * ci], c->events[2 * ci + 1]));
        ms += t;
    }
    c->last.render_kernel_ms = ms;
    c->last.shade_kernel_ms = 0;
    c->last.render_launches = (uint64_t)nchunks;
    c->last.kernel_launches = launches;
}

/* RtParams of a light-tracing call (whole film) */
RtParams particle_params(Ctx* c, const rt_render_params* p, int64_t first, int64_t count) {
    if (!c->has_scene) throw RtFail(RT_ERR_NO_SCENE, "no scene uploaded");
    if (!p) throw RtFail(RT_ERR_INVALID_ARG, "render_particles: null params");
    if (p->integrator != RT_INTEGRATOR_PARTICLE)
        throw RtFail(RT_ERR_INVALID_ARG, "render_particles: the integrator must be RT_INTEGRATOR_PARTICLE");
    if (p->x0 != 0 || p->y0 != 0 || p->width != 0 || p->height != 0)
        throw RtFail(RT_ERR_INVALID_ARG, "render_particles: particles splat into the whole film (crop fields must be 0)");
    if (first < 0 || count <= 0 || first > INT64_MAX - count)
        throw RtFail(RT_ERR_INVALID_ARG, "render_particles: bad particle range");
    RtParams P{};
    P.integrator = p->integrator; P.method = p->method; P.strategy = p->strategy;
    P.max_depth = p->max_depth; P.min_depth = p->min_depth; P.rr = p->rr_threshold;
    P.seed = p->seed; P.w = c->width; P.h = c->height;
    return P;
}

void ensure_wf_graph(Ctx* c, const WfState& W, bool vol, bool particle = false, bool sort = true, bool deep = false,
                     bool wide = false);

/* What a wavefront run shades, and how its kernels are chosen. */
struct WfMode {
    bool vol = false;        /* vol_path shade kernel */
    bool particle = false;   /* light-tracer start / shade kernels */
    bool sort = true;        /* regroup the active list by shade key before shading */
    bool deep = false;       /* trace kernels with the shared-memory stack (trees of 16+ levels) */
    bool wide = false;       /* the opt-in fast traversal over the wide nodes */
};
/* CUDA-event times and launch counts of a run, summed over its rounds */
struct WfTotals {
    double trace_ms = 0, shade_ms = 0;
    uint64_t launches = 0, trace_launches = 0;
};

/* One round of a wavefront run over the jobs already in c->d_jobs: every slot
 * takes a sample (or particle), then the loop bounces until no path is active
 * and no splat ray is queued (a finished particle leaves its last one behind).
 * The loop runs as one CUDA graph launch (render passes with `use_graph`) or
 * is driven from the host with per-phase event timing. */
void wf_round(Ctx* c, const WfState& W, cudaStream_t s, bool use_graph, const WfMode& m, int pass,
              const WfAdjoint* adj, int64_t total, int n_jobs, WfTotals* t) {
    std::memset(c->h_ctr, 0, sizeof(WfCounters));
    c->h_ctr->total = total;
    c->h_ctr->n_jobs = n_jobs;
    h2d(c, c->d_ctr, c->h_ctr, sizeof(WfCounters), s);
    CK(rt_wf_start(W, s, m.particle));
    t->launches += 2;
    if (use_graph && pass == WF_PASS_RENDER) {
        ensure_wf_graph(c, W, m.vol, m.particle, m.sort, m.deep, m.wide);
        CK(cudaEventRecord(c->events[0], s));
        CK(cudaGraphLaunch(c->wf_exec, s));
        CK(cudaEventRecord(c->events[1], s));
        CK(cudaMemcpyAsync(c->h_ctr, c->d_ctr, sizeof(WfCounters), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        const uint64_t iters = (uint64_t)std::max(0, c->h_ctr->iter);
        t->launches += (m.sort ? 7 : 5) * iters;
        t->trace_launches += 2 * iters;
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, c->events[0], c->events[1]));
        t->trace_ms += ms;                     /* the whole loop: not split by phase */
        return;
    }
    CK(cudaMemcpyAsync(c->h_ctr, c->d_ctr, sizeof(WfCounters), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    while (c->h_ctr->n_active[c->h_ctr->iter & 1] > 0 || c->h_ctr->n_shadow > 0) {
        if (c->cancel.load()) throw RtFail(RT_ERR_CANCELLED, "render cancelled");
        if (c->h_ctr->iter >= W.iter_cap) throw RtFail(RT_ERR_ITER_CAP, "wavefront: bounce iteration cap reached (WF_ITER_CAP)");
        NvtxRange nvtx_iter("rt.wavefront_iteration");
        CK(cudaEventRecord(c->events[0], s));
        CK(rt_wf_trace(W, c->status, c->stats, c->counting, s, m.deep, m.wide, &c->fork));
        CK(cudaEventRecord(c->events[1], s));
        CK(cudaEventRecord(c->events[2], s));
        CK(rt_wf_shade(W, c->h_ctr->n_active[c->h_ctr->iter & 1], c->status, c->stats, c->counting, 0, false, s,
                       &t->launches, pass, adj, m.vol, m.particle, m.sort));
        CK(cudaEventRecord(c->events[3], s));
        t->launches += 2;
        t->trace_launches += 2;
        CK(cudaMemcpyAsync(c->h_ctr, c->d_ctr, sizeof(WfCounters), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, c->events[0], c->events[1])); t->trace_ms += ms;
        CK(cudaEventElapsedTime(&ms, c->events[2], c->events[3])); t->shade_ms += ms;
    }
}

void wf_store_totals(Ctx* c, const WfTotals& t) {
    c->last.render_kernel_ms = t.trace_ms;
    c->last.shade_kernel_ms = t.shade_ms;
    c->last.render_launches = t.trace_launches;
    c->last.kernel_launches = t.launches;
}

/* The light tracer as a wavefront (rt_wavefront.cu): rounds of up to
 * 4 x sample_budget particles (cancellation is checked between rounds); in
 * a round, path slots are refilled with the next particle until none is
 * left.  The bounce loop is driven from the host or runs as one CUDA graph
 * launch per round. */
void particle_wavefront(Ctx* c, const RtParams& P, int64_t first, int64_t count, float* film, cudaStream_t s,
                        bool use_graph) {
    const int64_t round_max = std::max<int64_t>(1, 4 * c->sample_budget);
    const int slots = (int)std::min<int64_t>(std::min<int64_t>(c->wf_capacity, WF_MAX_SLOTS),
                                             std::min(count, round_max) + 31);
    ensure_wf(c, slots);
    ensure_events(c, 4);
    WfState W = c->wf;
    W.slots = slots;
    W.shadow_base = 2 * slots;
    W.refill = c->wf_refill;
    W.iter_cap = c->wf_iter_cap;
    W.dense_sort = 1;
    WfMode m;
    m.particle = true;
    m.sort = c->mat_types > 1;
    m.deep = c->tallest >= RT_DEEP_TREE;
    m.wide = c->traversal == RT_TRAVERSAL_WIDE && c->view.wide_ok;
    WfTotals t;
    for (int64_t done = 0; done < count;) {
        if (c->cancel.load()) throw RtFail(RT_ERR_CANCELLED, "render cancelled");
        const int64_t n = std::min(round_max, count - done);
        CK(cudaStreamSynchronize(s));          /* the pinned staging is free */
        WfJob& d = c->h_jobs[0];
        d.view = c->d_view;
        d.P = P;
        d.samples = film;
        d.first = first + done;
        d.count = n;
        h2d(c, c->d_jobs, c->h_jobs, sizeof(WfJob), s);
        wf_round(c, W, s, use_graph, m, WF_PASS_RENDER, nullptr, n, 1, &t);
        done += n;
    }
    wf_store_totals(c, t);
}

/* AdjointParticleRenderer (Renderers/AdjointParticleRenderer.cs:118-172): the
 * particles in launches of up to sample_budget, then the finishing pass */
void render_particles(Ctx* c, const rt_render_params* p, int64_t first, int64_t count, float* dst, bool dst_host,
                      cudaStream_t user) {
    NvtxRange nvtx_("rt.render_particles");
    RtParams P = particle_params(c, p, first, count);
    if (!dst) throw RtFail(RT_ERR_INVALID_ARG, "render_particles: null output");
    cudaStream_t s = user ? user : c->stream;
    const int64_t npix = (int64_t)P.w * P.h;
    ensure(&c->film, &c->film_bytes, (size_t)npix * 16);    /* float4 sums: one vector atomic per splat */
    float4* film = reinterpret_cast<float4*>(c->film);
    CK(cudaMemsetAsync(film, 0, (size_t)npix * 16, s));
    CK(cudaMemsetAsync(c->status, 0, 4, s));
    CK(cudaMemsetAsync(c->stats, 0, 8 * sizeof(unsigned long long), s));
    c->cancel.store(0);
    const bool mega = c->renderer == RT_RENDERER_MEGAKERNEL;
    const int64_t chunk = std::max<int64_t>(1, c->sample_budget);
    const int64_t nchunks = mega ? (count + chunk - 1) / chunk : 0;
    if (mega) {
        ensure_events(c, 2 * (size_t)nchunks);
        for (int64_t b = 0, ci = 0; b < count; b += chunk, ci++) {
            if (ci >= 2) CK(cudaEventSynchronize(c->events[2 * (ci - 2) + 1]));
            if (c->cancel.load()) {
                cudaStreamSynchronize(s);
                throw RtFail(RT_ERR_CANCELLED, "render cancelled");
            }
            CK(cudaEventRecord(c->events[2 * ci], s));
            CK(rt_launch_particles(c->d_view, P, first + b, std::min(chunk, count - b), film, c->status, c->stats,
                                   c->counting, s));
            CK(cudaEventRecord(c->events[2 * ci + 1], s));
        }
    } else {
        /* AUTO: the graph-driven loop (the particles' long Russian-roulette tails make many short iterations) */
        particle_wavefront(c, P, first, count, c->film, s,
                           c->renderer == RT_RENDERER_WAVEFRONT_GRAPH || c->renderer == RT_RENDERER_AUTO);
    }
    const rt_stats wf_last = c->last;
    float* out = dst;
    if (dst_host) {
        ensure(&c->out, &c->out_bytes, (size_t)npix * 12);
        out = c->out;
    }
    /* float v = (float)ScreenX * ScreenY / pathCount (AdjointParticleRenderer.cs:156-157) */
    const float v = (float)P.w * (float)P.h / (float)count;
    CK(rt_launch_particle_finish(c->d_view, npix, film, v, out, c->status, c->stats, c->counting, s));
    if (dst_host) CK(cudaMemcpyAsync(dst, out, (size_t)npix * 12, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    check_status(c);
    double ms = 0;
    for (int64_t ci = 0; ci < nchunks; ci++) {
        float t = 0;
        CK(cudaEventElapsedTime(&t, c->events[2 * ci], c->events[2 * ci + 1]));
        ms += t;
    }
    std::memset(&c->last, 0, sizeof(c->last));
    c->last.h2d_bytes = c->h2d;
    read_stats(c);
    c->last.samples = (uint64_t)count;
    if (mega) {
        c->last.render_kernel_ms = ms;
        c->last.render_launches = (uint64_t)nchunks;
        c->last.kernel_launches = (uint64_t)nchunks + 1;
    } else {
        c->last.render_kernel_ms = wf_last.render_kernel_ms;
        c->last.shade_kernel_ms = wf_last.shade_kernel_ms;
        c->last.render_launches = wf_last.render_launches;
        c->last.kernel_launches = wf_last.kernel_launches + 1;
    }
}

/* parity hook: each particle's camera connections into host arrays */
void particle_splats(Ctx* c, const rt_render_params* p, int64_t first, int64_t count, int max_per, int32_t* n,
                     int32_t* pix, float* rgb) {
    RtParams P = particle_params(c, p, first, count);
    if (max_per < 0 || !n || (max_per > 0 && (!pix || !rgb)) || count > (int64_t)1 << 26)
        throw RtFail(RT_ERR_INVALID_ARG, "particle_splats: bad output");
    const size_t nb = (size_t)count * 4, pb = (size_t)count * max_per * 4, rb = pb * 3;
    char* buf = nullptr;
    CK(rt_dev_malloc((void**)&buf, nb + pb + rb + 16));
    struct Free { char* b; ~Free() { cudaFree(b); } } guard{buf};
    int32_t* dn = (int32_t*)buf;
    int32_t* dp = (int32_t*)(buf + nb);
    float* dr = (float*)(buf + nb + pb);
    CK(cudaMemsetAsync(c->status, 0, 4, c->stream));
    CK(rt_launch_particle_records(c->d_view, P, first, count, dn, dp, dr, max_per, c->status, c->stream));
    CK(cudaMemcpyAsync(n, dn, nb, cudaMemcpyDeviceToHost, c->stream));
    if (max_per > 0) {
        CK(cudaMemcpyAsync(pix, dp, pb, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(rgb, dr, rb, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    check_status(c);
}

/* rt_render_device_noalloc: the megakernel render with every buffer carved
 * out of the fixed scratch array.  The first call on a device looks the array
 * up (which loads its module); after that a call issues only kernels,
 * memsets, one 4-byte read of the status word and a stream synchronisation,
 * and allocates nothing. */
void render_noalloc(Ctx* c, const rt_render_params* p, float* dst, cudaStream_t user) {
    if (!c->has_scene) throw RtFail(RT_ERR_NO_SCENE, "no scene uploaded");
    if (!c->noalloc) CK(rt_noalloc_scratch(c->device, (void**)&c->noalloc));
    if (!p || !dst || p->spp <= 0) throw RtFail(RT_ERR_INVALID_ARG, "render: null params/output or spp <= 0");
    if (p->integrator != RT_INTEGRATOR_PATH && p->integrator != RT_INTEGRATOR_VOL_PATH) throw RtFail(RT_ERR_INVALID_ARG, "render: unknown integrator");
    RtParams P{};
    P.integrator = p->integrator; P.method = p->method; P.strategy = p->strategy;
    P.max_depth = p->max_depth; P.min_depth = p->min_depth; P.rr = p->rr_threshold;
    P.seed = p->seed; P.x0 = p->x0; P.y0 = p->y0;
    P.w = p->width > 0 ? p->width : c->width - p->x0;
    P.h = p->height > 0 ? p->height : c->height - p->y0;
    if (P.x0 < 0 || P.y0 < 0 || P.w <= 0 || P.h <= 0 || P.x0 + P.w > c->width || P.y0 + P.h > c->height)
        throw RtFail(RT_ERR_INVALID_ARG, "render: crop outside the film");
    P.spp = p->spp; P.sample_begin = p->sample_begin;
    const int64_t npix = (int64_t)P.w * P.h;
    const int64_t plane = npix * 12, head = 512, film_bytes = (plane + 255) / 256 * 256;
    const int64_t room = (int64_t)RT_NOALLOC_SCRATCH_BYTES - head - film_bytes;
    if (room < plane) {
        char msg[192];
        std::snprintf(msg, sizeof(msg), "render_noalloc: a %d x %d crop needs %lld bytes of scratch, the fixed array holds %u",
                      P.w, P.h, (long long)(head + film_bytes + plane), RT_NOALLOC_SCRATCH_BYTES);
        throw RtFail(RT_ERR_INVALID_ARG, msg);
    }
    uint32_t* status = (uint32_t*)c->noalloc;
    unsigned long long* stats = (unsigned long long*)(c->noalloc + 256);
    float* film = (float*)(c->noalloc + head);
    float* samples = (float*)(c->noalloc + head + film_bytes);
    const int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(P.spp, room / plane));
    cudaStream_t s = user ? user : c->stream;
    CK(cudaMemsetAsync(c->noalloc, 0, (size_t)head, s));
    CK(cudaMemsetAsync(film, 0, (size_t)plane, s));
    c->cancel.store(0);
    uint64_t launches = 0, chunks = 0;
    for (int b = 0; b < P.spp; b += chunk) {
        if (c->cancel.load()) {
            /* the queued chunks still write the shared array: let them finish
             * so the next call, from any context, starts on an idle array */
            cudaStreamSynchronize(s);
            throw RtFail(RT_ERR_CANCELLED, "render cancelled");
        }
        P.chunk_begin = b;
        P.chunk_len = std::min(chunk, P.spp - b);
        CK(rt_launch_render(c->d_view, P, samples, status, stats, false, s));
        CK(rt_launch_accumulate(film, samples, npix, P.chunk_len, s));
        launches += 2;
        chunks++;
    }
    CK(rt_launch_finalize(dst, film, npix, (float)P.spp, s));
    uint32_t st = 0;
    CK(cudaMemcpyAsync(&st, status, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::memset(&c->last, 0, sizeof(c->last));
    c->last.h2d_bytes = c->h2d;
    c->last.samples = (uint64_t)npix * P.spp;
    c->last.render_launches = chunks;
    c->last.kernel_launches = launches + 1;
    throw_status(st);
}

/* one render of a wavefront run: scene, parameters (full spp), film sums */
struct WfJobIn {
    const RtSceneView* view;
    RtParams P;
    float* film;
    int mat_types;         /* distinct material types of the job's scene */
    int tallest;           /* levels of its tallest tree */
    bool wide_ok;          /* its wide trees fit the fast traversal's stack */
};

/* The bounce loop as a graph: a while node whose body is one iteration
 * (trace, phase, sort, shade, tail); the tail kernel clears the loop's
 * condition when no path is left.  Rebuilt when the path state moves or the
 * counting mode changes. */
void ensure_wf_graph(Ctx* c, const WfState& W, bool vol, bool particle, bool sort, bool deep, bool wide) {
    const uint64_t key = (c->wf_generation << 32) ^ ((uint64_t)wide << 63) ^ ((uint64_t)W.slots << 10) ^ ((uint64_t)deep << 9) ^
                         ((uint64_t)(uint32_t)W.iter_cap * 0x9E3779B97F4A7C15ull) ^
                         ((uint64_t)sort << 8) ^ ((uint64_t)particle << 7) ^ ((uint64_t)W.refill << 2) ^
                         ((uint64_t)vol << 1) ^ (c->counting ? 1u : 0u);
    if (c->wf_exec && c->wf_graph_key == key) return;
    if (c->wf_exec) { cudaGraphExecDestroy(c->wf_exec); c->wf_exec = nullptr; }
    if (c->wf_graph) { cudaGraphDestroy(c->wf_graph); c->wf_graph = nullptr; }
    CK(cudaGraphCreate(&c->wf_graph, 0));
    cudaGraphConditionalHandle loop;
    CK(cudaGraphConditionalHandleCreate(&loop, c->wf_graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = loop;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, c->wf_graph, nullptr, nullptr, 0, &np));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    CK(cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    uint64_t launches = 0;
    cudaError_t e1 = rt_wf_trace(W, c->status, c->stats, c->counting, c->stream, deep, wide, &c->fork);
    cudaError_t e2 = rt_wf_shade(W, -1, c->status, c->stats, c->counting, loop, true, c->stream, &launches,
                                 WF_PASS_RENDER, nullptr, vol, particle, sort);
    cudaGraph_t captured = nullptr;
    CK(cudaStreamEndCapture(c->stream, &captured));
    CK(e1);
    CK(e2);
    CK(cudaGraphInstantiate(&c->wf_exec, c->wf_graph, 0));
    c->wf_graph_key = key;
}

/* Renders every job: rounds of up to sample_budget samples (each job gets
 * the same number of sample indices per round); within a round all jobs'
 * paths share the path slots, queues and launches (rt_wavefront.cu).  The
 * bounce loop is driven from the host (per-phase timing) or, with
 * `use_graph`, runs as one CUDA graph launch per round. */
void wavefront_run(Ctx* c, const std::vector<WfJobIn>& jobs, cudaStream_t s, bool use_graph,
                   const WfAdjoint* adj = nullptr) {
    if (jobs.empty() || jobs.size() > WF_MAX_JOBS) throw RtFail(RT_ERR_INVALID_ARG, "wavefront: 1 to 256 jobs per run");
    std::vector<int> done(jobs.size(), 0);
    /* one integrator per run: the vol_path shade kernel or the path one */
    const bool vol = jobs[0].P.integrator == RT_INTEGRATOR_VOL_PATH;
    for (const WfJobIn& J : jobs)
        if ((J.P.integrator == RT_INTEGRATOR_VOL_PATH) != vol)
            throw RtFail(RT_ERR_UNSUPPORTED, "wavefront: a run renders one integrator");
    if (vol && adj) throw RtFail(RT_ERR_UNSUPPORTED, "adjoint: the path integrator is differentiated");
    /* the shade-key sort groups paths by material type: one `path` scene of one type gains nothing
     * from it when rendering.  vol_path keys also separate medium-boundary hits and paths advancing
     * boundary walks, and the adjoint replay's gradient scatter gains from grouped paths (C5: 22.1
     * gradients/s unsorted, 28.5 sorted), so both keep it. */
    WfMode mode;
    mode.vol = vol;
    mode.sort = vol || adj || jobs.size() > 1 || jobs[0].mat_types > 1;
    for (const WfJobIn& J : jobs) mode.deep = mode.deep || J.tallest >= RT_DEEP_TREE;
    mode.wide = c->traversal == RT_TRAVERSAL_WIDE;
    for (const WfJobIn& J : jobs) mode.wide = mode.wide && J.wide_ok;
    ensure_events(c, 4);
    WfTotals tot;
    while (true) {
        if (c->cancel.load()) throw RtFail(RT_ERR_CANCELLED, "render cancelled");
        std::vector<int> act;
        int64_t npix_total = 0;
        for (size_t j = 0; j < jobs.size(); j++)
            if (done[j] < jobs[j].P.spp) { act.push_back((int)j); npix_total += (int64_t)jobs[j].P.w * jobs[j].P.h; }
        if (act.empty()) break;
        const int64_t chunk = std::max<int64_t>(1, c->sample_budget / npix_total);
        int64_t total = 0;
        std::vector<int> clen(act.size());
        for (size_t k = 0; k < act.size(); k++) {
            const WfJobIn& J = jobs[act[k]];
            clen[k] = (int)std::min<int64_t>(chunk, J.P.spp - done[act[k]]);
            total += (int64_t)J.P.w * J.P.h * clen[k];
        }
        ensure(&c->samples, &c->samples_bytes, (size_t)total * 12);
        const int slots = (int)std::min<int64_t>(std::min<int64_t>(c->wf_capacity, WF_MAX_SLOTS), total + 31);
        ensure_wf(c, slots);
        CK(cudaStreamSynchronize(s));          /* the pinned staging of the last round has been read */
        int64_t first = 0;
        for (size_t k = 0; k < act.size(); k++) {
            const WfJobIn& J = jobs[act[k]];
            WfJob& d = c->h_jobs[k];
            d.view = J.view;
            d.P = J.P;
            d.P.chunk_begin = done[act[k]];
            d.P.chunk_len = clen[k];
            d.samples = c->samples + first * 3;
            d.first = first;
            d.count = (int64_t)J.P.w * J.P.h * clen[k];
            first += d.count;
        }
        h2d(c, c->d_jobs, c->h_jobs, act.size() * sizeof(WfJob), s);
        WfState W = c->wf;
        W.slots = slots;
        W.shadow_base = 2 * slots;
        W.refill = c->wf_refill;
        W.iter_cap = c->wf_iter_cap;
        /* vol_path's shade runs slower from slots walked in index order (C3: 115.3 -> 112.5 M samples/s) */
        W.dense_sort = mode.vol ? 0 : 1;
        /* one pass over the round's samples: start every slot, bounce until no path is left */
        auto run_pass = [&](int pass) {
            wf_round(c, W, s, use_graph, mode, pass, adj, total, (int)act.size(), &tot);
        };
        if (adj) {
            run_pass(WF_PASS_FORWARD_RAW);
            run_pass(WF_PASS_REPLAY);
            for (size_t k = 0; k < act.size(); k++) done[act[k]] += clen[k];
            continue;
        }
        run_pass(WF_PASS_RENDER);
        for (size_t k = 0; k < act.size(); k++) {
            const WfJobIn& J = jobs[act[k]];
            CK(rt_launch_accumulate(J.film, c->h_jobs[k].samples, (int64_t)J.P.w * J.P.h, clen[k], s));
            tot.launches += 1;
            done[act[k]] += clen[k];
        }
    }
    wf_store_totals(c, tot);
}

void render_wavefront(Ctx* c, RtParams P, int chunk, int64_t npix, cudaStream_t s) {
    (void)chunk; (void)npix;
    std::vector<WfJobIn> jobs(1);
    jobs[0].view = c->d_view;
    jobs[0].P = P;
    jobs[0].film = c->film;
    jobs[0].mat_types = c->mat_types;
    jobs[0].tallest = c->tallest;
    jobs[0].wide_ok = c->view.wide_ok != 0;
    /* AUTO drives vol_path's loop as a graph: its boundary walks make ~100 short iterations per
     * round, where the host loop's per-iteration synchronisation costs 9 % (C3) */
    const bool vol = P.integrator == RT_INTEGRATOR_VOL_PATH;
    wavefront_run(c, jobs, s, c->renderer == RT_RENDERER_WAVEFRONT_GRAPH ||
                              (c->renderer == RT_RENDERER_AUTO && (c->wf_graph_pref || vol)));
}

/* rt_render_batch(_device): every item's film through one wavefront run;
 * out_rgb are host pointers, or device pointers written on `user` */
void render_batch(Ctx* c, const rt_batch_item* items, int n, bool device_out, cudaStream_t user) {
    NvtxRange nvtx_("rt.render_batch");
    if (!items || n <= 0 || n > WF_MAX_JOBS) throw RtFail(RT_ERR_INVALID_ARG, "render_batch: 1 to 256 items");
    std::vector<WfJobIn> jobs((size_t)n);
    std::vector<int64_t> film_off((size_t)n);
    int64_t film_floats = 0;
    for (int i = 0; i < n; i++) {
        const rt_batch_item& it = items[i];
        Ctx* sc = (Ctx*)it.scene_ctx;
        const rt_render_params* p = &it.params;
        if (!sc || !it.out_rgb) throw RtFail(RT_ERR_INVALID_ARG, "render_batch: item " + std::to_string(i) + " has no scene context or output");
        if (sc->device != c->device) throw RtFail(RT_ERR_INVALID_ARG, "render_batch: item " + std::to_string(i) + " is on another device");
        if (!sc->has_scene) throw RtFail(RT_ERR_NO_SCENE, "render_batch: item " + std::to_string(i) + " has no uploaded scene");
        if (p->spp <= 0) throw RtFail(RT_ERR_INVALID_ARG, "render_batch: item " + std::to_string(i) + " has spp <= 0");
        if ((p->integrator != RT_INTEGRATOR_PATH && p->integrator != RT_INTEGRATOR_VOL_PATH) ||
            (p->strategy != RT_STRATEGY_UNIFORM && p->integrator != RT_INTEGRATOR_PATH) ||
            p->integrator != items[0].params.integrator)
            throw RtFail(RT_ERR_UNSUPPORTED, "render_batch: items must share the path or vol_path integrator; vol_path items use the Uniform light strategy");
        RtParams P{};
        P.integrator = p->integrator; P.method = p->method; P.strategy = p->strategy;
        P.max_depth = p->max_depth; P.min_depth = p->min_depth; P.rr = p->rr_threshold;
        P.seed = p->seed; P.x0 = p->x0; P.y0 = p->y0;
        P.w = p->width > 0 ? p->width : sc->width - p->x0;
        P.h = p->height > 0 ? p->height : sc->height - p->y0;
        if (P.x0 < 0 || P.y0 < 0 || P.w <= 0 || P.h <= 0 || P.x0 + P.w > sc->width || P.y0 + P.h > sc->height)
            throw RtFail(RT_ERR_INVALID_ARG, "render_batch: item " + std::to_string(i) + " crop outside the film");
        P.spp = p->spp; P.sample_begin = p->sample_begin;
        jobs[i].view = sc->d_view;
        jobs[i].P = P;
        jobs[i].mat_types = sc->mat_types;
        jobs[i].tallest = sc->tallest;
        jobs[i].wide_ok = sc->view.wide_ok != 0;
        film_off[i] = film_floats;
        film_floats += (int64_t)P.w * P.h * 3;
    }
    cudaStream_t s = device_out && user ? user : c->stream;
    ensure(&c->film, &c->film_bytes, (size_t)film_floats * 4);
    if (!device_out) ensure(&c->out, &c->out_bytes, (size_t)film_floats * 4);
    for (int i = 0; i < n; i++) jobs[i].film = c->film + film_off[i];
    CK(cudaMemsetAsync(c->film, 0, (size_t)film_floats * 4, s));
    CK(cudaMemsetAsync(c->status, 0, 4, s));
    CK(cudaMemsetAsync(c->stats, 0, 8 * sizeof(unsigned long long), s));
    c->cancel.store(0);
    wavefront_run(c, jobs, s, c->renderer == RT_RENDERER_WAVEFRONT_GRAPH ||
                              (c->renderer == RT_RENDERER_AUTO && c->wf_graph_pref));
    uint64_t samples = 0;
    for (int i = 0; i < n; i++) {
        const int64_t npix = (int64_t)jobs[i].P.w * jobs[i].P.h;
        if (device_out) {
            CK(rt_launch_finalize(items[i].out_rgb, c->film + film_off[i], npix, (float)jobs[i].P.spp, s));
        } else {
            CK(rt_launch_finalize(c->out + film_off[i], c->film + film_off[i], npix, (float)jobs[i].P.spp, s));
            CK(cudaMemcpyAsync(items[i].out_rgb, c->out + film_off[i], (size_t)npix * 12, cudaMemcpyDeviceToHost, s));
        }
        samples += (uint64_t)npix * jobs[i].P.spp;
    }
    CK(cudaStreamSynchronize(s));
    check_status(c);
    double rms = c->last.render_kernel_ms, sms = c->last.shade_kernel_ms;
    uint64_t launches = c->last.kernel_launches, rl = c->last.render_launches;
    std::memset(&c->last, 0, sizeof(c->last));
    c->last.h2d_bytes = c->h2d;
    read_stats(c);
    c->last.samples = samples;
    c->last.render_kernel_ms = rms;
    c->last.shade_kernel_ms = sms;
    c->last.render_launches = rl;
    c->last.kernel_launches = launches + (uint64_t)n;
}

/* rt_adjoint_backward: gradients of sum(dL/dI * I) through the MIS path tracer
 * (rt_adjoint.cu), chunked over samples like the megakernel render */
void adjoint_backward(Ctx* c, const rt_render_params* p, const rt_adjoint_desc* d, const float* dldi, float* g_albedo,
                      float* g_alpha) {
    NvtxRange nvtx_("rt.adjoint_backward");
    if (!c->has_scene) throw RtFail(RT_ERR_NO_SCENE, "no scene uploaded");
    if (!p || !d || !dldi || p->spp <= 0) throw RtFail(RT_ERR_INVALID_ARG, "adjoint: null params / descriptor / dL_dimage or spp <= 0");
    if (p->integrator != RT_INTEGRATOR_PATH || p->method != RT_METHOD_MIS)
        throw RtFail(RT_ERR_UNSUPPORTED, "adjoint: the path integrator with MIS is differentiated");
    const int ntex = (int)c->h_textures.size(), nmat = (int)c->h_materials.size();
    if (d->albedo_texture < -1 || d->albedo_texture >= ntex) throw RtFail(RT_ERR_INVALID_ARG, "adjoint: bad albedo texture");
    if (d->albedo_texture >= 0 && !g_albedo) throw RtFail(RT_ERR_INVALID_ARG, "adjoint: grad_albedo is null");
    if (d->alpha_count < 0 || d->alpha_count > RT_ADJ_MAX_ALPHA || (d->alpha_count > 0 && (!d->alpha_materials || !g_alpha)))
        throw RtFail(RT_ERR_INVALID_ARG, "adjoint: bad alpha parameter list");
    std::vector<int> slot((size_t)std::max(1, nmat), -1);
    for (int i = 0; i < d->alpha_count; i++) {
        const int m = d->alpha_materials[i];
        if (m < 0 || m >= nmat) throw RtFail(RT_ERR_INVALID_ARG, "adjoint: alpha material index out of range");
        if (slot[m] >= 0) throw RtFail(RT_ERR_INVALID_ARG, "adjoint: alpha material listed twice");
        const int t = c->h_materials[m].type;
        if (t != RT_MAT_ROUGH_PLASTIC && t != RT_MAT_ROUGH_METAL)
            throw RtFail(RT_ERR_UNSUPPORTED, "adjoint: alpha gradients are for rough_plastic and rough_metal");
        slot[m] = i;
    }
    RtParams P{};
    P.integrator = p->integrator; P.method = p->method; P.strategy = p->strategy;
    P.max_depth = p->max_depth; P.min_depth = p->min_depth; P.rr = p->rr_threshold;
    P.seed = p->seed; P.x0 = p->x0; P.y0 = p->y0;
    P.w = p->width > 0 ? p->width : c->width - p->x0;
    P.h = p->height > 0 ? p->height : c->height - p->y0;
    if (P.x0 < 0 || P.y0 < 0 || P.w <= 0 || P.h <= 0 || P.x0 + P.w > c->width || P.y0 + P.h > c->height)
        throw RtFail(RT_ERR_INVALID_ARG, "adjoint: crop outside the film");
    P.spp = p->spp; P.sample_begin = p->sample_begin;
    cudaStream_t s = c->stream;
    const int64_t npix = (int64_t)P.w * P.h;
    const int64_t texels = d->albedo_texture >= 0
        ? (int64_t)c->h_textures[d->albedo_texture].width * c->h_textures[d->albedo_texture].height : 0;
    ensure(&c->adj_dldi, &c->adj_dldi_bytes, (size_t)npix * 12);
    ensure(&c->adj_galb, &c->adj_galb_bytes, (size_t)std::max<int64_t>(1, texels) * 12);
    ensure(&c->adj_galpha, &c->adj_galpha_bytes, (size_t)std::max(1, d->alpha_count) * 4);
    ensure(&c->adj_slot, &c->adj_slot_bytes, slot.size() * 4);
    h2d(c, c->adj_dldi, dldi, (size_t)npix * 12, s);
    h2d(c, c->adj_slot, slot.data(), slot.size() * 4, s);
    CK(rt_launch_scale(c->adj_dldi, npix * 3, 1.0f / (float)P.spp, s));
    CK(cudaMemsetAsync(c->adj_galb, 0, (size_t)std::max<int64_t>(1, texels) * 12, s));
    CK(cudaMemsetAsync(c->adj_galpha, 0, (size_t)std::max(1, d->alpha_count) * 4, s));
    CK(cudaMemsetAsync(c->status, 0, 4, s));
    c->cancel.store(0);
    const int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(P.spp, c->sample_budget / std::max<int64_t>(1, npix)));
    ensure_events(c, 4);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, s));
    uint64_t launches = 2;
    if (P.strategy == RT_STRATEGY_UNIFORM) {
        /* the wavefront: a forward pass keeping each sample's radiance, then the replay */
        WfAdjoint A{d->albedo_texture, d->alpha_count, c->adj_slot, c->adj_galb, c->adj_galpha, c->adj_dldi};
        std::vector<WfJobIn> jobs(1);
        jobs[0].view = c->d_view;
        jobs[0].P = P;
        jobs[0].film = nullptr;
        jobs[0].mat_types = c->mat_types;
        jobs[0].tallest = c->tallest;
        jobs[0].wide_ok = c->view.wide_ok != 0;
        CK(cudaMemsetAsync(c->stats, 0, 8 * sizeof(unsigned long long), s));
        wavefront_run(c, jobs, s, false, &A);
        launches += c->last.kernel_launches;
    } else {
        for (int b = 0; b < P.spp; b += chunk) {
            if (c->cancel.load()) throw RtFail(RT_ERR_CANCELLED, "adjoint cancelled");
            P.chunk_begin = b;
            P.chunk_len = std::min(chunk, P.spp - b);
            CK(rt_launch_adjoint(c->d_view, P, d->albedo_texture, c->adj_slot, c->adj_galb, c->adj_galpha, d->alpha_count,
                                 c->adj_dldi, c->status, s));
            launches++;
        }
    }
    CK(cudaEventRecord(e1, s));
    if (texels > 0) CK(cudaMemcpyAsync(g_albedo, c->adj_galb, (size_t)texels * 12, cudaMemcpyDeviceToHost, s));
    if (d->alpha_count > 0) CK(cudaMemcpyAsync(g_alpha, c->adj_galpha, (size_t)d->alpha_count * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    check_status(c);
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::memset(&c->last, 0, sizeof(c->last));
    c->last.h2d_bytes = c->h2d;
    c->last.samples = (uint64_t)npix * P.spp;
    c->last.render_kernel_ms = ms;
    c->last.kernel_launches = launches;
    c->last.render_launches = launches - 1;
}

/* rt_update_texture: new texels for one texture of the uploaded scene */
void update_texture(Ctx* c, int tex, const float* texels) {
    if (!c->has_scene) throw RtFail(RT_ERR_NO_SCENE, "no scene uploaded");
    if (tex < 0 || tex >= (int)c->h_textures.size() || !texels) throw RtFail(RT_ERR_INVALID_ARG, "update_texture: bad texture or data");
    if (c->env_texture[tex]) throw RtFail(RT_ERR_UNSUPPORTED, "update_texture: the texture feeds an infinite light's sampling table; upload the scene again");
    const RtTexture& t = c->h_textures[tex];
    CK(cudaMemcpyAsync((void*)(c->view.texels + t.offset), texels, (size_t)t.width * t.height * 12, cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
}

/* rt_autotune: times the caller's batch under each setting that leaves films
 * unchanged (path slots in flight, trace-warp refill threshold, host- or
 * graph-driven bounce loop) and keeps the fastest on the context */
void autotune(Ctx* c, const rt_batch_item* items, int n, rt_tune_result* out) {
    NvtxRange nvtx_("rt.autotune");
    if (!items || n <= 0 || !out) throw RtFail(RT_ERR_INVALID_ARG, "autotune: no items or no result");
    const int caps[] = {WF_MAX_SLOTS, WF_MAX_SLOTS / 2, WF_MAX_SLOTS / 4};
    const int refills[] = {8, 4, 16};
    const int modes[] = {RT_RENDERER_WAVEFRONT, RT_RENDERER_WAVEFRONT_GRAPH};
    const int keep_cap = c->wf_capacity, keep_refill = c->wf_refill, keep_mode = c->renderer;
    const bool keep_pref = c->wf_graph_pref;
    auto probe = [&](int cap, int refill, int mode) {
        c->wf_capacity = cap; c->wf_refill = refill; c->renderer = mode;
        render_batch(c, items, n, false, nullptr);               /* warm: buffers, graph */
        const auto t0 = std::chrono::steady_clock::now();
        render_batch(c, items, n, false, nullptr);
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    };
    double best = 1e300, base = 0;
    int bc = keep_cap, br = keep_refill, bm = RT_RENDERER_WAVEFRONT;
    try {
        for (int mode : modes)
            for (int cap : caps)
                for (int refill : refills) {
                    const double ms = probe(cap, refill, mode);
                    if (mode == RT_RENDERER_WAVEFRONT && cap == WF_MAX_SLOTS && refill == 8) base = ms;
                    if (ms < best) { best = ms; bc = cap; br = refill; bm = mode; }
                }
    } catch (...) {
        c->wf_capacity = keep_cap; c->wf_refill = keep_refill; c->renderer = keep_mode; c->wf_graph_pref = keep_pref;
        throw;
    }
    c->wf_capacity = bc; c->wf_refill = br; c->renderer = keep_mode;
    c->wf_graph_pref = bm == RT_RENDERER_WAVEFRONT_GRAPH;
    out->capacity = bc; out->refill = br; out->renderer = bm;
    out->ms = (float)best; out->ms_default = (float)base;
}

void trace(Ctx* c, const rt_ray* rays, int64_t n, rt_hit* hits, uint8_t* occ, bool host, cudaStream_t user) {
    NvtxRange nvtx_("rt.trace");
    if (!c->has_scene) throw RtFail(RT_ERR_NO_SCENE, "no scene uploaded");
    if (n < 0 || (n > 0 && (!rays || (!hits && !occ)))) throw RtFail(RT_ERR_INVALID_ARG, "trace: bad arguments");
    cudaStream_t s = user ? user : c->stream;
    CK(cudaMemsetAsync(c->status, 0, 4, s));
    CK(cudaMemsetAsync(c->stats, 0, 8 * sizeof(unsigned long long), s));
    const rt_ray* dr = rays;
    rt_hit* dh = hits;
    uint8_t* dob = occ;
    if (host && n > 0) {
        size_t out_bytes = hits ? (size_t)n * sizeof(rt_hit) : (size_t)n;
        ensure(&c->io, &c->io_bytes, (size_t)n * sizeof(rt_ray) + out_bytes + 256);
        char* base = (char*)c->io;
        h2d(c, base, rays, (size_t)n * sizeof(rt_ray), s);
        dr = (const rt_ray*)base;
        char* ob = base + (((size_t)n * sizeof(rt_ray) + 255) & ~(size_t)255);
        if (hits) dh = (rt_hit*)ob; else dob = (uint8_t*)ob;
    }
    CK(rt_launch_trace(c->d_view, dr, n, dh, dob, c->status, c->stats, c->counting, s,
                       c->traversal == RT_TRAVERSAL_WIDE && c->view.wide_ok));
    if (host && n > 0) {
        if (hits) CK(cudaMemcpyAsync(hits, dh, (size_t)n * sizeof(rt_hit), cudaMemcpyDeviceToHost, s));
        else CK(cudaMemcpyAsync(occ, dob, (size_t)n, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
    check_status(c);
    std::memset(&c->last, 0, sizeof(c->last));
    c->last.h2d_bytes = c->h2d;
    read_stats(c);
    if (hits) c->last.rays_closest = (uint64_t)n; else c->last.rays_shadow = (uint64_t)n;
    c->last.kernel_launches = n > 0 ? 1 : 0;
}

template <class F>
int run(Ctx* c, F f) {
    if (!c) return RT_ERR_INVALID_ARG;
    try {
        CK(cudaSetDevice(c->device));
        c->h2d = 0;
        f();
        c->err.clear();
        return RT_OK;
    } catch (const RtFail& e) {
        c->err = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        c->err = "host allocation failed";
        return RT_ERR_OOM;
    } catch (const std::exception& e) {
        c->err = e.what();
        return RT_ERR_INVALID_ARG;
    }
}

}  // namespace

extern "C" {

int rt_abi_version(void) { return RT_ABI_VERSION; }

int rt_create(int device, void** out_ctx) {
    if (!out_ctx) return RT_ERR_INVALID_ARG;
    *out_ctx = nullptr;
    Ctx* c = new (std::nothrow) Ctx();
    if (!c) return RT_ERR_OOM;
    c->device = device;
    int rc = run(c, [&]() {
        CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&c->fork.side, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&c->fork.fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->fork.join, cudaEventDisableTiming));
        CK(rt_dev_malloc((void**)&c->status, 4));
        CK(rt_dev_malloc((void**)&c->stats, 8 * sizeof(unsigned long long)));
    });
    if (rc != RT_OK) { rt_destroy(c); return rc; }
    *out_ctx = c;
    return RT_OK;
}

void rt_destroy(void* ctx) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return;
    cudaSetDevice(c->device);
    free_scene(c);
    if (c->samples) cudaFree(c->samples);
    if (c->film) cudaFree(c->film);
    if (c->adj_dldi) cudaFree(c->adj_dldi);
    if (c->adj_galb) cudaFree(c->adj_galb);
    if (c->adj_galpha) cudaFree(c->adj_galpha);
    if (c->adj_slot) cudaFree(c->adj_slot);
    if (c->out) cudaFree(c->out);
    if (c->io) cudaFree(c->io);
    if (c->status) cudaFree(c->status);
    if (c->stats) cudaFree(c->stats);
    free_wf(c);
    if (c->wf_exec) cudaGraphExecDestroy(c->wf_exec);
    if (c->wf_graph) cudaGraphDestroy(c->wf_graph);
    if (c->d_ctr) cudaFree(c->d_ctr);
    if (c->h_ctr) cudaFreeHost(c->h_ctr);
    if (c->d_jobs) cudaFree(c->d_jobs);
    if (c->h_jobs) cudaFreeHost(c->h_jobs);
    for (cudaEvent_t e : c->events) cudaEventDestroy(e);
    if (c->fork.fork) cudaEventDestroy(c->fork.fork);
    if (c->fork.join) cudaEventDestroy(c->fork.join);
    if (c->fork.side) cudaStreamDestroy(c->fork.side);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char* rt_last_error(const void* ctx) {
    const Ctx* c = (const Ctx*)ctx;
    return c ? c->err.c_str() : "null context";
}

int rt_upload_scene(void* ctx, const rt_scene_desc* scene) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { upload_scene(c, scene); });
}

int rt_trace_closest(void* ctx, const rt_ray* rays, int64_t n, rt_hit* hits) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { if (!hits && n > 0) throw RtFail(RT_ERR_INVALID_ARG, "null hits"); trace(c, rays, n, hits, nullptr, true, nullptr); });
}
int rt_trace_any(void* ctx, const rt_ray* rays, int64_t n, uint8_t* occluded) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { if (!occluded && n > 0) throw RtFail(RT_ERR_INVALID_ARG, "null output"); trace(c, rays, n, nullptr, occluded, true, nullptr); });
}
int rt_trace_closest_device(void* ctx, const rt_ray* d_rays, int64_t n, rt_hit* d_hits, void* stream) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { if (!d_hits && n > 0) throw RtFail(RT_ERR_INVALID_ARG, "null hits"); trace(c, d_rays, n, d_hits, nullptr, false, (cudaStream_t)stream); });
}
int rt_trace_any_device(void* ctx, const rt_ray* d_rays, int64_t n, uint8_t* d_occ, void* stream) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { if (!d_occ && n > 0) throw RtFail(RT_ERR_INVALID_ARG, "null output"); trace(c, d_rays, n, nullptr, d_occ, false, (cudaStream_t)stream); });
}
int rt_render(void* ctx, const rt_render_params* params, float* out_rgb) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { render(c, params, out_rgb, true, nullptr); });
}
int rt_render_particles(void* ctx, const rt_render_params* params, int64_t first_particle, int64_t particle_count,
                        float* out_rgb) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { render_particles(c, params, first_particle, particle_count, out_rgb, true, nullptr); });
}
int rt_render_particles_device(void* ctx, const rt_render_params* params, int64_t first_particle,
                               int64_t particle_count, float* d_out_rgb, void* stream) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() {
        render_particles(c, params, first_particle, particle_count, d_out_rgb, false, (cudaStream_t)stream);
    });
}
int rt_render_device(void* ctx, const rt_render_params* params, float* d_out_rgb, void* stream) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { render(c, params, d_out_rgb, false, (cudaStream_t)stream); });
}
int rt_adjoint_forward(void* ctx, const rt_render_params* params, float* out_rgb) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { render(c, params, out_rgb, true, nullptr); });
}
int rt_adjoint_backward(void* ctx, const rt_render_params* params, const rt_adjoint_desc* desc, const float* dL_dimage,
                        float* grad_albedo, float* grad_alpha) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { adjoint_backward(c, params, desc, dL_dimage, grad_albedo, grad_alpha); });
}
int rt_update_texture(void* ctx, int texture, const float* texels) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { update_texture(c, texture, texels); });
}
int rt_autotune(void* ctx, const rt_batch_item* items, int n, rt_tune_result* out) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { autotune(c, items, n, out); });
}
int rt_render_batch(void* ctx, const rt_batch_item* items, int n) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { render_batch(c, items, n, false, nullptr); });
}
int rt_render_batch_device(void* ctx, const rt_batch_item* items, int n, void* stream) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { render_batch(c, items, n, true, (cudaStream_t)stream); });
}
int rt_render_device_noalloc(void* ctx, const rt_render_params* params, float* d_out_rgb, void* stream) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { render_noalloc(c, params, d_out_rgb, (cudaStream_t)stream); });
}
int rt_get_stats(void* ctx, rt_stats* out) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !out) return RT_ERR_INVALID_ARG;
    *out = c->last;
    return RT_OK;
}
int rt_set_counting(void* ctx, int enabled) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return RT_ERR_INVALID_ARG;
    c->counting = enabled != 0;
    return RT_OK;
}
int rt_set_renderer(void* ctx, int mode) {
    Ctx* c = (Ctx*)ctx;
    if (!c || mode < RT_RENDERER_AUTO || mode > RT_RENDERER_WAVEFRONT_GRAPH) return RT_ERR_INVALID_ARG;
    c->renderer = mode;
    return RT_OK;
}
int rt_cancel(void* ctx) {
    Ctx* c = (Ctx*)ctx;
    if (!c) return RT_ERR_INVALID_ARG;
    c->cancel.store(1);
    return RT_OK;
}
int rt_set_traversal(void* ctx, int mode) {
    Ctx* c = (Ctx*)ctx;
    if (!c || (mode != RT_TRAVERSAL_EXACT && mode != RT_TRAVERSAL_WIDE)) return RT_ERR_INVALID_ARG;
    c->traversal = mode;
    return RT_OK;
}
int rt_set_light_sampling(void* ctx, int mode) {
    Ctx* c = (Ctx*)ctx;
    if (!c || (mode != RT_LIGHT_SAMPLING_CDF && mode != RT_LIGHT_SAMPLING_ALIAS)) return RT_ERR_INVALID_ARG;
    return run(c, [&] {
        c->light_sampling = mode;
        if (!c->has_scene) return;
        /* the flag lives in the scene's device view, which every kernel reads */
        c->view.env_alias = mode == RT_LIGHT_SAMPLING_ALIAS ? 1 : 0;
        CK(cudaMemcpyAsync(c->d_view, &c->view, sizeof(RtSceneView), cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    });
}
int rt_get_light_sampling(void* ctx, int* mode) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !mode) return RT_ERR_INVALID_ARG;
    *mode = c->light_sampling;
    return RT_OK;
}
int rt_get_traversal(void* ctx, int* effective) {
    Ctx* c = (Ctx*)ctx;
    if (!c || !effective) return RT_ERR_INVALID_ARG;
    *effective = c->traversal == RT_TRAVERSAL_WIDE && c->has_scene && c->view.wide_ok ? RT_TRAVERSAL_WIDE
                                                                                     : RT_TRAVERSAL_EXACT;
    return RT_OK;
}

/* test hook (not part of radiantium.h): builds the SAH tree of n primitive
 * boxes (6 floats each) on the host exactly as rt_upload_scene does and
 * returns it in depth-first LinearBVHNode form.  Call with null arrays to get
 * the node count.  No CUDA call is made. */
/* test hook (not in the public header): shrinks the samples per round and
 * the path slots in flight so small renders exercise several rounds and
 * heavy slot reuse; 0 keeps a value */
/* test hook (not part of radiantium.h): each particle's camera connections,
 * laid out like the oracle's or_particle_splats */
int rt_debug_particle_splats(void* ctx, const rt_render_params* params, int64_t first, int64_t count, int max_per,
                             int32_t* n, int32_t* pix, float* rgb) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() { particle_splats(c, params, first, count, max_per, n, pix, rgb); });
}
int rt_debug_set_limits(void* ctx, int64_t sample_budget, int wf_capacity) {
    Ctx* c = (Ctx*)ctx;
    if (!c || sample_budget < 0 || wf_capacity < 0) return RT_ERR_INVALID_ARG;
    if (sample_budget > 0) c->sample_budget = sample_budget;
    if (wf_capacity > 0) c->wf_capacity = std::min(wf_capacity, WF_MAX_SLOTS);
    return RT_OK;
}

int rt_debug_bvh(const float* boxes, int n, int max_prims, int64_t* node_count, float* bounds, int32_t* idx,
                 int32_t* count, int32_t* axis, int32_t* order) {
    if (!boxes || n <= 0 || !node_count) return RT_ERR_INVALID_ARG;
    try {
        std::vector<rtb::Box> b(n);
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) { b[i].mn[k] = boxes[6 * i + k]; b[i].mx[k] = boxes[6 * i + 3 + k]; }
        rtb::BuildResult r = rtb::build_sah(b, max_prims, std::max(1u, std::thread::hardware_concurrency()));
        *node_count = (int64_t)r.nodes.size();
        if (bounds) {
            for (size_t i = 0; i < r.nodes.size(); i++) {
                for (int k = 0; k < 3; k++) { bounds[6 * i + k] = r.nodes[i].bounds.mn[k]; bounds[6 * i + 3 + k] = r.nodes[i].bounds.mx[k]; }
                idx[i] = r.nodes[i].second; count[i] = r.nodes[i].count; axis[i] = r.nodes[i].axis;
            }
            for (int i = 0; i < n; i++) order[i] = r.order[i];
        }
        return RT_OK;
    } catch (...) {
        return RT_ERR_OOM;
    }
}

/* test hook (not part of radiantium.h): the wide tree of the fast traversal
 * built from the host builder's tree of `boxes` (rtb::build_wide), one record
 * per wide node: p (3 floats), e (3 bytes), nchild, qlo / qhi (3 x 8 bytes
 * each, [axis][child]), child (8 binary node indices), wchild (8 wide indices
 * or -1).  Call with NULL arrays to query the node count. */
int rt_debug_wide(const float* boxes, int n, int max_prims, int64_t* node_count, float* p, uint8_t* e, uint8_t* nchild,
                  uint8_t* qlo, uint8_t* qhi, int32_t* child, int32_t* wchild, int32_t* max_push) {
    if (!boxes || n <= 0 || !node_count) return RT_ERR_INVALID_ARG;
    try {
        std::vector<rtb::Box> b(n);
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) { b[i].mn[k] = boxes[6 * i + k]; b[i].mx[k] = boxes[6 * i + 3 + k]; }
        rtb::BuildResult r = rtb::build_sah(b, max_prims, std::max(1u, std::thread::hardware_concurrency()));
        rtb::WideResult w = rtb::build_wide(r);
        *node_count = (int64_t)w.nodes.size();
        if (max_push) *max_push = w.max_push;
        if (!p) return RT_OK;
        for (size_t i = 0; i < w.nodes.size(); i++) {
            const rtb::WideNode& d = w.nodes[i];
            for (int a = 0; a < 3; a++) {
                p[3 * i + a] = d.p[a];
                e[3 * i + a] = d.e[a];
                std::memcpy(qlo + 24 * i + 8 * a, d.qlo[a], 8);
                std::memcpy(qhi + 24 * i + 8 * a, d.qhi[a], 8);
            }
            nchild[i] = d.nchild;
            std::memcpy(child + 8 * i, d.child, 32);
            std::memcpy(wchild + 8 * i, d.wchild, 32);
        }
        return RT_OK;
    } catch (...) {
        return RT_ERR_OOM;
    }
}

/* test hook (not part of radiantium.h): the GPU builder's tree in rt_debug_bvh's layout */
int rt_debug_bvh_gpu(void* ctx, const float* boxes, int n, int max_prims, int64_t* node_count, float* bounds,
                     int32_t* idx, int32_t* count, int32_t* axis, int32_t* order, int32_t* depth) {
    Ctx* c = (Ctx*)ctx;
    if (!boxes || n <= 0 || !node_count) return RT_ERR_INVALID_ARG;
    return run(c, [&]() {
        std::vector<rtb::Box> b(n);
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) { b[i].mn[k] = boxes[6 * i + k]; b[i].mx[k] = boxes[6 * i + 3 + k]; }
        rtb::BuildResult r;
        CK(rt_gpu_build_sah(b, max_prims, &r, c->stream));
        *node_count = (int64_t)r.nodes.size();
        if (depth) *depth = r.max_depth;
        if (bounds) {
            for (size_t i = 0; i < r.nodes.size(); i++) {
                for (int k = 0; k < 3; k++) { bounds[6 * i + k] = r.nodes[i].bounds.mn[k]; bounds[6 * i + 3 + k] = r.nodes[i].bounds.mx[k]; }
                idx[i] = r.nodes[i].second; count[i] = r.nodes[i].count; axis[i] = r.nodes[i].axis;
            }
            for (int i = 0; i < n; i++) order[i] = r.order[i];
        }
    });
}
/* test hook (not part of radiantium.h): how many device allocations the
 * library has made in this process, over every context */
int rt_debug_device_allocations(unsigned long long* out) {
    if (!out) return RT_ERR_INVALID_ARG;
    *out = g_device_allocs.load(std::memory_order_relaxed);
    return RT_OK;
}
/* test hook (not part of radiantium.h): the wavefront's bounce-iteration cap
 * per round (0 restores WF_ITER_CAP), so a test can make it run out */
int rt_debug_set_iter_cap(void* ctx, int cap) {
    Ctx* c = (Ctx*)ctx;
    if (!c || cap < 0) return RT_ERR_INVALID_ARG;
    c->wf_iter_cap = cap == 0 ? WF_ITER_CAP : cap;
    return RT_OK;
}
/* test hook: primitive count from which upload_scene builds trees on the GPU */
int rt_debug_set_gpu_build(void* ctx, int min_prims) {
    Ctx* c = (Ctx*)ctx;
    if (!c || min_prims < 0) return RT_ERR_INVALID_ARG;
    c->gpu_build_min = min_prims == 0 ? INT_MAX : min_prims;
    return RT_OK;
}

/* test hook (not part of radiantium.h): the alias table alias_from_cdf builds
 * for a CDF of n + 1 floats, as n {threshold, alias} pairs; no CUDA call */
int rt_debug_alias(const float* cdf, int n, int32_t* out) {
    if (!cdf || !out || n <= 0) return RT_ERR_INVALID_ARG;
    try {
        std::vector<int2> t;
        if (!alias_from_cdf(cdf, n, t)) return RT_ERR_UNSUPPORTED;
        std::memcpy(out, t.data(), t.size() * sizeof(int2));
        return RT_OK;
    } catch (...) {
        return RT_ERR_OOM;
    }
}

/* test hook (not part of radiantium.h): the texel (u, v offsets) and pdf that
 * infinite light `which` of the uploaded scene samples for each of n uniform
 * pairs (u[2i] for the column, u[2i + 1] for the row), in the context's light-
 * sampling mode, computed on the device */
int rt_debug_env_sample(void* ctx, int which, const float* u, int64_t n, int32_t* texel, float* pdf) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() {
        if (!c->has_scene) throw RtFail(RT_ERR_NO_SCENE, "no scene uploaded");
        if (which < 0 || which >= c->view.infinite_count || n < 0 || !u || !texel || !pdf)
            throw RtFail(RT_ERR_INVALID_ARG, "env_sample: bad light or arrays");
        char* d = nullptr;
        CK(rt_dev_malloc((void**)&d, (size_t)n * 20 + 16));
        float2* du = (float2*)d;
        int2* dt = (int2*)(d + (size_t)n * 8);
        float* dp = (float*)(d + (size_t)n * 16);
        cudaError_t e = cudaMemcpyAsync(du, u, (size_t)n * 8, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = rt_launch_env_sample(c->d_view, which, du, n, dt, dp, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(texel, dt, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(pdf, dp, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        cudaFree(d);
        CK(e);
    });
}

/* test hook (not part of radiantium.h): runs rt_detmath (fn 0..7) or CUDA's
 * own functions (fn 100..107) on the device over host arrays */
int rt_debug_detmath(void* ctx, int fn, const float* a, const float* b, float* out, int64_t n) {
    Ctx* c = (Ctx*)ctx;
    return run(c, [&]() {
        float* d = nullptr;
        CK(rt_dev_malloc((void**)&d, (size_t)n * 12 + 16));
        cudaError_t e = cudaSuccess;
        e = cudaMemcpyAsync(d, a, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d + n, b, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = rt_launch_detmath(fn, d, d + n, d + 2 * n, n, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out, d + 2 * n, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        cudaFree(d);
        CK(e);
    });
}

}  /* extern "C" */
