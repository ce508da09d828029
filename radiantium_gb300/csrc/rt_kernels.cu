/*
 * rt_kernels.cu - CUDA kernels of the GB300 path tracer and their launchers.
 *
 * Render pass structure (BlockBasedRenderer.RenderTask, BlockBasedRenderer.cs:107-179):
 *   k_render      one thread per camera sample of a chunk of sample indices;
 *                 a warp traces an 8x4 pixel tile at one sample index, so the
 *                 primary rays of a warp are coherent.  Each thread writes its
 *                 radiance to the chunk's sample buffer.
 *   k_accumulate  adds a chunk's samples to the film sums in sample order, so
 *                 every pixel sums exactly like the reference's
 *                 `RenderTarget += color` loop.
 *   k_finalize    divides by spp (BlockBasedRenderer.cs:169-178).
 * Ray-batch kernels k_trace_closest / k_trace_any serve the parity interface.
 */
#include <cuda_runtime.h>
#include "rt_integrators.cuh"
#include "rt_launch.h"

using namespace rtd;

namespace {

DF void warp_add(unsigned long long* dst, uint32_t v) {
    unsigned mask = __activemask();
    uint32_t s = __reduce_add_sync(mask, v);
    if ((threadIdx.x & 31) == (unsigned)(__ffs(mask) - 1) && s) atomicAdd(dst, (unsigned long long)s);
}

__global__ void __launch_bounds__(128) k_render(const RtSceneView* __restrict__ S, RtParams P, float* __restrict__ samples,
                                                  uint32_t* status, unsigned long long* stats, bool counting) {
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = (int)(gid & 31);
    const int64_t warp = gid >> 5;
    const int tw = (P.w + 7) >> 3, th = (P.h + 3) >> 2;
    const int64_t ntile = (int64_t)tw * th;
    const int64_t k = warp / ntile;
    if (k >= P.chunk_len) return;
    const int tile = (int)(warp - k * ntile);
    const int lx = (tile % tw) * 8 + (lane & 7);
    const int ly = (tile / tw) * 4 + (lane >> 3);
    if (lx >= P.w || ly >= P.h) return;
    int2 stack[2 * RT_STACK_SIZE];
    TravStats st = {0, 0, 0};
    Ctx c{S, stack, status, counting ? &st : nullptr, 0, 0};
    bool invalid;
    C3 col = RenderSample(c, P, P.x0 + lx, P.y0 + ly, P.sample_begin + P.chunk_begin + (int)k, &invalid);
    const int64_t npix = (int64_t)P.w * P.h;
    float* o = samples + (k * npix + (int64_t)lx * P.h + ly) * 3;
    o[0] = col.r; o[1] = col.g; o[2] = col.b;
    if (counting) {
        warp_add(stats + 0, 1u);
        warp_add(stats + 1, c.rays_closest);
        warp_add(stats + 2, c.rays_shadow);
        warp_add(stats + 3, st.nodes);
        warp_add(stats + 4, st.prims);
        warp_add(stats + 5, st.insts);
    }
    if (invalid) atomicAdd(stats + 6, 1ull);
}

__global__ void k_accumulate(float* __restrict__ film, const float* __restrict__ samples, int64_t npix, int chunk_len) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    float r = film[3 * p], g = film[3 * p + 1], b = film[3 * p + 2];
    for (int k = 0; k < chunk_len; k++) {
        const float* s = samples + ((int64_t)k * npix + p) * 3;
        r = r + s[0]; g = g + s[1]; b = b + s[2];
    }
    film[3 * p] = r; film[3 * p + 1] = g; film[3 * p + 2] = b;
}

__global__ void k_finalize(float* __restrict__ out, const float* __restrict__ film, int64_t npix, float spp) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    out[3 * p] = film[3 * p] / spp;
    out[3 * p + 1] = film[3 * p + 1] / spp;
    out[3 * p + 2] = film[3 * p + 2] / spp;
}

DF Ray ray_from(const rt_ray& r) {
    return mkray(v3(r.o[0], r.o[1], r.o[2]), v3(r.d[0], r.d[1], r.d[2]), r.min_t, r.max_t);
}

template <bool kWide>
__global__ void __launch_bounds__(128) k_trace_closest(const RtSceneView* __restrict__ S, const rt_ray* __restrict__ rays, int64_t n,
                                                         rt_hit* __restrict__ hits, uint32_t* status,
                                                         unsigned long long* stats, bool counting) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int2 stack[2 * RT_STACK_SIZE];
    TravStats st = {0, 0, 0};
    Ray ray = ray_from(rays[i]);
    Ray r = ray;
    Best b;
    rt_hit h;
    if (SceneClosest<kWide>(S, r, &b, stack, status, counting ? &st : nullptr)) {
        Isect it;
        Finish(S, ray, b, &it);
        h.t = it.T; h.u = it.bu; h.v = it.bv; h.prim = it.prim; h.sub = it.sub; h.flags = it.flags;
    } else {
        h.t = kFMax; h.u = 0; h.v = 0; h.prim = -1; h.sub = -1; h.flags = 0;
    }
    hits[i] = h;
    if (counting) {
        warp_add(stats + 3, st.nodes);
        warp_add(stats + 4, st.prims);
        warp_add(stats + 5, st.insts);
    }
}

template <bool kWide>
__global__ void __launch_bounds__(128) k_trace_any(const RtSceneView* __restrict__ S, const rt_ray* __restrict__ rays, int64_t n,
                                                     uint8_t* __restrict__ occ, uint32_t* status,
                                                     unsigned long long* stats, bool counting) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int2 stack[2 * RT_STACK_SIZE];
    TravStats st = {0, 0, 0};
    Ray ray = ray_from(rays[i]);
    occ[i] = SceneAny<kWide>(S, ray, stack, status, counting ? &st : nullptr) ? 1 : 0;
    if (counting) {
        warp_add(stats + 3, st.nodes);
        warp_add(stats + 4, st.prims);
        warp_add(stats + 5, st.insts);
    }
}

/* deterministic-math hook: runs rt_detmath on the device for the accuracy tests */
__global__ void k_detmath(int fn, const float* a, const float* b, float* out, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x = a[i], y = b[i], r;
    switch (fn) {
    case 0: r = rt_sinf(x); break;
    case 1: r = rt_cosf(x); break;
    case 2: r = rt_tanf(x); break;
    case 3: r = rt_atanf(x); break;
    case 4: r = rt_atan2f(x, y); break;
    case 5: r = rt_acosf(x); break;
    case 6: r = rt_expf(x); break;
    case 7: r = rt_logf(x); break;
    case 100: r = sinf(x); break;
    case 101: r = cosf(x); break;
    case 102: r = tanf(x); break;
    case 103: r = atanf(x); break;
    case 104: r = atan2f(x, y); break;
    case 105: r = acosf(x); break;
    case 106: r = expf(x); break;
    case 107: r = logf(x); break;
    default: r = 0.0f;
    }
    out[i] = r;
}

/* environment-sampling hook: Distribution2D.SampleContinuous's texel and pdf
 * (as SampleLi uses them) of infinite light `which` for each pair of uniforms,
 * in the scene's current light-sampling mode */
__global__ void k_env_sample(const RtSceneView* __restrict__ S, int which, const float2* __restrict__ u, int64_t n,
                             int2* __restrict__ texel, float* __restrict__ pdf) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const RtDist2D d = S->dists[S->lights[S->infinite_lights[which]].dist];
    const float2 uv = u[i];
    float p; int ov, ou;
    Sample2D(S, d, v2(uv.x, uv.y), &p, &ov, &ou);
    texel[i] = make_int2(ou, ov);
    pdf[i] = p;
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

cudaError_t rt_launch_render(const RtSceneView* S, const RtParams& P, float* samples, uint32_t* status,
                             unsigned long long* stats, bool counting, cudaStream_t stream) {
    const int tw = (P.w + 7) / 8, th = (P.h + 3) / 4;
    const int64_t threads = (int64_t)tw * th * 32 * P.chunk_len;
    const int block = 128;
    k_render<<<grid_for(threads, block), block, 0, stream>>>(S, P, samples, status, stats, counting);
    return cudaGetLastError();
}

cudaError_t rt_launch_accumulate(float* film, const float* samples, int64_t npix, int chunk_len, cudaStream_t stream) {
    k_accumulate<<<grid_for(npix, 256), 256, 0, stream>>>(film, samples, npix, chunk_len);
    return cudaGetLastError();
}

cudaError_t rt_launch_finalize(float* out, const float* film, int64_t npix, float spp, cudaStream_t stream) {
    k_finalize<<<grid_for(npix, 256), 256, 0, stream>>>(out, film, npix, spp);
    return cudaGetLastError();
}

cudaError_t rt_launch_trace(const RtSceneView* S, const rt_ray* rays, int64_t n, rt_hit* hits, uint8_t* occ,
                            uint32_t* status, unsigned long long* stats, bool counting, cudaStream_t stream,
                            bool wide) {
    if (n <= 0) return cudaSuccess;
    const int block = 128;
    if (hits && wide) k_trace_closest<true><<<grid_for(n, block), block, 0, stream>>>(S, rays, n, hits, status, stats, counting);
    else if (hits) k_trace_closest<false><<<grid_for(n, block), block, 0, stream>>>(S, rays, n, hits, status, stats, counting);
    else if (wide) k_trace_any<true><<<grid_for(n, block), block, 0, stream>>>(S, rays, n, occ, status, stats, counting);
    else k_trace_any<false><<<grid_for(n, block), block, 0, stream>>>(S, rays, n, occ, status, stats, counting);
    return cudaGetLastError();
}

cudaError_t rt_launch_detmath(int fn, const float* a, const float* b, float* out, int64_t n, cudaStream_t stream) {
    k_detmath<<<grid_for(n, 256), 256, 0, stream>>>(fn, a, b, out, n);
    return cudaGetLastError();
}

cudaError_t rt_launch_env_sample(const RtSceneView* S, int which, const float2* u, int64_t n, int2* texel, float* pdf,
                                 cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    k_env_sample<<<grid_for(n, 256), 256, 0, stream>>>(S, which, u, n, texel, pdf);
    return cudaGetLastError();
}
