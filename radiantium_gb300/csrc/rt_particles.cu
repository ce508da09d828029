/*
 * rt_particles.cu - light tracing: the "adjoint_particle" integrator and
 * renderer (Integrators/AdjointParticleIntegrator.cs,
 * Renderers/AdjointParticleRenderer.cs) on the device.
 *
 *   k_particles       one thread per particle: a light (Scene.SampleLight), an
 *                     emitted ray (Light.SampleEmit), then a bounce loop whose
 *                     every surface vertex is connected to the pinhole
 *                     (PerspectiveCamera.SampleWi + Scene.IsOccluded) and,
 *                     when visible, splatted into the film sums with float
 *                     atomics (the reference's `lock (renderTarget)` add).
 *                     The record variant writes each particle's splats to
 *                     per-particle slots instead, for the parity tests.
 *   k_particle_finish film * ScreenX*ScreenY/N + CameraTraceLight of the
 *                     camera ray through screen position (x, y).
 *
 * Particle i draws from the Philox stream (i mod 2^32, i / 2^32,
 * RT_PARTICLE_STREAM) keyed by the seed, in the reference's draw order.
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

/* where a particle's camera connections go: film sums, or per-particle records */
struct SplatSink {
    float4* film;          /* ScreenX * ScreenY sums (ColorBuffer pixel order, one vector atomic per splat) */
    int32_t* rec_n;        /* records: splat count of each particle */
    int32_t* rec_pix;      /* x * ScreenY + y of its first rec_max splats */
    float* rec_rgb;
    int rec_max;
};

/* AdjointParticleIntegrator.EmitParticle (AdjointParticleIntegrator.cs:24-79) */
template <bool kRec>
DF void EmitParticle(Ctx& c, const RtParams& P, int64_t i, int64_t slot, const SplatSink& out) {
    const RtSceneView* S = c.S;
    const int W = S->camera.width, H = S->camera.height;
    Rng rand;
    rng_init(rand, P.seed, (uint32_t)(uint64_t)i, (uint32_t)((uint64_t)i >> 32), RT_PARTICLE_STREAM);
    int nsplat = 0;
    int light;
    const float selectPdf = SampleLight(S, rand, &light);
    if (selectPdf != 0.0f) {
        const Emit e = LightSampleEmit(S, light, rand);
        if (!IsBlack(e.le)) {
            C3 coeff = e.le * AbsDot(e.dir, e.n) / (selectPdf * e.pdf_pos * e.pdf_dir);
            Ray ray = mkray(e.pos, e.dir, 0.0001f);
            int guard = 0;
            for (int bounces = 1;; bounces++) {
                if (++guard > RT_LOOP_CAP) { atomicOr(c.status, RT_STATUS_ITER); break; }
                if (P.max_depth != -1 && bounces >= P.max_depth) break;
                if (bounces > P.min_depth) {
                    if (NextFloat(rand) > P.rr) break;
                    coeff = coeff / P.rr;
                }
                Isect it;
                if (!SceneIntersect(c, ray, &it)) break;
                if (!HasSurface(S, it)) {
                    ray = mkray(it.P, ray.D, ray.MinT);
                    bounces--;
                    continue;
                }
                const int mat = PrimOf(S, it).material;
                const V3 wo = Lo(it, it.Wr);
                CamWi cw;
                /* SampleWi's pdf is 1 wherever it returns a sample, so `/ sample.Pdf` is exact */
                if (CameraSampleWi(S->camera, it.P, &cw) && cw.we != 0.0f && !IsOccluded(c, cw.pos, it.P)) {
                    const V3 wi = Lo(it, cw.dir);
                    const C3 f = MatFr<true>(S, mat, wo, wi, it.UV);
                    const float absCos = AbsCosTheta(wi);
                    const C3 color = coeff * f * cw.we * absCos;
                    if (cw.sx == cw.sx && cw.sy == cw.sy) { /* a NaN position throws in the reference */
                        const int x = (int)floorf(cw.sx), y = (int)floorf(cw.sy);
                        if (kRec) {
                            if (nsplat < out.rec_max) {
                                const int64_t o = slot * out.rec_max + nsplat;
                                out.rec_pix[o] = x * H + y;
                                out.rec_rgb[3 * o] = color.r; out.rec_rgb[3 * o + 1] = color.g;
                                out.rec_rgb[3 * o + 2] = color.b;
                            }
                        } else if (x >= 0 && x < W && y >= 0 && y < H) {
                            atomicAdd(out.film + ((int64_t)x * H + y), make_float4(color.r, color.g, color.b, 0.0f));
                        }
                        nsplat++;
                    }
                }
                const BSample bs = MatSample<true>(S, mat, wo, it.UV, rand);
                if (bs.Pdf > 0.0f) coeff = coeff * (bs.Fr * AbsCosTheta(bs.Wi) / bs.Pdf);
                else break;
                ray = Spawn(it, Wo(it, bs.Wi));
            }
        }
    }
    if (kRec) {
        out.rec_n[slot] = nsplat;
        for (int k = nsplat; k < out.rec_max; k++) {
            const int64_t o = slot * out.rec_max + k;
            out.rec_pix[o] = -1;
            out.rec_rgb[3 * o] = 0.0f; out.rec_rgb[3 * o + 1] = 0.0f; out.rec_rgb[3 * o + 2] = 0.0f;
        }
    }
}

template <bool kRec>
__global__ void __launch_bounds__(128) k_particles(const RtSceneView* __restrict__ S, RtParams P, int64_t first,
                                                     int64_t count, int64_t slot0, SplatSink out, uint32_t* status,
                                                     unsigned long long* stats, bool counting) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    int2 stack[2 * RT_STACK_SIZE];
    TravStats st = {0, 0, 0};
    Ctx c{S, stack, status, counting ? &st : nullptr, 0, 0};
    EmitParticle<kRec>(c, P, first + k, slot0 + k, out);
    if (counting) {
        warp_add(stats + 0, 1u);
        warp_add(stats + 1, c.rays_closest);
        warp_add(stats + 2, c.rays_shadow);
        warp_add(stats + 3, st.nodes);
        warp_add(stats + 4, st.prims);
        warp_add(stats + 5, st.insts);
    }
}

/* AdjointParticleRenderer.AfterRender (AdjointParticleRenderer.cs:156-172):
 * RefRGB(x, y) *= v, then += CameraTraceLight(camera.SampleRay((x, y)))
 * (AdjointParticleIntegrator.cs:81-84) */
__global__ void __launch_bounds__(128) k_particle_finish(const RtSceneView* __restrict__ S, const float4* __restrict__ film,
                                                           float v, float* __restrict__ out, uint32_t* status,
                                                           unsigned long long* stats, bool counting) {
    const int W = S->camera.width, H = S->camera.height;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)W * H) return;
    const int x = (int)(q / H), y = (int)(q - (int64_t)x * H);
    int2 stack[2 * RT_STACK_SIZE];
    TravStats st = {0, 0, 0};
    Ctx c{S, stack, status, counting ? &st : nullptr, 0, 0};
    const Ray ray = CameraRay(S->camera, v2((float)x, (float)y));
    Isect it;
    const C3 l = SceneIntersect(c, ray, &it) ? IsectLe(S, it, -ray.D) : EvalAllInfinite(S, ray.D);
    const float4 sum = film[q];
    C3 col = c3(sum.x, sum.y, sum.z) * v;
    col = col + l;
    out[3 * q] = col.r; out[3 * q + 1] = col.g; out[3 * q + 2] = col.b;
    if (counting) {
        warp_add(stats + 1, c.rays_closest);
        warp_add(stats + 3, st.nodes);
        warp_add(stats + 4, st.prims);
        warp_add(stats + 5, st.insts);
    }
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

cudaError_t rt_launch_particles(const RtSceneView* S, const RtParams& P, int64_t first, int64_t count, float4* film,
                                uint32_t* status, unsigned long long* stats, bool counting, cudaStream_t stream) {
    if (count <= 0) return cudaSuccess;
    SplatSink out{film, nullptr, nullptr, nullptr, 0};
    k_particles<false><<<grid_for(count, 128), 128, 0, stream>>>(S, P, first, count, 0, out, status, stats, counting);
    return cudaGetLastError();
}

cudaError_t rt_launch_particle_records(const RtSceneView* S, const RtParams& P, int64_t first, int64_t count,
                                       int32_t* rec_n, int32_t* rec_pix, float* rec_rgb, int rec_max,
                                       uint32_t* status, cudaStream_t stream) {
    if (count <= 0) return cudaSuccess;
    SplatSink out{nullptr, rec_n, rec_pix, rec_rgb, rec_max};
    k_particles<true><<<grid_for(count, 128), 128, 0, stream>>>(S, P, first, count, 0, out, status, nullptr, false);
    return cudaGetLastError();
}

cudaError_t rt_launch_particle_finish(const RtSceneView* S, int64_t npix, const float4* film, float v, float* out,
                                     uint32_t* status, unsigned long long* stats, bool counting, cudaStream_t stream) {
    k_particle_finish<<<grid_for(npix, 128), 128, 0, stream>>>(S, film, v, out, status, stats, counting);
    return cudaGetLastError();
}
