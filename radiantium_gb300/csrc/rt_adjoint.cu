/*
 * rt_adjoint.cu - gradients of an image loss with respect to material
 * parameters: the texels of one albedo texture (the `r` texture of diffuse /
 * rough_plastic materials) and the GGX / Beckmann alpha of chosen rough
 * materials.  The reference has no derivative code; this differentiates its
 * `path` integrator with MIS (PathTracer.Mis, Integrators/PathTracer.cs:192-270).
 *
 * Method: path replay with detached sampling.  The expected film is
 * E[I] = integral of f(x; theta) over paths, and the parameters change only
 * BSDF values, not the geometry, so dE[I]/dtheta = integral of df/dtheta:
 * every sampled path contributes its radiance times d ln f / dtheta of the
 * BSDF values it went through, with the sampling pdfs, the MIS weights (a
 * partition of unity for any theta) and the Russian-roulette probabilities
 * held fixed.  Each camera sample is traced twice with the same random
 * numbers: the first pass gives its total radiance L, the replay walks the
 * same path and, at a vertex k, credits
 *   - the albedo texel(s) under the hit with dL/dI * (L - L_before_k) / R
 *     (f is linear in R for these materials, so every term from vertex k on
 *     scales with R), spread over the bilinear footprint when the texture is
 *     filtered;
 *   - the vertex material's alpha with dL/dI * [each MIS-weighted direct
 *     light term times d ln (f w) / d alpha at its own direction (the
 *     power-heuristic weight moves with the BSDF pdf) + (L - L_after_direct_k)
 *     times d ln f / d alpha at the continuation direction].
 * The expectation of this estimator is the gradient of the expected loss
 * linearised at the film (dL/dI is the caller's), which central finite
 * differences of the renderer converge to.
 */
#include <cuda_runtime.h>
#include "rt_integrators.cuh"
#include "rt_adjoint.cuh"
#include "rt_launch.h"

using namespace rtd;

namespace {

constexpr int kMaxAlpha = RT_ADJ_MAX_ALPHA;

struct Adj {
    int albedo_tex;
    const int* alpha_slot;      /* per material: parameter index or -1 */
    float* grad_albedo;         /* the albedo texture's texels x rgb (ColorBuffer layout) */
    const float* dLdI;          /* crop film layout, already divided by spp */
};

/* MisEstimateDirect (rt_integrators.cuh) with its two terms and directions
 * returned separately; draws the same random numbers in the same order */
DF void MisDirectSplit(Ctx& c, Rng& rand, int light, const Isect& it, C3* tl, V3* wl, float* w_l, C3* tb, V3* wb,
                       float* w_b, C3* le_out) {
    const RtSceneView* S = c.S;
    const int mat = PrimOf(S, it).material;
    V3 wo = it.Wr;
    C3 le = c3s(0.0f);
    *tl = c3s(0.0f); *tb = c3s(0.0f); *w_l = 1.0f; *w_b = 1.0f;
    LSample ls = LightSampleLi(S, light, it.P, rand);
    *wl = Lo(it, ls.Wi);
    if (ls.Pdf > 0.0f && !IsBlack(ls.Li)) {
        C3 fr = MatFr(S, mat, Lo(it, wo), Lo(it, ls.Wi), it.UV);
        float scatteringPdf = MatPdf(S, mat, Lo(it, wo), Lo(it, ls.Wi), it.UV);
        if (!IsBlack(fr)) {
            if (!IsOccluded(c, it.P, ls.P)) {
                fr = fr * AbsCosTheta(Lo(it, ls.Wi));
                float weight = PowerHeuristic(ls.Pdf, scatteringPdf);
                *w_l = weight;
                *tl = fr * ls.Li * weight / ls.Pdf;
                le = le + *tl;
            }
        }
    }
    BSample sample = MatSample(S, mat, Lo(it, wo), it.UV, rand);
    *wb = sample.Wi;
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
            Ray toLight = Spawn(it, Wo(it, sample.Wi));
            Isect li_it;
            bool isHit = SceneIntersect(c, toLight, &li_it);
            C3 li = c3s(0);
            if (isHit) {
                if (LightOf(S, li_it) >= 0 && LightOf(S, li_it) == light) li = IsectLe(S, li_it, Wo(it, -sample.Wi));
            } else {
                li = EvalAllInfinite(S, toLight.D);
            }
            if (!IsBlack(li)) { *tb = fr * li * weight / scatteringPdf; le = le + *tb; }
            *w_b = sampledSpecular ? 2.0f : weight;       /* 2: no weight to differentiate */
        }
    }
    *le_out = le;
}

/* LiMis replayed with the same random numbers; Ltot is the first pass's radiance */
DF void LiMisReplay(Ctx& c, const RtParams& P, Ray ray, Rng& rand, C3 Ltot, C3 dL, const Adj& A, float* s_alpha) {
    const RtSceneView* S = c.S;
    C3 radiance = c3s(0.0f), coeff = c3s(1.0f);
    bool isSpecularPath = true;
    int guard = 0;
    for (int bounces = 0;; bounces++) {
        if (++guard > RT_LOOP_CAP) { atomicOr(c.status, RT_STATUS_ITER); break; }
        Isect it;
        bool isHit = SceneIntersect(c, ray, &it);
        V3 wo = -ray.D;
        if (bounces == 0 || isSpecularPath) {
            if (isHit) radiance = radiance + coeff * IsectLe(S, it, wo);
            else radiance = radiance + coeff * EvalAllInfinite(S, ray.D);
        }
        if (!isHit) break;
        if (P.max_depth != -1 && bounces >= P.max_depth) break;
        if (!HasSurface(S, it)) { ray = mkray(it.P, ray.D, ray.MinT); bounces--; continue; }
        const int mat = PrimOf(S, it).material;
        const int slot = A.alpha_slot ? A.alpha_slot[mat] : -1;
        const C3 before = radiance;
        float galpha = 0.0f;
        C3 direct = c3s(0);
        if (P.strategy == RT_STRATEGY_UNIFORM) {
            int light;
            float lightPdf = SampleLight(S, rand, &light);
            if (lightPdf > 0.0f) {
                C3 tl, tb, le; V3 wl, wb; float wtl, wtb;
                MisDirectSplit(c, rand, light, it, &tl, &wl, &wtl, &tb, &wb, &wtb, &le);
                direct = direct + le / lightPdf;
                if (slot >= 0) {
                    const V3 wol = Lo(it, it.Wr);
                    if (!IsBlack(tl)) galpha += DirectDln(S, mat, wol, wl, wtl, true, it.UV) * Dot3(dL, coeff * tl) / lightPdf;
                    if (!IsBlack(tb)) galpha += DirectDln(S, mat, wol, wb, wtb, false, it.UV) * Dot3(dL, coeff * tb) / lightPdf;
                }
            }
        } else {
            for (int l = 0; l < S->light_count; l++) {
                C3 tl, tb, le; V3 wl, wb; float wtl, wtb;
                MisDirectSplit(c, rand, l, it, &tl, &wl, &wtl, &tb, &wb, &wtb, &le);
                direct = direct + le;
                if (slot >= 0) {
                    const V3 wol = Lo(it, it.Wr);
                    if (!IsBlack(tl)) galpha += DirectDln(S, mat, wol, wl, wtl, true, it.UV) * Dot3(dL, coeff * tl);
                    if (!IsBlack(tb)) galpha += DirectDln(S, mat, wol, wb, wtb, false, it.UV) * Dot3(dL, coeff * tb);
                }
            }
        }
        radiance = radiance + coeff * direct;
        if (UsesAlbedo(S, A.albedo_tex, mat)) {
            const C3 R = TexSample(S, A.albedo_tex, it.UV);
            const C3 rest = Ltot - before;
            ScatterAlbedo(S, A.albedo_tex, A.grad_albedo, it.UV, c3(R.r > 0 ? dL.r * rest.r / R.r : 0.0f, R.g > 0 ? dL.g * rest.g / R.g : 0.0f,
                                         R.b > 0 ? dL.b * rest.b / R.b : 0.0f));
        }
        BSample sample = MatSample(S, mat, Lo(it, wo), it.UV, rand);
        if (slot >= 0) {
            float rc, rcp;
            if (sample.Pdf > 0.0f && DlnAlpha(S, mat, Lo(it, wo), sample.Wi, it.UV, &rc, &rcp))
                galpha += rc * Dot3(dL, Ltot - radiance);
            if (galpha != 0.0f) atomicAdd(s_alpha + slot, galpha);
        }
        isSpecularPath = (sample.Type & BX_SPECULAR) != 0;
        if (sample.Pdf > 0.0f) coeff = coeff * (sample.Fr * AbsCosTheta(sample.Wi) / sample.Pdf);
        else break;
        ray = Spawn(it, Wo(it, sample.Wi));
        if (bounces > P.min_depth) {
            float q = nmin(MaxElement(coeff), P.rr);
            if (NextFloat(rand) > q) break;
            coeff = coeff / q;
        }
    }
}

/* one thread per camera sample, warps on 8x4 pixel tiles (as k_render) */
__global__ void __launch_bounds__(128) k_adjoint(const RtSceneView* __restrict__ S, RtParams P, Adj A,
                                                   float* grad_alpha, int n_alpha, uint32_t* status) {
    __shared__ float s_alpha[kMaxAlpha];
    for (int i = threadIdx.x; i < n_alpha; i += blockDim.x) s_alpha[i] = 0.0f;
    __syncthreads();
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = (int)(gid & 31);
    const int64_t warp = gid >> 5;
    const int tw = (P.w + 7) >> 3, th = (P.h + 3) >> 2;
    const int64_t ntile = (int64_t)tw * th;
    const int64_t k = warp / ntile;
    const int tile = (int)(warp - k * ntile);
    const int lx = (tile % tw) * 8 + (lane & 7);
    const int ly = (tile / tw) * 4 + (lane >> 3);
    if (k < P.chunk_len && lx < P.w && ly < P.h) {
        int2 stack[2 * RT_STACK_SIZE];
        Ctx c{S, stack, status, nullptr, 0, 0};
        const int px = P.x0 + lx, py = P.y0 + ly, t = P.sample_begin + P.chunk_begin + (int)k;
        bool invalid;
        const C3 L = RenderSample(c, P, px, py, t, &invalid);
        if (!invalid) {
            const float* g = A.dLdI + ((int64_t)lx * P.h + ly) * 3;
            const C3 dL = c3(g[0], g[1], g[2]);
            if (dL.r != 0.0f || dL.g != 0.0f || dL.b != 0.0f) {
                Rng rand;
                rng_init(rand, P.seed, (uint32_t)px, (uint32_t)py, (uint32_t)t);
                V2 jit = NextVec2(rand);
                Ray ray = CameraRay(S->camera, v2((float)px + jit.x, (float)py + jit.y));
                LiMisReplay(c, P, ray, rand, L, dL, A, s_alpha);
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n_alpha; i += blockDim.x)
        if (s_alpha[i] != 0.0f) atomicAdd(grad_alpha + i, s_alpha[i]);
}

__global__ void k_scale(float* v, int64_t n, float s) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] *= s;
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

cudaError_t rt_launch_adjoint(const RtSceneView* S, const RtParams& P, int albedo_tex, const int* alpha_slot,
                              float* grad_albedo, float* grad_alpha, int n_alpha, const float* dLdI, uint32_t* status,
                              cudaStream_t stream) {
    if (n_alpha > kMaxAlpha) return cudaErrorInvalidValue;
    Adj A{albedo_tex, alpha_slot, grad_albedo, dLdI};
    const int tw = (P.w + 7) / 8, th = (P.h + 3) / 4;
    const int64_t threads = (int64_t)tw * th * 32 * P.chunk_len;
    k_adjoint<<<grid_for(threads, 128), 128, 0, stream>>>(S, P, A, grad_alpha, n_alpha, status);
    return cudaGetLastError();
}

cudaError_t rt_launch_scale(float* v, int64_t n, float s, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    k_scale<<<grid_for(n, 256), 256, 0, stream>>>(v, n, s);
    return cudaGetLastError();
}
