/*
 * or_integrators.cpp - CPU oracle, part 4: PathTracer (Bxdf / Nee / Mis),
 * VolumetricPathTracer, BlockBasedRenderer and the C entry points.
 *
 * TEST INFRASTRUCTURE ONLY (see or_core.h).
 */
#include <atomic>
#include <thread>
#include <unordered_map>
#include <vector>
#include <string>
#include "or_scene.h"
#include "oracle.h"

namespace orc {

extern thread_local bool tl_stack_overflow;
static const int kLoopCap = 1 << 16; /* cap on pass-through iterations (null-material boundaries) */

static inline LightEvalParam LEP(const Intersection& i) { LightEvalParam p; p.P = i.P; p.T = i.T; return p; }
static inline LightEvalParam LEP(const SampleMediumResult& m) { LightEvalParam p; p.P = m.P; p.T = m.T; return p; }
static inline C3 RR_Div(C3 c, float q) { return c / q; }

/* ---- PathTracer.OnlySampleBxdf (PathTracer.cs:43-93) ---------------------------------- */
static C3 OnlySampleBxdf(const Scene& scene, const rt_render_params& P, Ray ray, Rng& rand) {
    C3 radiance = c3s(0.0f), coeff = c3s(1.0f);
    int guard = 0;
    for (int bounces = 0;; bounces++) {
        if (++guard > kLoopCap) break;
        Intersection inct;
        if (!scene.Intersect(ray, &inct)) { radiance = radiance + coeff * scene.EvalAllInfiniteLights(ray); break; }
        if (P.max_depth != -1 && bounces >= P.max_depth) break;
        if (!inct.HasSurface()) { ray = Ray(inct.P, ray.D, ray.MinT); bounces--; continue; }
        V3 wo = -ray.D;
        if (inct.IsLight()) radiance = radiance + coeff * inct.Le(wo);
        SampleBxdfResult s = inct.Surface()->Sample(inct.ToLocal(-ray.D), inct, rand);
        if (s.Pdf > 0.0f) coeff = coeff * (s.Fr * AbsCosTheta(s.Wi) / s.Pdf);
        else break;
        ray = inct.SpawnRay(inct.ToWorld(s.Wi));
        if (bounces > P.min_depth) {
            float q = netMin(MaxElement(coeff), P.rr_threshold);
            if (rand.NextFloat() > q) break;
            coeff = RR_Div(coeff, q);
        }
    }
    return radiance;
}

/* ---- PathTracer.NextEventEstimation (PathTracer.cs:95-190) ------------------------------ */
static C3 NeeEstimateLight(const Scene& scene, Rng& rand, const Light* light, const Intersection& inct, V3 wo) {
    SampleLightResult r = light->SampleLi(LEP(inct), rand);
    if (r.Pdf <= 0.0f) return c3s(0);
    if (scene.IsOccluded(inct.P, r.P)) return c3s(0.0f);
    C3 fr = inct.Surface()->Fr(inct.ToLocal(wo), inct.ToLocal(r.Wi), inct);
    return fr * r.Li * AbsCosTheta(inct.ToLocal(r.Wi)) / r.Pdf;
}
static C3 NextEventEstimation(const Scene& scene, const rt_render_params& P, Ray ray, Rng& rand) {
    C3 radiance = c3s(0.0f), coeff = c3s(1.0f);
    bool isSpecularPath = true;
    int guard = 0;
    for (int bounces = 0;; bounces++) {
        if (++guard > kLoopCap) break;
        Intersection inct;
        bool isHit = scene.Intersect(ray, &inct);
        V3 wo = -ray.D;
        if (bounces == 0 || isSpecularPath) {
            if (isHit) radiance = radiance + coeff * inct.Le(wo);
            else radiance = radiance + coeff * scene.EvalAllInfiniteLights(ray);
        }
        if (!isHit) break;
        if (P.max_depth != -1 && bounces >= P.max_depth) break;
        if (!inct.HasSurface()) { ray = Ray(inct.P, ray.D, ray.MinT); bounces--; continue; }
        if (P.strategy == RT_STRATEGY_UNIFORM) {
            const Light* light;
            float lightPdf = scene.SampleLight(rand, &light);
            if (lightPdf > 0.0f) radiance = radiance + coeff * NeeEstimateLight(scene, rand, light, inct, wo) / lightPdf;
        } else {
            for (const Light* light : scene.Lights) radiance = radiance + coeff * NeeEstimateLight(scene, rand, light, inct, wo);
        }
        SampleBxdfResult s = inct.Surface()->Sample(inct.ToLocal(wo), inct, rand);
        isSpecularPath = (s.Type & Specular) != 0;
        if (s.Pdf > 0.0f) coeff = coeff * (s.Fr * AbsCosTheta(s.Wi) / s.Pdf);
        else break;
        ray = inct.SpawnRay(inct.ToWorld(s.Wi));
        if (bounces > P.min_depth) {
            float q = netMin(MaxElement(coeff), P.rr_threshold);
            if (rand.NextFloat() > q) break;
            coeff = RR_Div(coeff, q);
        }
    }
    return radiance;
}

/* ---- PathTracer.Mis (PathTracer.cs:192-399) ---------------------------------------------- */
static C3 MisEstimateDirect(const Scene& scene, Rng& rand, const Light* light, const Intersection& inct) {
    V3 wo = inct.Wr;
    C3 le = c3s(0.0f);
    SampleLightResult ls = light->SampleLi(LEP(inct), rand);
    if (ls.Pdf > 0.0f && ls.Li != c3s(0)) {
        C3 fr = inct.Surface()->Fr(inct.ToLocal(wo), inct.ToLocal(ls.Wi), inct);
        float scatteringPdf = inct.Surface()->Pdf(inct.ToLocal(wo), inct.ToLocal(ls.Wi), inct);
        if (fr != c3s(0)) {
            if (!scene.IsOccluded(inct.P, ls.P)) {
                fr = fr * AbsCosTheta(inct.ToLocal(ls.Wi));
                float weight = PowerHeuristic(1, ls.Pdf, 1, scatteringPdf);
                le = le + fr * ls.Li * weight / ls.Pdf;
            }
        }
    }
    /* light.IsDelta is false for area and infinite lights */
    SampleBxdfResult sample = inct.Surface()->Sample(inct.ToLocal(wo), inct, rand);
    C3 fr = sample.Fr * AbsCosTheta(sample.Wi);
    float scatteringPdf = sample.Pdf;
    bool sampledSpecular = (sample.Type & Specular) != 0;
    if (fr != c3s(0) && scatteringPdf > 0) {
        float weight = 1;
        if (!sampledSpecular) {
            float bxdfToLightPdf = light->PdfLi(LEP(inct), inct.ToWorld(sample.Wi));
            if (bxdfToLightPdf == 0.0f) return le;
            weight = PowerHeuristic(1, scatteringPdf, 1, bxdfToLightPdf);
        }
        Ray toLight = inct.SpawnRay(inct.ToWorld(sample.Wi));
        Intersection lightInct;
        bool isHit = scene.Intersect(toLight, &lightInct);
        C3 li = c3s(0);
        if (isHit) {
            if (lightInct.IsLight() && lightInct.Light() == light) li = lightInct.Le(inct.ToWorld(-sample.Wi));
        } else {
            li = scene.EvalAllInfiniteLights(toLight);
        }
        if (li != c3s(0)) le = le + fr * li * weight / scatteringPdf;
    }
    return le;
}
static C3 MisSampleLightToEstimateDirect(const Scene& scene, Rng& rand, const Intersection& inct, int strategy) {
    C3 result = c3s(0);
    if (strategy == RT_STRATEGY_UNIFORM) {
        const Light* light;
        float lightPdf = scene.SampleLight(rand, &light);
        if (lightPdf > 0.0f) result = result + MisEstimateDirect(scene, rand, light, inct) / lightPdf;
    } else {
        for (const Light* light : scene.Lights) result = result + MisEstimateDirect(scene, rand, light, inct);
    }
    return result;
}
static C3 Mis(const Scene& scene, const rt_render_params& P, Ray ray, Rng& rand) {
    C3 radiance = c3s(0.0f), coeff = c3s(1.0f);
    bool isSpecularPath = true;
    int guard = 0;
    for (int bounces = 0;; bounces++) {
        if (++guard > kLoopCap) break;
        Intersection inct;
        bool isHit = scene.Intersect(ray, &inct);
        V3 wo = -ray.D;
        if (bounces == 0 || isSpecularPath) {
            if (isHit) radiance = radiance + coeff * inct.Le(wo);
            else radiance = radiance + coeff * scene.EvalAllInfiniteLights(ray);
        }
        if (!isHit) break;
        if (P.max_depth != -1 && bounces >= P.max_depth) break;
        if (!inct.HasSurface()) { ray = Ray(inct.P, ray.D, ray.MinT); bounces--; continue; }
        radiance = radiance + coeff * MisSampleLightToEstimateDirect(scene, rand, inct, P.strategy);
        SampleBxdfResult sample = inct.Surface()->Sample(inct.ToLocal(wo), inct, rand);
        isSpecularPath = (sample.Type & Specular) != 0;
        if (sample.Pdf > 0.0f) coeff = coeff * (sample.Fr * AbsCosTheta(sample.Wi) / sample.Pdf);
        else break;
        ray = inct.SpawnRay(inct.ToWorld(sample.Wi));
        if (bounces > P.min_depth) {
            float q = netMin(MaxElement(coeff), P.rr_threshold);
            if (rand.NextFloat() > q) break;
            coeff = RR_Div(coeff, q);
        }
    }
    return radiance;
}

C3 PathLi(const Scene& s, const rt_render_params& p, Ray ray, Rng& rand) {
    switch (p.method) {
    case RT_METHOD_BXDF: return OnlySampleBxdf(s, p, ray, rand);
    case RT_METHOD_NEE: return NextEventEstimation(s, p, ray, rand);
    default: return Mis(s, p, ray, rand);
    }
}

/* ---- VolumetricPathTracer (VolumetricPathTracer.cs) ---------------------------------------- */
static C3 EstimateDirectSurface(const Scene& scene, Rng& rand, const Light* light, const Intersection& inct, const Medium* medium) {
    C3 le = c3s(0.0f);
    V3 wo = inct.Wr;
    SampleLightResult ls = light->SampleLi(LEP(inct), rand);
    C3 lightLi = ls.Li;
    if (ls.Pdf > 0.0f && lightLi != c3s(0)) {
        C3 fr = inct.Surface()->Fr(inct.ToLocal(wo), inct.ToLocal(ls.Wi), inct);
        float scatteringPdf = inct.Surface()->Pdf(inct.ToLocal(wo), inct.ToLocal(ls.Wi), inct);
        if (fr != c3s(0)) {
            lightLi = lightLi * scene.Transmittance(inct.P, ls.P, medium, rand);
            if (lightLi != c3s(0)) {
                fr = fr * AbsCosTheta(inct.ToLocal(ls.Wi));
                float weight = PowerHeuristic(1, ls.Pdf, 1, scatteringPdf);
                le = le + fr * lightLi * weight / ls.Pdf;
            }
        }
    }
    SampleBxdfResult sample = inct.Surface()->Sample(inct.ToLocal(wo), inct, rand);
    C3 fr = sample.Fr * AbsCosTheta(sample.Wi);
    float scatteringPdf = sample.Pdf;
    bool sampledSpecular = (sample.Type & Specular) != 0;
    if (fr != c3s(0) && scatteringPdf > 0) {
        float weight = 1;
        if (!sampledSpecular) {
            float bxdfToLightPdf = light->PdfLi(LEP(inct), inct.ToWorld(sample.Wi));
            if (bxdfToLightPdf == 0.0f) return le;
            weight = PowerHeuristic(1, scatteringPdf, 1, bxdfToLightPdf);
        }
        Ray toLight = inct.SpawnRay(inct.ToWorld(sample.Wi));
        Intersection lightInct; C3 tr;
        bool isHit = scene.IntersectTr(toLight, medium, rand, &lightInct, &tr);
        C3 li = c3s(0);
        if (isHit) {
            if (lightInct.IsLight() && lightInct.Light() == light) li = lightInct.Le(inct.ToWorld(-sample.Wi));
        } else {
            li = scene.EvalAllInfiniteLights(toLight);
        }
        if (li != c3s(0)) le = le + fr * li * tr * weight / scatteringPdf;
    }
    return le;
}
static C3 EstimateDirectMedium(const Scene& scene, Rng& rand, const Light* light, const SampleMediumResult& msr, const Medium* medium) {
    C3 le = c3s(0.0f);
    SampleLightResult ls = light->SampleLi(LEP(msr), rand);
    C3 lightLi = ls.Li;
    if (ls.Pdf > 0.0f && lightLi != c3s(0)) {
        float p = medium->P(msr.Wo, ls.Wi);
        float scatteringPdf = p;
        if (p != 0.0f) {
            lightLi = lightLi * scene.Transmittance(msr.P, ls.P, medium, rand);
            C3 f = c3s(p);
            if (lightLi != c3s(0) && f != c3s(0)) {
                float weight = PowerHeuristic(1, ls.Pdf, 1, scatteringPdf);
                le = le + f * lightLi * weight / ls.Pdf;
            }
        }
    }
    SamplePhaseFunctionResult sample = medium->SampleWi(msr.Wo, rand);
    C3 f = c3s(sample.P);
    float scatteringPdf = sample.P;
    if (scatteringPdf > 0) {
        float bxdfToLightPdf = light->PdfLi(LEP(msr), sample.Wi);
        if (bxdfToLightPdf == 0.0f) return le;
        float weight = PowerHeuristic(1, scatteringPdf, 1, bxdfToLightPdf);
        Ray toLight(msr.P, sample.Wi);
        Intersection lightInct; C3 tr;
        bool isHit = scene.IntersectTr(toLight, medium, rand, &lightInct, &tr);
        C3 li = c3s(0);
        if (isHit) {
            if (lightInct.IsLight() && lightInct.Light() == light) li = lightInct.Le(-sample.Wi);
        } else {
            li = scene.EvalAllInfiniteLights(toLight);
        }
        if (li != c3s(0)) le = le + f * li * tr * weight / scatteringPdf;
    }
    return le;
}
C3 VolPathLi(const Scene& scene, const rt_render_params& P, Ray ray, Rng& rand) {
    C3 radiance = c3s(0.0f), coeff = c3s(1.0f);
    bool isSpecularPath = true;
    const Medium* rayEnv = scene.GlobalMedium;
    int guard = 0;
    for (int bounces = 0;; bounces++) {
        if (++guard > kLoopCap) break;
        V3 wo = -ray.D;
        if (ray.MaxT <= ray.MinT) break;
        Intersection inct;
        bool isHit = scene.Intersect(ray, &inct);
        SampleMediumResult msr; msr.IsSampleMedium = false;
        if (rayEnv != nullptr) {
            Ray realRay(ray.O, ray.D, ray.MinT, isHit ? inct.T : kFloatMax);
            msr = rayEnv->Sample(realRay, rand);
            coeff = coeff * msr.Tr;
        }
        if (coeff == c3s(0)) break;
        if (msr.IsSampleMedium) {
            if (bounces >= P.max_depth) break; /* no -1 guard in the reference (VolumetricPathTracer.cs:55) */
            const Medium* envMedium = rayEnv;
            C3 direct = c3s(0);
            if (P.strategy == RT_STRATEGY_UNIFORM) {
                const Light* light;
                float lightPdf = scene.SampleLight(rand, &light);
                if (lightPdf > 0.0f) direct = direct + EstimateDirectMedium(scene, rand, light, msr, envMedium) / lightPdf;
            } else {
                for (const Light* light : scene.Lights) direct = direct + EstimateDirectMedium(scene, rand, light, msr, envMedium);
            }
            radiance = radiance + coeff * direct;
            SamplePhaseFunctionResult sample = envMedium->SampleWi(wo, rand);
            ray = Ray(msr.P, sample.Wi, ray.MinT);
            isSpecularPath = false;
        } else {
            if (bounces == 0 || isSpecularPath) {
                if (isHit) radiance = radiance + coeff * inct.Le(wo);
                else radiance = radiance + coeff * scene.EvalAllInfiniteLights(ray);
            }
            if (!isHit) break;
            if (P.max_depth != -1 && bounces >= P.max_depth) break;
            if (!inct.HasSurface()) {
                ray = Ray(inct.P, ray.D, ray.MinT);
                rayEnv = inct.GetMedium(ray.D);
                bounces--;
                continue;
            }
            C3 direct = c3s(0);
            if (P.strategy == RT_STRATEGY_UNIFORM) {
                const Light* light;
                float lightPdf = scene.SampleLight(rand, &light);
                if (lightPdf > 0.0f) direct = direct + EstimateDirectSurface(scene, rand, light, inct, rayEnv) / lightPdf;
            } else {
                for (const Light* light : scene.Lights) direct = direct + EstimateDirectSurface(scene, rand, light, inct, rayEnv);
            }
            radiance = radiance + coeff * direct;
            SampleBxdfResult sample = inct.Surface()->Sample(inct.ToLocal(wo), inct, rand);
            isSpecularPath = (sample.Type & Specular) != 0;
            if (sample.Pdf > 0.0f) coeff = coeff * (sample.Fr * AbsCosTheta(sample.Wi) / sample.Pdf);
            else break;
            V3 nextDir = inct.ToWorld(sample.Wi);
            ray = Ray(inct.P, nextDir, ray.MinT);
            rayEnv = inct.GetMedium(nextDir);
        }
        if (bounces > P.min_depth) {
            float q = netMin(MaxElement(coeff), P.rr_threshold);
            if (rand.NextFloat() > q) break;
            coeff = RR_Div(coeff, q);
        }
    }
    return radiance;
}

/* ---- AdjointParticleIntegrator (Integrators/AdjointParticleIntegrator.cs) ---------------- */
/* EmitParticle (:24-79): one particle from a light, every surface vertex connected to the camera */
void EmitParticle(const Scene& scene, const rt_render_params& P, Rng& rand, std::vector<Splat>* splats) {
    const Light* light = nullptr;
    float selectPdf = scene.SampleLight(rand, &light);
    if (selectPdf == 0.0f) return;
    LightEmitResult emit = light->SampleEmit(rand);
    if (IsBlack(emit.Radiance)) return;
    const PerspectiveCamera& camera = scene.Camera;
    C3 coeff = emit.Radiance * AbsDot(emit.Dir, emit.Normal) / (selectPdf * emit.PdfPos * emit.PdfDir);
    Ray lightRay(emit.Pos, emit.Dir, 0.0001f);
    int guard = 0;
    for (int bounces = 1;; bounces++) {
        if (++guard > kLoopCap) break;
        if (P.max_depth != -1 && bounces >= P.max_depth) break;
        if (bounces > P.min_depth) {
            if (rand.NextFloat() > P.rr_threshold) break;
            coeff = coeff / P.rr_threshold;
        }
        Intersection inct;
        if (!scene.Intersect(lightRay, &inct)) break;
        if (!inct.HasSurface()) {
            lightRay = Ray(inct.P, lightRay.D, lightRay.MinT);
            bounces--;
            continue;
        }
        SampleCameraWiResult sample = camera.SampleWi(inct.P);
        if (sample.Pdf > 0 && !IsBlack(sample.We)) {
            if (!scene.IsOccluded(sample.Pos, inct.P)) {
                C3 f = inct.Surface()->Fr(inct.ToLocal(inct.Wr), inct.ToLocal(sample.Dir), inct, true);
                float absCos = AbsCosTheta(inct.ToLocal(sample.Dir));
                C3 color = coeff * f * sample.We * absCos / sample.Pdf;
                V2 ss = sample.ScreenPos;
                /* the reference's ColorBuffer throws on a NaN position; it is dropped here */
                if (ss.x == ss.x && ss.y == ss.y) splats->push_back(Splat{(int)Floor(ss.x), (int)Floor(ss.y), color});
            }
        }
        SampleBxdfResult bs = inct.Surface()->Sample(inct.ToLocal(inct.Wr), inct, rand, true);
        if (bs.Pdf > 0.0f) coeff = coeff * (bs.Fr * AbsCosTheta(bs.Wi) / bs.Pdf);
        else break;
        lightRay = inct.SpawnRay(inct.ToWorld(bs.Wi));
    }
}
/* CameraTraceLight (:81-84) */
C3 CameraTraceLight(const Scene& scene, const Ray& ray) {
    Intersection inct;
    return scene.Intersect(ray, &inct) ? inct.Le(-ray.D) : scene.EvalAllInfiniteLights(ray);
}

/* one camera sample of BlockBasedRenderer.RenderTask (BlockBasedRenderer.cs:134-146) */
static inline C3 RenderSample(const Scene& scene, const rt_render_params& P, int px, int py, int t, bool* invalid) {
    Rng rand(P.seed, (uint32_t)px, (uint32_t)py, (uint32_t)t);
    V2 jitter = rand.NextVec2();
    V2 sp = v2((float)px + jitter.x, (float)py + jitter.y);
    Ray ray = scene.Camera.SampleRay(sp);
    C3 color = (P.integrator == RT_INTEGRATOR_VOL_PATH) ? VolPathLi(scene, P, ray, rand) : PathLi(scene, P, ray, rand);
    /* RT_INTEGRATOR_PARTICLE never gets here: the block renderer rejects it */
    *invalid = !IsValid(color);
    if (*invalid) color = c3s(0.0f);
    return color;
}

static int MaxThreads(int threads) {
    if (threads <= 0) threads = (int)std::thread::hardware_concurrency();
    return threads > 0 ? threads : 1;
}

template <class F>
static void ParallelFor(int64_t n, int threads, F fn) {
    if (threads <= 0) threads = (int)std::thread::hardware_concurrency();
    if (threads <= 0) threads = 1;
    if (n < threads) threads = (int)(n > 0 ? n : 1);
    std::atomic<int64_t> next(0);
    const int64_t chunk = 64;
    auto worker = [&](int tid) {
        while (true) {
            int64_t b = next.fetch_add(chunk);
            if (b >= n) break;
            int64_t e = b + chunk < n ? b + chunk : n;
            for (int64_t i = b; i < e; i++) fn(i, tid);
        }
    };
    std::vector<std::thread> ts;
    for (int i = 1; i < threads; i++) ts.emplace_back(worker, i);
    worker(0);
    for (auto& t : ts) t.join();
}

} /* namespace orc */

using namespace orc;

extern "C" {

void* or_scene_create(const rt_scene_desc* scene, char* err, int errlen) {
    std::string e;
    std::unique_ptr<Scene> s = BuildScene(scene, &e);
    if (!s) { if (err && errlen > 0) { snprintf(err, errlen, "%s", e.c_str()); } return nullptr; }
    return s.release();
}
void or_scene_destroy(void* s) { delete (Scene*)s; }

static inline Ray RayFrom(const rt_ray& r) { return Ray(v3(r.o[0], r.o[1], r.o[2]), v3(r.d[0], r.d[1], r.d[2]), r.min_t, r.max_t); }

/* traversal counters of a ray batch, summed over the worker threads */
static void SumTraceCounters(const std::vector<Counters>& counters, rt_stats* stats) {
    if (!stats) return;
    memset(stats, 0, sizeof(*stats));
    for (const Counters& c : counters) {
        stats->node_visits += c.node_visits; stats->prim_tests += c.prim_tests;
        stats->instance_visits += c.instance_visits;
    }
}

int or_trace_closest(void* sp, const rt_ray* rays, int64_t n, rt_hit* hits, int threads, rt_stats* stats) {
    const Scene* s = (const Scene*)sp;
    if (!s || n < 0) return RT_ERR_INVALID_ARG;
    std::atomic<int> overflow(0);
    std::vector<Counters> counters(MaxThreads(threads));
    ParallelFor(n, threads, [&](int64_t i, int tid) {
        tl_counters = stats ? &counters[tid] : nullptr;
        Intersection inct;
        tl_stack_overflow = false;
        bool hit = s->Aggregate->Intersect(RayFrom(rays[i]), &inct);
        if (tl_stack_overflow) overflow = 1;
        rt_hit& h = hits[i];
        if (hit) {
            h.t = inct.T; h.prim = inct.prim_id; h.sub = inct.sub_id; h.flags = inct.flags;
            h.u = inct.bu; h.v = inct.bv;
        } else {
            h.t = kFloatMax; h.u = 0; h.v = 0; h.prim = -1; h.sub = -1; h.flags = 0;
        }
        tl_counters = nullptr;
    });
    SumTraceCounters(counters, stats);
    return overflow ? RT_ERR_STACK : RT_OK;
}
int or_trace_any(void* sp, const rt_ray* rays, int64_t n, uint8_t* occ, int threads, rt_stats* stats) {
    const Scene* s = (const Scene*)sp;
    if (!s || n < 0) return RT_ERR_INVALID_ARG;
    std::atomic<int> overflow(0);
    std::vector<Counters> counters(MaxThreads(threads));
    ParallelFor(n, threads, [&](int64_t i, int tid) {
        tl_counters = stats ? &counters[tid] : nullptr;
        tl_stack_overflow = false;
        occ[i] = s->Aggregate->IntersectP(RayFrom(rays[i])) ? 1 : 0;
        if (tl_stack_overflow) overflow = 1;
        tl_counters = nullptr;
    });
    SumTraceCounters(counters, stats);
    return overflow ? RT_ERR_STACK : RT_OK;
}

static bool Crop(const Scene* s, const rt_render_params* p, int* x0, int* y0, int* w, int* h) {
    *x0 = p->x0; *y0 = p->y0;
    *w = p->width > 0 ? p->width : s->Camera.ScreenX - p->x0;
    *h = p->height > 0 ? p->height : s->Camera.ScreenY - p->y0;
    return *x0 >= 0 && *y0 >= 0 && *w > 0 && *h > 0 && *x0 + *w <= s->Camera.ScreenX && *y0 + *h <= s->Camera.ScreenY;
}

int or_render(void* sp, const rt_render_params* p, float* out, int threads, rt_stats* stats) {
    const Scene* s = (const Scene*)sp;
    int x0, y0, w, h;
    if (!s || !p || !out || p->spp <= 0 || !Crop(s, p, &x0, &y0, &w, &h)) return RT_ERR_INVALID_ARG;
    if (p->integrator == RT_INTEGRATOR_PARTICLE) return RT_ERR_INVALID_ARG;
    int nthreads = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    if (nthreads <= 0) nthreads = 1;
    std::vector<Counters> counters(nthreads);
    std::vector<uint64_t> invalid(nthreads, 0);
    std::atomic<int> overflow(0);
    /* 32x32 blocks like BlockBasedRenderer; each pixel sums its samples in order */
    const int B = 32;
    int nbx = (w + B - 1) / B, nby = (h + B - 1) / B;
    ParallelFor((int64_t)nbx * nby, nthreads, [&](int64_t bi, int tid) {
        tl_counters = stats ? &counters[tid] : nullptr;
        int bx = (int)(bi % nbx), by = (int)(bi / nbx);
        for (int lx = bx * B; lx < w && lx < bx * B + B; lx++) {
            for (int ly = by * B; ly < h && ly < by * B + B; ly++) {
                C3 sum = c3s(0.0f);
                for (int t = 0; t < p->spp; t++) {
                    bool inv;
                    tl_stack_overflow = false;
                    sum = sum + RenderSample(*s, *p, x0 + lx, y0 + ly, p->sample_begin + t, &inv);
                    if (tl_stack_overflow) overflow = 1;
                    if (inv) invalid[tid]++;
                }
                C3 c = sum / (float)p->spp;
                float* o = out + ((size_t)lx * h + ly) * 3;
                o[0] = c.r; o[1] = c.g; o[2] = c.b;
            }
        }
        tl_counters = nullptr;
    });
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->samples = (uint64_t)w * h * p->spp;
        for (int i = 0; i < nthreads; i++) {
            stats->rays_closest += counters[i].rays_closest; stats->rays_shadow += counters[i].rays_shadow;
            stats->node_visits += counters[i].node_visits; stats->prim_tests += counters[i].prim_tests;
            stats->instance_visits += counters[i].instance_visits; stats->invalid_samples += invalid[i];
        }
    }
    return overflow ? RT_ERR_STACK : RT_OK;
}

int or_render_samples(void* sp, const rt_render_params* p, float* out, int threads) {
    const Scene* s = (const Scene*)sp;
    int x0, y0, w, h;
    if (!s || !p || !out || p->spp <= 0 || !Crop(s, p, &x0, &y0, &w, &h)) return RT_ERR_INVALID_ARG;
    ParallelFor((int64_t)w * h, threads, [&](int64_t i, int) {
        int lx = (int)(i / h), ly = (int)(i % h);
        for (int t = 0; t < p->spp; t++) {
            bool inv;
            C3 c = RenderSample(*s, *p, x0 + lx, y0 + ly, p->sample_begin + t, &inv);
            float* o = out + (((size_t)lx * h + ly) * p->spp + t) * 3;
            o[0] = c.r; o[1] = c.g; o[2] = c.b;
        }
    });
    return RT_OK;
}

static inline Rng ParticleRng(uint64_t seed, int64_t i) {
    return Rng(seed, (uint32_t)(uint64_t)i, (uint32_t)((uint64_t)i >> 32), RT_PARTICLE_STREAM);
}
static bool ParticleArgs(const Scene* s, const rt_render_params* p, int64_t first, int64_t count) {
    return s && p && p->integrator == RT_INTEGRATOR_PARTICLE && first >= 0 && count > 0 &&
           p->x0 == 0 && p->y0 == 0 && p->width == 0 && p->height == 0;
}

/* AdjointParticleRenderer (Renderers/AdjointParticleRenderer.cs:118-172): each thread
 * takes a fixed contiguous share of the particles and splats into its own film; the
 * films are summed in thread order, so a fixed thread count gives a fixed film. */
int or_render_particles(void* sp, const rt_render_params* p, int64_t first, int64_t count, float* out,
                        int threads, rt_stats* stats) {
    const Scene* s = (const Scene*)sp;
    if (!ParticleArgs(s, p, first, count) || !out) return RT_ERR_INVALID_ARG;
    const int W = s->Camera.ScreenX, H = s->Camera.ScreenY;
    const size_t npix = (size_t)W * H;
    int nthreads = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    if (nthreads <= 0) nthreads = 1;
    if (count < nthreads) nthreads = (int)count;
    std::vector<std::vector<float>> films(nthreads, std::vector<float>(npix * 3, 0.0f));
    std::vector<Counters> counters(nthreads);
    std::vector<int> overflow(nthreads, 0);
    auto worker = [&](int tid) {
        tl_counters = &counters[tid];
        std::vector<Splat> splats;
        float* film = films[tid].data();
        int64_t b = first + count * tid / nthreads, e = first + count * (tid + 1) / nthreads;
        for (int64_t i = b; i < e; i++) {
            Rng rand = ParticleRng(p->seed, i);
            splats.clear();
            tl_stack_overflow = false;
            EmitParticle(*s, *p, rand, &splats);
            if (tl_stack_overflow) overflow[tid] = 1;
            for (const Splat& q : splats) {
                if (q.x < 0 || q.x >= W || q.y < 0 || q.y >= H) continue;
                float* o = film + ((size_t)q.x * H + q.y) * 3;
                o[0] = o[0] + q.color.r; o[1] = o[1] + q.color.g; o[2] = o[2] + q.color.b;
            }
        }
        tl_counters = nullptr;
    };
    std::vector<std::thread> ts;
    for (int t = 1; t < nthreads; t++) ts.emplace_back(worker, t);
    worker(0);
    for (auto& t : ts) t.join();
    /* film sums, then RefRGB *= v and += CameraTraceLight(SampleRay(x, y)) */
    const float v = (float)W * (float)H / (float)count;
    int fthreads = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    std::vector<Counters> fcount(fthreads > 0 ? fthreads : 1);
    ParallelFor((int64_t)npix, threads, [&](int64_t q, int tid) {
        tl_counters = &fcount[tid];
        int x = (int)(q / H), y = (int)(q % H);
        C3 sum = c3s(0.0f);
        for (int t = 0; t < nthreads; t++) {
            const float* f = films[t].data() + (size_t)q * 3;
            sum = sum + c3(f[0], f[1], f[2]);
        }
        C3 c = sum * v;
        c = c + CameraTraceLight(*s, s->Camera.SampleRay(v2((float)x, (float)y)));
        out[q * 3] = c.r; out[q * 3 + 1] = c.g; out[q * 3 + 2] = c.b;
        tl_counters = nullptr;
    });
    for (const Counters& f : fcount) counters.push_back(f);
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->samples = (uint64_t)count;
        for (size_t i = 0; i < counters.size(); i++) {
            stats->rays_closest += counters[i].rays_closest; stats->rays_shadow += counters[i].rays_shadow;
            stats->node_visits += counters[i].node_visits; stats->prim_tests += counters[i].prim_tests;
            stats->instance_visits += counters[i].instance_visits;
        }
    }
    for (int t = 0; t < nthreads; t++) if (overflow[t]) return RT_ERR_STACK;
    return RT_OK;
}

/* the camera connections of each particle, in emission order (parity hook) */
int or_particle_splats(void* sp, const rt_render_params* p, int64_t first, int64_t count, int max_per,
                       int32_t* n, int32_t* pix, float* rgb, int threads) {
    const Scene* s = (const Scene*)sp;
    if (!ParticleArgs(s, p, first, count) || max_per < 0 || !n || (max_per > 0 && (!pix || !rgb)))
        return RT_ERR_INVALID_ARG;
    const int H = s->Camera.ScreenY;
    ParallelFor(count, threads, [&](int64_t i, int) {
        std::vector<Splat> splats;
        Rng rand = ParticleRng(p->seed, first + i);
        EmitParticle(*s, *p, rand, &splats);
        n[i] = (int32_t)splats.size();
        for (int k = 0; k < max_per; k++) {
            int64_t o = i * max_per + k;
            if (k < (int)splats.size()) {
                pix[o] = splats[k].x * H + splats[k].y;
                rgb[o * 3] = splats[k].color.r; rgb[o * 3 + 1] = splats[k].color.g; rgb[o * 3 + 2] = splats[k].color.b;
            } else {
                pix[o] = -1; rgb[o * 3] = rgb[o * 3 + 1] = rgb[o * 3 + 2] = 0.0f;
            }
        }
    });
    return RT_OK;
}

int or_camera_rays(void* sp, const float* pos, int64_t n, rt_ray* out) {
    const Scene* s = (const Scene*)sp;
    if (!s) return RT_ERR_INVALID_ARG;
    for (int64_t i = 0; i < n; i++) {
        Ray r = s->Camera.SampleRay(v2(pos[2 * i], pos[2 * i + 1]));
        out[i].o[0] = r.O.x; out[i].o[1] = r.O.y; out[i].o[2] = r.O.z;
        out[i].d[0] = r.D.x; out[i].d[1] = r.D.y; out[i].d[2] = r.D.z;
        out[i].min_t = r.MinT; out[i].max_t = r.MaxT;
    }
    return RT_OK;
}

int or_bvh(void* sp, int which, int64_t* node_count, int64_t* prim_count, float* bounds, int32_t* idx,
           int32_t* count, int32_t* axis, int32_t* prim_order) {
    const Scene* s = (const Scene*)sp;
    if (!s) return RT_ERR_INVALID_ARG;
    const Bvh* b = nullptr;
    if (which < 0) b = s->Aggregate.get();
    else if (which < (int)s->blas.size()) b = s->blas[which].get();
    if (!b) return RT_ERR_INVALID_ARG;
    if (node_count) *node_count = (int64_t)b->nodes.size();
    if (prim_count) *prim_count = (int64_t)b->prims.size();
    for (size_t i = 0; bounds && i < b->nodes.size(); i++) {
        const LinearBVHNode& nd = b->nodes[i];
        float* o = bounds + 6 * i;
        o[0] = nd.Bounds.Min.x; o[1] = nd.Bounds.Min.y; o[2] = nd.Bounds.Min.z;
        o[3] = nd.Bounds.Max.x; o[4] = nd.Bounds.Max.y; o[5] = nd.Bounds.Max.z;
        idx[i] = nd.PrimitivesIndex; count[i] = nd.PrimitiveCount; axis[i] = nd.Axis;
    }
    for (size_t i = 0; prim_order && i < b->prims.size(); i++) prim_order[i] = b->prims[i]->id;
    return RT_OK;
}

int or_scene_lights(void* sp, int64_t* count, int32_t* kind, int32_t* prim, float* le) {
    const Scene* s = (const Scene*)sp;
    if (!s || !count) return RT_ERR_INVALID_ARG;
    *count = (int64_t)s->Lights.size();
    if (!kind || !prim || !le) return RT_OK;
    std::unordered_map<const Light*, int> owner;
    for (const Primitive* p : s->Aggregate->prims)
        if (const AreaLight* a = p->GetLight()) owner[a] = p->id;
    for (size_t i = 0; i < s->Lights.size(); i++) {
        const AreaLight* a = dynamic_cast<const AreaLight*>(s->Lights[i]);
        kind[i] = a ? 0 : 1;
        auto it = a ? owner.find(a) : owner.end();
        prim[i] = it != owner.end() ? it->second : -1;
        le[3 * i + 0] = a ? a->LightEmit.r : 0.0f;
        le[3 * i + 1] = a ? a->LightEmit.g : 0.0f;
        le[3 * i + 2] = a ? a->LightEmit.b : 0.0f;
    }
    return RT_OK;
}

int or_detmath(int fn, const float* a, const float* b, float* out, int64_t n) {
    for (int64_t i = 0; i < n; i++) {
        switch (fn) {
        case 0: out[i] = rt_sinf(a[i]); break;
        case 1: out[i] = rt_cosf(a[i]); break;
        case 2: out[i] = rt_tanf(a[i]); break;
        case 3: out[i] = rt_atanf(a[i]); break;
        case 4: out[i] = rt_atan2f(a[i], b[i]); break;
        case 5: out[i] = rt_acosf(a[i]); break;
        case 6: out[i] = rt_expf(a[i]); break;
        case 7: out[i] = rt_logf(a[i]); break;
        default: return RT_ERR_INVALID_ARG;
        }
    }
    return RT_OK;
}
int or_philox_raw(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    Philox4x32(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1], out);
    return RT_OK;
}
int or_philox(uint64_t seed, uint32_t x, uint32_t y, uint32_t s, int count, uint32_t* out) {
    Rng r(seed, x, y, s);
    for (int i = 0; i < count; i++) out[i] = r.NextU32();
    return RT_OK;
}

} /* extern "C" */
