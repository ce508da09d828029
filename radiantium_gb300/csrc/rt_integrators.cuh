/*
 * rt_integrators.cuh - PathTracer (Bxdf / Nee / Mis) and VolumetricPathTracer
 * Li loops on the device (Integrators/PathTracer.cs, VolumetricPathTracer.cs).
 */
#ifndef RT_INTEGRATORS_CUH
#define RT_INTEGRATORS_CUH

#include "rt_shading.cuh"

namespace rtd {

#ifndef RT_LOOP_CAP
#define RT_LOOP_CAP (1 << 16)          /* bounces of one path (the reference's loops have no cap) */
#endif

DF V3 Lo(const Isect& it, V3 v) { return ToLocal(it.F, v); }
DF V3 Wo(const Isect& it, V3 v) { return ToWorld(it.F, v); }
DF Ray Spawn(const Isect& it, V3 d) { return mkray(it.P, d, 0.0001f); }

/* PathTracer.OnlySampleBxdf (PathTracer.cs:43-93) */
DF C3 LiBxdf(Ctx& c, const RtParams& P, Ray ray, Rng& rand) {
    const RtSceneView* S = c.S;
    C3 radiance = c3s(0.0f), coeff = c3s(1.0f);
    int guard = 0;
    for (int bounces = 0;; bounces++) {
        if (++guard > RT_LOOP_CAP) { atomicOr(c.status, RT_STATUS_ITER); break; }
        Isect it;
        if (!SceneIntersect(c, ray, &it)) { radiance = radiance + coeff * EvalAllInfinite(S, ray.D); break; }
        if (P.max_depth != -1 && bounces >= P.max_depth) break;
        if (!HasSurface(S, it)) { ray = mkray(it.P, ray.D, ray.MinT); bounces--; continue; }
        V3 wo = -ray.D;
        if (LightOf(S, it) >= 0) radiance = radiance + coeff * IsectLe(S, it, wo);
        BSample s = MatSample(S, PrimOf(S, it).material, Lo(it, -ray.D), it.UV, rand);
        if (s.Pdf > 0.0f) coeff = coeff * (s.Fr * AbsCosTheta(s.Wi) / s.Pdf);
        else break;
        ray = Spawn(it, Wo(it, s.Wi));
        if (bounces > P.min_depth) {
            float q = nmin(MaxElement(coeff), P.rr);
            if (NextFloat(rand) > q) break;
            coeff = coeff / q;
        }
    }
    return radiance;
}

/* PathTracer.NextEventEstimation (PathTracer.cs:95-190) */
DF C3 NeeEstimateLight(Ctx& c, Rng& rand, int light, const Isect& it, V3 wo) {
    const RtSceneView* S = c.S;
    LSample r = LightSampleLi(S, light, it.P, rand);
    if (r.Pdf <= 0.0f) return c3s(0);
    if (IsOccluded(c, it.P, r.P)) return c3s(0.0f);
    C3 fr = MatFr(S, PrimOf(S, it).material, Lo(it, wo), Lo(it, r.Wi), it.UV);
    return fr * r.Li * AbsCosTheta(Lo(it, r.Wi)) / r.Pdf;
}
DF C3 LiNee(Ctx& c, const RtParams& P, Ray ray, Rng& rand) {
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
        if (P.strategy == RT_STRATEGY_UNIFORM) {
            int light;
            float lightPdf = SampleLight(S, rand, &light);
            if (lightPdf > 0.0f) radiance = radiance + coeff * NeeEstimateLight(c, rand, light, it, wo) / lightPdf;
        } else {
            for (int l = 0; l < S->light_count; l++) radiance = radiance + coeff * NeeEstimateLight(c, rand, l, it, wo);
        }
        BSample s = MatSample(S, PrimOf(S, it).material, Lo(it, wo), it.UV, rand);
        isSpecularPath = (s.Type & BX_SPECULAR) != 0;
        if (s.Pdf > 0.0f) coeff = coeff * (s.Fr * AbsCosTheta(s.Wi) / s.Pdf);
        else break;
        ray = Spawn(it, Wo(it, s.Wi));
        if (bounces > P.min_depth) {
            float q = nmin(MaxElement(coeff), P.rr);
            if (NextFloat(rand) > q) break;
            coeff = coeff / q;
        }
    }
    return radiance;
}

/* PathTracer.Mis EstimateDirect (PathTracer.cs:309-399) */
DF C3 MisEstimateDirect(Ctx& c, Rng& rand, int light, const Isect& it) {
    const RtSceneView* S = c.S;
    const int mat = PrimOf(S, it).material;
    V3 wo = it.Wr;
    C3 le = c3s(0.0f);
    LSample ls = LightSampleLi(S, light, it.P, rand);
    if (ls.Pdf > 0.0f && !IsBlack(ls.Li)) {
        C3 fr = MatFr(S, mat, Lo(it, wo), Lo(it, ls.Wi), it.UV);
        float scatteringPdf = MatPdf(S, mat, Lo(it, wo), Lo(it, ls.Wi), it.UV);
        if (!IsBlack(fr)) {
            if (!IsOccluded(c, it.P, ls.P)) {
                fr = fr * AbsCosTheta(Lo(it, ls.Wi));
                float weight = PowerHeuristic(ls.Pdf, scatteringPdf);
                le = le + fr * ls.Li * weight / ls.Pdf;
            }
        }
    }
    BSample sample = MatSample(S, mat, Lo(it, wo), it.UV, rand);
    C3 fr = sample.Fr * AbsCosTheta(sample.Wi);
    float scatteringPdf = sample.Pdf;
    bool sampledSpecular = (sample.Type & BX_SPECULAR) != 0;
    if (!IsBlack(fr) && scatteringPdf > 0) {
        float weight = 1;
        if (!sampledSpecular) {
            float bxdfToLightPdf = LightPdfLi(S, light, it.P, Wo(it, sample.Wi));
            if (bxdfToLightPdf == 0.0f) return le;
            weight = PowerHeuristic(scatteringPdf, bxdfToLightPdf);
        }
        Ray toLight = Spawn(it, Wo(it, sample.Wi));
        Isect li_it;
        bool isHit = SceneIntersect(c, toLight, &li_it);
        C3 li = c3s(0);
        if (isHit) {
            if (LightOf(S, li_it) >= 0 && LightOf(S, li_it) == light) li = IsectLe(S, li_it, Wo(it, -sample.Wi));
        } else {
            li = EvalAllInfinite(S, toLight.D);
        }
        if (!IsBlack(li)) le = le + fr * li * weight / scatteringPdf;
    }
    return le;
}
DF C3 LiMis(Ctx& c, const RtParams& P, Ray ray, Rng& rand) {
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
        C3 direct = c3s(0);
        if (P.strategy == RT_STRATEGY_UNIFORM) {
            int light;
            float lightPdf = SampleLight(S, rand, &light);
            if (lightPdf > 0.0f) direct = direct + MisEstimateDirect(c, rand, light, it) / lightPdf;
        } else {
            for (int l = 0; l < S->light_count; l++) direct = direct + MisEstimateDirect(c, rand, l, it);
        }
        radiance = radiance + coeff * direct;
        BSample sample = MatSample(S, PrimOf(S, it).material, Lo(it, wo), it.UV, rand);
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
    return radiance;
}

/* VolumetricPathTracer (VolumetricPathTracer.cs) */
DF C3 EstimateDirectSurface(Ctx& c, Rng& rand, int light, const Isect& it, int medium) {
    const RtSceneView* S = c.S;
    const int mat = PrimOf(S, it).material;
    C3 le = c3s(0.0f);
    V3 wo = it.Wr;
    LSample ls = LightSampleLi(S, light, it.P, rand);
    C3 lightLi = ls.Li;
    if (ls.Pdf > 0.0f && !IsBlack(lightLi)) {
        C3 fr = MatFr(S, mat, Lo(it, wo), Lo(it, ls.Wi), it.UV);
        float scatteringPdf = MatPdf(S, mat, Lo(it, wo), Lo(it, ls.Wi), it.UV);
        if (!IsBlack(fr)) {
            lightLi = lightLi * Transmittance(c, it.P, ls.P, medium);
            if (!IsBlack(lightLi)) {
                fr = fr * AbsCosTheta(Lo(it, ls.Wi));
                float weight = PowerHeuristic(ls.Pdf, scatteringPdf);
                le = le + fr * lightLi * weight / ls.Pdf;
            }
        }
    }
    BSample sample = MatSample(S, mat, Lo(it, wo), it.UV, rand);
    C3 fr = sample.Fr * AbsCosTheta(sample.Wi);
    float scatteringPdf = sample.Pdf;
    bool sampledSpecular = (sample.Type & BX_SPECULAR) != 0;
    if (!IsBlack(fr) && scatteringPdf > 0) {
        float weight = 1;
        if (!sampledSpecular) {
            float bxdfToLightPdf = LightPdfLi(S, light, it.P, Wo(it, sample.Wi));
            if (bxdfToLightPdf == 0.0f) return le;
            weight = PowerHeuristic(scatteringPdf, bxdfToLightPdf);
        }
        Ray toLight = Spawn(it, Wo(it, sample.Wi));
        Isect li_it; C3 tr;
        bool isHit = IntersectTr(c, toLight, medium, &li_it, &tr);
        C3 li = c3s(0);
        if (isHit) {
            if (LightOf(S, li_it) >= 0 && LightOf(S, li_it) == light) li = IsectLe(S, li_it, Wo(it, -sample.Wi));
        } else {
            li = EvalAllInfinite(S, toLight.D);
        }
        if (!IsBlack(li)) le = le + fr * li * tr * weight / scatteringPdf;
    }
    return le;
}
DF C3 EstimateDirectMedium(Ctx& c, Rng& rand, int light, const MedSample& msr, int medium) {
    const RtSceneView* S = c.S;
    const RtMedium& M = S->media[medium];
    C3 le = c3s(0.0f);
    LSample ls = LightSampleLi(S, light, msr.P, rand);
    C3 lightLi = ls.Li;
    if (ls.Pdf > 0.0f && !IsBlack(lightLi)) {
        float p = MedP(M, msr.Wo, ls.Wi);
        float scatteringPdf = p;
        if (p != 0.0f) {
            lightLi = lightLi * Transmittance(c, msr.P, ls.P, medium);
            C3 f = c3s(p);
            if (!IsBlack(lightLi) && !IsBlack(f)) {
                float weight = PowerHeuristic(ls.Pdf, scatteringPdf);
                le = le + f * lightLi * weight / ls.Pdf;
            }
        }
    }
    V3 swi;
    float sp = MedSampleWi(M, msr.Wo, rand, &swi);
    C3 f = c3s(sp);
    float scatteringPdf = sp;
    if (scatteringPdf > 0) {
        float bxdfToLightPdf = LightPdfLi(S, light, msr.P, swi);
        if (bxdfToLightPdf == 0.0f) return le;
        float weight = PowerHeuristic(scatteringPdf, bxdfToLightPdf);
        Ray toLight = mkray(msr.P, swi);
        Isect li_it; C3 tr;
        bool isHit = IntersectTr(c, toLight, medium, &li_it, &tr);
        C3 li = c3s(0);
        if (isHit) {
            if (LightOf(S, li_it) >= 0 && LightOf(S, li_it) == light) li = IsectLe(S, li_it, -swi);
        } else {
            li = EvalAllInfinite(S, toLight.D);
        }
        if (!IsBlack(li)) le = le + f * li * tr * weight / scatteringPdf;
    }
    return le;
}
DF C3 LiVol(Ctx& c, const RtParams& P, Ray ray, Rng& rand) {
    const RtSceneView* S = c.S;
    C3 radiance = c3s(0.0f), coeff = c3s(1.0f);
    bool isSpecularPath = true;
    int rayEnv = S->global_medium;
    int guard = 0;
    for (int bounces = 0;; bounces++) {
        if (++guard > RT_LOOP_CAP) { atomicOr(c.status, RT_STATUS_ITER); break; }
        V3 wo = -ray.D;
        if (ray.MaxT <= ray.MinT) break;
        Isect it;
        bool isHit = SceneIntersect(c, ray, &it);
        MedSample msr; msr.sampled = false;
        if (rayEnv >= 0) {
            Ray realRay = mkray(ray.O, ray.D, ray.MinT, isHit ? it.T : kFMax);
            msr = MedSampleDist(S->media[rayEnv], realRay, rand);
            coeff = coeff * msr.Tr;
        }
        if (IsBlack(coeff)) break;
        if (msr.sampled) {
            if (bounces >= P.max_depth) break; /* VolumetricPathTracer.cs:55 has no -1 guard */
            int envMedium = rayEnv;
            C3 direct = c3s(0);
            if (P.strategy == RT_STRATEGY_UNIFORM) {
                int light;
                float lightPdf = SampleLight(S, rand, &light);
                if (lightPdf > 0.0f) direct = direct + EstimateDirectMedium(c, rand, light, msr, envMedium) / lightPdf;
            } else {
                for (int l = 0; l < S->light_count; l++) direct = direct + EstimateDirectMedium(c, rand, l, msr, envMedium);
            }
            radiance = radiance + coeff * direct;
            V3 swi;
            MedSampleWi(S->media[envMedium], wo, rand, &swi);
            ray = mkray(msr.P, swi, ray.MinT);
            isSpecularPath = false;
        } else {
            if (bounces == 0 || isSpecularPath) {
                if (isHit) radiance = radiance + coeff * IsectLe(S, it, wo);
                else radiance = radiance + coeff * EvalAllInfinite(S, ray.D);
            }
            if (!isHit) break;
            if (P.max_depth != -1 && bounces >= P.max_depth) break;
            if (!HasSurface(S, it)) {
                ray = mkray(it.P, ray.D, ray.MinT);
                rayEnv = GetMedium(S, it, ray.D);
                bounces--;
                continue;
            }
            C3 direct = c3s(0);
            if (P.strategy == RT_STRATEGY_UNIFORM) {
                int light;
                float lightPdf = SampleLight(S, rand, &light);
                if (lightPdf > 0.0f) direct = direct + EstimateDirectSurface(c, rand, light, it, rayEnv) / lightPdf;
            } else {
                for (int l = 0; l < S->light_count; l++) direct = direct + EstimateDirectSurface(c, rand, l, it, rayEnv);
            }
            radiance = radiance + coeff * direct;
            BSample sample = MatSample(S, PrimOf(S, it).material, Lo(it, wo), it.UV, rand);
            isSpecularPath = (sample.Type & BX_SPECULAR) != 0;
            if (sample.Pdf > 0.0f) coeff = coeff * (sample.Fr * AbsCosTheta(sample.Wi) / sample.Pdf);
            else break;
            V3 nextDir = Wo(it, sample.Wi);
            ray = mkray(it.P, nextDir, ray.MinT);
            rayEnv = GetMedium(S, it, nextDir);
        }
        if (bounces > P.min_depth) {
            float q = nmin(MaxElement(coeff), P.rr);
            if (NextFloat(rand) > q) break;
            coeff = coeff / q;
        }
    }
    return radiance;
}

/* one camera sample of BlockBasedRenderer.RenderTask (BlockBasedRenderer.cs:134-146) */
DF C3 RenderSample(Ctx& c, const RtParams& P, int px, int py, int t, bool* invalid) {
    Rng rand;
    rng_init(rand, P.seed, (uint32_t)px, (uint32_t)py, (uint32_t)t);
    V2 jit = NextVec2(rand);
    V2 sp = v2((float)px + jit.x, (float)py + jit.y);
    Ray ray = CameraRay(c.S->camera, sp);
    C3 col;
    if (P.integrator == RT_INTEGRATOR_VOL_PATH) col = LiVol(c, P, ray, rand);
    else if (P.method == RT_METHOD_BXDF) col = LiBxdf(c, P, ray, rand);
    else if (P.method == RT_METHOD_NEE) col = LiNee(c, P, ray, rand);
    else col = LiMis(c, P, ray, rand);
    *invalid = !IsValid(col);
    if (*invalid) col = c3s(0.0f);
    return col;
}

}  /* namespace rtd */

#endif
