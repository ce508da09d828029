/*
 * rt_shading.cuh - BxDFs, materials, lights, media and scene services of the
 * GB300 path tracer (device code).
 *
 * Restates Radiantium.Offline's Bxdf/, Materials/, Lights/, Mediums/,
 * Distribution1D/2D and Scene.cs with switch dispatch over flat material and
 * light records instead of virtual calls.  Operand order follows the C#.
 */
#ifndef RT_SHADING_CUH
#define RT_SHADING_CUH

#include "rt_device.cuh"

namespace rtd {

#define NF static __device__ __noinline__

/* the scene services share one traversal context per path */
struct Ctx {
    const RtSceneView* S;
    int2* stack;
    uint32_t* status;
    TravStats* st;
    uint32_t rays_closest, rays_shadow;
};

/* Scene.Intersect (Scene.cs:32-35) */
NF bool SceneIntersect(Ctx& c, const Ray& ray, Isect* it) {
    if (c.st) c.rays_closest++;
    Ray r = ray;
    Best b;
    if (!SceneClosest(c.S, r, &b, c.stack, c.status, c.st)) return false;
    Finish(c.S, ray, b, it);
    return true;
}
NF bool SceneIntersectP(Ctx& c, const Ray& ray) {
    if (c.st) c.rays_shadow++;
    return SceneAny(c.S, ray, c.stack, c.status, c.st);
}
DF const RtPrim& PrimOf(const RtSceneView* S, const Isect& it) { return S->prims[it.prim]; }
DF bool HasSurface(const RtSceneView* S, const Isect& it) { return S->prims[it.prim].material >= 0; }
DF int LightOf(const RtSceneView* S, const Isect& it) { return S->prims[it.prim].light; }
/* Intersection.GetMedium */
DF int GetMedium(const RtSceneView* S, const Isect& it, V3 w) {
    const RtPrim& p = S->prims[it.prim];
    return Dot(w, it.F.Z) > 0 ? p.med_out : p.med_in;
}

/* ---- microfacet distributions (Bxdf/Microfacet.cs) ---------------------------- */
struct Dist {
    int type; float ax, ay;
};
DF Dist mkdist(int type, float roughness, float anis) {
    Dist d; d.type = type;
    float k = anis;
    d.ax = nmax(roughness * roughness * (1 + k), 0.001f);
    d.ay = nmax(roughness * roughness * (1 - k), 0.001f);
    return d;
}
DF float DistD(const Dist& d, V3 wh) {
    float tan2Theta = Tan2Theta(wh);
    if (isinff_(tan2Theta)) return 0.0f;
    float cos4Theta = Cos2Theta(wh) * Cos2Theta(wh);
    if (d.type == RT_DIST_BECKMANN)
        return rt_expf(-tan2Theta * (Cos2Phi(wh) / (d.ax * d.ax) + Sin2Phi(wh) / (d.ay * d.ay))) / (kPI * d.ax * d.ay * cos4Theta);
    float e = (Cos2Phi(wh) / (d.ax * d.ax) + Sin2Phi(wh) / (d.ay * d.ay)) * tan2Theta;
    return 1 / (kPI * d.ax * d.ay * cos4Theta * (1 + e) * (1 + e));
}
DF float DistLambda(const Dist& d, V3 w) {
    float absTanTheta = Abs(TanTheta(w));
    if (isinff_(absTanTheta)) return 0.0f;
    float alpha = Sqrt(Cos2Phi(w) * d.ax * d.ax + Sin2Phi(w) * d.ay * d.ay);
    if (d.type == RT_DIST_BECKMANN) {
        float a = 1 / (alpha * absTanTheta);
        if (a >= 1.6f) return 0;
        return (1 - 1.259f * a + 0.396f * a * a) / (3.535f * a + 2.181f * a * a);
    }
    float a2t2 = (alpha * absTanTheta) * (alpha * absTanTheta);
    return (-1 + Sqrt(1.0f + a2t2)) / 2;
}
DF float DistG(const Dist& d, V3 wo, V3 wi) { return 1 / (1 + DistLambda(d, wo) + DistLambda(d, wi)); }
DF float DistPdf(const Dist& d, V3 wh) { return DistD(d, wh) * AbsCosTheta(wh); }
DF V3 DistSampleWh(const Dist& d, V3 wo, Rng& rand) {
    if (d.type == RT_DIST_BECKMANN) {
        float tan2Theta, phi;
        V2 u = NextVec2(rand);
        if (d.ax == d.ay) {
            float logSample = rt_logf(1 - u.x);
            tan2Theta = -d.ax * d.ax * logSample;
            phi = u.y * 2 * kPI;
        } else {
            float logSample = rt_logf(1 - u.x);
            phi = rt_atanf(d.ay / d.ax * rt_tanf(2 * kPI * u.y + 0.5f * kPI));
            if (u.y > 0.5f) phi += kPI;
            float sinPhi = rt_sinf(phi), cosPhi = rt_cosf(phi);
            float ax2 = d.ax * d.ax, ay2 = d.ay * d.ay;
            tan2Theta = -logSample / (cosPhi * cosPhi / ax2 + sinPhi * sinPhi / ay2);
        }
        float cosTheta = 1 / Sqrt(1 + tan2Theta);
        float sinTheta = Sqrt(nmax(0, 1 - cosTheta * cosTheta));
        V3 wh = SphDir(sinTheta, cosTheta, phi);
        if (!SameHemisphere(wo, wh)) wh = -wh;
        return wh;
    }
    V2 u = NextVec2(rand);
    float phi = (2 * kPI) * u.y;
    float cosTheta;
    if (d.ax == d.ay) {
        float tanTheta2 = d.ax * d.ax * u.x / (1.0f - u.x);
        cosTheta = 1 / Sqrt(1 + tanTheta2);
    } else {
        phi = rt_atanf(d.ay / d.ax * rt_tanf(2 * kPI * u.y + .5f * kPI));
        if (u.y > 0.5f) phi += kPI;
        float sinPhi = rt_sinf(phi), cosPhi = rt_cosf(phi);
        float ax2 = d.ax * d.ax, ay2 = d.ay * d.ay;
        float alpha2 = 1 / (cosPhi * cosPhi / ax2 + sinPhi * sinPhi / ay2);
        float tanTheta2 = alpha2 * u.x / (1 - u.x);
        cosTheta = 1 / Sqrt(1 + tanTheta2);
    }
    float sinTheta = Sqrt(nmax(0.0f, 1.0f - cosTheta * cosTheta));
    V3 wh = SphDir(sinTheta, cosTheta, phi);
    if (!SameHemisphere(wo, wh)) wh = -wh;
    return wh;
}

/* ---- Fresnel (Bxdf/Fresnel.cs) ------------------------------------------------- */
DF float DielectricFunc(float cosThetaI, float etaI, float etaT) {
    cosThetaI = nclamp(cosThetaI, -1, 1);
    bool entering = cosThetaI > 0.0f;
    if (!entering) { float t = etaI; etaI = etaT; etaT = t; cosThetaI = Abs(cosThetaI); }
    float sinThetaI = Sqrt(nmax(0, 1 - cosThetaI * cosThetaI));
    float sinThetaT = etaI / etaT * sinThetaI;
    if (sinThetaT >= 1) return 1;
    float cosThetaT = Sqrt(nmax(0, 1 - sinThetaT * sinThetaT));
    float rparl = ((etaT * cosThetaI) - (etaI * cosThetaT)) / ((etaT * cosThetaI) + (etaI * cosThetaT));
    float rperp = ((etaI * cosThetaI) - (etaT * cosThetaT)) / ((etaI * cosThetaI) + (etaT * cosThetaT));
    return (rparl * rparl + rperp * rperp) / 2;
}
DF C3 ConductorFunc(float cosThetaI, C3 etai, C3 etat, C3 k) {
    cosThetaI = nclamp(cosThetaI, -1, 1);
    C3 eta = etat / etai;
    C3 etak = k / etai;
    float cosThetaI2 = cosThetaI * cosThetaI;
    float sinThetaI2 = 1.0f - cosThetaI2;
    C3 eta2 = eta * eta;
    C3 etak2 = etak * etak;
    C3 t0 = eta2 - etak2 - sinThetaI2;
    C3 s = t0 * t0 + 4 * eta2 * etak2;
    C3 a2plusb2 = c3(Sqrt(s.r), Sqrt(s.g), Sqrt(s.b));
    C3 t1 = a2plusb2 + cosThetaI2;
    C3 s2 = 0.5f * (a2plusb2 + t0);
    C3 a = c3(Sqrt(s2.r), Sqrt(s2.g), Sqrt(s2.b));
    C3 t2 = 2 * cosThetaI * a;
    C3 Rs = (t1 - t2) / (t1 + t2);
    C3 t3 = cosThetaI2 * a2plusb2 + sinThetaI2 * sinThetaI2;
    C3 t4 = t2 * sinThetaI2;
    C3 Rp = Rs * (t3 - t4) / (t3 + t4);
    return 0.5f * (Rp + Rs);
}

struct BSample { V3 Wi; C3 Fr; float Pdf; int Type; };
DF BSample empty_sample() { BSample r; r.Wi = v3s(0); r.Fr = c3s(0); r.Pdf = 0; r.Type = 0; return r; }
enum { BX_REFLECTION = 1, BX_TRANSMISSION = 2, BX_DIFFUSE = 4, BX_GLOSSY = 8, BX_SPECULAR = 16 };

/* MicrofacetReflectionBrdf with conductor (frKind 0) or dielectric (1) Fresnel */
struct MicroRefl { C3 R; int frKind; C3 etaT, k; float dEtaI, dEtaT; Dist D; };
DF C3 MRFresnel(const MicroRefl& m, float cosI) {
    if (m.frKind == 0) return ConductorFunc(cosI, c3s(1.0f), m.etaT, m.k);
    return c3s(DielectricFunc(cosI, m.dEtaI, m.dEtaT));
}
DF C3 MRFr(const MicroRefl& m, V3 wo, V3 wi) {
    if (!SameHemisphere(wo, wi)) return c3s(0.0f);
    float cosThetaO = AbsCosTheta(wo), cosThetaI = AbsCosTheta(wi);
    V3 wh = wi + wo;
    if (cosThetaI == 0 || cosThetaO == 0) return c3s(0);
    if (wh.x == 0 && wh.y == 0 && wh.z == 0) return c3s(0);
    wh = Normalize(wh);
    C3 f = MRFresnel(m, Dot(wi, Faceforward(wh, v3(0, 0, 1))));
    float d = DistD(m.D, wh);
    float g = DistG(m.D, wo, wi);
    return m.R * CAbs((d * g * f) / (4 * cosThetaI * cosThetaO));
}
DF float MRPdf(const MicroRefl& m, V3 wo, V3 wi) {
    if (!SameHemisphere(wo, wi)) return 0;
    V3 wh = Normalize(wo + wi);
    return DistPdf(m.D, wh) / (4 * Dot(wo, wh));
}
DF BSample MRSample(const MicroRefl& m, V3 wo, Rng& rand) {
    BSample r = empty_sample();
    if (CosTheta(wo) == 0) return r;
    V3 wh = DistSampleWh(m.D, wo, rand);
    if (Dot(wo, wh) < 0) return r;
    V3 wi = Reflect(-wo, wh);
    if (!SameHemisphere(wo, wi)) return r;
    r.Pdf = DistPdf(m.D, wh) / (4 * Dot(wi, wh));
    r.Fr = MRFr(m, wo, wi);
    r.Wi = wi; r.Type = BX_REFLECTION | BX_GLOSSY;
    return r;
}
/* LambertianReflectionBrdf */
DF C3 LambFr(C3 R, V3 wo, V3 wi) { return SameHemisphere(wo, wi) ? R / kPI : c3s(0); }
DF float LambPdf(V3 wo, V3 wi) { return SameHemisphere(wo, wi) ? AbsCosTheta(wi) / kPI : 0.0f; }
DF BSample LambSample(C3 R, V3 wo, Rng& rand) {
    BSample r = empty_sample();
    V3 wi = Normalize(SquareToCosineHemisphere(NextVec2(rand)));
    if (wo.z < 0) wi.z *= -1;
    if (!SameHemisphere(wo, wi)) return r;
    r.Pdf = LambPdf(wo, wi); r.Fr = R / kPI; r.Wi = wi; r.Type = BX_REFLECTION | BX_DIFFUSE;
    return r;
}

/* RoughGlass (Materials/RoughGlass.cs).  kImp: TransportMode.Importance, which
 * drops the 1/eta^2 scaling of refraction (RoughGlass.cs:63,161). */
template <bool kImp = false>
DF C3 GlassFr(const RtSceneView* S, const RtMaterial& m, V3 wo, V3 wi, V2 uv, const Dist& dist) {
    C3 r = TexSample(S, m.tex_r, uv), t = TexSample(S, m.tex_t, uv);
    bool isReflect = SameHemisphere(wo, wi);
    bool entering = CosTheta(wo) > 0;
    float etaI = entering ? m.eta_a : m.eta_b;
    float etaT = entering ? m.eta_b : m.eta_a;
    float eta = isReflect ? 1 : etaT / etaI;
    V3 wh = Normalize(wo + wi * eta);
    if (CosTheta(wh) < 0) wh = -wh;
    float sqrtDenom = Dot(wo, wh) + eta * Dot(wi, wh);
    float d = DistD(dist, wh);
    float g = DistG(dist, wo, wi);
    float f = DielectricFunc(Dot(wo, wh), etaI, etaT);
    C3 bsdf;
    if (isReflect) {
        bsdf = r * (d * g * f / (4.0f * CosTheta(wi) * CosTheta(wo)));
    } else {
        if (Dot(wo, wh) * Dot(wi, wh) > 0) return c3s(0);
        float factor = kImp ? 1.0f : 1 / eta;
        bsdf = (1 - f) * t * Abs(d * g * eta * eta * AbsDot(wi, wh) * AbsDot(wo, wh) * factor * factor /
                                  (CosTheta(wo) * CosTheta(wi) * sqrtDenom * sqrtDenom));
    }
    return IsValid(bsdf) ? bsdf : c3s(0.0f);
}
DF float GlassPdf(const RtMaterial& m, V3 wo, V3 wi, const Dist& dist) {
    bool isReflect = SameHemisphere(wo, wi);
    bool entering = CosTheta(wo) > 0;
    float etaI = entering ? m.eta_a : m.eta_b;
    float etaT = entering ? m.eta_b : m.eta_a;
    float pdf;
    if (isReflect) {
        V3 wh = Normalize(wo + wi);
        if (CosTheta(wh) < 0) wh = -wh;
        if (Dot(wo, wh) * CosTheta(wo) <= 0 || Dot(wi, wh) * CosTheta(wi) <= 0) return 0.0f;
        float jacobian = 1.0f / (4.0f * AbsDot(wh, wi));
        float f = DielectricFunc(Dot(wo, wh), etaI, etaT);
        pdf = DistPdf(dist, wh) * jacobian * f;
    } else {
        float eta = etaT / etaI;
        V3 wh = Normalize(wo + wi * eta);
        if (CosTheta(wh) < 0) wh = -wh;
        if (Dot(wo, wh) * Dot(wi, wh) > 0) return 0.0f;
        if (Dot(wo, wh) * CosTheta(wo) <= 0 || Dot(wi, wh) * CosTheta(wi) <= 0) return 0.0f;
        float sqrtDenom = Dot(wo, wh) + eta * Dot(wi, wh);
        float dwhdwi = Abs((eta * eta * Dot(wi, wh)) / (sqrtDenom * sqrtDenom));
        float f = DielectricFunc(Dot(wo, wh), etaI, etaT);
        pdf = DistPdf(dist, wh) * dwhdwi * (1 - f);
    }
    return (isinff_(pdf) || isnanf_(pdf)) ? 0.0f : pdf;
}
template <bool kImp = false>
DF BSample GlassSample(const RtSceneView* S, const RtMaterial& m, V3 wo, V2 uv, Rng& rand, const Dist& dist) {
    BSample res = empty_sample();
    C3 r = TexSample(S, m.tex_r, uv), t = TexSample(S, m.tex_t, uv);
    V3 wh = DistSampleWh(dist, wo, rand);
    float f = DielectricFunc(Dot(wo, wh), m.eta_a, m.eta_b);
    if (NextFloat(rand) < f) {
        V3 wi = Reflect(-wo, wh);
        if (!SameHemisphere(wo, wi)) return res;
        float d = DistD(dist, wh);
        float g = DistG(dist, wo, wi);
        C3 brdf = r * (d * g * f / (4.0f * CosTheta(wi) * CosTheta(wo)));
        float jacobian = 1.0f / (4.0f * AbsDot(wh, wi));
        float pdf = DistPdf(dist, wh) * jacobian * f;
        if (isinff_(pdf) || isnanf_(pdf) || !IsValid(brdf)) return res;
        res.Wi = wi; res.Fr = brdf; res.Pdf = pdf; res.Type = BX_REFLECTION | BX_GLOSSY;
        return res;
    }
    bool entering = CosTheta(wo) > 0;
    float etaI = entering ? m.eta_a : m.eta_b;
    float etaT = entering ? m.eta_b : m.eta_a;
    float eta = etaT / etaI;
    V3 wi;
    if (Refract(wo, wh, etaI / etaT, &wi)) {
        if (Dot(wo, wh) * Dot(wi, wh) > 0) return res;
    } else {
        wi = Reflect(-wo, wh);
        eta = 1;
    }
    float sqrtDenom = Dot(wo, wh) + eta * Dot(wi, wh);
    float factor = kImp ? 1.0f : 1 / eta;
    float d = DistD(dist, wh);
    float g = DistG(dist, wo, wi);
    C3 btdf = (1 - f) * t * Abs(d * g * eta * eta * AbsDot(wi, wh) * AbsDot(wo, wh) * factor * factor /
                                 (CosTheta(wo) * CosTheta(wi) * sqrtDenom * sqrtDenom));
    float dwhdwi = Abs((eta * eta * Dot(wi, wh)) / (sqrtDenom * sqrtDenom));
    float pdf = DistPdf(dist, wh) * dwhdwi * (1 - f);
    if (isinff_(pdf) || isnanf_(pdf) || !IsValid(btdf)) return res;
    res.Wi = wi; res.Fr = btdf; res.Pdf = pdf; res.Type = BX_TRANSMISSION | BX_GLOSSY;
    return res;
}
DF bool OneSidedReject(const RtMaterial& m, V3 wo, V3 wi) { return (CosTheta(wo) <= 0 || CosTheta(wi) <= 0) && !m.two_sided; }
DF C3 PlasticFr(const RtMaterial& m, V3 wo, V3 wi, const Dist& dist, C3 r) {
    if (OneSidedReject(m, wo, wi)) return c3s(0.0f);
    C3 diffuse = LambFr(r, wo, wi);
    MicroRefl mr{r, 1, c3s(0), c3s(0), m.eta_a, m.eta_b, dist};
    C3 glossy = MRFr(mr, wo, wi);
    return m.kd * diffuse + m.ks * glossy;
}
DF float PlasticPdf(const RtMaterial& m, V3 wo, V3 wi, const Dist& dist, C3 r) {
    if (OneSidedReject(m, wo, wi)) return 0.0f;
    float p = m.ks / (m.kd + m.ks);
    float diffuse = LambPdf(wo, wi);
    MicroRefl mr{r, 1, c3s(0), c3s(0), m.eta_a, m.eta_b, dist};
    float glossy = MRPdf(mr, wo, wi);
    return (1 - p) * diffuse + p * glossy;
}
DF Dist MatDist(const RtSceneView* S, const RtMaterial& m, V2 uv) {
    return mkdist(m.dist, TexSample(S, m.tex_rough, uv).r, TexSample(S, m.tex_anis, uv).r);
}

/* Material.Fr (Material.cs:28); kImp: TransportMode.Importance */
template <bool kImp = false>
NF C3 MatFr(const RtSceneView* S, int mi, V3 wo, V3 wi, V2 uv) {
    const RtMaterial m = S->materials[mi];
    switch (m.type) {
    case RT_MAT_DIFFUSE:
        if (OneSidedReject(m, wo, wi)) return c3s(0.0f);
        return LambFr(TexSample(S, m.tex_r, uv), wo, wi);
    case RT_MAT_ROUGH_METAL: {
        Dist d = MatDist(S, m, uv);
        if (OneSidedReject(m, wo, wi)) return c3s(0.0f);
        MicroRefl mr{c3s(1.0f), 0, c3(m.eta[0], m.eta[1], m.eta[2]), c3(m.k[0], m.k[1], m.k[2]), 0, 0, d};
        return MRFr(mr, wo, wi);
    }
    case RT_MAT_ROUGH_GLASS: return GlassFr<kImp>(S, m, wo, wi, uv, MatDist(S, m, uv));
    case RT_MAT_ROUGH_PLASTIC: return PlasticFr(m, wo, wi, MatDist(S, m, uv), TexSample(S, m.tex_r, uv));
    default: return c3s(0.0f);
    }
}
/* Material.Pdf (Material.cs:48) */
NF float MatPdf(const RtSceneView* S, int mi, V3 wo, V3 wi, V2 uv) {
    const RtMaterial m = S->materials[mi];
    switch (m.type) {
    case RT_MAT_DIFFUSE:
        if (OneSidedReject(m, wo, wi)) return 0.0f;
        return LambPdf(wo, wi);
    case RT_MAT_ROUGH_METAL: {
        Dist d = MatDist(S, m, uv);
        if (OneSidedReject(m, wo, wi)) return 0.0f;
        MicroRefl mr{c3s(1.0f), 0, c3(m.eta[0], m.eta[1], m.eta[2]), c3(m.k[0], m.k[1], m.k[2]), 0, 0, d};
        return MRPdf(mr, wo, wi);
    }
    case RT_MAT_ROUGH_GLASS: return GlassPdf(m, wo, wi, MatDist(S, m, uv));
    case RT_MAT_ROUGH_PLASTIC: return PlasticPdf(m, wo, wi, MatDist(S, m, uv), TexSample(S, m.tex_r, uv));
    default: return 0.0f;
    }
}
/* Material.Sample (Material.cs:38); kImp: TransportMode.Importance */
template <bool kImp = false>
NF BSample MatSample(const RtSceneView* S, int mi, V3 wo, V2 uv, Rng& rand) {
    const RtMaterial m = S->materials[mi];
    BSample res = empty_sample();
    switch (m.type) {
    case RT_MAT_DIFFUSE:
        if (CosTheta(wo) <= 0 && !m.two_sided) return res;
        return LambSample(TexSample(S, m.tex_r, uv), wo, rand);
    case RT_MAT_ROUGH_METAL: {
        Dist d = MatDist(S, m, uv);
        if (CosTheta(wo) <= 0 && !m.two_sided) return res;
        MicroRefl mr{c3s(1.0f), 0, c3(m.eta[0], m.eta[1], m.eta[2]), c3(m.k[0], m.k[1], m.k[2]), 0, 0, d};
        return MRSample(mr, wo, rand);
    }
    case RT_MAT_ROUGH_GLASS: return GlassSample<kImp>(S, m, wo, uv, rand, MatDist(S, m, uv));
    case RT_MAT_ROUGH_PLASTIC: {
        Dist d = MatDist(S, m, uv);
        if (CosTheta(wo) <= 0 && !m.two_sided) return res;
        C3 r = TexSample(S, m.tex_r, uv);
        float p = m.ks / (m.kd + m.ks);
        MicroRefl mr{r, 1, c3s(0), c3s(0), m.eta_a, m.eta_b, d};
        BSample glossy = MRSample(mr, wo, rand);
        BSample diffuse = LambSample(r, wo, rand);
        V3 wi; int tp;
        if (NextFloat(rand) < p) { wi = glossy.Wi; tp = glossy.Type; }
        else { wi = diffuse.Wi; tp = diffuse.Type; }
        res.Pdf = PlasticPdf(m, wo, wi, d, r);
        res.Fr = PlasticFr(m, wo, wi, d, r);
        res.Wi = wi; res.Type = tp;
        return res;
    }
    case RT_MAT_PERFECT_MIRROR: {
        if (CosTheta(wo) <= 0 && !m.two_sided) return res;
        C3 R = TexSample(S, m.tex_r, uv);
        if (AbsCosTheta(wo) == 0) return res;
        V3 wi = v3(-wo.x, -wo.y, wo.z);
        res.Wi = wi; res.Fr = R / AbsCosTheta(wi); res.Pdf = 1.0f; res.Type = BX_REFLECTION | BX_SPECULAR;
        return res;
    }
    case RT_MAT_PERFECT_GLASS: {
        C3 R = TexSample(S, m.tex_r, uv), T = TexSample(S, m.tex_t, uv);
        float f = DielectricFunc(CosTheta(wo), m.eta_a, m.eta_b);
        if (NextFloat(rand) < f) {
            if (CosTheta(wo) == 0) return res;
            V3 wi = v3(-wo.x, -wo.y, wo.z);
            res.Wi = wi; res.Fr = f * R / AbsCosTheta(wi); res.Pdf = f; res.Type = BX_REFLECTION | BX_SPECULAR;
            return res;
        }
        bool entering = CosTheta(wo) > 0;
        float etaI = entering ? m.eta_a : m.eta_b;
        float etaT = entering ? m.eta_b : m.eta_a;
        V3 n = entering ? v3(0, 0, 1) : v3(0, 0, -1);
        V3 wi;
        if (!Refract(wo, n, etaI / etaT, &wi) || CosTheta(wi) == 0.0f) return res;
        C3 ft = T * (1.0f - f);
        if (!kImp) ft = ft * ((etaI * etaI) / (etaT * etaT)); /* FresnelSpecularBsdf.cs:58-61 */
        ft = ft / AbsCosTheta(wi);
        res.Wi = wi; res.Fr = ft; res.Pdf = 1 - f; res.Type = BX_TRANSMISSION | BX_SPECULAR;
        return res;
    }
    }
    return res;
}

/* ---- media (Mediums/Homogeneous.cs, IPhaseFunction.cs) ------------------------------ */
DF C3 MedTr(const RtMedium& m, const Ray& ray) {
    float negLength = ray.MinT - ray.MaxT;
    C3 tr;
    tr.r = m.sig_t[0] == 0 ? 1.0f : rt_expf(m.sig_t[0] * negLength);
    tr.g = m.sig_t[1] == 0 ? 1.0f : rt_expf(m.sig_t[1] * negLength);
    tr.b = m.sig_t[2] == 0 ? 1.0f : rt_expf(m.sig_t[2] * negLength);
    return tr;
}
struct MedSample { V3 P; V3 Wo; C3 Tr; float T; bool sampled; };
DF MedSample MedSampleDist(const RtMedium& m, const Ray& ray, Rng& rand) {
    int channel = NextInt(rand, 3);
    C3 sigmaT = c3(m.sig_t[0], m.sig_t[1], m.sig_t[2]);
    C3 sigmaS = c3(m.sig_s[0], m.sig_s[1], m.sig_s[2]);
    float samplingDensity = CGet(sigmaT, channel);
    float sampledDistance = -rt_logf(1 - NextFloat(rand)) / samplingDensity;
    float distSurf = ray.MaxT - ray.MinT;
    MedSample r;
    if (sampledDistance < distSurf) {
        float t = ray.MinT + sampledDistance;
        V3 p = At(ray, t);
        C3 tr;
        tr.r = rt_expf(-sigmaT.r * sampledDistance);
        tr.g = rt_expf(-sigmaT.g * sampledDistance);
        tr.b = rt_expf(-sigmaT.b * sampledDistance);
        float pdf = (tr.r * sigmaT.r + tr.g * sigmaT.g + tr.b * sigmaT.b) / 3;
        if (pdf == 0) pdf = 0.0001f;
        r.P = p; r.Wo = -ray.D; r.Tr = tr * sigmaS / pdf; r.T = t; r.sampled = true;
        return r;
    }
    C3 tr;
    tr.r = rt_expf(-sigmaT.r * distSurf);
    tr.g = rt_expf(-sigmaT.g * distSurf);
    tr.b = rt_expf(-sigmaT.b * distSurf);
    float pdf = (tr.r + tr.g + tr.b) / 3;
    if (pdf == 0) pdf = 0.0001f;
    r.Tr = tr / pdf; r.sampled = false; r.P = v3s(0); r.Wo = v3s(0); r.T = 0;
    return r;
}
DF float HGValue(float cosTheta, float g) {
    float denom = 1 + g * g + 2 * g * cosTheta;
    return (1 / (4 * kPI)) * (1 - g * g) / (denom * Sqrt(denom));
}
DF float HGClamp(float g) { return nclamp(g, -0.999f, 0.999f); }
DF float MedP(const RtMedium& m, V3 wo, V3 wi) { return HGValue(Dot(wo, wi), HGClamp(m.g)); }
DF float MedSampleWi(const RtMedium& m, V3 wo, Rng& rand, V3* wiOut) {
    float g = HGClamp(m.g);
    V2 rng = NextVec2(rand);
    float cosTheta;
    if (Abs(g) < 0.001f) cosTheta = 1 - 2 * rng.x;
    else {
        float sqrTerm = (1 - g * g) / (1 + g - 2 * g * rng.x);
        cosTheta = -(1 + g * g - sqrTerm * sqrTerm) / (2 * g);
    }
    float sinTheta = Sqrt(nmax(0, 1 - cosTheta * cosTheta));
    float phi = 2 * kPI * rng.y;
    Frame f = mkframe(wo);
    float sinPhi = rt_sinf(phi), cosPhi = rt_cosf(phi);
    *wiOut = sinTheta * cosPhi * f.X + sinTheta * sinPhi * f.Y + cosTheta * f.Z;
    return HGValue(cosTheta, g);
}

/* ---- Distribution1D / 2D (Distribution1D.cs, Distribution2D.cs) --------------------- */
DF int FindInterval(const float* cdf, int size, float u) {
    int first = 0, len = size;
    while (len > 0) {
        int half = len >> 1, middle = first + half;
        if (__ldg(cdf + middle) <= u) { first = middle + 1; len -= half + 1; }
        else len = half;
    }
    return nclampi(first - 1, 0, size - 2);
}
DF float Sample1D(const float* pdf, const float* cdf, float integ, int n, float u, float* pdfOut, int* off) {
    *off = FindInterval(cdf, n + 1, u);
    float du = u - __ldg(cdf + *off);
    if ((__ldg(cdf + *off + 1) - __ldg(cdf + *off)) > 0) du /= __ldg(cdf + *off + 1) - __ldg(cdf + *off);
    *pdfOut = integ > 0 ? __ldg(pdf + *off) / integ : 0;
    return ((float)*off + du) / (float)n;
}
/* The alias pick of an n-entry table (built by alias_from_cdf in rt_host.cpp)
 * for u = k / 2^24, as every NextFloat is: bucket floor(k n / 2^24), kept when
 * the remainder k n mod 2^24 is below its threshold, else its alias.  The
 * arithmetic is exact integer arithmetic, so every k lands where the host's
 * count of the table assumes. */
DF int AliasPick(const int2* tab, int n, float u) {
    const uint32_t k = min((uint32_t)(u * 16777216.0f), 16777215u);   /* u < 1 always; kept in range anyway */
    const uint64_t s = (uint64_t)k * (uint32_t)n;
    const int i = (int)(s >> 24);
    const int2 e = __ldg(tab + i);
    return (uint32_t)(s & 0xFFFFFFu) < (uint32_t)e.x ? i : e.y;
}
DF void Sample2D(const RtSceneView* S, const RtDist2D& d, V2 u, float* pdf, int* ov, int* ou) {
    float pdf1, pdf0;
    const float* P = S->dist_pool;
    if (S->env_alias && d.marg_alias >= 0) {
        /* the same texel pmf and the same pdf arithmetic as the search below;
         * SampleLi and SampleEmit use only the offsets and the pdf */
        *ov = AliasPick(S->alias_pool + d.marg_alias, d.nv, u.y);
        *ou = AliasPick(S->alias_pool + d.cond_alias + (int64_t)(*ov) * d.nu, d.nu, u.x);
        pdf1 = d.marg_int > 0 ? __ldg(P + d.marg_pdf + *ov) / d.marg_int : 0;
        const float ci = __ldg(P + d.cond_int + *ov);
        pdf0 = ci > 0 ? __ldg(P + d.cond_pdf + (int64_t)(*ov) * d.nu + *ou) / ci : 0;
        *pdf = pdf0 * pdf1;
        return;
    }
    Sample1D(P + d.marg_pdf, P + d.marg_cdf, d.marg_int, d.nv, u.y, &pdf1, ov);
    const float* cpdf = P + d.cond_pdf + (int64_t)(*ov) * d.nu;
    const float* ccdf = P + d.cond_cdf + (int64_t)(*ov) * (d.nu + 1);
    Sample1D(cpdf, ccdf, __ldg(P + d.cond_int + *ov), d.nu, u.x, &pdf0, ou);
    *pdf = pdf0 * pdf1;
}
DF float Pdf2D(const RtSceneView* S, const RtDist2D& d, float u, float v) {
    int iu = nclampi(nf2i(u * (float)d.nu), 0, d.nu - 1);
    int iv = nclampi(nf2i(v * (float)d.nv), 0, d.nv - 1);
    return __ldg(S->dist_pool + d.cond_pdf + (int64_t)iv * d.nu + iu) / d.marg_int;
}

/* ---- lights (Lights/DiffuseAreaLight.cs, Lights/InfiniteAreaLight.cs) ------------------- */
struct LSample { V3 P; C3 Li; V3 Wi; float Pdf; };
DF LSample empty_lsample() { LSample r; r.P = v3s(0); r.Li = c3s(0); r.Wi = v3s(0); r.Pdf = 0; return r; }

/* Shape.Sample of the light's shape */
DF void ShapeSample(const RtSceneView* S, const RtLight& L, Rng& rand, V3* p, V3* n, float* pdf) {
    if (L.kind == RT_LIGHT_AREA_TRI) {
        V2 rng = NextVec2(rand);
        float alpha = 1 - Sqrt(1 - rng.x);
        float beta = rng.y * Sqrt(1 - rng.x);
        V3 bary = v3(alpha, beta, (1 - alpha - beta));
        V2 uv;
        TriAttrs(S, L.ref, bary, p, n, &uv);
        *pdf = 1.0f / L.area;
    } else {
        const RtSphere sph = S->spheres[L.ref];
        V3 rng = SquareToUniformSphere(NextVec2(rand));
        V3 nn = Normalize(rng);
        *n = nn;
        *p = nn * sph.radius + v3(sph.center[0], sph.center[1], sph.center[2]);
        *pdf = 1 / (4 * sph.radius * sph.radius * kPI);
    }
}
DF float ShapeArea(const RtSceneView* S, const RtLight& L) {
    if (L.kind == RT_LIGHT_AREA_TRI) return L.area;
    const RtSphere sph = S->spheres[L.ref];
    return 4 * sph.radius * sph.radius * kPI;
}
/* Shape.Intersect + GetIntersection of the light's own shape for PdfLi */
DF bool ShapeHit(const RtSceneView* S, const RtLight& L, const Ray& ray, V3* p, V3* n) {
    if (L.kind == RT_LIGHT_AREA_TRI) {
        RtTri t = S->tris[L.ref];
        V3 pa = f4xyz(S->pos[t.v0]), pb = f4xyz(S->pos[t.v1]), pc = f4xyz(S->pos[t.v2]);
        SurfPt sp;
        if (!TriTest(pa, pb - pa, pc - pa, ray, &sp)) return false;
        V3 bary = v3(1 - (sp.u + sp.v), sp.u, sp.v);
        V2 uv;
        TriAttrs(S, L.ref, bary, p, n, &uv);
        return true;
    }
    const RtSphere sph = S->spheres[L.ref];
    V3 c = v3(sph.center[0], sph.center[1], sph.center[2]);
    float t;
    if (!SphereTest(c, sph.radius, ray, &t)) return false;
    V3 nn = Normalize(At(ray, t) - c);
    *n = nn; *p = nn * sph.radius + c;
    return true;
}
DF C3 InfLe(const RtSceneView* S, const RtLight& L, V3 rd) {
    V3 dir = Normalize(XfN12(rd, L.w2m));
    float phi = rt_atan2f(dir.x, -dir.z);
    phi = (phi < 0) ? (phi + 2 * kPI) : phi;
    float theta = rt_acosf(nclamp(dir.y, -1, 1));
    float u = phi / (2 * kPI), v = theta / kPI;
    return TexSample(S, L.ref, v2(u, v));
}
DF float InfPdfDir(const RtSceneView* S, const RtLight& L, V3 wi) {
    V3 dir = Normalize(XfN12(wi, L.w2m));
    float phi = rt_atan2f(dir.x, -dir.z);
    phi = (phi < 0) ? (phi + 2 * kPI) : phi;
    float theta = rt_acosf(nclamp(dir.y, -1, 1));
    float sinTheta = rt_sinf(theta);
    if (sinTheta == 0.0f) return 0.0f;
    float u = phi / (2 * kPI), v = theta / kPI;
    return Pdf2D(S, S->dists[L.dist], u, v) / (2 * kPI * kPI * sinTheta);
}
/* Light.SampleLi */
NF LSample LightSampleLi(const RtSceneView* S, int li, V3 refP, Rng& rand) {
    const RtLight& L = S->lights[li];
    LSample r = empty_lsample();
    if (L.kind == RT_LIGHT_INFINITE) {
        const RtDist2D d = S->dists[L.dist];
        float pdf; int ov, ou;
        Sample2D(S, d, NextVec2(rand), &pdf, &ov, &ou);
        if (pdf <= 0) return r;
        float y = (float)ov / (float)d.nv;
        float x = (float)ou / (float)d.nu;
        float theta = y * kPI;
        float phi = x * 2 * kPI;
        float sinTheta = rt_sinf(theta);
        if (sinTheta == 0) return r;
        pdf /= (2 * kPI * kPI * sinTheta);
        float cosTheta = rt_cosf(theta);
        float sinPhi = rt_sinf(phi), cosPhi = rt_cosf(phi);
        V3 sph = v3(cosPhi * sinTheta, sinPhi * sinTheta, cosTheta);
        V3 dir = v3(sph.y, sph.z, -sph.x);
        V3 worldDir = Normalize(XfN12(dir, L.m2w));
        C3 radiance = TexSample(S, L.ref, v2(x, y));
        V3 pos = worldDir * L.world_radius * 20 + v3(L.world_center[0], L.world_center[1], L.world_center[2]);
        r.P = pos; r.Li = radiance; r.Wi = Normalize(pos - refP); r.Pdf = pdf;
        return r;
    }
    V3 sp, sn; float shapePdf;
    ShapeSample(S, L, rand, &sp, &sn, &shapePdf);
    V3 wi = sp - refP;
    C3 li_ = (Dot(sn, -wi) > 0) ? c3(L.le[0], L.le[1], L.le[2]) : c3s(0.0f);
    float pdf;
    if (LengthSq(wi) == 0) pdf = 0.0f;
    else {
        wi = Normalize(wi);
        pdf = shapePdf * LengthSq(refP - sp) / AbsDot(sn, -wi);
        if (isinff_(pdf)) pdf = 0.0f;
    }
    r.P = sp; r.Li = li_; r.Wi = wi; r.Pdf = pdf;
    return r;
}
/* Light.PdfLi */
NF float LightPdfLi(const RtSceneView* S, int li, V3 refP, V3 wi) {
    const RtLight& L = S->lights[li];
    if (L.kind == RT_LIGHT_INFINITE) return InfPdfDir(S, L, wi);
    Ray ray = mkray(refP, wi);
    V3 hp, hn;
    if (!ShapeHit(S, L, ray, &hp, &hn)) return 0.0f;
    float pdf = LengthSq(refP - hp) / (AbsDot(hn, -wi) * ShapeArea(S, L));
    if (isinff_(pdf)) pdf = 0.0f;
    return pdf;
}
/* Intersection.Le -> DiffuseAreaLight.L */
DF C3 IsectLe(const RtSceneView* S, const Isect& it, V3 w) {
    int li = LightOf(S, it);
    if (li < 0) return c3s(0.0f);
    const RtLight& L = S->lights[li];
    return (Dot(it.F.Z, w) > 0) ? c3(L.le[0], L.le[1], L.le[2]) : c3s(0.0f);
}
/* Scene.EvalAllInfiniteLights */
DF C3 EvalAllInfinite(const RtSceneView* S, V3 rd) {
    C3 l = c3s(0.0f);
    for (int i = 0; i < S->infinite_count; i++) l = l + InfLe(S, S->lights[S->infinite_lights[i]], rd);
    return l;
}
/* Scene.SampleLight: uniform choice, pdf 1/N */
DF float SampleLight(const RtSceneView* S, Rng& rand, int* light) {
    if (S->light_count == 0) { *light = -1; return 0.0f; }
    *light = NextInt(rand, S->light_count);
    return 1.0f / (float)S->light_count;
}
/* Scene.IsOccluded */
DF bool IsOccluded(Ctx& c, V3 from, V3 to) {
    V3 vec = to - from;
    float dis = Length(vec);
    if (dis < 0.001f) return true;
    V3 dir = Normalize(vec);
    return SceneIntersectP(c, mkray(from, dir, 0.0001f, dis - 0.0001f));
}
#ifndef RT_WALK_CAP
#define RT_WALK_CAP 4096               /* segments of one null-boundary walk */
#endif
/* Scene.Transmittance (Scene.cs:72-103); a walk that reaches RT_WALK_CAP
 * segments stops and reports RT_STATUS_WALK */
DF C3 Transmittance(Ctx& c, V3 from, V3 to, int rayEnv) {
    C3 tr = c3s(1.0f);
    V3 start = from;
    V3 dir = Normalize(to - start);
    for (int it = 0;; it++) {
        if (it == RT_WALK_CAP) { atomicOr(c.status, RT_STATUS_WALK); break; }
        V3 vec = to - start;
        float dis = Length(vec);
        if (dis < 0.0001f) break;
        Ray ray = mkray(start, dir, 0.0001f, dis - 0.0001f);
        Isect inct;
        bool anyHit = SceneIntersect(c, ray, &inct);
        if (anyHit && HasSurface(c.S, inct)) return c3s(0.0f);
        if (rayEnv >= 0) tr = tr * MedTr(c.S->media[rayEnv], ray);
        if (!anyHit) break;
        start = inct.P;
        rayEnv = GetMedium(c.S, inct, dir);
    }
    return tr;
}
/* Scene.IntersectTr (Scene.cs:105-131) */
DF bool IntersectTr(Ctx& c, Ray ray, int rayEnv, Isect* inct, C3* tr) {
    *tr = c3s(1.0f);
    for (int it = 0;; it++) {
        if (it == RT_WALK_CAP) { atomicOr(c.status, RT_STATUS_WALK); break; }
        bool anyHit = SceneIntersect(c, ray, inct);
        if (!anyHit) {
            if (rayEnv >= 0) *tr = *tr * MedTr(c.S->media[rayEnv], ray);
            return false;
        }
        if (rayEnv >= 0) {
            Ray realPath = mkray(ray.O, ray.D, ray.MinT, Length(At(ray, inct->T)));
            *tr = *tr * MedTr(c.S->media[rayEnv], realPath);
        }
        if (HasSurface(c.S, *inct)) return true;
        ray = mkray(inct->P, ray.D, 0.001f);
        rayEnv = GetMedium(c.S, *inct, ray.D);
    }
    return false;
}

/* PerspectiveCamera.SampleRay (Camera.cs:182-191) */
DF Ray CameraRay(const RtCamera& cam, V2 sp) {
    V3 ndc = v3(sp.x * cam.inv_res_x, sp.y * cam.inv_res_y, 0.0f);
    V3 near_ = Xf16(ndc, cam.clip_to_camera);
    V3 dir = Normalize(near_);
    float invZ = 1.0f / dir.z;
    V3 o = Xf16(v3(0, 0, 0), cam.camera_to_world);
    V3 d = Normalize(XfN16(dir, cam.camera_to_world));
    return mkray(o, d, cam.near_z * invZ, cam.far_z * invZ);
}

/* ---- light tracing: Light.SampleEmit and PerspectiveCamera.SampleWi -------------------- */
/* Probability.SquareToConcentricDisk (Probability.cs:157-174) */
DF V2 SquareToConcentricDisk(V2 u) {
    V2 uOffset = v2(2.0f * u.x - 1.0f, 2.0f * u.y - 1.0f);
    if (uOffset.x == 0 && uOffset.y == 0) return v2(0, 0);
    float theta, r;
    if (Abs(uOffset.x) > Abs(uOffset.y)) {
        r = uOffset.x;
        theta = (kPI / 4) * (uOffset.y / uOffset.x);
    } else {
        r = uOffset.y;
        theta = (kPI / 2) - (kPI / 4) * (uOffset.x / uOffset.y);
    }
    float sinTheta = rt_sinf(theta), cosTheta = rt_cosf(theta);
    return v2(r * cosTheta, r * sinTheta);
}
/* LightEmitResult (Light.cs:61-107) without the unused uv */
struct Emit { V3 pos, dir, n; C3 le; float pdf_pos, pdf_dir; };
/* Light.SampleEmit: DiffuseAreaLight.cs:70-77, InfiniteAreaLight.cs:122-133 */
NF Emit LightSampleEmit(const RtSceneView* S, int li, Rng& rand) {
    const RtLight& L = S->lights[li];
    Emit e;
    if (L.kind == RT_LIGHT_INFINITE) {
        /* SampleLightDir (InfiniteAreaLight.cs:92-109): a zero direction and pdf 0
         * when the sample fails, which SampleEmit passes on unchecked */
        const RtDist2D d = S->dists[L.dist];
        float pdf; int ov, ou;
        Sample2D(S, d, NextVec2(rand), &pdf, &ov, &ou);
        V2 uv = v2(0, 0);
        V3 worldDir = v3s(0);
        float pdfDir = 0;
        if (pdf > 0) {
            float y = (float)ov / (float)d.nv;
            float x = (float)ou / (float)d.nu;
            uv = v2(x, y);
            float theta = y * kPI;
            float phi = x * 2 * kPI;
            float sinTheta = rt_sinf(theta);
            if (sinTheta != 0) {
                pdf /= (2 * kPI * kPI * sinTheta);
                float cosTheta = rt_cosf(theta);
                float sinPhi = rt_sinf(phi), cosPhi = rt_cosf(phi);
                V3 sph = v3(cosPhi * sinTheta, sinPhi * sinTheta, cosTheta);
                V3 dir = v3(sph.y, sph.z, -sph.x);
                worldDir = Normalize(XfN12(dir, L.m2w));
                pdfDir = pdf;
            }
        }
        C3 radiance = TexSample(S, L.ref, uv);
        V3 normal = -worldDir;
        Frame coord = mkframe(normal);
        V2 cd = SquareToConcentricDisk(NextVec2(rand));
        V3 center = v3(L.world_center[0], L.world_center[1], L.world_center[2]);
        V3 disk = center + L.world_radius * (cd.x * coord.X + cd.y * coord.Y);
        e.pos = disk + worldDir * L.world_radius;
        e.dir = -worldDir; e.n = -worldDir; e.le = radiance;
        e.pdf_pos = 1 / (kPI * (L.world_radius * L.world_radius));
        e.pdf_dir = pdfDir;
        return e;
    }
    V3 sp, sn; float pdfPos;
    ShapeSample(S, L, rand, &sp, &sn, &pdfPos);
    V3 localW = Normalize(SquareToCosineHemisphere(NextVec2(rand)));
    float pdfDir = CosTheta(localW) / kPI; /* SquareToCosineHemispherePdf */
    Frame F = mkframe(sn);
    e.pos = sp; e.dir = Normalize(ToWorld(F, localW)); e.n = sn;
    e.le = c3(L.le[0], L.le[1], L.le[2]);
    e.pdf_pos = pdfPos; e.pdf_dir = pdfDir;
    return e;
}
/* PerspectiveCamera.Importance (Camera.cs:193-204); d normalized, camera space */
DF float CameraImportance(const RtCamera& cam, V3 d) {
    float cosTheta = CosTheta(d);
    if (cosTheta <= 0) return 0;
    float focus = 1 / cosTheta;
    float px = d.x * focus, py = d.y * focus;
    if (px < cam.min_x || px > cam.max_x || py < cam.min_y || py > cam.max_y) return 0.0f;
    return cam.normalization * focus * focus * focus;
}
/* SampleCameraWiResult (Camera.cs:21-48) fields the light tracer reads; pdf is 1 */
struct CamWi { V3 pos, dir; float we, sx, sy; };
/* PerspectiveCamera.SampleWi (Camera.cs:221-241); false where it returns the
 * empty result (pdf 0).  The clip-space point comes from Vector3.Transform (no
 * w divide) and is divided by its own z, the reference's projection as written. */
DF bool CameraSampleWi(const RtCamera& cam, V3 pos, CamWi* r) {
    V3 lt = Xf16(pos, cam.world_to_camera);
    if (lt.z < cam.near_z || lt.z > cam.far_z) return false;
    V3 screen = Xf16(lt, cam.camera_to_clip);
    float sx = screen.x / screen.z, sy = screen.y / screen.z;
    if (sx < 0 || sx > 1 || sy < 0 || sy > 1) return false;
    r->sx = sx * (float)(cam.width - 1);
    r->sy = sy * (float)(cam.height - 1);
    float dist = Length(lt);
    float inv = 1 / dist;
    V3 localDir = lt * inv;
    r->pos = Xf16(v3(0, 0, 0), cam.camera_to_world);
    r->dir = (r->pos - pos) / dist;
    r->we = CameraImportance(cam, localDir) * inv * inv;
    return true;
}

}  /* namespace rtd */

#endif
