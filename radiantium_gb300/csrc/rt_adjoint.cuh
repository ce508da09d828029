/*
 * rt_adjoint.cuh - derivatives shared by the megakernel adjoint
 * (rt_adjoint.cu) and the wavefront adjoint (rt_wavefront.cu): d ln f and
 * d ln pdf of the rough BSDFs with respect to alpha, the MIS-weight
 * derivative of a direct-light term, and the scatter of albedo gradients
 * over a texture lookup's footprint.
 */
#ifndef RT_ADJOINT_CUH
#define RT_ADJOINT_CUH
#include "rt_shading.cuh"

namespace rtd {

/* d ln D / d alpha and d ln G / d alpha of Microfacet (Bxdf/Microfacet.cs) for
 * ax = max(alpha (1 + k), 0.001), ay = max(alpha (1 - k), 0.001) */
DF float DlnD(const Dist& d, float dax, float day, V3 wh) {
    const float tan2 = Tan2Theta(wh);
    if (isinff_(tan2)) return 0.0f;
    const float c2 = Cos2Phi(wh), s2 = Sin2Phi(wh);
    const float ax = d.ax, ay = d.ay;
    const float e = (c2 / (ax * ax) + s2 / (ay * ay)) * tan2;
    const float de = tan2 * (-2.0f * c2 / (ax * ax * ax) * dax - 2.0f * s2 / (ay * ay * ay) * day);
    if (d.type == RT_DIST_BECKMANN) return -dax / ax - day / ay - de;
    return -dax / ax - day / ay - 2.0f * de / (1.0f + e);
}
DF float Lambda(const Dist& d, V3 w, float dax, float day, float* dlam) {
    *dlam = 0.0f;
    const float absTan = Abs(TanTheta(w));
    if (isinff_(absTan)) return 0.0f;
    const float c2 = Cos2Phi(w), s2 = Sin2Phi(w);
    const float alpha = Sqrt(c2 * d.ax * d.ax + s2 * d.ay * d.ay);
    const float dalpha = alpha > 0.0f ? (c2 * d.ax * dax + s2 * d.ay * day) / alpha : 0.0f;
    if (d.type == RT_DIST_BECKMANN) {
        const float a = 1 / (alpha * absTan);
        if (a >= 1.6f) return 0.0f;
        const float num = 1 - 1.259f * a + 0.396f * a * a, den = 3.535f * a + 2.181f * a * a;
        const float dnum = -1.259f + 0.792f * a, dden = 3.535f + 4.362f * a;
        const float da = -a / alpha * dalpha;
        *dlam = (dnum * den - num * dden) / (den * den) * da;
        return num / den;
    }
    const float a2t2 = (alpha * absTan) * (alpha * absTan);
    const float r = Sqrt(1.0f + a2t2);
    *dlam = alpha * absTan * absTan * dalpha / (2.0f * r);
    return (-1 + r) / 2;
}
DF float DlnG(const Dist& d, float dax, float day, V3 wo, V3 wi) {
    float dlo, dli;
    const float lo = Lambda(d, wo, dax, day, &dlo), li = Lambda(d, wi, dax, day, &dli);
    return -(dlo + dli) / (1 + lo + li);
}

/* d ln f / d alpha and d ln pdf / d alpha of a rough material at (wo, wi);
 * false where f = 0 or the material has no differentiable alpha (same
 * branches as MatFr / MatPdf) */
DF bool DlnAlpha(const RtSceneView* S, int mi, V3 wo, V3 wi, V2 uv, float* out, float* outp) {
    *out = 0.0f;
    *outp = 0.0f;
    const RtMaterial m = S->materials[mi];
    if (m.type != RT_MAT_ROUGH_PLASTIC && m.type != RT_MAT_ROUGH_METAL) return false;
    if (OneSidedReject(m, wo, wi)) return false;
    const float r = TexSample(S, m.tex_rough, uv).r, k = TexSample(S, m.tex_anis, uv).r;
    const Dist d = mkdist(m.dist, r, k);
    const float dax = r * r * (1 + k) > 0.001f ? 1 + k : 0.0f;
    const float day = r * r * (1 - k) > 0.001f ? 1 - k : 0.0f;
    if (!SameHemisphere(wo, wi)) return false;
    const float cosO = AbsCosTheta(wo), cosI = AbsCosTheta(wi);
    V3 wh = wi + wo;
    if (cosI == 0 || cosO == 0 || (wh.x == 0 && wh.y == 0 && wh.z == 0)) return false;
    wh = Normalize(wh);
    const float D = DistD(d, wh);
    if (!(D > 0.0f)) return false;
    const float dlnD = DlnD(d, dax, day, wh);
    const float dln = dlnD + DlnG(d, dax, day, wo, wi);
    /* the glossy pdf D |cos theta_h| / (4 wo.wh) scales with D */
    if (m.type == RT_MAT_ROUGH_METAL) { *out = dln; *outp = dlnD; return true; }
    /* plastic: f = R (kd / pi + ks spec), spec = D G F / (4 cos cos);
     * pdf = (1 - p) cos / pi + p D |cos theta_h| / (4 wo.wh), p = ks / (kd + ks) */
    const float F = DielectricFunc(Dot(wi, Faceforward(wh, v3(0, 0, 1))), m.eta_a, m.eta_b);
    const float spec = Abs((D * DistG(d, wo, wi) * F) / (4 * cosI * cosO));
    const float s = m.kd / kPI + m.ks * spec;
    if (!(s > 0.0f)) return false;
    *out = m.ks * spec * dln / s;
    const float pl = m.ks / (m.kd + m.ks);
    const float gp = DistPdf(d, wh) / (4 * Dot(wo, wh));
    const float pdf = (1 - pl) * LambPdf(wo, wi) + pl * gp;
    if (pdf > 0.0f && gp > 0.0f) *outp = pl * gp * dlnD / pdf;
    return true;
}

DF bool UsesAlbedo(const RtSceneView* S, int albedo_tex, int mi) {
    if (albedo_tex < 0) return false;
    const RtMaterial& m = S->materials[mi];
    return (m.type == RT_MAT_DIFFUSE || m.type == RT_MAT_ROUGH_PLASTIC) && m.tex_r == albedo_tex;
}

/* adds v to the three floats at o with one atomic per distinct address per
 * warp: the lanes that reach this call together are grouped by address
 * (__match_any_sync), each group sums its values by shuffles in lane order
 * and its lowest lane adds the sums.  Lanes with o == nullptr only take part
 * in the exchange. */
DF void WarpAggregatedAdd3(float* o, C3 v) {
    const unsigned active = __activemask();
    const unsigned peers = __match_any_sync(active, (unsigned long long)o);
    const int lane = (int)(threadIdx.x & 31);
    float r = 0.0f, g = 0.0f, b = 0.0f;
    for (unsigned m = peers; m; m &= m - 1) {
        const int src = __ffs(m) - 1;
        r += __shfl_sync(peers, v.r, src);
        g += __shfl_sync(peers, v.g, src);
        b += __shfl_sync(peers, v.b, src);
    }
    if (o && lane == __ffs(peers) - 1) {
        if (r != 0.0f) atomicAdd(o + 0, r);
        if (g != 0.0f) atomicAdd(o + 1, g);
        if (b != 0.0f) atomicAdd(o + 2, b);
    }
}

/* credits g (rgb, per unit R) to the texel footprint of TexSample at uv; the
 * lanes of a warp that credit the same texel share one atomic per channel */
DF void ScatterAlbedo(const RtSceneView* S, int albedo_tex, float* grad_albedo, V2 uv, C3 g) {
    const RtTexture t = S->textures[albedo_tex];
    const float u = Wrapper(uv.x, t.wrap), v = Wrapper(uv.y, t.wrap);
    const float fu = u * (float)(t.width - 1), fv = v * (float)(t.height - 1);
    const int pu = nclampi(nf2i(fu), 0, t.width - 1), pv = nclampi(nf2i(fv), 0, t.height - 1);
    int xs[4] = {pu, pu, pu, pu}, ys[4] = {pv, pv, pv, pv};
    float ws[4] = {1.0f, 0.0f, 0.0f, 0.0f};
    if (t.filter == RT_FILTER_LINEAR) {
        const int dpu = (fu > (float)nf2i(fu) + 0.5f) ? 1 : -1;
        const int dpv = (fv > (float)nf2i(fv) + 0.5f) ? 1 : -1;
        const int apu = nclampi(nf2i(fu) + dpu, 0, t.width - 1), apv = nclampi(nf2i(fv) + dpv, 0, t.height - 1);
        const float du = nmin(Abs(fu - (float)nf2i(fu) - 0.5f), 1), dv = nmin(Abs(fv - (float)nf2i(fv) - 0.5f), 1);
        xs[1] = apu; ys[1] = pv; xs[2] = pu; ys[2] = apv; xs[3] = apu; ys[3] = apv;
        ws[0] = (1 - du) * (1 - dv); ws[1] = du * (1 - dv); ws[2] = (1 - du) * dv; ws[3] = du * dv;
    }
    for (int q = 0; q < 4; q++) {
        const bool any = ws[q] != 0.0f && (g.r != 0.0f || g.g != 0.0f || g.b != 0.0f);
        float* o = any ? grad_albedo + ((int64_t)xs[q] * t.height + ys[q]) * 3 : nullptr;
        WarpAggregatedAdd3(o, c3(g.r * ws[q], g.g * ws[q], g.b * ws[q]));
    }
}

DF float Dot3(C3 a, C3 b) { return a.r * b.r + a.g * b.g + a.b * b.b; }

/* d ln / d alpha of the two MIS-weighted direct terms: the BSDF value and the
 * power-heuristic weight, whose BSDF pdf moves with alpha (both terms are
 * differentiated: the environment light's sampler follows its texels, not
 * the pdf it reports, so the two weights do not cancel in expectation) */
DF float DirectDln(const RtSceneView* S, int mat, V3 wo, V3 w, float weight, bool light_term, V2 uv) {
    float rf, rp;
    if (!DlnAlpha(S, mat, wo, w, uv, &rf, &rp)) return 0.0f;
    if (weight > 1.0f) return rf;
    return light_term ? rf - 2.0f * (1.0f - weight) * rp : rf + 2.0f * (1.0f - weight) * rp;
}

}  /* namespace rtd */

#endif
