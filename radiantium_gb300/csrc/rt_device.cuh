/*
 * rt_device.cuh - device code of the GB300 path tracer: math, RNG, textures,
 * BVH traversal, BxDFs, lights, media and the scene services the integrators
 * call.
 *
 * Every expression keeps the operand order of the reference C# (cited per
 * function) and the file is compiled with --fmad=false, IEEE division and
 * square root, so a path computes the same bits as the reference's arithmetic
 * restated on the CPU.  Transcendentals come from rt_detmath.h.
 */
#ifndef RT_DEVICE_CUH
#define RT_DEVICE_CUH

#include <stdint.h>
#include "rt_types.h"
#include "../../include/radiantium.h"
#include "../../include/rt_detmath.h"

#define DF __device__ __forceinline__

namespace rtd {

constexpr float kPI = 3.14159265f;
constexpr float kEps = 1.401298464324817e-45f;   /* float.Epsilon */
constexpr float kFMax = 3.40282347e+38f;         /* float.MaxValue */

DF bool isnanf_(float x) { return x != x; }
DF bool isinff_(float x) { return (__float_as_uint(x) & 0x7fffffffu) == 0x7f800000u; }
DF bool isneg_(float x) { return (__float_as_uint(x) >> 31) != 0; }
/* System.Math.Max / Min (float), NaN-propagating, +0 > -0 */
DF float nmax(float a, float b) {
    if (a != b) { if (!isnanf_(a)) return b < a ? a : b; return a; }
    return isneg_(b) ? a : b;
}
DF float nmin(float a, float b) {
    if (a != b) { if (!isnanf_(a)) return a < b ? a : b; return a; }
    return isneg_(a) ? a : b;
}
DF float nclamp(float v, float lo, float hi) { if (v < lo) return lo; if (v > hi) return hi; return v; }
DF int nclampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
/* (int)float as the .NET x64 JIT converts: truncation, NaN / overflow -> int.MinValue */
DF int nf2i(float f) {
    if (isnanf_(f) || f >= 2147483648.0f || f < -2147483648.0f) return (int)0x80000000;
    return __float2int_rz(f);
}
DF float Sqrt(float x) { return __fsqrt_rn(x); }
DF float Abs(float x) { return fabsf(x); }
DF float Sqr(float v) { return v * v; }
DF float MulSign(float a1, float a2) { return a1 * rt_dm_copysign(1.0f, a2); }
DF float SafeSqrt(float a) { return Sqrt(nmax(a, 0.0f)); }

struct V2 { float x, y; };
struct V3 { float x, y, z; };
DF V2 v2(float x, float y) { V2 r; r.x = x; r.y = y; return r; }
DF V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
DF V3 v3s(float s) { return v3(s, s, s); }
DF V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
DF V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
DF V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
DF V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
DF V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
DF V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
DF V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
DF V2 operator+(V2 a, V2 b) { return v2(a.x + b.x, a.y + b.y); }
DF V2 operator*(float s, V2 a) { return v2(s * a.x, s * a.y); }
DF float Dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DF float AbsDot(V3 a, V3 b) { return Abs(Dot(a, b)); }
DF V3 Cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
DF float LengthSq(V3 a) { return Dot(a, a); }
DF float Length(V3 a) { return Sqrt(LengthSq(a)); }
DF V3 Normalize(V3 a) { float l = Length(a); return a / l; }
DF float Distance(V3 a, V3 b) { return Length(a - b); }
DF V3 Reflect(V3 v, V3 n) { float d = Dot(v, n); return v - ((2.0f * d) * n); }
DF float Get(V3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
DF V3 f4xyz(float4 f) { return v3(f.x, f.y, f.z); }

/* Matrix rows: m[0..2] row 1, m[3..5] row 2, m[6..8] row 3, m[9..11] translation */
DF V3 Xf12(V3 p, const float* m) {
    return v3(p.x * m[0] + p.y * m[3] + p.z * m[6] + m[9],
              p.x * m[1] + p.y * m[4] + p.z * m[7] + m[10],
              p.x * m[2] + p.y * m[5] + p.z * m[8] + m[11]);
}
DF V3 XfN12(V3 v, const float* m) {
    return v3(v.x * m[0] + v.y * m[3] + v.z * m[6],
              v.x * m[1] + v.y * m[4] + v.z * m[7],
              v.x * m[2] + v.y * m[5] + v.z * m[8]);
}
/* full Matrix4x4 (16 floats, M11..M44) used by the camera */
DF V3 Xf16(V3 p, const float* m) {
    return v3(p.x * m[0] + p.y * m[4] + p.z * m[8] + m[12],
              p.x * m[1] + p.y * m[5] + p.z * m[9] + m[13],
              p.x * m[2] + p.y * m[6] + p.z * m[10] + m[14]);
}
DF V3 XfN16(V3 v, const float* m) {
    return v3(v.x * m[0] + v.y * m[4] + v.z * m[8],
              v.x * m[1] + v.y * m[5] + v.z * m[9],
              v.x * m[2] + v.y * m[6] + v.z * m[10]);
}

struct C3 { float r, g, b; };
DF C3 c3(float r, float g, float b) { C3 c; c.r = r; c.g = g; c.b = b; return c; }
DF C3 c3s(float v) { return c3(v, v, v); }
DF C3 operator+(C3 a, C3 b) { return c3(a.r + b.r, a.g + b.g, a.b + b.b); }
DF C3 operator-(C3 a, C3 b) { return c3(a.r - b.r, a.g - b.g, a.b - b.b); }
DF C3 operator*(C3 a, C3 b) { return c3(a.r * b.r, a.g * b.g, a.b * b.b); }
DF C3 operator/(C3 a, C3 b) { return c3(a.r / b.r, a.g / b.g, a.b / b.b); }
DF C3 operator+(C3 a, float s) { return c3(a.r + s, a.g + s, a.b + s); }
DF C3 operator-(C3 a, float s) { return c3(a.r - s, a.g - s, a.b - s); }
DF C3 operator*(C3 a, float s) { return c3(a.r * s, a.g * s, a.b * s); }
DF C3 operator/(C3 a, float s) { return c3(a.r / s, a.g / s, a.b / s); }
DF C3 operator*(float s, C3 a) { return c3(s * a.r, s * a.g, s * a.b); }
DF C3 operator-(float s, C3 a) { return c3(s - a.r, s - a.g, s - a.b); }
DF bool IsBlack(C3 a) { return a.r == 0.0f && a.g == 0.0f && a.b == 0.0f; }
DF bool Same(C3 a, C3 b) { return a.r == b.r && a.g == b.g && a.b == b.b; }
DF bool IsValid(C3 c) {
    if (c.r < 0 || isinff_(c.r) || isnanf_(c.r)) return false;
    if (c.g < 0 || isinff_(c.g) || isnanf_(c.g)) return false;
    if (c.b < 0 || isinff_(c.b) || isnanf_(c.b)) return false;
    return true;
}
DF C3 CAbs(C3 c) { return c3(Abs(c.r), Abs(c.g), Abs(c.b)); }
DF float MaxElement(C3 c) { return nmax(nmax(c.r, c.g), c.b); }
DF float Luminance(C3 c) { return c.r * 0.212671f + c.g * 0.715160f + c.b * 0.072169f; }
DF float CGet(C3 c, int i) { return i == 0 ? c.r : (i == 1 ? c.g : c.b); }

/* Ray3F (Radiantium.Core/Ray3F.cs) */
struct Ray { V3 O, D; float MinT, MaxT; V3 InvD; };
DF Ray mkray(V3 o, V3 d, float minT = kEps, float maxT = kFMax) {
    Ray r; r.O = o; r.D = d; r.MinT = minT; r.MaxT = maxT;
    r.InvD = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    return r;
}
DF V3 At(const Ray& r, float t) { return r.O + t * r.D; }
/* Ray3F.Transform */
DF Ray XfRay(const Ray& ray, const float* m) {
    V3 o = Xf12(ray.O, m);
    V3 d = Normalize(XfN12(ray.D, m));
    V3 mx = Xf12(At(ray, ray.MaxT), m);
    float maxT = Distance(o, mx);
    return mkray(o, d, ray.MinT, maxT);
}

/* Coordinate (Coordinate.cs:14-34, Duff et al. 2017) */
struct Frame { V3 X, Y, Z; };
DF Frame mkframe(V3 n) {
    float sign = rt_dm_copysign(1.0f, n.z);
    float a = -1 / (sign + n.z);
    float b = n.x * n.y * a;
    Frame f;
    f.X = v3(MulSign(Sqr(n.x) * a, n.z) + 1.0f, MulSign(b, n.z), MulSign(n.x, -n.z));
    f.Y = v3(b, sign + Sqr(n.y) * a, -n.y);
    f.Z = n;
    return f;
}
DF V3 ToLocal(const Frame& f, V3 v) { return v3(Dot(v, f.X), Dot(v, f.Y), Dot(v, f.Z)); }
DF V3 ToWorld(const Frame& f, V3 v) { return f.X * v.x + f.Y * v.y + f.Z * v.z; }
DF float CosTheta(V3 v) { return v.z; }
DF float AbsCosTheta(V3 v) { return Abs(v.z); }
DF float Cos2Theta(V3 v) { return Sqr(v.z); }
DF float Sin2Theta(V3 v) { return v.x * v.x + Sqr(v.y); }
DF float TanTheta(V3 v) { return SafeSqrt(-v.z * v.z + 1.0f) / v.z; }
DF float Tan2Theta(V3 v) { return nmax(-v.z * v.z + 1.0f, 0.0f) / Sqr(v.z); }
DF float Cos2Phi(V3 v) { float s2 = Sin2Theta(v); return Abs(s2) <= 4.0f * kEps ? 1.0f : nclamp(Sqr(v.x) / s2, -1.0f, 1.0f); }
DF float Sin2Phi(V3 v) { float s2 = Sin2Theta(v); return Abs(s2) <= 4.0f * kEps ? 0.0f : nclamp(Sqr(v.y) / s2, -1.0f, 1.0f); }
DF bool SameHemisphere(V3 a, V3 b) { return a.z * b.z > 0; }
DF V3 Faceforward(V3 v, V3 w) { return (Dot(v, w) < 0.0f) ? -v : v; }
/* MathExt.Refract */
DF bool Refract(V3 wi, V3 n, float eta, V3* wt) {
    float cosThetaI = Dot(n, wi);
    float sin2ThetaI = nmax(0, 1 - cosThetaI * cosThetaI);
    float sin2ThetaT = eta * eta * sin2ThetaI;
    if (sin2ThetaT >= 1) { *wt = v3s(0); return false; }
    float cosThetaT = Sqrt(1 - sin2ThetaT);
    *wt = Normalize(eta * -wi + (eta * cosThetaI - cosThetaT) * n);
    return true;
}
DF V3 SphDir(float sinTheta, float cosTheta, float phi) {
    float sinPhi = rt_sinf(phi), cosPhi = rt_cosf(phi);
    return v3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
}

/* ---- Philox4x32-10 stream (stands in for System.Random) ------------------- */
struct Rng {
    uint32_t k0, k1, c0, c1, c2, n;
    uint32_t buf[4];
};
DF void philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t* out) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
DF void rng_init(Rng& r, uint64_t seed, uint32_t x, uint32_t y, uint32_t s) {
    r.k0 = (uint32_t)seed; r.k1 = (uint32_t)(seed >> 32); r.c0 = x; r.c1 = y; r.c2 = s; r.n = 0;
}
DF uint32_t next_u32(Rng& r) {
    if ((r.n & 3u) == 0) philox(r.c0, r.c1, r.c2, r.n >> 2, r.k0, r.k1, r.buf);
    uint32_t v;
    switch (r.n & 3u) { case 0: v = r.buf[0]; break; case 1: v = r.buf[1]; break; case 2: v = r.buf[2]; break; default: v = r.buf[3]; }
    r.n++;
    return v;
}
DF float NextFloat(Rng& r) { return (float)(next_u32(r) >> 8) * (1.0f / 16777216.0f); }
DF int NextInt(Rng& r, int n) { return (int)(((uint64_t)next_u32(r) * (uint64_t)(uint32_t)n) >> 32); }
DF V2 NextVec2(Rng& r) { float a = NextFloat(r); float b = NextFloat(r); return v2(a, b); }

/* Probability.cs warps */
DF V3 SquareToCosineHemisphere(V2 s) {
    float radius = Sqrt(s.x);
    float angle = s.y * kPI * 2;
    float x = radius * rt_cosf(angle), y = radius * rt_sinf(angle);
    return v3(x, y, Sqrt(1 - x * x - y * y));
}
DF V3 SquareToUniformSphere(V2 s) {
    float phi = s.x * kPI * 2;
    float theta = rt_acosf(1 - 2 * s.y);
    float sinTheta = rt_sinf(theta), cosTheta = rt_cosf(theta);
    float sinPhi = rt_sinf(phi), cosPhi = rt_cosf(phi);
    return v3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
}
/* PathUtility.PowerHeuristic (double) */
DF float PowerHeuristic(float fPdf, float gPdf) {
    double f = (double)(1.0f * fPdf), g = (double)(1.0f * gPdf);
    return (float)((f * f) / (f * f + g * g));
}

/* ---- textures (TextureSampler.cs:28-72) ------------------------------------ */
DF C3 TexRead(const RtSceneView* S, const RtTexture& t, int x, int y) {
    x = nclampi(x, 0, t.width - 1); y = nclampi(y, 0, t.height - 1);
    const float* p = S->texels + t.offset + ((int64_t)x * t.height + y) * 3;
    return c3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}
DF float Wrapper(float a, int mode) {
    if (mode == RT_WRAP_CLAMP) return nclamp(a, 0, 1);
    return nclamp(a - floorf(a), 0, 1);
}
DF C3 TexSample(const RtSceneView* S, int ti, V2 uv) {
    const RtTexture t = S->textures[ti];
    float u = Wrapper(uv.x, t.wrap), v = Wrapper(uv.y, t.wrap);
    float fu = u * (float)(t.width - 1);
    float fv = v * (float)(t.height - 1);
    int pu = nf2i(fu), pv = nf2i(fv);
    if (t.filter == RT_FILTER_LINEAR) {
        int dpu = (fu > (float)pu + 0.5f) ? 1 : -1;
        int dpv = (fv > (float)pv + 0.5f) ? 1 : -1;
        int apu = nclampi(pu + dpu, 0, t.width - 1);
        int apv = nclampi(pv + dpv, 0, t.height - 1);
        float du = nmin(Abs(fu - (float)pu - 0.5f), 1);
        float dv = nmin(Abs(fv - (float)pv - 0.5f), 1);
        C3 a = TexRead(S, t, pu, pv), b = TexRead(S, t, apu, pv), c = TexRead(S, t, pu, apv), d = TexRead(S, t, apu, apv);
        return (a * (1 - du) + b * du) * (1 - dv) + (c * (1 - du) + d * du) * dv;
    }
    return TexRead(S, t, pu, pv);
}

/* ---- shapes ----------------------------------------------------------------- */
struct SurfPt { float u, v, t; };
/* Moller-Trumbore exactly as Triangle.Intersect (Shapes/Triangle.cs:149-177) */
DF bool TriTest(V3 pa, V3 e1, V3 e2, const Ray& ray, SurfPt* sp) {
    V3 pvec = Cross(ray.D, e2);
    float det = Dot(e1, pvec);
    if (Abs(det) < kEps) return false;
    float invDet = 1.0f / det;
    V3 tvec = ray.O - pa;
    float u = Dot(tvec, pvec) * invDet;
    if (u < 0.0f || u > 1.0f) return false;
    V3 qvec = Cross(tvec, e1);
    float v = Dot(ray.D, qvec) * invDet;
    if (v < 0.0f || u + v > 1.0f) return false;
    float t = Dot(e2, qvec) * invDet;
    if (!(t >= ray.MinT && t <= ray.MaxT)) return false;
    sp->u = u; sp->v = v; sp->t = t;
    return true;
}
DF double dmin_(double a, double b) { if (a != b) { if (a == a) return a < b ? a : b; return a; } return signbit(a) ? a : b; }
DF double dmax_(double a, double b) { if (a != b) { if (a == a) return b < a ? a : b; return a; } return signbit(b) ? a : b; }
/* Sphere.Intersect (Shapes/Sphere.cs:65-80) with MathExt.SolveQuadratic in double */
DF bool SphereTest(V3 c, float radius, const Ray& ray, float* tOut) {
    double ox = (double)ray.O.x - (double)c.x, oy = (double)ray.O.y - (double)c.y, oz = (double)ray.O.z - (double)c.z;
    double dx = ray.D.x, dy = ray.D.y, dz = ray.D.z;
    double a = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    double b = __dmul_rn(2.0, __dadd_rn(__dadd_rn(__dmul_rn(ox, dx), __dmul_rn(oy, dy)), __dmul_rn(oz, dz)));
    double cc = __dsub_rn(__dadd_rn(__dadd_rn(__dmul_rn(ox, ox), __dmul_rn(oy, oy)), __dmul_rn(oz, oz)), (double)Sqr(radius));
    bool linearCase = a == 0.0;
    bool validLinear = linearCase && b != 0.0;
    double x0 = __ddiv_rn(-cc, b), x1 = x0;
    double discrim = __dsub_rn(__dmul_rn(b, b), __dmul_rn(__dmul_rn(4.0, a), cc));
    bool validQuadratic = !linearCase && (discrim >= 0.0);
    if (validQuadratic) {
        double root = __dsqrt_rn(discrim);
        double temp = __dmul_rn(-0.5, __dadd_rn(b, copysign(root, b)));
        double x0p = __ddiv_rn(temp, a), x1p = __ddiv_rn(cc, temp);
        double x0m = dmin_(x0p, x1p), x1m = dmax_(x0p, x1p);
        x0 = x0m; x1 = x1m;
    }
    bool found = validLinear || validQuadratic;
    double mint = ray.MinT, maxt = ray.MaxT;
    bool outB = !(x0 <= maxt && x1 >= mint);
    bool inB = x0 < mint && x1 > maxt;
    *tOut = x0 < mint ? (float)x1 : (float)x0;
    return found && !outB && !inB;
}

/* triangle attributes at barycentrics (Triangle.GetIntersection / Sample) */
DF void TriAttrs(const RtSceneView* S, int tri, V3 bary, V3* p, V3* n, V2* uv) {
    RtTri t = S->tris[tri];
    V3 pa = f4xyz(S->pos[t.v0]), pb = f4xyz(S->pos[t.v1]), pc = f4xyz(S->pos[t.v2]);
    *p = bary.x * pa + bary.y * pb + bary.z * pc;
    if (t.flags & 1) *n = Normalize(bary.x * f4xyz(S->nrm[t.v0]) + bary.y * f4xyz(S->nrm[t.v1]) + bary.z * f4xyz(S->nrm[t.v2]));
    else *n = Normalize(Cross(pb - pa, pc - pa));
    if (t.flags & 2) {
        float2 a = S->uv[t.v0], b = S->uv[t.v1], c = S->uv[t.v2];
        *uv = bary.x * v2(a.x, a.y) + bary.y * v2(b.x, b.y) + bary.z * v2(c.x, c.y);
    } else {
        *uv = bary.x * v2(0, 0) + bary.y * v2(1, 0) + bary.z * v2(1, 1);
    }
}
DF V2 SphereUV(const RtSphere& s, V3 n) {
    V3 local = XfN12(n, s.w2m);
    float theta = rt_acosf(-local.y);
    float phi = rt_atan2f(-local.z, local.x) + kPI;
    return v2(phi / (2 * kPI), theta / kPI);
}

/* ---- Intersection (Intersection.cs) ------------------------------------------- */
struct Isect {
    V3 P; V2 UV; float T; Frame F; V3 Wr;
    int prim;       /* top-level primitive id */
    int sub;        /* instanced prototype primitive id or -1 */
    int slot;       /* winning slot (absolute), for parity reporting */
    float bu, bv;
    uint32_t flags;
};

/* ---- BVH traversal ------------------------------------------------------------ */
struct TravStats { uint32_t nodes, prims, insts; };

struct Trav {
    const RtSceneView* S;
    uint32_t* status;
    TravStats* st;
    int2* stack;   /* 2 x RT_STACK_SIZE entries: top level, then instanced prototype */
};

/* Slab test (BoundingBox3F.cs:155-176) split into the part that does not
 * depend on MaxT (returns false) and tMin; the caller compares tMin < MaxT.
 * Gamma(3) is computed from float.Epsilon, a denormal, so 1 + 2*Gamma(3) == 1. */
DF bool SlabA(float mnx, float mny, float mnz, float mxx, float mxy, float mxz, const Ray& r, float* tminOut) {
    bool nx = r.InvD.x < 0, ny = r.InvD.y < 0, nz = r.InvD.z < 0;
    float tMin = ((nx ? mxx : mnx) - r.O.x) * r.InvD.x;
    float tMax = ((nx ? mnx : mxx) - r.O.x) * r.InvD.x;
    float tyMin = ((ny ? mxy : mny) - r.O.y) * r.InvD.y;
    float tyMax = ((ny ? mny : mxy) - r.O.y) * r.InvD.y;
    if (tMin > tyMax || tyMin > tMax) return false;
    if (tyMin > tMin) tMin = tyMin;
    if (tyMax < tMax) tMax = tyMax;
    float tzMin = ((nz ? mxz : mnz) - r.O.z) * r.InvD.z;
    float tzMax = ((nz ? mnz : mxz) - r.O.z) * r.InvD.z;
    if (tMin > tzMax || tzMin > tMax) return false;
    if (tzMin > tMin) tMin = tzMin;
    if (tzMax < tMax) tMax = tzMax;
    *tminOut = tMin;
    return tMax > 0;
}

/* closest-hit result inside one BVH */
struct Best {
    float t; float u, v; int slot; uint32_t flags;
    int sub;         /* for instance candidates: winning prototype slot */
    V3 pw;           /* for instance candidates: world-space point */
};

#ifndef RT_TRAVERSAL_CAP
#define RT_TRAVERSAL_CAP (1u << 26)   /* loop steps of one two-level traversal */
#endif
#ifndef RT_DESCEND
/* interior nodes one traversal step may visit in shallow trees (Cornell box / light tracer,
 * M samples / particles per s: 415 / 223 at 2, 421 / 229 at 3, 426 / 227 at 4, 418 / 224 at 5) */
#define RT_DESCEND 3
#endif
#define RT_NO_NODE ((int)0x80000000)

/* Leaf primitive of either level against ray r: triangle or sphere (the
 * instance case is handled by the callers).  Bvh.Intersect's leaf loop
 * (Accelerators/Bvh.cs:193-204, 140-152). */
DF bool PrimHit(const RtSceneView* S, uint32_t kind, uint32_t ref, float4 s0, float4 s1, float4 s2, const Ray& r,
                float* t, float* u, float* v) {
    if (kind == RT_KIND_TRI) {
        SurfPt sp;
        if (!TriTest(f4xyz(s0), f4xyz(s1), f4xyz(s2), r, &sp)) return false;
        *t = sp.t; *u = sp.u; *v = sp.v;
        return true;
    }
    RtSphere sph = S->spheres[ref];
    *u = 0; *v = 0;
    return SphereTest(v3(sph.center[0], sph.center[1], sph.center[2]), sph.radius, r, t);
}

/* Root box of tree `bvh`: RT_NO_NODE if the tree is empty or the box is
 * missed, else the root's reference (counts one node visit if non-empty);
 * kWide: the root of the tree's wide form. */
template <bool kWide = false>
DF int RootRef(const RtSceneView* S, int bvh, const Ray& r, TravStats* st) {
    const RtBvh h = S->bvhs[bvh];
    if (h.root_ref == RT_NO_NODE) return RT_NO_NODE;
    if (st) st->nodes++;
    float tmin;
    if (!SlabA(h.root_min[0], h.root_min[1], h.root_min[2], h.root_max[0], h.root_max[1], h.root_max[2], r, &tmin) ||
        !(tmin < r.MaxT))
        return RT_NO_NODE;
    return kWide ? h.wide_root : h.root_ref;
}

/* Traversal stack storage: a thread-local array, or (SplitStack) the first
 * RT_SH_STACK entries in shared memory - one column of a block-wide array per
 * thread, so a warp's accesses fall in distinct banks - and the rest in the
 * thread's local array.  Both levels share one index range (the prototype's
 * entries start where the top level's end), so the shared entries hold the
 * bottom of the combined stack. */
#ifndef RT_SH_STACK
#define RT_SH_STACK 16
#endif
#define RT_TRACE_BLOCK 128            /* threads per block of the kernels that use SplitStack */
struct SplitStack {
    int2* sh;                         /* &block_array[threadIdx.x]; entry i at sh[i * RT_TRACE_BLOCK] */
    int2* loc;                        /* 2 * RT_STACK_SIZE entries */
};
DF int2 stk_get(int2* s, int i) { return s[i]; }
DF void stk_put(int2* s, int i, int2 v) { s[i] = v; }
DF int2 stk_get(const SplitStack& s, int i) { return i < RT_SH_STACK ? s.sh[i * RT_TRACE_BLOCK] : s.loc[i]; }
DF void stk_put(const SplitStack& s, int i, int2 v) {
    if (i < RT_SH_STACK) s.sh[i * RT_TRACE_BLOCK] = v;
    else s.loc[i] = v;
}

/* One interior node: both child boxes are read from the parent, the far child
 * is pushed with its entry distance and re-checked against the MaxT current
 * when it is popped, which is exactly when the reference tests it.  A far
 * child whose slab test already failed is pushed by the reference only to be
 * rejected when popped (NaN < MaxT is false), so it is not stored at all -
 * except while counting node visits (an any-hit traversal that stops early
 * never pops, nor counts, what is left on its stack) and for trees tall
 * enough to overflow the stack.  Returns the near child to descend into, or
 * RT_NO_NODE. */
template <class Stk>
DF int VisitNode(const RtSceneView* S, int node, const Ray& r, Stk stack, int* sp, TravStats* st) {
    const float4* np = S->nodes + 4 * (int64_t)node;
    const float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3);
    const int lref = __float_as_int(n3.x), rref = __float_as_int(n3.y), axis = __float_as_int(n3.z);
    float tl, tr;
    const bool al = SlabA(n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, r, &tl);
    const bool ar = SlabA(n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, r, &tr);
    const float ia = axis == 0 ? r.InvD.x : (axis == 1 ? r.InvD.y : r.InvD.z);
    const bool rightFirst = ia < 0;
    const int nearRef = rightFirst ? rref : lref, farRef = rightFirst ? lref : rref;
    const bool nearA = rightFirst ? ar : al, farA = rightFirst ? al : ar;
    const float nearT = rightFirst ? tr : tl, farT = rightFirst ? tl : tr;
    if (farA || st || S->deep_trees)
        stk_put(stack, (*sp)++, make_int2(farRef, __float_as_int(farA ? farT : __int_as_float(0x7fc00000))));
    return (nearA && nearT < r.MaxT) ? nearRef : RT_NO_NODE;
}

/* two candidate distances within 4 ulp of each other: the fast traversal
 * reports these as ties too (its conservative boxes can meet a candidate
 * the reference's rounding-scale box test culled) */
DF bool NearTie(float a, float b) {
    const int d = __float_as_int(a) - __float_as_int(b);
    return a >= 0.0f && b >= 0.0f && d >= -4 && d <= 4;
}

/* ---- the opt-in fast traversal: 8-wide nodes with quantised child boxes ----------------------
 * One node holds up to eight children of the reference's tree (rtb::build_wide)
 * with boxes quantised outwards on a per-node grid, read with six 16-byte
 * loads.  The plane distances t = q * (s / d) + (p - o) / d are one fused
 * multiply-add each - the only place the fast mode contracts - and every
 * interval is widened by 2^-20 of its ends, so a child box is never missed
 * where its exact box is hit: the fast traversal visits a superset of the
 * boxes the reference's slab test accepts and finds every primitive hit the
 * reference finds.  Hit children are ordered near to far by a sorting network
 * over 32-bit keys (entry distance with its low three bits replaced by the
 * child's index, which rounds the distance down); the nearest is descended
 * into and the others are pushed far-first with the rounded-down distance,
 * which PopNext checks against MaxT.  Primitive tests, instance entry and
 * exit and the closest-hit rule are the exact traversal's; only the order in
 * which equal-t candidates are met can differ.  Such ties are flagged
 * RT_HIT_TIE as in the exact traversal, and so are candidates within 4 ulp
 * of the best one (coplanar surfaces a ulp apart, of which the reference's
 * box test culls the second at rounding scale). */
/* byte k of `word` as a float: the byte placed in the mantissa of 2^23, minus 2^23 (exact) */
DF float wq(uint32_t word, int k) {
    return __uint_as_float(__byte_perm(word, 0x4B000000u, 0x7650u | (uint32_t)k)) - 8388608.0f;
}
DF void ucas(uint32_t& a, uint32_t& b) { const uint32_t lo = umin(a, b), hi = umax(a, b); a = lo; b = hi; }

template <class Stk>
DF int VisitWideNode(const RtSceneView* S, int node, const Ray& r, Stk stack, int* sp) {
    const float4* np = S->wnodes + RT_WIDE_F4 * (int64_t)node;
    const float4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3);
    const int4 ra = __ldg(reinterpret_cast<const int4*>(np + 4)), rb = __ldg(reinterpret_cast<const int4*>(np + 5));
    const uint32_t meta = __float_as_uint(w0.w);
    const float kWiden = 9.5367431640625e-07f;   /* 2^-20 */
    uint32_t key[8];
    /* 1/d clamped to +-2^95.  The split form q (s/d) + (p - o)/d needs both
     * terms finite: for a direction component of zero (or so small that 1/d
     * times a grid step or node origin overflows) it would add infinities of
     * opposite sign, and fmaxf / fminf would drop the NaN - every box would
     * count as unbounded along that axis and the traversal would visit most
     * of the tree.  Clamped, the plane distances of such an axis are 0 or
     * +-huge with the sign of (plane - origin), so the test keeps exactly the
     * boxes whose quantised slab contains the origin's coordinate.  A
     * quantised box contains its exact box with a grid step to spare, so an
     * origin on a quantised plane lies outside the exact box, where the
     * reference's slab test (which ignores only NaN bounds) rejects it too:
     * the test still accepts a superset of the reference's boxes. */
    const float kClamp = 3.9614081257132169e28f;   /* 2^95 */
    const float ix = fminf(fmaxf(r.InvD.x, -kClamp), kClamp);
    const float iy = fminf(fmaxf(r.InvD.y, -kClamp), kClamp);
    const float iz = fminf(fmaxf(r.InvD.z, -kClamp), kClamp);
    const float ax = __uint_as_float((meta & 0xffu) << 23) * ix;
    const float ay = __uint_as_float(((meta >> 8) & 0xffu) << 23) * iy;
    const float az = __uint_as_float(((meta >> 16) & 0xffu) << 23) * iz;
    const float bx = (w0.x - r.O.x) * ix, by = (w0.y - r.O.y) * iy, bz = (w0.z - r.O.z) * iz;
    /* near and far planes per axis by the direction's sign: words of children 0-3 and 4-7 */
    const bool fx = r.InvD.x < 0, fy = r.InvD.y < 0, fz = r.InvD.z < 0;
    const uint32_t nx0 = __float_as_uint(fx ? w1.z : w1.x), nx1 = __float_as_uint(fx ? w1.w : w1.y);
    const uint32_t gx0 = __float_as_uint(fx ? w1.x : w1.z), gx1 = __float_as_uint(fx ? w1.y : w1.w);
    const uint32_t ny0 = __float_as_uint(fy ? w2.z : w2.x), ny1 = __float_as_uint(fy ? w2.w : w2.y);
    const uint32_t gy0 = __float_as_uint(fy ? w2.x : w2.z), gy1 = __float_as_uint(fy ? w2.y : w2.w);
    const uint32_t nz0 = __float_as_uint(fz ? w3.z : w3.x), nz1 = __float_as_uint(fz ? w3.w : w3.y);
    const uint32_t gz0 = __float_as_uint(fz ? w3.x : w3.z), gz1 = __float_as_uint(fz ? w3.y : w3.w);
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int b = k & 3;
        const float tx0 = __fmaf_rn(wq(k < 4 ? nx0 : nx1, b), ax, bx), tx1 = __fmaf_rn(wq(k < 4 ? gx0 : gx1, b), ax, bx);
        const float ty0 = __fmaf_rn(wq(k < 4 ? ny0 : ny1, b), ay, by), ty1 = __fmaf_rn(wq(k < 4 ? gy0 : gy1, b), ay, by);
        const float tz0 = __fmaf_rn(wq(k < 4 ? nz0 : nz1, b), az, bz), tz1 = __fmaf_rn(wq(k < 4 ? gz0 : gz1, b), az, bz);
        float tlo = fmaxf(fmaxf(tx0, ty0), tz0), thi = fminf(fminf(tx1, ty1), tz1);
        tlo = __fmaf_rn(-fabsf(tlo), kWiden, tlo);
        thi = __fmaf_rn(fabsf(thi), kWiden, thi);
        const bool hit = k < (int)(meta >> 24) && tlo <= thi && thi >= 0.0f && tlo <= r.MaxT;
        const float te = tlo > 0.0f ? tlo : 0.0f;
        key[k] = hit ? ((__float_as_uint(te) & ~7u) | (uint32_t)k) : 0xffffffffu;
    }
    /* Batcher's odd-even merge sort of eight keys (19 compare-exchanges) */
    ucas(key[0], key[1]); ucas(key[2], key[3]); ucas(key[4], key[5]); ucas(key[6], key[7]);
    ucas(key[0], key[2]); ucas(key[1], key[3]); ucas(key[4], key[6]); ucas(key[5], key[7]);
    ucas(key[1], key[2]); ucas(key[5], key[6]);
    ucas(key[0], key[4]); ucas(key[1], key[5]); ucas(key[2], key[6]); ucas(key[3], key[7]);
    ucas(key[2], key[4]); ucas(key[3], key[5]);
    ucas(key[1], key[2]); ucas(key[3], key[4]); ucas(key[5], key[6]);
    if (key[0] == 0xffffffffu) return RT_NO_NODE;
#pragma unroll
    for (int j = 7; j >= 1; j--) {
        if (key[j] != 0xffffffffu) {
            const uint32_t c = key[j] & 7u;
            const int4 q = (c & 4u) ? rb : ra;
            const int ref = (c & 2u) ? ((c & 1u) ? q.w : q.z) : ((c & 1u) ? q.y : q.x);
            stk_put(stack, (*sp)++, make_int2(ref, (int)(key[j] & ~7u)));
        }
    }
    const uint32_t c = key[0] & 7u;
    const int4 q = (c & 4u) ? rb : ra;
    return (c & 2u) ? ((c & 1u) ? q.w : q.z) : ((c & 1u) ? q.y : q.x);
}

/* Pops until an entry passes the MaxT check (Bvh.cs:205-229 / 153-169). */
template <class Stk>
DF int PopNext(Stk stack, int* sp, int base, float maxT, TravStats* st) {
    while (*sp > base) {
        const int2 e = stk_get(stack, --*sp);
        if (st) st->nodes++;
        if (__int_as_float(e.y) < maxT) return e.x;
    }
    return RT_NO_NODE;
}

/* Leaf references become a primitive cursor (count in the first slot). */
DF void EnterLeaf(const RtSceneView* S, int* cur, int* leafSlot, int* leafLeft) {
    if (*cur != RT_NO_NODE && *cur < 0) {
        *leafSlot = ~*cur;
        *leafLeft = __float_as_int(__ldg(S->slots + 3 * (int64_t)*leafSlot + 2).w);
        *cur = RT_NO_NODE;
    }
}

/* Scene.Intersect(ray, out inct) over the two-level scene: Bvh.Intersect
 * (Accelerators/Bvh.cs:174-232) on the top-level tree and, for each instance
 * leaf, InstancedPrimitive.Intersect (Primitive.cs:169-188) on its prototype
 * tree in model space with world T = Distance(ray.O, p).  Boxes, MaxT culls
 * and primitive tests happen in exactly the order of the recursive form; the
 * recursion is unrolled into a state machine: a step visits up to kDescend
 * interior nodes (with the pops that follow them) and then, if that reached a
 * leaf, tests its next primitive, or leaves a prototype.  A lane that has just
 * reached a leaf tests it together with the lanes already in leaves, and rays
 * at different levels run the same step code together; a persistent kernel
 * can hand a lane a new ray between any two steps.  stack[0, base) holds
 * top-level entries, stack[base, base + RT_STACK_SIZE) the prototype's, so
 * `stack` has 2 * RT_STACK_SIZE entries. */
struct TravClosest {
    Ray r;                       /* world ray, or the model-space ray inside a prototype */
    V3 wO, wD;                   /* the world ray */
    float wMaxT;                 /* the world ray's MaxT while a prototype is traversed */
    Best best;
    float pt, pu, pv; int pslot; uint32_t pflags;     /* the prototype's own closest hit */
    int cur, sp, base, leafSlot, leafLeft, topSlot, topLeft, inst;
    bool any, inProto, pany;
    uint32_t guard;
};

/* Returns true when the traversal is already over (empty scene or root box missed). */
template <bool kWide = false>
DF bool ClosestBegin(const RtSceneView* S, const Ray& ray, TravClosest& T, TravStats* st) {
    Best& b = T.best;
    b.t = kFMax; b.flags = 0; b.slot = -1; b.sub = -1; b.u = 0; b.v = 0; b.pw = v3s(0);
    T.r = ray; T.wO = ray.O; T.wD = ray.D; T.wMaxT = ray.MaxT;
    T.any = false; T.inProto = false; T.pany = false;
    T.base = 0; T.sp = 0; T.leafLeft = 0; T.leafSlot = 0; T.topSlot = 0; T.topLeft = 0; T.inst = 0;
    T.pt = kFMax; T.pu = 0; T.pv = 0; T.pslot = -1; T.pflags = 0;
    T.guard = 0;
    T.cur = RootRef<kWide>(S, 0, ray, st);
    if (T.cur == RT_NO_NODE) return true;
    EnterLeaf(S, &T.cur, &T.leafSlot, &T.leafLeft);
    return false;
}

/* One step; true when the traversal has finished.  kWide: the fast traversal's
 * wide nodes (a visit may push up to seven entries). */
template <class Stk, int kDescend = RT_DESCEND, bool kWide = false>
DF bool ClosestStep(const RtSceneView* S, TravClosest& T, Stk stack, uint32_t* status, TravStats* st) {
    if (++T.guard > RT_TRAVERSAL_CAP) { atomicOr(status, RT_STATUS_TRAV); return true; }
    if (T.cur != RT_NO_NODE) {
        /* up to kDescend interior nodes (with the pops that follow them) per step */
        for (int k = 0; k < kDescend && T.cur >= 0; k++) {
            if (kWide ? T.sp - T.base > RT_STACK_SIZE - 8 : T.sp - T.base == RT_STACK_SIZE) {
                atomicOr(status, RT_STATUS_STACK);
                if (!T.inProto) return true;
                T.sp = T.base;                  /* the prototype's traversal stops here */
                T.cur = RT_NO_NODE;
                return false;
            }
            if (st) st->nodes++;
            T.cur = kWide ? VisitWideNode(S, T.cur, T.r, stack, &T.sp) : VisitNode(S, T.cur, T.r, stack, &T.sp, st);
            if (T.cur == RT_NO_NODE) T.cur = PopNext(stack, &T.sp, T.base, T.r.MaxT, st);
        }
        EnterLeaf(S, &T.cur, &T.leafSlot, &T.leafLeft);
        if (T.cur != RT_NO_NODE) return false;      /* still descending: the next step goes on */
    }
    if (T.leafLeft > 0) {
        const int slot = T.leafSlot++;
        T.leafLeft--;
        const float4 s0 = __ldg(S->slots + 3 * (int64_t)slot);
        const float4 s1 = __ldg(S->slots + 3 * (int64_t)slot + 1);
        const float4 s2 = __ldg(S->slots + 3 * (int64_t)slot + 2);
        const uint32_t kr = __float_as_uint(s1.w);
        const uint32_t kind = kr >> RT_KIND_SHIFT, ref = kr & RT_REF_MASK;
        if (st) st->prims++;
        if (kind != RT_KIND_INSTANCE) {
            float t, u, v;
            if (!PrimHit(S, kind, ref, s0, s1, s2, T.r, &t, &u, &v)) {
            } else if (T.inProto) {
                T.pany = true;
                if (kWide && NearTie(t, T.pt)) T.pflags |= RT_HIT_TIE;
                if (t < T.pt) { T.pt = t; T.pu = u; T.pv = v; T.pslot = slot; T.r.MaxT = t; }
                else if (t == T.pt) T.pflags |= RT_HIT_TIE;
            } else {
                T.any = true;
                if (kWide && NearTie(t, T.best.t)) T.best.flags |= RT_HIT_TIE;
                if (t < T.best.t) {
                    T.best.t = t; T.best.u = u; T.best.v = v; T.best.slot = slot; T.best.sub = -1; T.best.pw = v3s(0);
                    T.r.MaxT = t;
                } else if (t == T.best.t) {
                    T.best.flags |= RT_HIT_TIE;
                }
            }
        } else if (T.inProto) {
            atomicOr(status, RT_STATUS_BADREF);
        }
        if (kind != RT_KIND_INSTANCE || T.inProto) {
            if (T.leafLeft == 0) {
                T.cur = PopNext(stack, &T.sp, T.base, T.r.MaxT, st);
                EnterLeaf(S, &T.cur, &T.leafSlot, &T.leafLeft);
            }
            return false;
        }
        /* enter the instance's prototype */
        if (st) st->insts++;
        T.inst = (int)ref;
        T.topSlot = T.leafSlot; T.topLeft = T.leafLeft; T.leafLeft = 0;
        T.wMaxT = T.r.MaxT;
        const RtInstance& I = S->instances[T.inst];
        float w2m[12];
#pragma unroll
        for (int i = 0; i < 12; i++) w2m[i] = __ldg(I.w2m + i);
        T.r = XfRay(T.r, w2m);
        T.pt = kFMax; T.pu = 0; T.pv = 0; T.pslot = -1; T.pflags = 0; T.pany = false;
        T.inProto = true;
        T.base = T.sp;
        T.cur = RootRef<kWide>(S, 1 + __ldg(&I.blas), T.r, st);
        EnterLeaf(S, &T.cur, &T.leafSlot, &T.leafLeft);
        return false;
    }
    if (!T.inProto) return true;
    /* leave the prototype: the instance's candidate in world space */
    T.inProto = false;
    if (T.pany) {
        const RtInstance& I = S->instances[T.inst];
        const float4 s1 = __ldg(S->slots + 3 * (int64_t)T.pslot + 1);
        const uint32_t kr = __float_as_uint(s1.w);
        V3 pm;
        if ((kr >> RT_KIND_SHIFT) == RT_KIND_TRI) {
            const V3 bary = v3(1 - (T.pu + T.pv), T.pu, T.pv);
            const RtTri t = S->tris[kr & RT_REF_MASK];
            pm = bary.x * f4xyz(S->pos[t.v0]) + bary.y * f4xyz(S->pos[t.v1]) + bary.z * f4xyz(S->pos[t.v2]);
        } else {
            const RtSphere sph = S->spheres[kr & RT_REF_MASK];
            const V3 c = v3(sph.center[0], sph.center[1], sph.center[2]);
            const V3 n = Normalize(At(T.r, T.pt) - c);
            pm = n * sph.radius + c;
        }
        float m2w[12];
#pragma unroll
        for (int i = 0; i < 12; i++) m2w[i] = __ldg(I.m2w + i);
        const V3 pw = Xf12(pm, m2w);
        const float t = Distance(T.wO, pw);
        T.any = true;
        T.best.flags |= T.pflags;
        if (kWide && NearTie(t, T.best.t)) T.best.flags |= RT_HIT_TIE;
        if (t < T.best.t) {
            T.best.t = t; T.best.u = T.pu; T.best.v = T.pv; T.best.slot = T.topSlot - 1; T.best.sub = T.pslot; T.best.pw = pw;
            T.wMaxT = t;
        } else if (t == T.best.t) {
            T.best.flags |= RT_HIT_TIE;
        }
    }
    T.r = mkray(T.wO, T.wD, T.r.MinT, T.wMaxT);
    T.leafSlot = T.topSlot; T.leafLeft = T.topLeft;
    T.sp = T.base;
    T.base = 0;
    if (T.leafLeft == 0) {
        T.cur = PopNext(stack, &T.sp, 0, T.r.MaxT, st);
        EnterLeaf(S, &T.cur, &T.leafSlot, &T.leafLeft);
    }
    return false;
}

/* The whole closest-hit traversal of one ray; ray.MaxT ends at the closest hit. */
template <bool kWide = false>
DF bool SceneClosest(const RtSceneView* S, Ray& ray, Best* best, int2* stack, uint32_t* status, TravStats* st) {
    TravClosest T;
    if (!ClosestBegin<kWide>(S, ray, T, st))
        while (!ClosestStep<int2*, RT_DESCEND, kWide>(S, T, stack, status, st)) {}
    *best = T.best;
    ray.MaxT = T.inProto ? T.wMaxT : T.r.MaxT;
    return T.any;
}

/* Scene.Intersect(ray): the any-hit form (Bvh.cs:126-172,
 * InstancedPrimitive.Intersect(ray), Primitive.cs:162-167). */
struct TravAny {
    Ray r;
    V3 wO, wD;
    float wMaxT;
    int cur, sp, base, leafSlot, leafLeft, topSlot, topLeft;
    bool inProto, hit;
    uint32_t guard;
};

template <bool kWide = false>
DF bool AnyBegin(const RtSceneView* S, const Ray& ray, TravAny& T, TravStats* st) {
    T.r = ray; T.wO = ray.O; T.wD = ray.D; T.wMaxT = ray.MaxT;
    T.inProto = false; T.hit = false;
    T.base = 0; T.sp = 0; T.leafLeft = 0; T.leafSlot = 0; T.topSlot = 0; T.topLeft = 0;
    T.guard = 0;
    T.cur = RootRef<kWide>(S, 0, ray, st);
    if (T.cur == RT_NO_NODE) return true;
    EnterLeaf(S, &T.cur, &T.leafSlot, &T.leafLeft);
    return false;
}

/* One step; true when the traversal has finished (T.hit holds the answer). */
template <class Stk, int kDescend = RT_DESCEND, bool kWide = false>
DF bool AnyStep(const RtSceneView* S, TravAny& T, Stk stack, uint32_t* status, TravStats* st) {
    if (++T.guard > RT_TRAVERSAL_CAP) { atomicOr(status, RT_STATUS_TRAV); return true; }
    if (T.cur != RT_NO_NODE) {
        for (int k = 0; k < kDescend && T.cur >= 0; k++) {
            if (kWide ? T.sp - T.base > RT_STACK_SIZE - 8 : T.sp - T.base == RT_STACK_SIZE) {
                atomicOr(status, RT_STATUS_STACK);
                if (!T.inProto) return true;
                T.sp = T.base;
                T.cur = RT_NO_NODE;
                return false;
            }
            if (st) st->nodes++;
            T.cur = kWide ? VisitWideNode(S, T.cur, T.r, stack, &T.sp) : VisitNode(S, T.cur, T.r, stack, &T.sp, st);
            if (T.cur == RT_NO_NODE) T.cur = PopNext(stack, &T.sp, T.base, T.r.MaxT, st);
        }
        EnterLeaf(S, &T.cur, &T.leafSlot, &T.leafLeft);
        if (T.cur != RT_NO_NODE) return false;
    }
    if (T.leafLeft > 0) {
        const int slot = T.leafSlot++;
        T.leafLeft--;
        const float4 s0 = __ldg(S->slots + 3 * (int64_t)slot);
        const float4 s1 = __ldg(S->slots + 3 * (int64_t)slot + 1);
        const float4 s2 = __ldg(S->slots + 3 * (int64_t)slot + 2);
        const uint32_t kr = __float_as_uint(s1.w);
        const uint32_t kind = kr >> RT_KIND_SHIFT, ref = kr & RT_REF_MASK;
        if (st) st->prims++;
        if (kind != RT_KIND_INSTANCE) {
            float t, u, v;
            if (PrimHit(S, kind, ref, s0, s1, s2, T.r, &t, &u, &v)) { T.hit = true; return true; }
        } else if (T.inProto) {
            atomicOr(status, RT_STATUS_BADREF);
        }
        if (kind != RT_KIND_INSTANCE || T.inProto) {
            if (T.leafLeft == 0) {
                T.cur = PopNext(stack, &T.sp, T.base, T.r.MaxT, st);
                EnterLeaf(S, &T.cur, &T.leafSlot, &T.leafLeft);
            }
            return false;
        }
        if (st) st->insts++;
        T.topSlot = T.leafSlot; T.topLeft = T.leafLeft; T.leafLeft = 0;
        const RtInstance& I = S->instances[(int)ref];
        float w2m[12];
#pragma unroll
        for (int i = 0; i < 12; i++) w2m[i] = __ldg(I.w2m + i);
        T.r = XfRay(T.r, w2m);
        T.inProto = true;
        T.base = T.sp;
        T.cur = RootRef<kWide>(S, 1 + __ldg(&I.blas), T.r, st);
        EnterLeaf(S, &T.cur, &T.leafSlot, &T.leafLeft);
        return false;
    }
    if (!T.inProto) return true;
    T.inProto = false;
    T.r = mkray(T.wO, T.wD, T.r.MinT, T.wMaxT);
    T.leafSlot = T.topSlot; T.leafLeft = T.topLeft;
    T.sp = T.base;
    T.base = 0;
    if (T.leafLeft == 0) {
        T.cur = PopNext(stack, &T.sp, 0, T.r.MaxT, st);
        EnterLeaf(S, &T.cur, &T.leafSlot, &T.leafLeft);
    }
    return false;
}

template <bool kWide = false>
DF bool SceneAny(const RtSceneView* S, const Ray& ray, int2* stack, uint32_t* status, TravStats* st) {
    TravAny T;
    if (!AnyBegin<kWide>(S, ray, T, st))
        while (!AnyStep<int2*, RT_DESCEND, kWide>(S, T, stack, status, st)) {}
    return T.hit;
}

/* Builds the full Intersection of the winning primitive (GetIntersection /
 * InstancedPrimitive.Intersect). */
DF void Finish(const RtSceneView* S, const Ray& ray, const Best& b, Isect* it) {
    float4 s0 = __ldg(S->slots + 3 * (int64_t)b.slot);
    float4 s1 = __ldg(S->slots + 3 * (int64_t)b.slot + 1);
    uint32_t kr = __float_as_uint(s1.w);
    uint32_t kind = kr >> RT_KIND_SHIFT, ref = kr & RT_REF_MASK;
    it->prim = __float_as_int(s0.w); it->sub = -1; it->slot = b.slot; it->flags = b.flags;
    it->bu = b.u; it->bv = b.v;
    if (kind == RT_KIND_TRI) {
        V3 bary = v3(1 - (b.u + b.v), b.u, b.v);
        V3 n;
        TriAttrs(S, (int)ref, bary, &it->P, &n, &it->UV);
        it->F = mkframe(n); it->T = b.t; it->Wr = -ray.D;
    } else if (kind == RT_KIND_SPHERE) {
        RtSphere sph = S->spheres[ref];
        V3 c = v3(sph.center[0], sph.center[1], sph.center[2]);
        V3 n = Normalize(At(ray, b.t) - c);
        it->P = n * sph.radius + c; it->UV = SphereUV(sph, n); it->F = mkframe(n); it->T = b.t; it->Wr = -ray.D;
    } else {
        const RtInstance& I = S->instances[ref];
        float w2m[12], m2w[12];
        for (int i = 0; i < 12; i++) { w2m[i] = I.w2m[i]; m2w[i] = I.m2w[i]; }
        V3 dm = Normalize(XfN12(ray.D, w2m));
        float4 p0 = __ldg(S->slots + 3 * (int64_t)b.sub);
        float4 p1 = __ldg(S->slots + 3 * (int64_t)b.sub + 1);
        uint32_t pkr = __float_as_uint(p1.w);
        V3 nm; V2 uvm;
        if ((pkr >> RT_KIND_SHIFT) == RT_KIND_TRI) {
            V3 bary = v3(1 - (b.u + b.v), b.u, b.v);
            V3 pm;
            TriAttrs(S, (int)(pkr & RT_REF_MASK), bary, &pm, &nm, &uvm);
        } else {
            /* sphere inside a prototype: normal from the model-space ray */
            RtSphere sph = S->spheres[pkr & RT_REF_MASK];
            Ray mr = XfRay(ray, w2m);
            V3 c = v3(sph.center[0], sph.center[1], sph.center[2]);
            float tm = 0; SphereTest(c, sph.radius, mr, &tm);
            nm = Normalize(At(mr, tm) - c); uvm = SphereUV(sph, nm);
        }
        it->P = b.pw;
        V3 n = Normalize(XfN12(nm, m2w));
        it->F = mkframe(n);
        it->Wr = Normalize(XfN12(-dm, m2w));
        it->UV = uvm; it->T = b.t;
        it->sub = __float_as_int(p0.w);
    }
}

}  /* namespace rtd */

#endif
