/*
 * or_core.h - CPU oracle, part 1: System.Numerics / Radiantium.Core value types.
 *
 * TEST INFRASTRUCTURE ONLY.  This directory is the CPU restatement of the
 * Radiantium path-tracing hot path that the CUDA library is checked against;
 * only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use it.
 *
 * Parity status: the reference is C#/.NET 6 and cannot run on this machine
 * (no dotnet/mono) and ships no tests or golden vectors, so this restatement
 * cannot be compared with the reference binary's outputs.  It is pinned by
 * the reference's own example scenes (tests/fixtures/reference: the scene
 * files load into the primitive list and Scene.Lights RendererBuilder.Build
 * makes, and render on the GPU library bit for bit like here), by analytic
 * known answers, and by the GPU library, bit for bit, up to the benchmark
 * sizes.
 *
 * Every operation keeps the reference's expression order; compile with
 * -ffp-contract=off so no multiply-add is fused (the C# JIT never fuses).
 */
#ifndef OR_CORE_H
#define OR_CORE_H

#include <stdint.h>
#include <math.h>
#include <string.h>
#include <limits.h>
#include "../include/rt_detmath.h"

namespace orc {

static const float kPI = 3.14159265f;                      /* MathF.PI */
static const float kFloatEpsilon = 1.401298464324817e-45f; /* float.Epsilon (denormal) */
static const float kFloatMax = 3.40282347e+38f;            /* float.MaxValue */

static inline bool isnan_(float x) { return x != x; }
static inline bool isinf_(float x) { return rt_dm_isinf(x) != 0; }
static inline bool isneg_(float x) { return (rt_dm_f2u(x) >> 31) != 0; }

/* System.Math.Max/Min(float, float) of .NET Core 3.0+ (NaN-propagating,
 * +0 > -0). */
static inline float netMax(float a, float b) {
    if (a != b) { if (!isnan_(a)) return b < a ? a : b; return a; }
    return isneg_(b) ? a : b;
}
static inline float netMin(float a, float b) {
    if (a != b) { if (!isnan_(a)) return a < b ? a : b; return a; }
    return isneg_(a) ? a : b;
}
/* System.Math.Clamp(float, min, max) */
static inline float netClamp(float v, float lo, float hi) {
    if (v < lo) return lo;
    if (v > hi) return hi;
    return v;
}
static inline int netClampI(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
/* (int)float in C# on x64: truncation, NaN/out-of-range -> int.MinValue */
static inline int netF2I(float f) {
    if (isnan_(f) || f >= 2147483648.0f || f < -2147483648.0f) return INT_MIN;
    return (int)f;
}
static inline float netCopySign(float m, float s) { return rt_dm_copysign(m, s); }
static inline float Sqrt(float x) { return sqrtf(x); }
static inline float Abs(float x) { return fabsf(x); }
static inline float Sin(float x) { return rt_sinf(x); }
static inline float Cos(float x) { return rt_cosf(x); }
static inline float Tan(float x) { return rt_tanf(x); }
static inline float Atan(float x) { return rt_atanf(x); }
static inline float Atan2(float y, float x) { return rt_atan2f(y, x); }
static inline float Acos(float x) { return rt_acosf(x); }
static inline float Exp(float x) { return rt_expf(x); }
static inline float Log(float x) { return rt_logf(x); }
static inline float Sqr(float v) { return v * v; }                      /* MathExt.Sqr */
static inline float Fma(float a, float b, float c) { return a * b + c; } /* MathExt.Fma (not fused) */
static inline float MulSign(float a1, float a2) { return a1 * netCopySign(1.0f, a2); }
static inline float SafeSqrt(float a) { return Sqrt(netMax(a, 0.0f)); }
static inline float Rsqrt(float a) { return 1.0f / Sqrt(a); }
static inline float Radian(float v) { return v * (kPI / 180.0f); }

/* ---- Vector2 / Vector3 ------------------------------------------------ */
struct V2 { float x, y; };
static inline V2 v2(float x, float y) { V2 r; r.x = x; r.y = y; return r; }
static inline V2 operator+(V2 a, V2 b) { return v2(a.x + b.x, a.y + b.y); }
static inline V2 operator*(float s, V2 a) { return v2(s * a.x, s * a.y); }

struct V3 { float x, y, z; };
static inline V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline V3 v3s(float s) { return v3(s, s, s); }
static inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
static inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
static inline V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); } /* element-wise divide */
static inline float Dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float AbsDot(V3 a, V3 b) { return Abs(Dot(a, b)); }
static inline V3 Cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float LengthSquared(V3 a) { return Dot(a, a); }
static inline float Length(V3 a) { return Sqrt(LengthSquared(a)); }
static inline V3 Normalize(V3 a) { float l = Length(a); return a / l; }
static inline float Distance(V3 a, V3 b) { return Length(a - b); }
static inline V3 VMin(V3 a, V3 b) { return v3(a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z); }
static inline V3 VMax(V3 a, V3 b) { return v3(a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z); }
static inline float& At(V3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
static inline float Get(const V3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
/* Vector3.Reflect(vector, normal) */
static inline V3 Reflect(V3 v, V3 n) { float d = Dot(v, n); return v - ((2.0f * d) * n); }
static inline V3 SquareRoot(V3 v) { return v3(Sqrt(v.x), Sqrt(v.y), Sqrt(v.z)); }

/* ---- Matrix4x4 (row vectors) ---------------------------------------- */
struct M44 { float m[16]; };
static inline V3 Transform(V3 p, const M44& M) {
    const float* m = M.m;
    return v3(p.x * m[0] + p.y * m[4] + p.z * m[8] + m[12],
              p.x * m[1] + p.y * m[5] + p.z * m[9] + m[13],
              p.x * m[2] + p.y * m[6] + p.z * m[10] + m[14]);
}
static inline V3 TransformNormal(V3 v, const M44& M) {
    const float* m = M.m;
    return v3(v.x * m[0] + v.y * m[4] + v.z * m[8],
              v.x * m[1] + v.y * m[5] + v.z * m[9],
              v.x * m[2] + v.y * m[6] + v.z * m[10]);
}
static inline bool IsIdentity(const M44& M) {
    for (int i = 0; i < 16; i++) { if (M.m[i] != ((i % 5 == 0) ? 1.0f : 0.0f)) return false; }
    return true;
}

/* ---- Color3F (Radiantium.Core/Color3F.cs) ------------------------------ */
struct C3 { float r, g, b; };
static inline C3 c3(float r, float g, float b) { C3 c; c.r = r; c.g = g; c.b = b; return c; }
static inline C3 c3s(float v) { return c3(v, v, v); }
static inline C3 operator+(C3 a, C3 b) { return c3(a.r + b.r, a.g + b.g, a.b + b.b); }
static inline C3 operator-(C3 a, C3 b) { return c3(a.r - b.r, a.g - b.g, a.b - b.b); }
static inline C3 operator*(C3 a, C3 b) { return c3(a.r * b.r, a.g * b.g, a.b * b.b); }
static inline C3 operator/(C3 a, C3 b) { return c3(a.r / b.r, a.g / b.g, a.b / b.b); }
static inline C3 operator+(C3 a, float s) { return c3(a.r + s, a.g + s, a.b + s); }
static inline C3 operator-(C3 a, float s) { return c3(a.r - s, a.g - s, a.b - s); }
static inline C3 operator*(C3 a, float s) { return c3(a.r * s, a.g * s, a.b * s); }
static inline C3 operator/(C3 a, float s) { return c3(a.r / s, a.g / s, a.b / s); }
static inline C3 operator+(float s, C3 a) { return c3(s + a.r, s + a.g, s + a.b); }
static inline C3 operator-(float s, C3 a) { return c3(s - a.r, s - a.g, s - a.b); }
static inline C3 operator*(float s, C3 a) { return c3(s * a.r, s * a.g, s * a.b); }
static inline C3 operator/(float s, C3 a) { return c3(s / a.r, s / a.g, s / a.b); }
static inline bool operator==(C3 a, C3 b) { return a.r == b.r && a.g == b.g && a.b == b.b; }
static inline bool operator!=(C3 a, C3 b) { return !(a == b); }
static inline bool IsBlack(C3 a) { return a == c3s(0.0f); }
static inline float Floor(float x) { return std::floor(x); }
static inline bool IsValid(C3 c) {
    if (c.r < 0 || isinf_(c.r) || isnan_(c.r)) return false;
    if (c.g < 0 || isinf_(c.g) || isnan_(c.g)) return false;
    if (c.b < 0 || isinf_(c.b) || isnan_(c.b)) return false;
    return true;
}
static inline C3 CAbs(C3 c) { return c3(Abs(c.r), Abs(c.g), Abs(c.b)); }
static inline float MaxElement(C3 c) { return netMax(netMax(c.r, c.g), c.b); }
static inline float Luminance(C3 c) { return c.r * 0.212671f + c.g * 0.715160f + c.b * 0.072169f; }
static inline float CGet(const C3& c, int i) { return i == 0 ? c.r : (i == 1 ? c.g : c.b); }
static inline C3 FromV3(V3 v) { return c3(v.x, v.y, v.z); }

/* ---- Ray3F (Radiantium.Core/Ray3F.cs) ------------------------------------ */
struct Ray {
    V3 O, D;
    float MinT, MaxT;
    V3 InvD;
    Ray() {}
    Ray(V3 o, V3 d, float minT = kFloatEpsilon, float maxT = kFloatMax) : O(o), D(d), MinT(minT), MaxT(maxT) {
        InvD = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    }
    V3 At(float t) const { return O + t * D; }
};
/* Ray3F.Transform */
static inline Ray TransformRay(const Ray& ray, const M44& m) {
    V3 o = Transform(ray.O, m);
    V3 d = Normalize(TransformNormal(ray.D, m));
    V3 mx = Transform(ray.At(ray.MaxT), m);
    float maxT = Distance(o, mx);
    return Ray(o, d, ray.MinT, maxT);
}

/* ---- BoundingBox3F (Radiantium.Core/BoundingBox3F.cs) ------------------ */
struct BBox {
    V3 Min, Max;
    BBox() { Min = v3s(kFloatMax); Max = v3s(-kFloatMax); }
    BBox(V3 p) : Min(p), Max(p) {}
    BBox(V3 mn, V3 mx) : Min(mn), Max(mx) {}
    V3 Diagonal() const { return Max - Min; }
    float SurfaceArea() const { V3 d = Diagonal(); return 2 * (d.x * d.y + d.x * d.z + d.y * d.z); }
    V3 Center() const { return (Max + Min) * 0.5f; }
    void ExpendBy(V3 p) { Min = VMin(Min, p); Max = VMax(Max, p); }
    void Union(const BBox& b) { Min = VMin(Min, b.Min); Max = VMax(Max, b.Max); }
    V3 Offset(V3 p) const {
        V3 o = p - Min;
        if (Max.x > Min.x) o.x /= Max.x - Min.x;
        if (Max.y > Min.y) o.y /= Max.y - Min.y;
        if (Max.z > Min.z) o.z /= Max.z - Min.z;
        return o;
    }
    int MaximumExtent() const {
        V3 d = Diagonal();
        if (d.x > d.y && d.x > d.z) return 0;
        else if (d.y > d.z) return 1;
        else return 2;
    }
    /* Slab test, BoundingBox3F.cs:155-176.  Gamma(3) uses float.Epsilon
     * (a denormal) so the 1 + 2*gamma factor is exactly 1.0f. */
    bool Intersect(const Ray& ray) const {
        bool nx = ray.InvD.x < 0, ny = ray.InvD.y < 0, nz = ray.InvD.z < 0;
        float tMin = ((nx ? Max : Min).x - ray.O.x) * ray.InvD.x;
        float tMax = ((nx ? Min : Max).x - ray.O.x) * ray.InvD.x;
        float tyMin = ((ny ? Max : Min).y - ray.O.y) * ray.InvD.y;
        float tyMax = ((ny ? Min : Max).y - ray.O.y) * ray.InvD.y;
        const float g = 1.0f; /* 1 + 2 * Gamma(3) */
        tMax *= g; tyMax *= g;
        if (tMin > tyMax || tyMin > tMax) return false;
        if (tyMin > tMin) tMin = tyMin;
        if (tyMax < tMax) tMax = tyMax;
        float tzMin = ((nz ? Max : Min).z - ray.O.z) * ray.InvD.z;
        float tzMax = ((nz ? Min : Max).z - ray.O.z) * ray.InvD.z;
        tzMax *= g;
        if (tMin > tzMax || tzMin > tMax) return false;
        if (tzMin > tMin) tMin = tzMin;
        if (tzMax < tMax) tMax = tzMax;
        return (tMin < ray.MaxT) && (tMax > 0);
    }
};
static inline BBox BUnion(const BBox& a, const BBox& b) { return BBox(VMin(a.Min, b.Min), VMax(a.Max, b.Max)); }
static inline BBox BTransform(const BBox& b, const M44& m) {
    BBox r(Transform(v3(b.Min.x, b.Min.y, b.Min.z), m));
    r.ExpendBy(Transform(v3(b.Max.x, b.Min.y, b.Min.z), m));
    r.ExpendBy(Transform(v3(b.Min.x, b.Max.y, b.Min.z), m));
    r.ExpendBy(Transform(v3(b.Min.x, b.Min.y, b.Max.z), m));
    r.ExpendBy(Transform(v3(b.Min.x, b.Max.y, b.Max.z), m));
    r.ExpendBy(Transform(v3(b.Max.x, b.Max.y, b.Min.z), m));
    r.ExpendBy(Transform(v3(b.Max.x, b.Min.y, b.Max.z), m));
    r.ExpendBy(Transform(v3(b.Max.x, b.Max.y, b.Max.z), m));
    return r;
}

/* ---- Coordinate (Radiantium.Offline/Coordinate.cs) ------------------------ */
struct Coordinate {
    V3 X, Y, Z;
    Coordinate() {}
    /* Duff et al., JCGT 6(1) 2017, as written in Coordinate.cs:14-34 */
    explicit Coordinate(V3 n) {
        float sign = netCopySign(1.0f, n.z);
        float a = -1 / (sign + n.z);
        float b = n.x * n.y * a;
        X = v3(MulSign(Sqr(n.x) * a, n.z) + 1.0f, MulSign(b, n.z), MulSign(n.x, -n.z));
        Y = v3(b, sign + Sqr(n.y) * a, -n.y);
        Z = n;
    }
    V3 ToLocal(V3 v) const { return v3(Dot(v, X), Dot(v, Y), Dot(v, Z)); }
    V3 ToWorld(V3 v) const { return X * v.x + Y * v.y + Z * v.z; }
};
static inline float CosTheta(V3 v) { return v.z; }
static inline float AbsCosTheta(V3 v) { return Abs(CosTheta(v)); }
static inline float Cos2Theta(V3 v) { return Sqr(v.z); }
static inline float Sin2Theta(V3 v) { return Fma(v.x, v.x, Sqr(v.y)); }
static inline float TanTheta(V3 v) { return SafeSqrt(Fma(-v.z, v.z, 1.0f)) / v.z; }
static inline float Tan2Theta(V3 v) { return netMax(Fma(-v.z, v.z, 1.0f), 0.0f) / Sqr(v.z); }
static inline float Cos2Phi(V3 v) {
    float s2 = Sin2Theta(v);
    return Abs(s2) <= 4.0f * kFloatEpsilon ? 1.0f : netClamp(Sqr(v.x) / s2, -1.0f, 1.0f);
}
static inline float Sin2Phi(V3 v) {
    float s2 = Sin2Theta(v);
    return Abs(s2) <= 4.0f * kFloatEpsilon ? 0.0f : netClamp(Sqr(v.y) / s2, -1.0f, 1.0f);
}
static inline bool SameHemisphere(V3 a, V3 b) { return a.z * b.z > 0; }
static inline V3 Faceforward(V3 v, V3 v2_) { return (Dot(v, v2_) < 0.0f) ? -v : v; }

/* MathExt.Refract (Radiantium.Core/MathExt.cs:83-92) */
static inline bool Refract(V3 wi, V3 n, float eta, V3* wt) {
    float cosThetaI = Dot(n, wi);
    float sin2ThetaI = netMax(0, 1 - cosThetaI * cosThetaI);
    float sin2ThetaT = eta * eta * sin2ThetaI;
    if (sin2ThetaT >= 1) { *wt = v3s(0); return false; }
    float cosThetaT = Sqrt(1 - sin2ThetaT);
    *wt = Normalize(eta * -wi + (eta * cosThetaI - cosThetaT) * n);
    return true;
}
/* MathExt.SphericalDirection(sinTheta, cosTheta, phi) */
static inline V3 SphericalDirection(float sinTheta, float cosTheta, float phi) {
    float sinPhi = Sin(phi), cosPhi = Cos(phi);
    return v3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
}
static inline V3 SphericalDirectionF(float sinTheta, float cosTheta, float phi, V3 x, V3 y, V3 z) {
    float sinPhi = Sin(phi), cosPhi = Cos(phi);
    return sinTheta * cosPhi * x + sinTheta * sinPhi * y + cosTheta * z;
}
static inline V3 SphericalCoordinates(float theta, float phi) {
    float sinTheta = Sin(theta), cosTheta = Cos(theta);
    float sinPhi = Sin(phi), cosPhi = Cos(phi);
    return v3(cosPhi * sinTheta, sinPhi * sinTheta, cosTheta);
}

/* ---- counter-based RNG (stands in for System.Random) -------------------- */
/* Philox4x32-10 of Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3" (SC 2011). */
static inline void Philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                              uint32_t k0, uint32_t k1, uint32_t out[4]) {
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
struct Rng {
    uint32_t k0, k1, c0, c1, c2, n;
    uint32_t buf[4];
    Rng(uint64_t seed, uint32_t x, uint32_t y, uint32_t s)
        : k0((uint32_t)seed), k1((uint32_t)(seed >> 32)), c0(x), c1(y), c2(s), n(0) {}
    uint32_t NextU32() {
        if ((n & 3u) == 0) Philox4x32(c0, c1, c2, n >> 2, k0, k1, buf);
        return buf[n++ & 3u];
    }
    /* (float)rand.NextDouble() */
    float NextFloat() { return (float)(NextU32() >> 8) * (1.0f / 16777216.0f); }
    /* rand.Next(n) */
    int Next(int n_) { return (int)(((uint64_t)NextU32() * (uint64_t)(uint32_t)n_) >> 32); }
    V2 NextVec2() { float a = NextFloat(); float b = NextFloat(); return v2(a, b); }
};

/* ---- Probability.cs warps used on the path --------------------------------- */
static inline V2 SquareToUniformDisk(V2 s) {
    float radius = Sqrt(s.x);
    float angle = s.y * kPI * 2;
    return v2(radius * Cos(angle), radius * Sin(angle));
}
static inline V3 SquareToCosineHemisphere(V2 s) {
    V2 b = SquareToUniformDisk(s);
    float x = b.x, y = b.y;
    return v3(x, y, Sqrt(1 - x * x - y * y));
}
static inline V3 SquareToUniformSphere(V2 s) {
    float phi = s.x * kPI * 2;
    float theta = Acos(1 - 2 * s.y);
    float sinTheta = Sin(theta), cosTheta = Cos(theta);
    float sinPhi = Sin(phi), cosPhi = Cos(phi);
    return v3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
}

/* Probability.SquareToConcentricDisk (Probability.cs:157-174), Shirley-Chiu mapping */
static inline V2 SquareToConcentricDisk(V2 u) {
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
    float sinTheta = Sin(theta), cosTheta = Cos(theta);
    return v2(r * cosTheta, r * sinTheta);
}
/* Probability.SquareToCosineHemispherePdf (Probability.cs:102-105) */
static inline float SquareToCosineHemispherePdf(V3 v) { return v.z / kPI; }

/* PathUtility.PowerHeuristic (computed in double) */
static inline float PowerHeuristic(int nf, float fPdf, int ng, float gPdf) {
    double f = (double)((float)nf * fPdf), g = (double)((float)ng * gPdf);
    return (float)((f * f) / (f * f + g * g));
}

} /* namespace orc */

#endif /* OR_CORE_H */
