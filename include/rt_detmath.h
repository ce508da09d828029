/*
 * rt_detmath.h - deterministic single-precision elementary functions.
 *
 * The path tracer reproduces the reference renderer's estimator bit for bit
 * between the CPU restatement and the CUDA kernels.  That only works when
 * every transcendental function returns the same bits on x86-64, aarch64 and
 * sm_103a.  The platform libraries (glibc libm, CUDA's libdevice) are each
 * accurate to 1-2 ulp but disagree with each other in the last bit, so both
 * sides call the functions below instead.
 *
 * Every function is built from IEEE-754 binary32 +, -, *, / and sqrt (all
 * correctly rounded on every target) plus integer bit manipulation.  The file
 * MUST be compiled without floating-point contraction (gcc/g++:
 * -ffp-contract=off, nvcc: --fmad=false) and without fast-math, otherwise a
 * compiler may fuse a multiply-add and change the last bit.
 *
 * Methods (all standard textbook constructions):
 *  - sin/cos/tan: Cody & Waite additive range reduction by pi/2 with a
 *    four-term split of pi/2 (W. J. Cody, W. Waite, "Software Manual for the
 *    Elementary Functions", 1980), then the Taylor series of sin and cos on
 *    [-pi/4, pi/4] truncated after the x^9 / x^10 terms (truncation error
 *    < 3e-9, below half an ulp).
 *  - exp: Cody-Waite reduction x = k ln2 + r, |r| <= ln2/2, Taylor series of
 *    e^r to r^8, exact scaling by 2^k (two steps for subnormal results).
 *  - log: x = m 2^e with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s) with
 *    s = (m-1)/(m+1), odd series in s to s^11.
 *  - atan: argument reduction atan(x) = pi/2 - atan(1/x) for |x| > 1 and
 *    atan(x) = pi/6 + atan((x sqrt3 - 1)/(x + sqrt3)) for x > 2 - sqrt3, then
 *    the Taylor series of atan to t^15 (|t| <= 0.268).
 *  - atan2: C99 Annex F special cases plus quadrant correction of atan(|y/x|).
 *  - acos: acos(x) = 2 atan(sqrt((1 - x) / (1 + x))).
 * Accuracy is checked against libm and CUDA in the test-suite (<= 4 ulp over
 * the ranges the renderer uses).
 */
#ifndef RT_DETMATH_H
#define RT_DETMATH_H

#include <stdint.h>
#ifndef __CUDACC__
#include <string.h>
#include <math.h>
#endif

#if defined(__CUDACC__)
#define RT_DM_FN __host__ __device__ __forceinline__
#else
#define RT_DM_FN static inline
#endif

RT_DM_FN uint32_t rt_dm_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u; memcpy(&u, &f, 4); return u;
#endif
}
RT_DM_FN float rt_dm_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f; memcpy(&f, &u, 4); return f;
#endif
}
RT_DM_FN int rt_dm_isnan(float x) { return x != x; }
RT_DM_FN int rt_dm_isinf(float x) { return (rt_dm_f2u(x) & 0x7fffffffu) == 0x7f800000u; }
RT_DM_FN float rt_dm_sqrt(float x) {
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(x);
#else
    return sqrtf(x);
#endif
}
RT_DM_FN float rt_dm_qnan(void) { return rt_dm_u2f(0x7fc00000u); }
RT_DM_FN float rt_dm_inf(void) { return rt_dm_u2f(0x7f800000u); }
RT_DM_FN float rt_dm_copysign(float mag, float sgn) {
    return rt_dm_u2f((rt_dm_f2u(mag) & 0x7fffffffu) | (rt_dm_f2u(sgn) & 0x80000000u));
}
/* round-to-nearest-even of x for |x| < 2^22 (magic-number addition). */
RT_DM_FN float rt_dm_rint_small(float x) {
    const float magic = 12582912.0f; /* 1.5 * 2^23 */
    if (x >= 0.0f) { float t = x + magic; return t - magic; }
    float t = x - magic; return t + magic;
}
/* 2^k as a float for -126 <= k <= 127 */
RT_DM_FN float rt_dm_pow2i(int k) { return rt_dm_u2f((uint32_t)(k + 127) << 23); }

/* ---- sin / cos / tan ------------------------------------------------- */
#define RT_DM_PIO2_1 1.5703125f
#define RT_DM_PIO2_2 0.0004837512969970703f
#define RT_DM_PIO2_3 7.549533620476723e-08f
#define RT_DM_PIO2_4 2.5633440682570896e-12f
#define RT_DM_2_OVER_PI 0.6366197466850281f

/* Reduce x to r in [-pi/4, pi/4] (approximately) and quadrant q (0..3). */
RT_DM_FN float rt_dm_reduce_pio2(float x, int* q) {
    float ax = x < 0.0f ? -x : x;
    if (ax < 8192.0f) {
        float k = rt_dm_rint_small(x * RT_DM_2_OVER_PI);
        float r = x - k * RT_DM_PIO2_1;
        r = r - k * RT_DM_PIO2_2;
        r = r - k * RT_DM_PIO2_3;
        r = r - k * RT_DM_PIO2_4;
        int ki = (int)k;
        *q = ki & 3;
        return r;
    }
    /* large arguments: reduction in binary64 (IEEE, identical everywhere) */
    double xd = (double)x;
    double kd = xd * 0.63661977236758134308;
    double kr = (kd >= 0.0) ? (double)(int64_t)(kd + 0.5) : -(double)(int64_t)(-kd + 0.5);
    double r = xd - kr * 1.5707963267341256;
    r = r - kr * 6.077100506506192e-11;
    r = r - kr * 2.0222662487959506e-21;
    int64_t ki = (int64_t)kr;
    *q = (int)(ki & 3);
    return (float)r;
}
RT_DM_FN float rt_dm_sin_poly(float r) {
    float r2 = r * r;
    float p = 2.7557319e-6f;            /*  1/9! */
    p = p * r2 + -1.9841270e-4f;         /* -1/7! */
    p = p * r2 + 8.3333333e-3f;          /*  1/5! */
    p = p * r2 + -1.6666667e-1f;         /* -1/3! */
    return r + (r * r2) * p;
}
RT_DM_FN float rt_dm_cos_poly(float r) {
    float r2 = r * r;
    float p = -2.7557319e-7f;           /* -1/10! */
    p = p * r2 + 2.4801587e-5f;          /*  1/8! */
    p = p * r2 + -1.3888889e-3f;         /* -1/6! */
    p = p * r2 + 4.1666667e-2f;          /*  1/4! */
    float hr = 0.5f * r2;
    float w = 1.0f - hr;
    /* add back the rounding error of (1 - hr) before the small tail */
    float tail = ((1.0f - w) - hr) + (r2 * r2) * p;
    return w + tail;
}
RT_DM_FN float rt_sinf(float x) {
    if (rt_dm_isnan(x) || rt_dm_isinf(x)) return rt_dm_qnan();
    int q; float r = rt_dm_reduce_pio2(x, &q);
    float s;
    switch (q) {
        case 0: s = rt_dm_sin_poly(r); break;
        case 1: s = rt_dm_cos_poly(r); break;
        case 2: s = -rt_dm_sin_poly(r); break;
        default: s = -rt_dm_cos_poly(r); break;
    }
    return s;
}
RT_DM_FN float rt_cosf(float x) {
    if (rt_dm_isnan(x) || rt_dm_isinf(x)) return rt_dm_qnan();
    int q; float r = rt_dm_reduce_pio2(x, &q);
    float c;
    switch (q) {
        case 0: c = rt_dm_cos_poly(r); break;
        case 1: c = -rt_dm_sin_poly(r); break;
        case 2: c = -rt_dm_cos_poly(r); break;
        default: c = rt_dm_sin_poly(r); break;
    }
    return c;
}
RT_DM_FN float rt_tanf(float x) {
    if (rt_dm_isnan(x) || rt_dm_isinf(x)) return rt_dm_qnan();
    int q; float r = rt_dm_reduce_pio2(x, &q);
    float s = rt_dm_sin_poly(r), c = rt_dm_cos_poly(r);
    return (q & 1) ? -(c / s) : (s / c);
}

/* ---- exp ---------------------------------------------------------------- */
#define RT_DM_LN2_1 0.693115234375f
#define RT_DM_LN2_2 3.193318843841553e-05f
#define RT_DM_LN2_3 1.2996506981721723e-08f
#define RT_DM_LOG2E 1.4426950216293335f
RT_DM_FN float rt_expf(float x) {
    if (rt_dm_isnan(x)) return x;
    if (x > 88.72284f) return rt_dm_inf();
    if (x < -103.97209f) return 0.0f;
    float k = rt_dm_rint_small(x * RT_DM_LOG2E);
    float r = x - k * RT_DM_LN2_1;
    r = r - k * RT_DM_LN2_2;
    r = r - k * RT_DM_LN2_3;
    float p = 2.4801587e-5f;             /* 1/8! */
    p = p * r + 1.9841270e-4f;           /* 1/7! */
    p = p * r + 1.3888889e-3f;           /* 1/6! */
    p = p * r + 8.3333333e-3f;           /* 1/5! */
    p = p * r + 4.1666667e-2f;           /* 1/4! */
    p = p * r + 1.6666667e-1f;           /* 1/3! */
    p = p * r + 0.5f;
    float e = 1.0f + (r + (r * r) * p);
    int ki = (int)k;
    if (ki > 127) return (e * rt_dm_pow2i(127)) * 2.0f;
    if (ki >= -126) return e * rt_dm_pow2i(ki);
    return (e * rt_dm_pow2i(ki + 100)) * rt_dm_pow2i(-100);
}

/* ---- log ---------------------------------------------------------------- */
RT_DM_FN float rt_logf(float x) {
    if (rt_dm_isnan(x)) return x;
    if (x < 0.0f) return rt_dm_qnan();
    if (x == 0.0f) return -rt_dm_inf();
    if (rt_dm_isinf(x)) return x;
    uint32_t u = rt_dm_f2u(x);
    int e = 0;
    if (u < 0x00800000u) { /* subnormal */
        x = x * 8388608.0f; /* 2^23 */
        u = rt_dm_f2u(x);
        e = -23;
    }
    e += (int)(u >> 23) - 127;
    float m = rt_dm_u2f((u & 0x007fffffu) | 0x3f800000u); /* [1, 2) */
    if (m > 1.4142135381698608f) { m = m * 0.5f; e += 1; }
    float f = m - 1.0f;
    float s = f / (2.0f + f);
    float s2 = s * s;
    float p = 1.0f / 11.0f;
    p = p * s2 + 1.0f / 9.0f;
    p = p * s2 + 1.0f / 7.0f;
    p = p * s2 + 0.2f;
    p = p * s2 + 1.0f / 3.0f;
    /* log(m) = 2s + 2s*s2*p, written as f - (f - 2s) to keep leading bits */
    float two_s = 2.0f * s;
    float lm = two_s + (two_s * s2) * p;
    float ef = (float)e;
    return ef * RT_DM_LN2_1 + (ef * RT_DM_LN2_2 + (ef * RT_DM_LN2_3 + lm));
}

/* ---- atan / atan2 / acos -------------------------------------------------- */
#define RT_DM_PIO2_HI 1.5707963705062866f
#define RT_DM_PIO2_LO (-4.3711390001862428e-08f)
#define RT_DM_PIO6_HI 0.5235987901687622f
#define RT_DM_PIO6_LO (-1.4570463e-08f)
#define RT_DM_PI_HI 3.1415927410125732f
#define RT_DM_PI_LO (-8.7422780003724856e-08f)
#define RT_DM_SQRT3 1.7320507764816284f
RT_DM_FN float rt_dm_atan_series(float t) {
    float t2 = t * t;
    float p = -1.0f / 15.0f;
    p = p * t2 + 1.0f / 13.0f;
    p = p * t2 + -1.0f / 11.0f;
    p = p * t2 + 1.0f / 9.0f;
    p = p * t2 + -1.0f / 7.0f;
    p = p * t2 + 0.2f;
    p = p * t2 + -1.0f / 3.0f;
    return t + (t * t2) * p;
}
/* atan of a non-negative finite argument */
RT_DM_FN float rt_dm_atan_pos(float ax) {
    int inv = 0;
    float t = ax;
    if (t > 1.0f) { t = 1.0f / t; inv = 1; }
    float a;
    if (t > 0.26794919f) {
        float u = (t * RT_DM_SQRT3 - 1.0f) / (t + RT_DM_SQRT3);
        a = RT_DM_PIO6_HI + (rt_dm_atan_series(u) + RT_DM_PIO6_LO);
    } else {
        a = rt_dm_atan_series(t);
    }
    if (inv) a = RT_DM_PIO2_HI - (a - RT_DM_PIO2_LO);
    return a;
}
RT_DM_FN float rt_atanf(float x) {
    if (rt_dm_isnan(x)) return x;
    if (rt_dm_isinf(x)) return rt_dm_copysign(RT_DM_PIO2_HI, x);
    float ax = x < 0.0f ? -x : x;
    float a = rt_dm_atan_pos(ax);
    return rt_dm_copysign(a, x);
}
RT_DM_FN float rt_atan2f(float y, float x) {
    if (rt_dm_isnan(x) || rt_dm_isnan(y)) return rt_dm_qnan();
    int xneg = (rt_dm_f2u(x) >> 31) != 0;
    if (y == 0.0f) {
        if (!xneg) return y; /* +-0 */
        return rt_dm_copysign(RT_DM_PI_HI, y);
    }
    if (x == 0.0f) return rt_dm_copysign(RT_DM_PIO2_HI, y);
    if (rt_dm_isinf(x)) {
        if (rt_dm_isinf(y)) {
            float v = xneg ? 2.3561944961547852f : 0.78539818525314331f;
            return rt_dm_copysign(v, y);
        }
        return xneg ? rt_dm_copysign(RT_DM_PI_HI, y) : rt_dm_copysign(0.0f, y);
    }
    if (rt_dm_isinf(y)) return rt_dm_copysign(RT_DM_PIO2_HI, y);
    float ay = y < 0.0f ? -y : y;
    float ax = x < 0.0f ? -x : x;
    float a;
    if (ay > ax) {
        /* atan(ay/ax) = pi/2 - atan(ax/ay): avoids overflow of the quotient */
        float t = ax / ay;
        a = RT_DM_PIO2_HI - (rt_dm_atan_pos(t) - RT_DM_PIO2_LO);
    } else {
        a = rt_dm_atan_pos(ay / ax);
    }
    if (xneg) a = RT_DM_PI_HI - (a - RT_DM_PI_LO);
    return rt_dm_copysign(a, y);
}
RT_DM_FN float rt_acosf(float x) {
    if (rt_dm_isnan(x)) return x;
    if (x > 1.0f || x < -1.0f) return rt_dm_qnan();
    if (x == -1.0f) return RT_DM_PI_HI;
    float q = (1.0f - x) / (1.0f + x);
    return 2.0f * rt_dm_atan_pos(rt_dm_sqrt(q));
}

#endif /* RT_DETMATH_H */
