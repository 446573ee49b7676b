/*
 * oracle_pmath.h -- deterministic single-precision math for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links this file; the
 * product's GPU kernel carries its own copy of the same published methods
 * (mcxcl_gb300/csrc/mcx_pmath.cuh) for its "exact" instantiation, and a CPU
 * test checks that both produce identical bits over a sweep of inputs.
 *
 * Every function below uses only IEEE-754 basic operations (+, -, *, /,
 * sqrt, rint, floor) evaluated in float with no contraction, so the results
 * are the same bits on x86-64 (SSE), aarch64 and an sm_103a GPU compiled
 * with -fmad=false -prec-div=true -prec-sqrt=true -ftz=false.
 *
 * Methods (textbook, no vendor code):
 *   log : x = 2^k m, m in [sqrt(1/2), sqrt(2)); ln m = 2 atanh(s),
 *         s = (m-1)/(m+1), atanh series to s^9; k ln2 with a two-part
 *         Cody-Waite split of ln2 (12-bit head).
 *   exp : Cody-Waite reduction x = k ln2 + r, |r| <= ln2/2, Taylor
 *         polynomial to r^7, scaling by 2^k built from exponent bits.
 *         Results below FLT_MIN are returned as 0 (no subnormal output).
 *   sin/cos : k = rint(x 2/pi), three-part Cody-Waite split of pi/2 (12-bit
 *         heads, exact for |k| < 2^11), Taylor polynomials on |r| <= pi/4.
 *   acos: |x| <= 1/2: pi/2 - asin(x); else 2 asin(sqrt((1-|x|)/2)) folded
 *         by sign; asin by its Taylor series to t^23 on [0, 1/2].
 * Accuracy against a double-precision reference: a few ulp (tested).
 */
#ifndef MCX_ORACLE_PMATH_H
#define MCX_ORACLE_PMATH_H

#include <math.h>
#include <stdint.h>
#include <string.h>

static inline float opm_bits2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static inline uint32_t opm_f2bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

static inline float opm_logf(float x) {
    uint32_t u = opm_f2bits(x);
    int k = 0;
    float m, f, s, z, p, lnm, kf;
    if (!(x > 0.0f)) {
        return (x == 0.0f) ? -INFINITY : NAN;
    }
    if (u >= 0x7f800000u) {
        return x;
    }
    if (u < 0x00800000u) {              /* subnormal input: scale by 2^24 */
        x = x * 16777216.0f;
        u = opm_f2bits(x);
        k = -24;
    }
    k += (int)(u >> 23) - 127;
    m = opm_bits2f((u & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        k += 1;
    }
    f = m - 1.0f;
    s = f / (2.0f + f);
    z = s * s;
    p = z * (0.666666667f + z * (0.4f + z * (0.285714286f + z * 0.222222222f)));
    lnm = 2.0f * s + s * p;
    kf = (float)k;
    return kf * 0.693115234375f + (lnm + kf * 3.19461833e-05f);
}

static inline float opm_expf(float x) {
    float kf, r, p;
    int k;
    if (x != x) {
        return x;
    }
    if (x > 88.7228394f) {
        return INFINITY;
    }
    if (x < -87.3365479f) {
        return 0.0f;
    }
    kf = rintf(x * 1.44269502f);
    r = x - kf * 0.693115234375f;
    r = r - kf * 3.19461833e-05f;
    p = 1.0f + r * (1.0f + r * (0.5f + r * (0.166666667f + r * (0.0416666667f +
                    r * (0.00833333333f + r * (0.00138888889f + r * 0.000198412698f))))));
    k = (int)kf;
    if (k > 127) {
        p = p * 2.0f;
        k -= 1;
    }
    return p * opm_bits2f((uint32_t)(k + 127) << 23);
}

static inline void opm_sincosf(float x, float* sn, float* cs) {
    float kf = rintf(x * 0.636619747f);
    float r = x - kf * 1.57080078125f;
    float z, s, c;
    int q;
    r = r - kf * -4.45358455e-06f;
    r = r - kf * -8.70551631e-10f;
    z = r * r;
    s = r + r * z * (-0.166666667f + z * (0.00833333333f + z * (-0.000198412698f +
                     z * 2.75573192e-06f)));
    c = 1.0f + z * (-0.5f + z * (0.0416666667f + z * (-0.00138888889f +
                    z * (2.48015873e-05f + z * -2.75573192e-07f))));
    q = ((int)kf) & 3;
    switch (q) {
        case 0: *sn = s;  *cs = c;  break;
        case 1: *sn = c;  *cs = -s; break;
        case 2: *sn = -s; *cs = -c; break;
        default: *sn = -c; *cs = s; break;
    }
}

static inline float opm_sinf(float x) {
    float s, c;
    opm_sincosf(x, &s, &c);
    return s;
}

static inline float opm_cosf(float x) {
    float s, c;
    opm_sincosf(x, &s, &c);
    return c;
}

static inline float opm_asin_poly(float t) {
    float z = t * t;
    float p = 0.00731252587f;
    p = p * z + 0.00839033581f;
    p = p * z + 0.00976160953f;
    p = p * z + 0.0115518009f;
    p = p * z + 0.0139648438f;
    p = p * z + 0.0173527644f;
    p = p * z + 0.0223721591f;
    p = p * z + 0.0303819444f;
    p = p * z + 0.0446428571f;
    p = p * z + 0.075f;
    p = p * z + 0.166666667f;
    return t + t * z * p;
}

static inline float opm_acosf(float x) {
    float ax = fabsf(x);
    if (x != x || ax > 1.0f) {
        return NAN;
    }
    if (ax <= 0.5f) {
        return 1.57079637f + (-4.37113901e-08f - opm_asin_poly(x));
    } else {
        float t = sqrtf(0.5f * (1.0f - ax));
        float a = 2.0f * opm_asin_poly(t);
        return (x > 0.0f) ? a : (3.14159274f + (-8.74227801e-08f - a));
    }
}

#endif
