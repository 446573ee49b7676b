/*
 * mcx_pmath.cuh -- deterministic single-precision math for the kernel's
 * "exact" instantiation.
 *
 * The exact instantiation exists so that a GPU run can be compared with the
 * CPU oracle photon for photon: every function here uses only IEEE-754 basic
 * operations (+ - * / sqrt rint) with no contraction, so the same inputs give
 * the same bits on the GPU (compiled -fmad=false -prec-div=true
 * -prec-sqrt=true -ftz=false) and on any host compiled -ffp-contract=off.
 * The fast instantiation uses the hardware MUFU approximations instead.
 *
 * Methods (textbook):
 *   log : x = 2^k m, m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh((m-1)/(m+1))
 *         by its series to s^9; k ln2 with a 12-bit Cody-Waite split of ln2.
 *   exp : Cody-Waite reduction x = k ln2 + r, Taylor polynomial to r^7,
 *         2^k from exponent bits; results below FLT_MIN return 0.
 *   sin/cos: k = rint(2x/pi), three-part Cody-Waite split of pi/2 (12-bit
 *         heads, exact for |k| < 2^11), Taylor polynomials on |r| <= pi/4.
 *   acos: |x| <= 1/2: pi/2 - asin(x); else 2 asin(sqrt((1-|x|)/2)),
 *         asin by its Taylor series to t^23.
 * A CPU test checks these bit for bit against the oracle's copy and within a
 * few ulp of a double-precision evaluation.
 */
#ifndef MCX_PMATH_CUH
#define MCX_PMATH_CUH

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define MCX_HD __host__ __device__ __forceinline__
#else
#define MCX_HD static inline
#endif

MCX_HD float pm_bits2f(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

MCX_HD uint32_t pm_f2bits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

MCX_HD float pm_logf(float x) {
    uint32_t u = pm_f2bits(x);
    int k = 0;
    if (!(x > 0.0f)) {
        return (x == 0.0f) ? -INFINITY : NAN;
    }
    if (u >= 0x7f800000u) {
        return x;
    }
    if (u < 0x00800000u) {
        x = x * 16777216.0f;
        u = pm_f2bits(x);
        k = -24;
    }
    k += (int)(u >> 23) - 127;
    float m = pm_bits2f((u & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        k += 1;
    }
    float f = m - 1.0f;
    float s = f / (2.0f + f);
    float z = s * s;
    float p = z * (0.666666667f + z * (0.4f + z * (0.285714286f + z * 0.222222222f)));
    float lnm = 2.0f * s + s * p;
    float kf = (float)k;
    return kf * 0.693115234375f + (lnm + kf * 3.19461833e-05f);
}

MCX_HD float pm_expf(float x) {
    if (x != x) {
        return x;
    }
    if (x > 88.7228394f) {
        return INFINITY;
    }
    if (x < -87.3365479f) {
        return 0.0f;
    }
    float kf = rintf(x * 1.44269502f);
    float r = x - kf * 0.693115234375f;
    r = r - kf * 3.19461833e-05f;
    float p = 1.0f + r * (1.0f + r * (0.5f + r * (0.166666667f + r * (0.0416666667f +
                          r * (0.00833333333f + r * (0.00138888889f + r * 0.000198412698f))))));
    int k = (int)kf;
    if (k > 127) {
        p = p * 2.0f;
        k -= 1;
    }
    return p * pm_bits2f((uint32_t)(k + 127) << 23);
}

MCX_HD void pm_sincosf(float x, float* sn, float* cs) {
    float kf = rintf(x * 0.636619747f);
    float r = x - kf * 1.57080078125f;
    r = r - kf * -4.45358455e-06f;
    r = r - kf * -8.70551631e-10f;
    float z = r * r;
    float s = r + r * z * (-0.166666667f + z * (0.00833333333f + z * (-0.000198412698f +
                           z * 2.75573192e-06f)));
    float c = 1.0f + z * (-0.5f + z * (0.0416666667f + z * (-0.00138888889f +
                          z * (2.48015873e-05f + z * -2.75573192e-07f))));
    int q = ((int)kf) & 3;
    if (q == 0) {
        *sn = s;
        *cs = c;
    } else if (q == 1) {
        *sn = c;
        *cs = -s;
    } else if (q == 2) {
        *sn = -s;
        *cs = -c;
    } else {
        *sn = -c;
        *cs = s;
    }
}

MCX_HD float pm_sinf(float x) {
    float s, c;
    pm_sincosf(x, &s, &c);
    return s;
}

MCX_HD float pm_cosf(float x) {
    float s, c;
    pm_sincosf(x, &s, &c);
    return c;
}

MCX_HD float pm_asin_poly(float t) {
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

MCX_HD float pm_acosf(float x) {
    float ax = fabsf(x);
    if (x != x || ax > 1.0f) {
        return NAN;
    }
    if (ax <= 0.5f) {
        return 1.57079637f + (-4.37113901e-08f - pm_asin_poly(x));
    }
    float t = sqrtf(0.5f * (1.0f - ax));
    float a = 2.0f * pm_asin_poly(t);
    return (x > 0.0f) ? a : (3.14159274f + (-8.74227801e-08f - a));
}

#endif
