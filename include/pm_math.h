/*
 * pm_math.h -- deterministic single-precision math shared by the GPU kernels
 * and the CPU oracle: the Philox4x32-10 counter-based generator and the
 * few transcendental functions photon tracing needs.
 *
 * Every function here is built from IEEE operations that round the same way
 * on the host and on the GPU: +, -, *, /, sqrtf and fmaf (each correctly
 * rounded), and exact bit manipulation. Compiled with contraction disabled
 * (nvcc -fmad=false, gcc -ffp-contract=off) the host and the device return
 * identical bits, which is what lets GPU photon positions be compared with
 * the CPU restatement exactly. Accuracy against double-precision libm is
 * checked by tests/test_pm_math.py (a few ulp).
 *
 *  - Philox4x32-10: Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
 *    as easy as 1, 2, 3", SC 2011 (round function, multipliers and Weyl
 *    key schedule as published there).
 *  - pm_log1: log(x) for x in (0, 1], via x = m * 2^e with m in
 *    [sqrt(1/2), sqrt(2)) and log(m) = 2 atanh(s), s = (m-1)/(m+1), a
 *    truncated odd series in s.
 *  - pm_sincos2pi: sin and cos of 2*pi*u, reduced to an eighth of a turn
 *    and evaluated with Taylor polynomials in Horner form.
 *  - pm_expf: exp(x) for x <= 0, via x = k ln2 + r, |r| <= ln2/2 and a
 *    degree-7 Taylor polynomial, scaled by 2^k through the exponent bits.
 */
#ifndef PM_MATH_H
#define PM_MATH_H

#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define PMM_FN static __host__ __device__ __forceinline__
#else
#define PMM_FN static inline
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { uint32_t v[4]; } pm_u32x4;

PMM_FN uint32_t pmm_mulhilo(uint32_t a, uint32_t b, uint32_t *hi) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    return (uint32_t)p;
}

/* Philox4x32 with 10 rounds. ctr = 4 words, key = 2 words. */
PMM_FN pm_u32x4 pm_philox4x32_10(pm_u32x4 c, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, hi1;
        uint32_t lo0 = pmm_mulhilo(0xD2511F53u, c.v[0], &hi0);
        uint32_t lo1 = pmm_mulhilo(0xCD9E8D57u, c.v[2], &hi1);
        pm_u32x4 n;
        n.v[0] = hi1 ^ c.v[1] ^ k0;
        n.v[1] = lo1;
        n.v[2] = hi0 ^ c.v[3] ^ k1;
        n.v[3] = lo0;
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

/* Uniform float in [0, 1) with 24 random bits (exactly representable). */
PMM_FN float pm_u01(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-08f; }

PMM_FN float pmm_bits_to_float(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
PMM_FN uint32_t pmm_float_to_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

/* Natural logarithm of a normal positive float. */
PMM_FN float pm_logf(float x) {
    uint32_t b = pmm_float_to_bits(x);
    int e = (int)((b >> 23) & 0xFF) - 127;
    float m = pmm_bits_to_float((b & 0x007FFFFFu) | 0x3F800000u); /* [1, 2) */
    if (m > 1.41421356f) { m = m * 0.5f; e += 1; }                /* [0.7071, 1.4142] */
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    /* 2 atanh(s) = 2s (1 + s^2/3 + s^4/5 + s^6/7 + s^8/9 + s^10/11) */
    float p = fmaf(s2, 0.0909090909f, 0.111111111f);
    p = fmaf(s2, p, 0.142857143f);
    p = fmaf(s2, p, 0.2f);
    p = fmaf(s2, p, 0.333333333f);
    p = fmaf(s2, p, 1.0f);
    float lm = 2.0f * s * p;
    float fe = (float)e;
    /* ln2 split so fe * ln2_hi is exact for |e| < 2^12 */
    return fmaf(fe, 0.693145752f, fmaf(fe, 1.42860677e-06f, lm));
}

/* sin and cos of 2*pi*u for u in [0, 1]. */
PMM_FN void pm_sincos2pi(float u, float *s, float *c) {
    float q = rintf(u * 4.0f);           /* nearest quarter turn */
    float t = u - q * 0.25f;             /* exact, in [-1/8, 1/8] turn */
    int quad = ((int)q) & 3;
    float th = t * 6.28318548f;          /* |th| <= pi/4 */
    float x2 = th * th;
    float sp = fmaf(x2, 2.75573192e-06f, -1.98412698e-04f);
    sp = fmaf(x2, sp, 8.33333333e-03f);
    sp = fmaf(x2, sp, -1.66666667e-01f);
    float sn = fmaf(th * x2, sp, th);
    float cp = fmaf(x2, -2.75573192e-07f, 2.48015873e-05f);
    cp = fmaf(x2, cp, -1.38888889e-03f);
    cp = fmaf(x2, cp, 4.16666667e-02f);
    cp = fmaf(x2, cp, -0.5f);
    float cs = fmaf(x2, cp, 1.0f);
    switch (quad) {
        case 0: *s = sn; *c = cs; break;
        case 1: *s = cs; *c = -sn; break;
        case 2: *s = -sn; *c = -cs; break;
        default: *s = -cs; *c = sn; break;
    }
}

/* exp(x) for x <= 0 (returns 0 below -87). */
PMM_FN float pm_expf(float x) {
    if (x < -87.0f) return 0.0f;
    float k = rintf(x * 1.44269504f);
    float r = fmaf(k, -0.693145752f, x);
    r = fmaf(k, -1.42860677e-06f, r);
    float p = fmaf(r, 1.98412698e-04f, 1.38888889e-03f);
    p = fmaf(r, p, 8.33333333e-03f);
    p = fmaf(r, p, 4.16666667e-02f);
    p = fmaf(r, p, 1.66666667e-01f);
    p = fmaf(r, p, 0.5f);
    p = fmaf(r, p, 1.0f);
    p = fmaf(r, p, 1.0f);
    int ki = (int)k;
    /* 2^ki for ki in [-126, 0], as two exact factors to stay normal */
    int k1 = ki / 2, k2 = ki - k1;
    float s1 = pmm_bits_to_float((uint32_t)(k1 + 127) << 23);
    float s2 = pmm_bits_to_float((uint32_t)(k2 + 127) << 23);
    return (p * s1) * s2;
}

#ifdef __cplusplus
}
#endif
#endif /* PM_MATH_H */
