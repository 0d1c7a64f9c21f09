/*
 * cnncrf_fmath.h -- single-precision exp / expm1 / tanh written from the
 * mathematics, shared verbatim by the CUDA kernels and the CPU oracle so the
 * bit-exact FP32 path produces identical bits on both sides.
 *
 * Method (published): Cody & Waite argument reduction ("Software Manual for
 * the Elementary Functions", 1980): x = n*ln2 + r with |r| <= ln2/2, where
 * ln2 is split into a 12-bit "hi" part (so n*hi is exact for |n| < 4096) and
 * the float remainder "lo".  expm1(r) is then the degree-8 Taylor polynomial
 * r + r^2 * (1/2! + r/3! + ... + r^6/8!) evaluated by Horner's rule with
 * fused multiply-adds; the truncation error r^9/9! <= 2e-10 is far below one
 * float ulp.  Reconstruction: exp(x) = 2^n * (1 + expm1(r)) and
 * expm1(x) = 2^n * expm1(r) + (2^n - 1), each as one fused multiply-add.
 * tanh(y) = E / (E + 2) with E = expm1(2|y|), odd-extended; |y| >= 9 gives
 * +-1 (tanh(9) = 1 - 3e-8 rounds to 1.0f).
 *
 * Constants were derived from ln 2 = 0.6931471805599453094... and the
 * factorials 1/k!, each rounded to the nearest float.
 *
 * Only IEEE-754 correctly rounded operations are used (add, mul, fma, div,
 * rint), so any compiler that does not contract or reassociate (host:
 * -ffp-contract=off; device: explicit __fmaf_rn, --fmad=false) gives the same
 * result on x86-64, aarch64 and sm_103a.
 *
 * Accuracy (checked by tests/test_oracle.py::test_tanh_exp_accuracy against
 * float64 references):
 * exp, expm1 <= 2 ulp; tanh <= 3 ulp.  Results below FLT_MIN flush to 0.
 */
#ifndef CNNCRF_FMATH_H
#define CNNCRF_FMATH_H

#if defined(__CUDACC__)
#define CNNCRF_HD __host__ __device__ __forceinline__
#else
#define CNNCRF_HD static inline
#endif

#if !defined(__CUDA_ARCH__)
#include <math.h>
#include <stdint.h>
#include <string.h>
#endif

#define CNNCRF_LN2_HI 0.693115234375f          /* 0x3f317000 */
#define CNNCRF_LN2_LO 3.194618329871446e-05f
#define CNNCRF_INV_LN2 1.4426950216293335f
#define CNNCRF_C2 0.5f
#define CNNCRF_C3 0.1666666716337204f
#define CNNCRF_C4 0.0416666679084301f
#define CNNCRF_C5 0.008333333767950535f
#define CNNCRF_C6 0.0013888889225199819f
#define CNNCRF_C7 0.00019841270113829523f
#define CNNCRF_C8 2.4801587642286904e-05f

CNNCRF_HD float cnncrf_fma(float a, float b, float c)
{
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

CNNCRF_HD float cnncrf_mul(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}

CNNCRF_HD float cnncrf_add(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}

CNNCRF_HD float cnncrf_div(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

CNNCRF_HD float cnncrf_rint(float x)
{
#if defined(__CUDA_ARCH__)
    return rintf(x);
#else
    return rintf(x);
#endif
}

/* 2^n as a float for -126 <= n <= 127 (exact). */
CNNCRF_HD float cnncrf_pow2i(int n)
{
#if defined(__CUDA_ARCH__)
    return __int_as_float((n + 127) << 23);
#else
    uint32_t bits = (uint32_t)(n + 127) << 23;
    float f;
    memcpy(&f, &bits, sizeof f);
    return f;
#endif
}

/* expm1 of the reduced argument, |r| <= ~0.35. */
CNNCRF_HD float cnncrf_expm1_reduced(float r)
{
    float q = CNNCRF_C8;
    q = cnncrf_fma(q, r, CNNCRF_C7);
    q = cnncrf_fma(q, r, CNNCRF_C6);
    q = cnncrf_fma(q, r, CNNCRF_C5);
    q = cnncrf_fma(q, r, CNNCRF_C4);
    q = cnncrf_fma(q, r, CNNCRF_C3);
    q = cnncrf_fma(q, r, CNNCRF_C2);
    return cnncrf_fma(cnncrf_mul(r, r), q, r);
}

/* Cody-Waite reduction: returns r, writes n. */
CNNCRF_HD float cnncrf_reduce_ln2(float x, int *n_out)
{
    float n = cnncrf_rint(cnncrf_mul(x, CNNCRF_INV_LN2));
    float r = cnncrf_fma(-n, CNNCRF_LN2_HI, x);
    r = cnncrf_fma(-n, CNNCRF_LN2_LO, r);
    *n_out = (int)n;
    return r;
}

CNNCRF_HD float cnncrf_expf(float x)
{
    if (x > 88.72f) return 1.0f / 0.0f;
    if (x < -87.33f) return 0.0f;
    int n;
    float r = cnncrf_reduce_ln2(x, &n);
    float em1 = cnncrf_expm1_reduced(r);
    if (n > 127) { /* x in (88.38, 88.72]: scale in two steps */
        float s = cnncrf_pow2i(127);
        return cnncrf_mul(cnncrf_fma(s, em1, s), cnncrf_pow2i(n - 127));
    }
    if (n < -126) return 0.0f;
    float s = cnncrf_pow2i(n);
    return cnncrf_fma(s, em1, s);
}

CNNCRF_HD float cnncrf_expm1f(float x)
{
    if (x > 88.72f) return 1.0f / 0.0f;
    if (x < -17.5f) return -1.0f;
    int n;
    float r = cnncrf_reduce_ln2(x, &n);
    float em1 = cnncrf_expm1_reduced(r);
    if (n == 0) return em1;
    if (n > 127) {
        float s = cnncrf_pow2i(127);
        return cnncrf_mul(cnncrf_fma(s, em1, s), cnncrf_pow2i(n - 127));
    }
    float s = cnncrf_pow2i(n);
    return cnncrf_fma(s, em1, cnncrf_add(s, -1.0f));
}

CNNCRF_HD float cnncrf_tanhf(float x)
{
    float a = x < 0.0f ? -x : x;
    float t;
    if (a >= 9.0f) {
        t = 1.0f;
    } else if (a < 2.44140625e-4f) { /* 2^-12: tanh(a) = a to float precision */
        return x;
    } else {
        float e = cnncrf_expm1f(cnncrf_add(a, a));
        t = cnncrf_div(e, cnncrf_add(e, 2.0f));
    }
    return x < 0.0f ? -t : t;
}

/* log(x) for finite x > 0 (0 -> -inf, x < 0 -> NaN).  Method (published,
 * e.g. Muller, "Elementary Functions", ch. 6): x = 2^e * m with m in
 * [sqrt(1/2), sqrt(2)), s = (m - 1) / (m + 1), log(m) = 2 atanh(s) =
 * 2 (s + s^3/3 + s^5/5 + ... + s^11/11) with |s| <= 0.1716 (truncation
 * below 1e-11 relative), log(x) = e ln2 + log(m) with ln2 split hi / lo as
 * above.  The coefficients are 1/(2k+1) rounded to the nearest float. */
CNNCRF_HD float cnncrf_logf(float x)
{
    if (!(x > 0.0f)) return x == 0.0f ? -1.0f / 0.0f : 0.0f / 0.0f;
    if (x == 1.0f / 0.0f) return x;
    int32_t bits;
#if defined(__CUDA_ARCH__)
    bits = __float_as_int(x);
#else
    memcpy(&bits, &x, sizeof bits);
#endif
    int e = 0;
    if (((bits >> 23) & 0xff) == 0) { /* subnormal: scale by 2^23 (exact) */
        x = cnncrf_mul(x, 8388608.0f);
#if defined(__CUDA_ARCH__)
        bits = __float_as_int(x);
#else
        memcpy(&bits, &x, sizeof bits);
#endif
        e = -23;
    }
    e += ((bits >> 23) & 0xff) - 127;
    int32_t mb = (bits & 0x7fffff) | 0x3f800000; /* m in [1, 2) */
    float m;
#if defined(__CUDA_ARCH__)
    m = __int_as_float(mb);
#else
    memcpy(&m, &mb, sizeof m);
#endif
    if (m > 1.41421356f) { /* m in [sqrt(1/2), sqrt(2)) */
        m = cnncrf_mul(m, 0.5f);
        e += 1;
    }
    const float s = cnncrf_div(cnncrf_add(m, -1.0f), cnncrf_add(m, 1.0f));
    const float s2 = cnncrf_mul(s, s);
    float p = 0.09090909090909091f;          /* 1/11 */
    p = cnncrf_fma(p, s2, 0.1111111111111111f); /* 1/9 */
    p = cnncrf_fma(p, s2, 0.14285714285714285f); /* 1/7 */
    p = cnncrf_fma(p, s2, 0.2f);                /* 1/5 */
    p = cnncrf_fma(p, s2, 0.3333333432674408f);  /* 1/3 */
    const float s2x = cnncrf_add(s, s);
    const float lm = cnncrf_fma(s2x, cnncrf_mul(s2, p), s2x); /* 2s + 2s * s^2 p */
    const float ef = (float)e;
    return cnncrf_fma(ef, CNNCRF_LN2_HI, cnncrf_fma(ef, CNNCRF_LN2_LO, lm));
}

/* x^y for x >= 0 as exp(y log x); 0^y = 0 for y > 0, 1 for y == 0. */
CNNCRF_HD float cnncrf_powf(float x, float y)
{
    if (x == 0.0f) return y > 0.0f ? 0.0f : (y == 0.0f ? 1.0f : 1.0f / 0.0f);
    return cnncrf_expf(cnncrf_mul(y, cnncrf_logf(x)));
}

#endif /* CNNCRF_FMATH_H */
