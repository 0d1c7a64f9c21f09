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
 * Accuracy (checked by tests/test_fmath.py against float64 references):
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

#endif /* CNNCRF_FMATH_H */
