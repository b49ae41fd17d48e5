/*
 * pfref_internal.h -- exact-arithmetic helpers of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links or includes this.
 *
 * The reference's rasteriser runs on AVX2 (src/internal/simd.h).  Its results
 * depend on x86 rules that plain C does not give for free:
 *   - MINPS/MAXPS return the SECOND operand when the compare is false or
 *     unordered (NaN), unlike fminf/fmaxf;
 *   - CVTPS2DQ rounds to nearest-even and returns 0x80000000 for NaN and
 *     out-of-range inputs; CVTTPS2DQ is the truncating form;
 *   - packing a colour ORs shifted channels without masking them.
 * These helpers restate those rules so that the scalar oracle reproduces the
 * SIMD path lane by lane on any host (x86-64 or aarch64).
 */
#ifndef PFREF_INTERNAL_H
#define PFREF_INTERNAL_H

#include <stdint.h>
#include <string.h>
#include <math.h>

static inline float ox_min(float a, float b) { return (a < b) ? a : b; }   /* MINPS(a, b) */
static inline float ox_max(float a, float b) { return (a > b) ? a : b; }   /* MAXPS(a, b) */

static inline uint32_t ox_fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float ox_bitsf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* CVTPS2DQ with MXCSR at its default (round to nearest even). */
static inline int32_t ox_cvt_rne(float x)
{
    if (!(x > -2147483648.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int32_t)nearbyintf(x);
}

/* CVTTPS2DQ (truncation). */
static inline int32_t ox_cvt_trunc(float x)
{
    if (!(x > -2147483649.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int32_t)x;
}

/* Scalar C conversion of a float to int as GCC emits it on x86-64
 * (cvttss2si: truncation, 0x80000000 when out of range). */
static inline int32_t ox_ftoi(float x) { return ox_cvt_trunc(x); }

/* (PFubyte)(float) as GCC emits it on x86-64: truncate to int32, keep the
 * low 8 bits. */
static inline uint8_t ox_ftoub(float x) { return (uint8_t)(uint32_t)ox_ftoi(x); }

/* (PFubyte)(double), same rule (cvttsd2si, low 8 bits). */
static inline uint8_t ox_dtoub(double x)
{
    if (!(x > -2147483649.0 && x < 2147483648.0)) return 0;
    return (uint8_t)(uint32_t)(int32_t)x;
}

static inline int32_t ox_iabs(int32_t v) { return (v < 0) ? (int32_t)(0u - (uint32_t)v) : v; }

/* Natural logarithm, Cephes polynomial as adapted by J. Pommier for SSE and
 * G. Garberoglio for AVX (zlib licence), which the reference uses for its
 * per-fragment power function (src/internal/simd.h:183-252).  Every step is
 * a separate IEEE single operation; non-positive inputs give NaN. */
static inline float ox_log_cephes(float x)
{
    const int invalid = (x <= 0.0f);          /* _CMP_LE_OS: false for NaN */
    x = ox_max(x, ox_bitsf(0x00800000u));
    int32_t e_i = (int32_t)(ox_fbits(x) >> 23);
    x = ox_bitsf((ox_fbits(x) & ~0x7f800000u) | ox_fbits(0.5f));
    e_i -= 0x7f;
    float e = (float)e_i;
    e = e + 1.0f;
    const int lt = (x < 0.707106781186547524f);
    float tmp = lt ? x : 0.0f;
    x = x - 1.0f;
    e = e - (lt ? 1.0f : 0.0f);
    x = x + tmp;
    float z = x * x;
    float y = 7.0376836292E-2f;
    y = y * x; y = y + -1.1514610310E-1f;
    y = y * x; y = y + 1.1676998740E-1f;
    y = y * x; y = y + -1.2420140846E-1f;
    y = y * x; y = y + 1.4249322787E-1f;
    y = y * x; y = y + -1.6668057665E-1f;
    y = y * x; y = y + 2.0000714765E-1f;
    y = y * x; y = y + -2.4999993993E-1f;
    y = y * x; y = y + 3.3333331174E-1f;
    y = y * x;
    y = y * z;
    tmp = e * -2.12194440e-4f;
    y = y + tmp;
    tmp = z * 0.5f;
    y = y - tmp;
    tmp = e * 0.693359375f;
    x = x + y;
    x = x + tmp;
    if (invalid) x = ox_bitsf(0xffffffffu);
    return x;
}

/* exp(x), same provenance (src/internal/simd.h:254-300). */
static inline float ox_exp_cephes(float x)
{
    x = ox_min(x, 88.3762626647949f);
    x = ox_max(x, -88.3762626647949f);
    float fx = x * 1.44269504088896341f;
    fx = fx + 0.5f;
    float tmp = floorf(fx);
    fx = tmp - ((tmp > fx) ? 1.0f : 0.0f);
    tmp = fx * 0.693359375f;
    float z = fx * -2.12194440e-4f;
    x = x - tmp;
    x = x - z;
    z = x * x;
    float y = 1.9875691500E-4f;
    y = y * x; y = y + 1.3981999507E-3f;
    y = y * x; y = y + 8.3334519073E-3f;
    y = y * x; y = y + 4.1665795894E-2f;
    y = y * x; y = y + 1.6666665459E-1f;
    y = y * x; y = y + 5.0000001201E-1f;
    y = y * z;
    y = y + x;
    y = y + 1.0f;
    int32_t n = ox_cvt_trunc(fx);
    n = n + 0x7f;
    float pow2n = ox_bitsf((uint32_t)n << 23);
    return y * pow2n;
}

/* pfiSimdPow_F32 (src/internal/simd.h:1158-1170). */
static inline float ox_pow_cephes(float base, float exponent)
{
    return ox_exp_cephes(ox_log_cephes(base) * exponent);
}

#endif /* PFREF_INTERNAL_H */
