/*
 * Forced-include header for the "shim" build of the reference PixelForge
 * (oracle/Makefile, target `shim`).  Test infrastructure only.
 *
 * The reference's AVX2 path uses the approximate reciprocal and reciprocal
 * square root instructions (src/internal/simd.h:1218-1225 `pfiSimdRCP_F32`,
 * src/internal/simd.h:1238-1245 `pfiSimdRSqrt_F32`).  Their result bits are
 * implementation-defined (they differ between CPU vendors), so they cannot be
 * reproduced on another machine.  This header replaces both with the
 * correctly rounded IEEE forms (1/x and 1/sqrt(x)), which the GPU kernels and
 * the portable restatement (oracle/pfref.c) compute exactly.  Everything else
 * in the reference is compiled unmodified.
 */
#ifndef PF_ORACLE_REF_SHIM_H
#define PF_ORACLE_REF_SHIM_H

#include <immintrin.h>

#define _mm256_rcp_ps(x)   _mm256_div_ps(_mm256_set1_ps(1.0f), (x))
#define _mm256_rsqrt_ps(x) _mm256_div_ps(_mm256_set1_ps(1.0f), _mm256_sqrt_ps(x))
#define _mm_rcp_ps(x)      _mm_div_ps(_mm_set1_ps(1.0f), (x))
#define _mm_rsqrt_ps(x)    _mm_div_ps(_mm_set1_ps(1.0f), _mm_sqrt_ps(x))

#endif /* PF_ORACLE_REF_SHIM_H */
