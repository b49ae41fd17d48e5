/*
 * pf_pixfmt.h -- framebuffer pixel formats: the reference's pixel getters
 * and setters for the formats a framebuffer may have, on raw pixels.
 *
 * A framebuffer pixel is carried as its raw bytes, little-endian in four
 * 32-bit words (2 to 16 bytes).  Triangles read the destination through the
 * format's SIMD getter and write through its SIMD setter (one unmasked lane:
 * src/internal/primitives/triangles.c:378-379, 525-528); points, lines,
 * rectangles, pixel transfers, fog, post-processing and the framebuffer
 * functions use the scalar getter and setter (src/internal/pixel.h:52-760).
 *
 * Compiled by nvcc for the kernels and by the host compiler for what the
 * host does with framebuffer pixels (the clear values it precomputes, the
 * framebuffer functions, pfReadPixels, host post-processing); both follow
 * the reference's x86-64 build: CVTPS2DQ / CVTTSS2SI conversions, no fused
 * multiply-add.
 */
#ifndef PF_PIXFMT_H
#define PF_PIXFMT_H

#include <stdint.h>
#include <stddef.h>
#include <string.h>
#include <math.h>

#ifdef __CUDACC__
#define PFF_HD __host__ __device__ __forceinline__
#else
#define PFF_HD static inline
#endif

/* Framebuffer format codes (PFTarget.fmt). */
enum {
    PFF_RGBA8 = 0,
    PFF_RGB8, PFF_BGR8,
    PFF_RGB565, PFF_BGR565,
    PFF_RGBA5551, PFF_BGRA5551, PFF_RGBA4444, PFF_BGRA4444,
    PFF_LA16F, PFF_RGB16F, PFF_BGR16F, PFF_RGBA16F, PFF_BGRA16F,
    PFF_LA32F, PFF_RGB32F, PFF_BGR32F, PFF_RGBA32F, PFF_BGRA32F,
    PFF_BGRA8,                    /* BGRA / unsigned byte: see pff_swap_rb */
    PFF_COUNT
};

PFF_HD int pff_bytes(uint32_t f)
{
    switch (f) {
    case PFF_RGBA8: case PFF_BGRA8: return 4;
    case PFF_RGB8: case PFF_BGR8: return 3;
    case PFF_LA16F: return 4;
    case PFF_RGB16F: case PFF_BGR16F: return 6;
    case PFF_RGBA16F: case PFF_BGRA16F: case PFF_LA32F: return 8;
    case PFF_RGB32F: case PFF_BGR32F: return 12;
    case PFF_RGBA32F: case PFF_BGRA32F: return 16;
    default: return 2;                                    /* packed shorts */
    }
}

/* ------------------------------------------------------------------------ */
/* x86 conversions and the half-float maps of src/pfm.h                      */
/* ------------------------------------------------------------------------ */
PFF_HD uint32_t pff_fbits(float x) { uint32_t u; memcpy(&u, &x, 4); return u; }
PFF_HD float pff_bitsf(uint32_t u) { float x; memcpy(&x, &u, 4); return x; }

/* CVTPS2DQ: to nearest even; 0x80000000 for NaN and out of range */
PFF_HD uint32_t pff_cvt_rne(float x)
{
    if (!(x > -2147483648.0f && x < 2147483648.0f)) return 0x80000000u;
#ifdef __CUDA_ARCH__
    return (uint32_t)__float2int_rn(x);
#else
    return (uint32_t)(int32_t)nearbyintf(x);
#endif
}
/* (PFubyte)(float): truncation to int32 (0x80000000 out of range), low byte */
PFF_HD uint32_t pff_ftoub(float x)
{
    if (!(x > -2147483649.0f && x < 2147483648.0f)) return 0u;
    return (uint32_t)(int32_t)x & 255u;
}
/* pfmHalfToFloat (src/pfm.h:129-161): subnormal halves flush to zero */
PFF_HD float pff_half_to_float(uint32_t h)
{
    const uint32_t s = (h & 0x8000u) << 16;
    const int32_t em = (int32_t)(h & 0x7fffu);
    int32_t r = (int32_t)((uint32_t)(em + (112 << 10)) << 13);
    r = (em < (1 << 10)) ? 0 : r;
    r += (em >= (31 << 10)) ? (112 << 23) : 0;
    return pff_bitsf(s | (uint32_t)r);
}
/* pfmFloatToHalfI (src/pfm.h:108-126): the dropped bits round half up,
 * below 2^-14 flushes to zero, 2^16 and above is infinity, NaNs are quiet */
PFF_HD uint32_t pff_float_to_half(float x)
{
    const uint32_t ui = pff_fbits(x);
    const int s = (int)((ui >> 16) & 0x8000u);
    const int em = (int)(ui & 0x7fffffffu);
    int h = (em - (112 << 23) + (1 << 12)) >> 13;
    h = (em < (113 << 23)) ? 0 : h;
    h = (em >= (143 << 23)) ? 0x7c00 : h;
    h = (em > (255 << 23)) ? 0x7e00 : h;
    return (uint32_t)(s | h);
}

PFF_HD uint32_t pff_half(const uint32_t *r, int k) { return (r[k >> 1] >> (16 * (k & 1))) & 0xffffu; }
PFF_HD void pff_put_half(uint32_t *r, int k, uint32_t h)
{
    const int sh = 16 * (k & 1);
    r[k >> 1] = (r[k >> 1] & ~(0xffffu << sh)) | (h & 0xffffu) << sh;
}
PFF_HD int pff_is_half(uint32_t f) { return f >= PFF_LA16F && f <= PFF_BGRA16F; }
PFF_HD int pff_channels(uint32_t f)               /* half / float formats */
{
    switch (f) {
    case PFF_LA16F: case PFF_LA32F: return 2;
    case PFF_RGB16F: case PFF_BGR16F: case PFF_RGB32F: case PFF_BGR32F: return 3;
    default: return 4;
    }
}
/* channel k of a half / float pixel */
PFF_HD float pff_chan(uint32_t f, const uint32_t *r, int k)
{
    return pff_is_half(f) ? pff_half_to_float(pff_half(r, k)) : pff_bitsf(r[k]);
}
PFF_HD void pff_put_chan(uint32_t f, uint32_t *r, int k, float v)
{
    if (pff_is_half(f)) pff_put_half(r, k, pff_float_to_half(v));
    else r[k] = pff_fbits(v);
}

/* BGRA / unsigned byte: a pixel's bytes are B, G, R, A; every getter and
 * setter swaps R and B of the packed RGBA colour (pixel.h:356-363,
 * 703-707, 2070-2078, 2916-2921).  The SIMD pair does so with one shuffle
 * mask for the whole vector, which repeats the bytes of the first pixel of
 * each 4-pixel half (simd.h:564-583): a triangle writes the first pixel's
 * value to every pixel of the half its mask lets through.  That rule is the
 * rasterizer's (k_rows); one pixel's conversion is the swap. */
PFF_HD uint32_t pff_swap_rb(uint32_t w) { return (w & 0xff00ff00u) | ((w >> 16) & 255u) | ((w & 255u) << 16); }

/* ------------------------------------------------------------------------ */
/* raw pixels in memory                                                      */
/* ------------------------------------------------------------------------ */
/* Pixel i of a buffer of format f into r[0..3] (unused bytes 0).  Pixel
 * addresses are multiples of their size, so 2-, 4-, 8- and 16-byte pixels
 * load whole and 6- and 12-byte pixels as halves and words. */
PFF_HD void pff_load(uint32_t f, const void *base, size_t i, uint32_t *r)
{
    r[0] = r[1] = r[2] = r[3] = 0u;
    switch (pff_bytes(f)) {
    case 2: r[0] = ((const uint16_t *)base)[i]; break;
    case 3: {
        const uint8_t *p = (const uint8_t *)base + 3 * i;
        r[0] = (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16;
    } break;
    case 4: r[0] = ((const uint32_t *)base)[i]; break;
    case 6: {
        const uint16_t *p = (const uint16_t *)base + 3 * i;
        r[0] = (uint32_t)p[0] | (uint32_t)p[1] << 16; r[1] = p[2];
    } break;
    case 8: { const uint32_t *p = (const uint32_t *)base + 2 * i; r[0] = p[0]; r[1] = p[1]; } break;
    case 12: { const uint32_t *p = (const uint32_t *)base + 3 * i; r[0] = p[0]; r[1] = p[1]; r[2] = p[2]; } break;
    default: { const uint32_t *p = (const uint32_t *)base + 4 * i; r[0] = p[0]; r[1] = p[1]; r[2] = p[2]; r[3] = p[3]; } break;
    }
}
PFF_HD void pff_store(uint32_t f, void *base, size_t i, const uint32_t *r)
{
    switch (pff_bytes(f)) {
    case 2: ((uint16_t *)base)[i] = (uint16_t)r[0]; break;
    case 3: {
        uint8_t *p = (uint8_t *)base + 3 * i;
        p[0] = (uint8_t)r[0]; p[1] = (uint8_t)(r[0] >> 8); p[2] = (uint8_t)(r[0] >> 16);
    } break;
    case 4: ((uint32_t *)base)[i] = r[0]; break;
    case 6: {
        uint16_t *p = (uint16_t *)base + 3 * i;
        p[0] = (uint16_t)r[0]; p[1] = (uint16_t)(r[0] >> 16); p[2] = (uint16_t)r[1];
    } break;
    case 8: { uint32_t *p = (uint32_t *)base + 2 * i; p[0] = r[0]; p[1] = r[1]; } break;
    case 12: { uint32_t *p = (uint32_t *)base + 3 * i; p[0] = r[0]; p[1] = r[1]; p[2] = r[2]; } break;
    default: { uint32_t *p = (uint32_t *)base + 4 * i; p[0] = r[0]; p[1] = r[1]; p[2] = r[2]; p[3] = r[3]; } break;
    }
}

/* ------------------------------------------------------------------------ */
/* getters                                                                   */
/* ------------------------------------------------------------------------ */
/* The SIMD getter (src/internal/pixel.h:2253-3045): packed fields widened
 * by shifts (5551 alpha x255, 4444 x17), half / float channels
 * CVTPS2DQ(v * 255) with no clamp, RGB / BGR half and float read R first. */
PFF_HD uint32_t pff_get_simd(uint32_t f, const uint32_t *r)
{
    const uint32_t w = r[0];
    switch (f) {
    case PFF_RGBA8: return w;
    case PFF_BGRA8: return pff_swap_rb(w);
    case PFF_RGB8: return (w & 0xffffffu) | 0xff000000u;
    case PFF_BGR8: return ((w >> 16) & 255u) | (w & 0xff00u) | (w & 255u) << 16 | 0xff000000u;
    case PFF_RGB565: case PFF_BGR565: {
        const uint32_t hi = ((w & 0xf800u) >> 11) << 3, g = ((w & 0x07e0u) >> 5) << 2, lo = (w & 0x1fu) << 3;
        return f == PFF_RGB565 ? (0xff000000u | lo << 16 | g << 8 | hi) : (0xff000000u | hi << 16 | g << 8 | lo);
    }
    case PFF_RGBA5551: case PFF_BGRA5551: {
        const uint32_t c0 = ((w >> 11) & 0x1fu) * 8u, c1 = ((w >> 6) & 0x1fu) * 8u, c2 = ((w >> 1) & 0x1fu) * 8u, a = (w & 1u) * 255u;
        return f == PFF_RGBA5551 ? (a << 24 | c2 << 16 | c1 << 8 | c0) : (a << 24 | c0 << 16 | c1 << 8 | c2);
    }
    case PFF_RGBA4444: case PFF_BGRA4444: {
        const uint32_t c0 = ((w >> 12) & 0xfu) * 17u, c1 = ((w >> 8) & 0xfu) * 17u, c2 = ((w >> 4) & 0xfu) * 17u, a = (w & 0xfu) * 17u;
        return f == PFF_RGBA4444 ? (a << 24 | c2 << 16 | c1 << 8 | c0) : (a << 24 | c0 << 16 | c1 << 8 | c2);
    }
    default: break;
    }
    uint32_t c[4];
    const int n = pff_channels(f);
    for (int k = 0; k < n; k++) c[k] = pff_cvt_rne(pff_chan(f, r, k) * 255.0f);
    switch (f) {
    case PFF_LA16F: case PFF_LA32F: return c[1] << 24 | c[0] << 16 | c[0] << 8 | c[0];
    case PFF_RGB16F: case PFF_BGR16F: case PFF_RGB32F: case PFF_BGR32F: return 0xff000000u | c[2] << 16 | c[1] << 8 | c[0];
    case PFF_RGBA16F: case PFF_RGBA32F: return c[3] << 24 | c[2] << 16 | c[1] << 8 | c[0];
    default: return c[3] << 24 | c[0] << 16 | c[1] << 8 | c[2];                  /* BGRA */
    }
}

/* The scalar getter (src/internal/pixel.h:410-760): (PFubyte)(255 v) for
 * half / float channels, (PFubyte)(field * 255/(2^n - 1)) for packed ones;
 * BGR and BGRA of every type read B first. */
PFF_HD uint32_t pff_get_sisd(uint32_t f, const uint32_t *r)
{
    const uint32_t w = r[0];
    uint32_t cr = 0, cg = 0, cb = 0, ca = 255;
    switch (f) {
    case PFF_RGBA8: return w;
    case PFF_BGRA8: return pff_swap_rb(w);
    case PFF_RGB8: return (w & 0xffffffu) | 0xff000000u;
    case PFF_BGR8: return ((w >> 16) & 255u) | (w & 0xff00u) | (w & 255u) << 16 | 0xff000000u;
    case PFF_RGB565: case PFF_BGR565: {
        const uint32_t hi = pff_ftoub((float)((w & 0xF800u) >> 11) * (255.0f / 31));
        const uint32_t mid = pff_ftoub((float)((w & 0x7E0u) >> 5) * (255.0f / 63));
        const uint32_t lo = pff_ftoub((float)(w & 0x1Fu) * (255.0f / 31));
        cr = f == PFF_RGB565 ? hi : lo; cg = mid; cb = f == PFF_RGB565 ? lo : hi;
    } break;
    case PFF_RGBA5551: case PFF_BGRA5551: {
        const uint32_t hi = pff_ftoub((float)((w & 0xF800u) >> 11) * (255.0f / 31));
        const uint32_t mid = pff_ftoub((float)((w & 0x7C0u) >> 6) * (255.0f / 31));
        const uint32_t lo = pff_ftoub((float)((w & 0x3Eu) >> 1) * (255.0f / 31));
        cr = f == PFF_RGBA5551 ? hi : lo; cg = mid; cb = f == PFF_RGBA5551 ? lo : hi;
        ca = (w & 1u) * 255u;
    } break;
    case PFF_RGBA4444: case PFF_BGRA4444: {
        const uint32_t c3 = pff_ftoub((float)((w & 0xF000u) >> 12) * (255.0f / 15));
        const uint32_t c2 = pff_ftoub((float)((w & 0xF00u) >> 8) * (255.0f / 15));
        const uint32_t c1 = pff_ftoub((float)((w & 0xF0u) >> 4) * (255.0f / 15));
        ca = pff_ftoub((float)(w & 0xFu) * (255.0f / 15));
        cr = f == PFF_RGBA4444 ? c3 : c1; cg = c2; cb = f == PFF_RGBA4444 ? c1 : c3;
    } break;
    default: {
        uint32_t v[4] = { 0, 0, 0, 0 };
        const int n = pff_channels(f);
        for (int k = 0; k < n; k++) v[k] = pff_ftoub(255.0f * pff_chan(f, r, k));
        switch (f) {
        case PFF_LA16F: case PFF_LA32F: cr = cg = cb = v[0]; ca = v[1]; break;
        case PFF_RGB16F: case PFF_RGB32F: cr = v[0]; cg = v[1]; cb = v[2]; break;
        case PFF_BGR16F: case PFF_BGR32F: cr = v[2]; cg = v[1]; cb = v[0]; break;
        case PFF_RGBA16F: case PFF_RGBA32F: cr = v[0]; cg = v[1]; cb = v[2]; ca = v[3]; break;
        default: cr = v[2]; cg = v[1]; cb = v[0]; ca = v[3]; break;           /* BGRA */
        }
    } break;
    }
    return cr | cg << 8 | cb << 16 | ca << 24;
}

/* ------------------------------------------------------------------------ */
/* setters                                                                   */
/* ------------------------------------------------------------------------ */
/* The SIMD setter, one unmasked lane (src/internal/pixel.h:976-1090,
 * 1492-2250): channels to 5 / 6 / 4 bits by (c (2^n - 1)) >> 8, the 1-bit
 * alpha a > 127, half / float channels c * (1/255); BGR half / float keep R
 * first, BGR unsigned byte and BGRA of every type put B first; luminance
 * (77 r + 150 g + 29 b) >> 8 (src/internal/color.h:206-240). */
PFF_HD void pff_set_simd(uint32_t f, uint32_t col, uint32_t *r)
{
    const uint32_t cr = col & 255u, cg = (col >> 8) & 255u, cb = (col >> 16) & 255u, ca = col >> 24;
    const int bFirst = f == PFF_BGR8 || f == PFF_BGR565 || f == PFF_BGRA5551 || f == PFF_BGRA4444 ||
                       f == PFF_BGRA16F || f == PFF_BGRA32F;
    const uint32_t c0 = bFirst ? cb : cr, c2 = bFirst ? cr : cb;
    r[0] = r[1] = r[2] = r[3] = 0u;
    switch (f) {
    case PFF_RGBA8: r[0] = col; return;
    case PFF_BGRA8: r[0] = pff_swap_rb(col); return;
    case PFF_RGB8: case PFF_BGR8: r[0] = c0 | cg << 8 | c2 << 16; return;
    case PFF_RGB565: case PFF_BGR565: r[0] = ((c0 * 31u) >> 8) << 11 | ((cg * 63u) >> 8) << 5 | ((c2 * 31u) >> 8); return;
    case PFF_RGBA5551: case PFF_BGRA5551:
        r[0] = ((c0 * 31u) >> 8) << 11 | ((cg * 31u) >> 8) << 6 | ((c2 * 31u) >> 8) << 1 | (ca > 127u ? 1u : 0u);
        return;
    case PFF_RGBA4444: case PFF_BGRA4444:
        r[0] = ((c0 * 15u) >> 8) << 12 | ((cg * 15u) >> 8) << 8 | ((c2 * 15u) >> 8) << 4 | ((ca * 15u) >> 8);
        return;
    default: break;
    }
    const float inv = 1.0f / 255.0f;
    if (f == PFF_LA16F || f == PFF_LA32F) {
        const uint32_t gray = (cb * 29u + cg * 150u + cr * 77u) >> 8;
        pff_put_chan(f, r, 0, (float)(gray & 255u) * inv);
        pff_put_chan(f, r, 1, (float)ca * inv);
        return;
    }
    pff_put_chan(f, r, 0, (float)c0 * inv);
    pff_put_chan(f, r, 1, (float)cg * inv);
    pff_put_chan(f, r, 2, (float)c2 * inv);
    if (pff_channels(f) == 4) pff_put_chan(f, r, 3, (float)ca * inv);
}

/* The scalar setter (src/internal/pixel.h:52-405): channels normalised by
 * 1/255 and rounded (roundf) to packed fields, the 1-bit alpha a / 255 >
 * 50 / 255 in double; only BGR swaps R and B in the normalised colour (the
 * BGRA one keeps RGBA order, pixel.h:36-66), unsigned-byte BGR puts B first;
 * luminance 0.299 r + 0.587 g + 0.114 b of the normalised channels. */
PFF_HD void pff_set_sisd(uint32_t f, uint32_t col, uint32_t *r)
{
    const uint32_t cr = col & 255u, cg = (col >> 8) & 255u, cb = (col >> 16) & 255u, ca = col >> 24;
    const float inv = (float)(1.0 / 255);
    r[0] = r[1] = r[2] = r[3] = 0u;
    switch (f) {
    case PFF_RGBA8: r[0] = col; return;
    case PFF_BGRA8: r[0] = pff_swap_rb(col); return;
    case PFF_RGB8: r[0] = cr | cg << 8 | cb << 16; return;
    case PFF_BGR8: r[0] = cb | cg << 8 | cr << 16; return;
    default: break;
    }
    if (f == PFF_LA16F || f == PFF_LA32F) {
        const float gray = (float)cr * inv * 0.299f + (float)cg * inv * 0.587f + (float)cb * inv * 0.114f;
        pff_put_chan(f, r, 0, gray);
        pff_put_chan(f, r, 1, (float)ca * inv);
        return;
    }
    const int bgr = f == PFF_BGR565 || f == PFF_BGR16F || f == PFF_BGR32F;
    const float n0 = (float)(bgr ? cb : cr) * inv, n1 = (float)cg * inv, n2 = (float)(bgr ? cr : cb) * inv;
    const float n3 = (float)ca * inv;
    switch (f) {
    case PFF_RGB565: case PFF_BGR565:
        r[0] = (uint32_t)(uint8_t)roundf(n0 * 31.0f) << 11 | (uint32_t)(uint8_t)roundf(n1 * 63.0f) << 5 |
               (uint32_t)(uint8_t)roundf(n2 * 31.0f);
        return;
    case PFF_RGBA5551: case PFF_BGRA5551:
        r[0] = ((uint32_t)(uint8_t)roundf(n0 * 31.0f) << 11 | (uint32_t)(uint8_t)roundf(n1 * 31.0f) << 6 |
                (uint32_t)(uint8_t)roundf(n2 * 31.0f) << 1 | (((double)n3 > (double)(float)50 * (1.0 / 255)) ? 1u : 0u)) & 0xffffu;
        return;
    case PFF_RGBA4444: case PFF_BGRA4444:
        r[0] = ((uint32_t)(uint8_t)roundf(n0 * 15.0f) << 12 | (uint32_t)(uint8_t)roundf(n1 * 15.0f) << 8 |
                (uint32_t)(uint8_t)roundf(n2 * 15.0f) << 4 | (uint32_t)(uint8_t)roundf(n3 * 15.0f)) & 0xffffu;
        return;
    default: break;
    }
    pff_put_chan(f, r, 0, n0);
    pff_put_chan(f, r, 1, n1);
    pff_put_chan(f, r, 2, n2);
    if (pff_channels(f) == 4) pff_put_chan(f, r, 3, n3);
}

#endif /* PF_PIXFMT_H */
