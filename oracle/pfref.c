/*
 * pfref.c -- CPU ORACLE for the PixelForge triangle pipeline.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the smoke
 * check and bench.py's CPU-baseline leg load it; the product never does.
 *
 * It is a plain-C restatement (portable: x86-64 and aarch64, no intrinsics)
 * of the reference's barycentric AVX2 path, evaluated one pixel at a time,
 * exporting the same pf* API (include/pixelforge.h) so that one scene driver
 * can run the reference build, this oracle and the GPU library alike.
 * Each function cites the reference lines it restates.  Floating-point
 * expressions keep the reference's operation order; the Makefile builds it
 * with -ffp-contract=off so that no multiply-add is fused (the reference is
 * compiled for AVX2 without FMA, CMakeLists.txt:44-47).
 *
 * Pinned semantics where the reference is not reproducible:
 *   - depth and Phong use exact 1/x and 1/sqrt(x) where the reference uses
 *     the approximate rcp/rsqrt instructions (src/internal/simd.h:1218-1245);
 *     the reference "shim" build (oracle/ref_shim.h) makes the same choice and
 *     this oracle is checked bit-exactly against it;
 *   - the bilinear colour lerp reads an uninitialised vector in the reference
 *     (src/internal/color.h:138-144); here both endpoints are loaded, i.e.
 *     lerp(a, b, t) per channel on 1/255-normalised floats;
 *   - pfDepthMask (extension) gates the depth write; the reference always
 *     writes depth (src/internal/primitives/triangles.c:529);
 *   - a texel whose linear offset y*w+x falls outside the texture reads as 0
 *     (the reference reads past its buffer: its SIMD mirrored and clamped
 *     maps round a coordinate of exactly 1.0 to row h,
 *     src/internal/sampler.h:222-258).
 * Framebuffer formats: see fb_format_ok.
 */
#include "pixelforge.h"
#include "pfref_internal.h"

#include <float.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>
#include <math.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define REF_PI 3.14159265358979323846
#define REF_DEG2RAD (REF_PI / 180.0)
#define CLIP_EPS 1e-5f
#define MAX_LIGHTS 8
#define MAX_POLY 12

typedef float mat4[16];

/* ------------------------------------------------------------------------ */
/* objects                                                                   */
/* ------------------------------------------------------------------------ */

typedef struct {
    void *pixels;
    PFpixelformat format;
    PFdatatype type;
    PFsizei w, h;
    float tx, ty;
    PFtexturewrap wrap;
    PFtexturefilter filter;
} RTex;

typedef struct {
    float position[3];
    float direction[3];
    float innerCutOff, outerCutOff;
    float attConstant, attLinear, attQuadratic;
    PFcolor ambient, diffuse, specular;
    int active;
} RLight;

typedef struct {
    PFcolor ambient, diffuse, specular, emission;
    float shininess;
} RMat;

typedef struct {
    float homogeneous[4];
    float screen[2];
    float position[4];
    float normal[3];
    float texcoord[2];
    PFcolor color;
} RVert;

typedef struct { const void *buf; PFsizei stride; PFint size; PFenum type; } RAttrib;

typedef struct {
    PFframebuffer main;
    PFframebuffer *current;
    PFframebuffer *bound;
    RTex *texture;
    void *aux;

    PFint vpPos[2]; PFsizei vpDim[2]; PFint vpMin[2]; PFint vpMax[2];

    RAttrib positions, normals, colors, texcoords;
    RVert vbuf[6];
    PFsizei vcount;
    float curNormal[3]; float curTex[2]; PFcolor curColor;

    PFcolor clearColor; float clearDepth;
    PFdrawmode drawMode;
    PFpolygonmode polygonMode[2];
    RMat mat[2];
    PFface colMatFace; PFenum colMatMode;
    RLight lights[MAX_LIGHTS];
    int lightOrder[MAX_LIGHTS]; int nActive;   /* active list, in insertion order */

    mat4 proj, tex, model, view, mvp, normal;
    mat4 stackProj[2], stackMV[8], stackTex[4];
    PFsizei nProj, nMV, nTex;
    PFmatrixmode matMode; int modelUsed;
    float *cur;

    PFshademode shade; PFlightmode lightMode; PFface cullFace;
    PFblendmode blend; PFdepthmode depthFunc;
    PFerrcode err; PFuint state;
    PFboolean depthMask;
    float pointSize, lineWidth;
    float rasterPos[4]; float pixelZoom[2];
    struct { uint32_t mode; float density, start, end; PFcolor color; } fog;
    struct RList *curList;             /* render list being recorded, or NULL */
    struct { RMat mat[2]; float tex[2]; float nrm[3]; PFcolor col; RTex *texture; PFuint state; } backup;
    PFstats stats;
} RCtx;

/* Render lists (src/renderlist.c): per pfBegin, the draw mode, both
 * materials, the texture, and per vertex its position, texcoord, normal and
 * colour as they were current. */
typedef struct {
    PFdrawmode mode;
    RMat mat[2];
    RTex *texture;
    float (*pos)[4]; float (*uv)[2]; float (*nrm)[3]; PFcolor *col;
    size_t n, cap;
} RCall;
typedef struct RList { RCall *calls; size_t n, cap; } RList;

static RCtx *G = NULL;   /* current context (one per process, as in GCC+OpenMP builds) */

/* ------------------------------------------------------------------------ */
/* pfm.h math in the reference's operation order                             */
/* ------------------------------------------------------------------------ */

static void m_identity(float *d) { memset(d, 0, 64); d[0] = d[5] = d[10] = d[15] = 1.0f; }

/* pfmMat4Mul (src/pfm.h:2176-2199): result[i*4+j] = sum_k left[i*4+k]*right[k*4+j] */
static void m_mul(float *dst, const float *l, const float *r)
{
    float res[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            float s = 0.0f;
            for (int k = 0; k < 4; k++) s += l[i * 4 + k] * r[k * 4 + j];
            res[i * 4 + j] = s;
        }
    memcpy(dst, res, 64);
}

/* pfmMat4Invert (src/pfm.h:2082-2121) */
static void m_invert(float *dst, const float *s)
{
    float a00 = s[0], a01 = s[1], a02 = s[2], a03 = s[3];
    float a10 = s[4], a11 = s[5], a12 = s[6], a13 = s[7];
    float a20 = s[8], a21 = s[9], a22 = s[10], a23 = s[11];
    float a30 = s[12], a31 = s[13], a32 = s[14], a33 = s[15];
    float b00 = a00*a11 - a01*a10, b01 = a00*a12 - a02*a10, b02 = a00*a13 - a03*a10;
    float b03 = a01*a12 - a02*a11, b04 = a01*a13 - a03*a11, b05 = a02*a13 - a03*a12;
    float b06 = a20*a31 - a21*a30, b07 = a20*a32 - a22*a30, b08 = a20*a33 - a23*a30;
    float b09 = a21*a32 - a22*a31, b10 = a21*a33 - a23*a31, b11 = a22*a33 - a23*a32;
    float invDet = 1.0f/(b00*b11 - b01*b10 + b02*b09 + b03*b08 - b04*b07 + b05*b06);
    float d[16];
    d[0] = (a11*b11 - a12*b10 + a13*b09)*invDet;
    d[1] = (-a01*b11 + a02*b10 - a03*b09)*invDet;
    d[2] = (a31*b05 - a32*b04 + a33*b03)*invDet;
    d[3] = (-a21*b05 + a22*b04 - a23*b03)*invDet;
    d[4] = (-a10*b11 + a12*b08 - a13*b07)*invDet;
    d[5] = (a00*b11 - a02*b08 + a03*b07)*invDet;
    d[6] = (-a30*b05 + a32*b02 - a33*b01)*invDet;
    d[7] = (a20*b05 - a22*b02 + a23*b01)*invDet;
    d[8] = (a10*b10 - a11*b08 + a13*b06)*invDet;
    d[9] = (-a00*b10 + a01*b08 - a03*b06)*invDet;
    d[10] = (a30*b04 - a31*b02 + a33*b00)*invDet;
    d[11] = (-a20*b04 + a21*b02 - a23*b00)*invDet;
    d[12] = (-a10*b09 + a11*b07 - a12*b06)*invDet;
    d[13] = (a00*b09 - a01*b07 + a02*b06)*invDet;
    d[14] = (-a30*b03 + a31*b01 - a32*b00)*invDet;
    d[15] = (a20*b03 - a21*b01 + a22*b00)*invDet;
    memcpy(dst, d, 64);
}

static void m_transpose(float *dst, const float *s)
{
    float r[16];
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) r[i * 4 + j] = s[j * 4 + i];
    memcpy(dst, r, 64);
}

/* pfmVec4Transform (src/pfm.h:1996-2006) */
static void v4_transform(float *dst, const float *v, const float *m)
{
    float t[4] = {
        m[0]*v[0] + m[4]*v[1] + m[8]*v[2] + m[12]*v[3],
        m[1]*v[0] + m[5]*v[1] + m[9]*v[2] + m[13]*v[3],
        m[2]*v[0] + m[6]*v[1] + m[10]*v[2] + m[14]*v[3],
        m[3]*v[0] + m[7]*v[1] + m[11]*v[2] + m[15]*v[3] };
    memcpy(dst, t, 16);
}

/* pfmVec3Transform (src/pfm.h:1507-1516) */
static void v3_transform(float *dst, const float *v, const float *m)
{
    float t[3] = {
        m[0]*v[0] + m[4]*v[1] + m[8]*v[2] + m[12],
        m[1]*v[0] + m[5]*v[1] + m[9]*v[2] + m[13],
        m[2]*v[0] + m[6]*v[1] + m[10]*v[2] + m[14] };
    memcpy(dst, t, 12);
}

/* pfmVec3Normalize (src/pfm.h:1183-1197): rsqrtf is 1.0f/sqrtf (src/pfm.h:30-31) */
static void v3_normalize(float *v)
{
    float sq = v[0]*v[0] + v[1]*v[1] + v[2]*v[2];
    if (sq == 0.0f) return;
    float inv = 1.0f / sqrtf(sq);
    for (int i = 0; i < 3; i++) v[i] = v[i] * inv;
}

static float v3_dot(const float *a, const float *b) { return a[0]*b[0] + a[1]*b[1] + a[2]*b[2]; }

/* pfmVec3DirectionR (src/pfm.h:1322-1342) */
static void v3_direction(float *dst, const float *a, const float *b)
{
    float lsq = 0.0f;
    for (int i = 0; i < 3; i++) { dst[i] = a[i] - b[i]; lsq += dst[i]*dst[i]; }
    float inv = 1.0f / sqrtf(lsq);
    for (int i = 0; i < 3; i++) dst[i] = dst[i] * inv;
}

/* ------------------------------------------------------------------------ */
/* scalar colour helpers                                                     */
/* ------------------------------------------------------------------------ */

static inline uint32_t col_pack(PFcolor c) { uint32_t u; memcpy(&u, &c, 4); return u; }
static inline PFcolor col_unpack(uint32_t u) { PFcolor c; memcpy(&c, &u, 4); return c; }
#define MIN255(n) ((uint8_t)(((int32_t)(n)) | ((255 - (int32_t)(n)) >> 31)))

/* pfiBlendMultiplicative, scalar (src/internal/blend.h:77-86) */
static PFcolor blend_mul_scalar(PFcolor s, PFcolor d)
{
    PFcolor r = { (uint8_t)((s.r*d.r)/255), (uint8_t)((s.g*d.g)/255),
                  (uint8_t)((s.b*d.b)/255), (uint8_t)((s.a*d.a)/255) };
    return r;
}

/* Channel i of a packed SIMD colour; packing ORs without masks
 * (src/internal/color.h:66-71 and 112-121). */
static inline int32_t ch(uint32_t p, int i) { return (int32_t)((p >> (8 * i)) & 255u); }
static inline uint32_t pack4(const int32_t *v)
{
    uint32_t r = 0;
    for (int i = 0; i < 4; i++) r |= ((uint32_t)v[i]) << (8 * i);
    return r;
}

/* SIMD blend functions (src/internal/blend.h:140-277), one lane. */
static uint32_t blend_simd(PFblendmode mode, uint32_t src, uint32_t dst)
{
    int32_t s[4], d[4], o[4];
    for (int i = 0; i < 4; i++) { s[i] = ch(src, i); d[i] = ch(dst, i); }
    switch (mode) {
    case PF_BLEND_AVERAGE: for (int i = 0; i < 4; i++) o[i] = (int32_t)((uint32_t)(s[i] + d[i]) >> 1); break;
    case PF_BLEND_ALPHA: {
        int32_t a = s[3] + 1, ia = 256 - a;
        for (int i = 0; i < 3; i++) o[i] = (int32_t)((uint32_t)(s[i]*a + d[i]*ia) >> 8);
        o[3] = (int32_t)((uint32_t)(255*a + d[3]*ia) >> 8);
    } break;
    case PF_BLEND_ADD: for (int i = 0; i < 4; i++) { int32_t t = s[i] + d[i]; o[i] = t < 255 ? t : 255; } break;
    case PF_BLEND_SUB: for (int i = 0; i < 4; i++) { int32_t t = s[i] + d[i]; o[i] = t > 0 ? t : 0; } break;
    case PF_BLEND_MUL: for (int i = 0; i < 4; i++) o[i] = (int32_t)((uint32_t)(s[i]*d[i]) >> 8); break;
    case PF_BLEND_SCREEN: for (int i = 0; i < 4; i++) {
        int32_t t = (int32_t)((uint32_t)(d[i]*(255 - s[i])) >> 8) + s[i]; o[i] = t < 255 ? t : 255; } break;
    case PF_BLEND_LIGHTEN: for (int i = 0; i < 4; i++) o[i] = s[i] > d[i] ? s[i] : d[i]; break;
    case PF_BLEND_DARKEN: for (int i = 0; i < 4; i++) o[i] = s[i] < d[i] ? s[i] : d[i]; break;
    default: return src;
    }
    return pack4(o);
}

/* SIMD depth tests (src/internal/depth.h:80-124); NOTEQUAL compares equal there. */
static inline int depth_simd(PFdepthmode m, float src, float dst)
{
    switch (m) {
    case PF_EQUAL: case PF_NOTEQUAL: return src == dst;
    case PF_LESS: return src < dst;
    case PF_LEQUAL: return src <= dst;
    case PF_GREATER: return src > dst;
    case PF_GEQUAL: return src >= dst;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* texture sampling, SIMD semantics (src/internal/sampler.h:203-420)          */
/* ------------------------------------------------------------------------ */

static const float INV255 = 1.0f / 255.0f;

static void map_repeat(const RTex *t, float u, float v, int32_t *x, int32_t *y)
{
    u = (u - truncf(u)) * (float)(t->w - 1);
    v = (v - truncf(v)) * (float)(t->h - 1);
    *x = ox_iabs(ox_cvt_rne(u));
    *y = ox_iabs(ox_cvt_rne(v));
}

static inline float mod2(float x)   /* pfiSimdMod_F32 (src/internal/simd.h:1182-1195) */
{
    float q = x / 2.0f;
    float f = floorf(q);
    return x - f * 2.0f;
}

static void map_mirror(const RTex *t, float u, float v, int32_t *x, int32_t *y)
{
    u = mod2(fabsf(u));
    v = mod2(fabsf(v));
    float um = 1.0f - (u - 1.0f), vm = 1.0f - (v - 1.0f);
    u = (u > 1.0f) ? um : u;
    v = (v > 1.0f) ? vm : v;
    u = u * (float)(t->w - 1);
    v = v * (float)(t->h - 1);
    *x = ox_cvt_rne(u + 0.5f);
    *y = ox_cvt_rne(v + 0.5f);
}

static void map_clamp(const RTex *t, float u, float v, int32_t *x, int32_t *y)
{
    u = ox_min(ox_max(u, 0.0f), 1.0f) * (float)(t->w - 1);
    v = ox_min(ox_max(v, 0.0f), 1.0f) * (float)(t->h - 1);
    *x = ox_cvt_rne(u + 0.5f);
    *y = ox_cvt_rne(v + 0.5f);
}

static void tex_map(const RTex *t, float u, float v, int32_t *x, int32_t *y)
{
    switch (t->wrap) {
    case PF_REPEAT: map_repeat(t, u, v, x, y); break;
    case PF_MIRRORED_REPEAT: map_mirror(t, u, v, x, y); break;
    default: map_clamp(t, u, v, x, y); break;
    }
}

/* ------------------------------------------------------------------------ */
/* texel formats: the SIMD pixel getters (src/internal/pixel.h:2253-3045)     */
/* ------------------------------------------------------------------------ */

/* Bytes of one texel of a sampling format, 0 when the reference has no SIMD
 * getter for the combination (src/internal/pixel.h:3046-3097). */
static int texel_bytes(PFpixelformat f, PFdatatype t)
{
    int comps;
    switch (f) {
    case PF_RED: case PF_GREEN: case PF_BLUE: case PF_ALPHA: case PF_LUMINANCE: comps = 1; break;
    case PF_LUMINANCE_ALPHA: comps = 2; break;
    case PF_RGB: case PF_BGR: comps = 3; break;
    case PF_RGBA: case PF_BGRA: comps = 4; break;
    default: return 0;
    }
    switch (t) {
    case PF_UNSIGNED_BYTE: return comps;
    case PF_HALF_FLOAT: return 2 * comps;
    case PF_FLOAT: return 4 * comps;
    case PF_UNSIGNED_SHORT_5_6_5: return (f == PF_RGB || f == PF_BGR) ? 2 : 0;
    case PF_UNSIGNED_SHORT_5_5_5_1: case PF_UNSIGNED_SHORT_4_4_4_4: return (f == PF_RGBA || f == PF_BGRA) ? 2 : 0;
    default: return 0;
    }
}

/* Byte b of the texture buffer; bytes past its end read 0 (the reference's
 * 32-bit gathers read past the buffer). */
static inline uint32_t tbyte(const RTex *t, int64_t b)
{
    const int64_t n = (int64_t)t->w * t->h * texel_bytes(t->format, t->type);
    return (b >= 0 && b < n) ? ((const uint8_t *)t->pixels)[b] : 0u;
}
static inline uint32_t tword(const RTex *t, int64_t b)   /* little-endian 32-bit gather */
{
    return tbyte(t, b) | tbyte(t, b + 1) << 8 | tbyte(t, b + 2) << 16 | tbyte(t, b + 3) << 24;
}
/* pfmHalfToFloat (src/pfm.h:129-161): denormals flush to zero */
static inline float half_to_float(uint32_t h)
{
    uint32_t s = (h & 0x8000u) << 16;
    int32_t em = (int32_t)(h & 0x7fffu);
    int32_t r = (int32_t)((uint32_t)(em + (112 << 10)) << 13);
    r = (em < (1 << 10)) ? 0 : r;
    r += (em >= (31 << 10)) ? (112 << 23) : 0;
    return ox_bitsf(s | (uint32_t)r);
}
static inline uint32_t h8(const RTex *t, int64_t halfIndex)      /* cvt(half * 255) */
{
    return (uint32_t)ox_cvt_rne(half_to_float(tword(t, 2 * halfIndex) & 0xffffu) * 255.0f);
}
static inline uint32_t f8(const RTex *t, int64_t floatIndex)     /* cvt(float * 255) */
{
    return (uint32_t)ox_cvt_rne(ox_bitsf(tword(t, 4 * floatIndex)) * 255.0f);
}

/* RGBA8 value the reference's SIMD getter returns for texel o. */
static uint32_t texel_rgba8(const RTex *t, int64_t o)
{
    const PFpixelformat f = t->format;
    switch (t->type) {
    case PF_UNSIGNED_BYTE:
        switch (f) {
        case PF_RED: return (tword(t, o) >> 24) | 0xff000000u;           /* the gather's top byte: texel o+3 */
        case PF_GREEN: return ((tword(t, o) >> 24) << 8) | 0xff000000u;
        case PF_BLUE: return ((tword(t, o) >> 24) << 16) | 0xff000000u;
        case PF_ALPHA: return tword(t, o) << 24;
        case PF_LUMINANCE: { uint32_t v = tword(t, o) >> 24; return v | v << 8 | v << 16 | 0xff000000u; }
        case PF_LUMINANCE_ALPHA: {                                         /* bytes 2o+2, 2o+3: texel o+1 */
            uint32_t w = tword(t, 2 * o), l = (w >> 16) & 255u, a = w >> 24;
            return l | l << 8 | l << 16 | a << 24;
        }
        case PF_RGB: { uint32_t w = tword(t, 3 * o); return (w & 0xffffffu) | 0xff000000u; }
        case PF_BGR: { uint32_t w = tword(t, 3 * o); return ((w >> 16) & 255u) | (w & 0xff00u) | (w & 255u) << 16 | 0xff000000u; }
        case PF_RGBA: return tword(t, 4 * o);
        case PF_BGRA: { uint32_t w = tword(t, 4 * o); return ((w >> 16) & 255u) | (w & 0xff00u) | (w & 255u) << 16 | (w & 0xff000000u); }
        default: return 0;
        }
    case PF_HALF_FLOAT:
        switch (f) {
        case PF_RED: return h8(t, o) | 0xff000000u;
        case PF_GREEN: return h8(t, o) << 8 | 0xff000000u;
        case PF_BLUE: return h8(t, o) << 16 | 0xff000000u;
        case PF_ALPHA: return h8(t, o) << 24;
        case PF_LUMINANCE: { uint32_t v = h8(t, o); return 0xff000000u | v << 16 | v << 8 | v; }
        case PF_LUMINANCE_ALPHA: { uint32_t v = h8(t, 2 * o), a = h8(t, 2 * o + 1); return a << 24 | v << 16 | v << 8 | v; }
        case PF_RGB: return 0xff000000u | h8(t, 3 * o + 2) << 16 | h8(t, 3 * o + 1) << 8 | h8(t, 3 * o);
        case PF_BGR: return 0xff000000u | h8(t, 3 * o + 2) << 16 | h8(t, 3 * o + 1) << 8 | h8(t, 3 * o);
        case PF_RGBA: return h8(t, 4 * o + 3) << 24 | h8(t, 4 * o + 2) << 16 | h8(t, 4 * o + 1) << 8 | h8(t, 4 * o);
        case PF_BGRA: return h8(t, 4 * o + 3) << 24 | h8(t, 4 * o) << 16 | h8(t, 4 * o + 1) << 8 | h8(t, 4 * o + 2);
        default: return 0;
        }
    case PF_FLOAT:
        switch (f) {
        case PF_RED: return f8(t, o) | 0xff000000u;
        case PF_GREEN: return f8(t, o) << 8 | 0xff000000u;
        case PF_BLUE: return f8(t, o) << 16 | 0xff000000u;
        case PF_ALPHA: return f8(t, o) << 24;
        case PF_LUMINANCE: { uint32_t v = f8(t, o); return 0xff000000u | v << 16 | v << 8 | v; }
        case PF_LUMINANCE_ALPHA: { uint32_t v = f8(t, 2 * o), a = f8(t, 2 * o + 1); return a << 24 | v << 16 | v << 8 | v; }
        case PF_RGB: return 0xff000000u | f8(t, 3 * o + 2) << 16 | f8(t, 3 * o + 1) << 8 | f8(t, 3 * o);
        case PF_BGR: return 0xff000000u | f8(t, 3 * o + 2) << 16 | f8(t, 3 * o + 1) << 8 | f8(t, 3 * o);
        case PF_RGBA: return f8(t, 4 * o + 3) << 24 | f8(t, 4 * o + 2) << 16 | f8(t, 4 * o + 1) << 8 | f8(t, 4 * o);
        case PF_BGRA: return f8(t, 4 * o + 3) << 24 | f8(t, 4 * o) << 16 | f8(t, 4 * o + 1) << 8 | f8(t, 4 * o + 2);
        default: return 0;
        }
    case PF_UNSIGNED_SHORT_5_6_5: {
        uint32_t w = tword(t, 2 * o);
        uint32_t hi = ((w & 0xf800u) >> 11) << 3, g = ((w & 0x07e0u) >> 5) << 2, lo = (w & 0x1fu) << 3;
        return (f == PF_RGB) ? (0xff000000u | lo << 16 | g << 8 | hi) : (0xff000000u | hi << 16 | g << 8 | lo);
    }
    case PF_UNSIGNED_SHORT_5_5_5_1: {
        uint32_t w = tword(t, 2 * o);
        uint32_t c0 = ((w >> 11) & 0x1fu) * 8u, c1 = ((w >> 6) & 0x1fu) * 8u, c2 = ((w >> 1) & 0x1fu) * 8u, a = (w & 1u) * 255u;
        return (f == PF_RGBA) ? (a << 24 | c2 << 16 | c1 << 8 | c0) : (a << 24 | c0 << 16 | c1 << 8 | c2);
    }
    case PF_UNSIGNED_SHORT_4_4_4_4: {
        uint32_t w = tword(t, 2 * o);
        uint32_t c0 = ((w >> 12) & 0xfu) * 17u, c1 = ((w >> 8) & 0xfu) * 17u, c2 = ((w >> 4) & 0xfu) * 17u, a = (w & 0xfu) * 17u;
        return (f == PF_RGBA) ? (a << 24 | c2 << 16 | c1 << 8 | c0) : (a << 24 | c0 << 16 | c1 << 8 | c2);
    }
    default: return 0;
    }
}

/* ------------------------------------------------------------------------ */
/* framebuffer formats                                                       */
/* ------------------------------------------------------------------------ */

static uint32_t pixel_sisd(PFpixelformat f, PFdatatype t, const void *p, size_t o);
static void pixel_set_sisd(PFpixelformat f, PFdatatype t, void *dst, size_t o, uint32_t col);
static uint16_t float_to_half(float x);

/* Formats a framebuffer may have.  The reference draws triangles through
 * the framebuffer format's SIMD getter and setter (triangles.c:378-379,
 * 525-528) and everything else through the scalar ones.  Refused, because
 * one pixel's result would depend on other pixels or on its SIMD lane:
 * single-channel and luminance(-alpha) unsigned byte (their SIMD getters
 * read the texel three places on, or the next texel, pixel.h:2253-2420),
 * single-channel and luminance half / float (their SIMD setters rewrite,
 * requantised, the pixels of the vector that the mask leaves out,
 * pixel.h:905-970, 1219-1490).  BGRA unsigned byte, whose SIMD getter and
 * setter shuffle a half vector with its first pixel's bytes, is accepted:
 * raster_tri follows the halves. */
static int fb_format_ok(PFpixelformat f, PFdatatype t)
{
    if (!texel_bytes(f, t)) return 0;
    switch (f) {
    case PF_RGB: case PF_BGR: case PF_RGBA: case PF_BGRA: return 1;
    case PF_LUMINANCE_ALPHA: return t == PF_HALF_FLOAT || t == PF_FLOAT;
    default: return 0;
    }
}
static inline int fb_rgba8(const RTex *t) { return t->format == PF_RGBA && t->type == PF_UNSIGNED_BYTE; }
static inline int fb_bgra8(const RTex *t) { return t->format == PF_BGRA && t->type == PF_UNSIGNED_BYTE; }

/* Destination colour as the SIMD getter reads it (blending of triangles). */
static inline uint32_t fb_get_simd(const RTex *t, size_t o)
{
    return fb_rgba8(t) ? ((const uint32_t *)t->pixels)[o] : texel_rgba8(t, (int64_t)o);
}

/* The SIMD setter writing one unmasked lane (pixel.h:976-1090, 1492-2250):
 * 8-bit channels to 5/6/4 bits by (c * (2^n - 1)) >> 8, the 1-bit alpha
 * a > 127, half / float channels c * (1/255) (BGR half / float keep R first,
 * BGR unsigned byte and BGRA of every type put B first), luminance
 * (77 r + 150 g + 29 b) >> 8 (color.h:206-240). */
static void fb_set_simd(RTex *t, size_t o, uint32_t col)
{
    if (fb_rgba8(t)) { ((uint32_t *)t->pixels)[o] = col; return; }
    const uint32_t r = col & 255u, g = (col >> 8) & 255u, b = (col >> 16) & 255u, a = col >> 24;
    uint8_t *p8 = (uint8_t *)t->pixels;
    uint16_t *p16 = (uint16_t *)t->pixels;
    float *pf = (float *)t->pixels;
    const PFpixelformat f = t->format;
    const int bFirst = f == PF_BGRA || (f == PF_BGR && (t->type == PF_UNSIGNED_BYTE ||
                                                        t->type == PF_UNSIGNED_SHORT_5_6_5));
    const uint32_t c0 = bFirst ? b : r, c2 = bFirst ? r : b;
    switch (t->type) {
    case PF_UNSIGNED_SHORT_5_6_5:
        p16[o] = (uint16_t)(((c0 * 31u) >> 8) << 11 | ((g * 63u) >> 8) << 5 | ((c2 * 31u) >> 8));
        return;
    case PF_UNSIGNED_SHORT_5_5_5_1:
        p16[o] = (uint16_t)(((c0 * 31u) >> 8) << 11 | ((g * 31u) >> 8) << 6 | ((c2 * 31u) >> 8) << 1 | (a > 127u ? 1u : 0u));
        return;
    case PF_UNSIGNED_SHORT_4_4_4_4:
        p16[o] = (uint16_t)(((c0 * 15u) >> 8) << 12 | ((g * 15u) >> 8) << 8 | ((c2 * 15u) >> 8) << 4 | ((a * 15u) >> 8));
        return;
    case PF_UNSIGNED_BYTE:                                  /* RGB, BGR, BGRA */
        if (f == PF_BGRA) {
            p8[4 * o] = (uint8_t)b; p8[4 * o + 1] = (uint8_t)g; p8[4 * o + 2] = (uint8_t)r; p8[4 * o + 3] = (uint8_t)a;
            return;
        }
        p8[3 * o] = (uint8_t)c0; p8[3 * o + 1] = (uint8_t)g; p8[3 * o + 2] = (uint8_t)c2;
        return;
    default: break;
    }
    float n[4];
    int k;
    if (f == PF_LUMINANCE_ALPHA) {
        const uint32_t gray = (b * 29u + g * 150u + r * 77u) >> 8;
        n[0] = (float)(gray & 255u) * INV255; n[1] = (float)a * INV255; k = 2;
    } else {
        n[0] = (float)c0 * INV255; n[1] = (float)g * INV255; n[2] = (float)c2 * INV255; n[3] = (float)a * INV255;
        k = (f == PF_RGB || f == PF_BGR) ? 3 : 4;
    }
    for (int i = 0; i < k; i++) {
        if (t->type == PF_HALF_FLOAT) p16[(size_t)k * o + (size_t)i] = float_to_half(n[i]);
        else pf[(size_t)k * o + (size_t)i] = n[i];
    }
}

/* The scalar getter and setter (points, lines, rectangles, pixel
 * transfers, fog, post-processing, the framebuffer functions). */
static inline uint32_t fb_get(const RTex *t, size_t o)
{
    return fb_rgba8(t) ? ((const uint32_t *)t->pixels)[o] : pixel_sisd(t->format, t->type, t->pixels, o);
}
static inline void fb_set(RTex *t, size_t o, uint32_t col)
{
    if (fb_rgba8(t)) ((uint32_t *)t->pixels)[o] = col;
    else pixel_set_sisd(t->format, t->type, t->pixels, o, col);
}

static uint32_t tex_fetch(const RTex *t, int32_t x, int32_t y)
{
    int64_t off = (int64_t)(int32_t)((uint32_t)y * t->w + (uint32_t)x);
    /* The reference reads past the texture buffer here (mirrored or clamped
     * coordinates of exactly 1.0 round to row h); pinned to 0. */
    if (off < 0 || off >= (int64_t)t->w * t->h) return 0;
    if (t->format == PF_RGBA && t->type == PF_UNSIGNED_BYTE) return ((const uint32_t *)t->pixels)[off];
    return texel_rgba8(t, off);
}

/* Colour lerp with both endpoints defined (see header). */
static uint32_t lerp_color(uint32_t a, uint32_t b, float t)
{
    int32_t o[4];
    for (int i = 0; i < 4; i++) {
        float af = (float)ch(a, i) * INV255;
        float bf = (float)ch(b, i) * INV255;
        float r = af + t * (bf - af);
        o[i] = ox_cvt_rne(ox_min(ox_max(r, 0.0f), 1.0f) * 255.0f);
    }
    return pack4(o);
}

static uint32_t tex_sample(const RTex *t, float u, float v)
{
    int32_t x0, y0;
    tex_map(t, u, v, &x0, &y0);
    if (t->filter == PF_NEAREST) return tex_fetch(t, x0, y0);
    int32_t x1, y1;
    tex_map(t, u + t->tx, v + t->ty, &x1, &y1);
    float fx = u * (float)t->w - (float)x0;
    float fy = v * (float)t->h - (float)y0;
    fx = ox_min(ox_max(fx, 0.0f), 1.0f);
    fy = ox_min(ox_max(fy, 0.0f), 1.0f);
    uint32_t c00 = tex_fetch(t, x0, y0), c10 = tex_fetch(t, x1, y0);
    uint32_t c01 = tex_fetch(t, x0, y1), c11 = tex_fetch(t, x1, y1);
    uint32_t c0 = lerp_color(c00, c10, fx);
    uint32_t c1 = lerp_color(c01, c11, fx);
    return lerp_color(c0, c1, fy);
}

/* ------------------------------------------------------------------------ */
/* lighting                                                                  */
/* ------------------------------------------------------------------------ */

/* pfiLightingProcess (src/internal/lighting/lighting.c:24-134), Blinn-Phong. */
static PFcolor light_gouraud(const RCtx *c, const RMat *m, PFcolor diffuse,
                             const float *viewPos, const float *P, const float *N)
{
    uint8_t R = m->emission.r, Gc = m->emission.g, B = m->emission.b;
    uint8_t aR = (uint8_t)((m->ambient.r*diffuse.r)/255);
    uint8_t aG = (uint8_t)((m->ambient.g*diffuse.g)/255);
    uint8_t aB = (uint8_t)((m->ambient.b*diffuse.b)/255);
    float V[3]; v3_direction(V, viewPos, P);
    float shin = m->shininess; PFcolor spc = m->specular;
    for (int li = 0; li < c->nActive; li++) {
        const RLight *l = &c->lights[c->lightOrder[li]];
        uint8_t lR = 0, lG = 0, lB = 0;
        float L[3] = { l->position[0] - P[0], l->position[1] - P[1], l->position[2] - P[2] };
        float dsq = L[0]*L[0] + L[1]*L[1] + L[2]*L[2];
        float dist = 0;
        if (dsq != 0.0f) {
            dist = sqrtf(dsq);
            float inv = 1.0f / dist;
            for (int i = 0; i < 3; i++) L[i] *= inv;
        }
        uint8_t intensity = 255;
        if ((double)l->innerCutOff < REF_PI) {
            float nd[3] = { -l->direction[0], -l->direction[1], -l->direction[2] };
            float theta = v3_dot(L, nd);
            float eps = l->innerCutOff - l->outerCutOff;
            int32_t iv = ox_ftoi(255*(theta - l->outerCutOff)/eps);
            intensity = (uint8_t)(iv < 0 ? 0 : (iv > 255 ? 255 : iv));
            if (intensity == 0) goto apply;
        }
        {
            uint8_t att = 255;
            if (l->attLinear != 0.0f || l->attQuadratic != 0.0f) {
                att = ox_ftoub(255 / (l->attConstant + l->attLinear*dist + l->attQuadratic*dsq));
                if (att == 0) goto apply;
            }
            uint8_t factor = (uint8_t)((intensity*att)/255);
            int32_t dI = ox_ftoi(255*v3_dot(N, L));
            uint8_t diff = (uint8_t)(dI > 0 ? dI : 0);
            lR = MIN255(lR + (diffuse.r*l->diffuse.r*diff)/(255*255));
            lG = MIN255(lG + (diffuse.g*l->diffuse.g*diff)/(255*255));
            lB = MIN255(lB + (diffuse.b*l->diffuse.b*diff)/(255*255));
            float H[3] = { L[0] + V[0], L[1] + V[1], L[2] + V[2] };
            v3_normalize(H);
            uint8_t spec = ox_ftoub(255 * powf(fmaxf(v3_dot(N, H), 0.0f), shin));
            lR = MIN255(lR + (spc.r*l->specular.r*spec)/(255*255));
            lG = MIN255(lG + (spc.g*l->specular.g*spec)/(255*255));
            lB = MIN255(lB + (spc.b*l->specular.b*spec)/(255*255));
            lR = (uint8_t)((lR*factor)/255);
            lG = (uint8_t)((lG*factor)/255);
            lB = (uint8_t)((lB*factor)/255);
        }
    apply:
        R = MIN255(R + lR + (aR*l->ambient.r)/255);
        Gc = MIN255(Gc + lG + (aG*l->ambient.g)/255);
        B = MIN255(B + lB + (aB*l->ambient.b)/255);
    }
    PFcolor out = { R, Gc, B, diffuse.a };
    return out;
}

/* pfiVec3DirectionR_simd (src/internal/simd.h:2469-2490) with exact rsqrt */
static void v3_direction_simd(float *d, const float *a, const float *b)
{
    d[0] = a[0] - b[0]; d[1] = a[1] - b[1]; d[2] = a[2] - b[2];
    float lsq = d[0]*d[0] + d[1]*d[1];
    lsq = lsq + d[2]*d[2];
    lsq = ox_max(lsq, 1e-5f);
    float inv = 1.0f / sqrtf(lsq);
    d[0] *= inv; d[1] *= inv; d[2] *= inv;
}

static inline float dot_simd(const float *a, const float *b)
{
    float d = a[0]*b[0] + a[1]*b[1];
    return d + a[2]*b[2];
}

/* pfiSimdLightingProcess (src/internal/lighting/lighting.c:149-258), one lane. */
static uint32_t light_phong(const RCtx *c, uint32_t frag, const RMat *m,
                            const float *viewPos, const float *P, const float *N)
{
    float cd[3], ca[3], cs[3];
    for (int i = 0; i < 3; i++) {
        cd[i] = (float)ch(frag, i) * INV255;
        ca[i] = (float)((const uint8_t *)&m->ambient)[i] * INV255;
        cs[i] = (float)((const uint8_t *)&m->specular)[i] * INV255;
    }
    for (int i = 0; i < 3; i++) ca[i] = ca[i] * cd[i];
    float V[3]; v3_direction_simd(V, viewPos, P);
    float acc[3] = { 0.0f, 0.0f, 0.0f };
    for (int li = 0; li < c->nActive; li++) {
        const RLight *l = &c->lights[c->lightOrder[li]];
        float la[3], ld[3], ls[3];
        for (int i = 0; i < 3; i++) {
            la[i] = (float)((const uint8_t *)&l->ambient)[i] * INV255;
            ld[i] = (float)((const uint8_t *)&l->diffuse)[i] * INV255;
            ls[i] = (float)((const uint8_t *)&l->specular)[i] * INV255;
        }
        float L[3]; v3_direction_simd(L, l->position, P);
        float amb[3], dif[3], spe[3];
        for (int i = 0; i < 3; i++) amb[i] = la[i] * ca[i];
        float diff = ox_max(dot_simd(N, L), 0.0f);
        for (int i = 0; i < 3; i++) { dif[i] = ld[i] * diff; dif[i] = dif[i] * cd[i]; }
        float H[3] = { L[0] + V[0], L[1] + V[1], L[2] + V[2] };
        float hs = H[0]*H[0] + H[1]*H[1];
        hs = hs + H[2]*H[2];
        float hinv = 1.0f / sqrtf(hs);
        for (int i = 0; i < 3; i++) H[i] = H[i] * hinv;
        float spec = ox_max(dot_simd(N, H), 0.0f);
        spec = ox_pow_cephes(spec, m->shininess);
        for (int i = 0; i < 3; i++) { spe[i] = ls[i] * spec; spe[i] = spe[i] * cs[i]; }
        if ((double)l->innerCutOff < REF_PI) {
            float nd[3] = { -l->direction[0], -l->direction[1], -l->direction[2] };
            float theta = dot_simd(L, nd);
            float eps = l->innerCutOff - l->outerCutOff;
            float it = (theta - l->outerCutOff) / eps;
            it = ox_min(ox_max(it, 0.0f), 1.0f);
            for (int i = 0; i < 3; i++) { dif[i] *= it; spe[i] *= it; }
        }
        if (l->attLinear != 0.0f || l->attQuadratic != 0.0f) {
            /* pfiVec3DistanceSq_simd (src/internal/simd.h:2423-2442) uses y twice */
            float d0 = l->position[0] - P[0], d1 = l->position[1] - P[1], d2 = l->position[1] - P[1];
            float dsq = d0*d0 + (d1*d1 + d2*d2);
            float dist = sqrtf(dsq);
            float att = 1.0f / (l->attConstant + (l->attLinear*dist + l->attQuadratic*dsq));
            for (int i = 0; i < 3; i++) { amb[i] *= att; dif[i] *= att; spe[i] *= att; }
        }
        for (int i = 0; i < 3; i++) { acc[i] = acc[i] + amb[i]; acc[i] = acc[i] + dif[i]; acc[i] = acc[i] + spe[i]; }
    }
    int32_t o[4] = { 0, 0, 0, 0 };
    for (int i = 0; i < 3; i++) o[i] = ox_cvt_rne(ox_min(ox_max(acc[i], 0.0f), 1.0f) * 255.0f);
    return pack4(o);
}

/* ------------------------------------------------------------------------ */
/* rasterizer (src/internal/primitives/triangles.c:287-558)                  */
/* ------------------------------------------------------------------------ */

/* What a triangle's fragments are shaded with (triangles.c:356-397). */
typedef struct {
    const RCtx *c;
    int is3D;
    const RVert *v1, *v2, *v3;
    const float *viewPos;
    uint32_t c1, c2, c3;
    const RTex *tex;
    int phong;
    const RMat *fm;
    int smooth;
} TriFrag;

/* Source colour of a fragment with normalised weights wn1..wn3 and depth z
 * (triangles.c:500-521): colour interpolation, texturing, per-fragment
 * lighting.  texOn 0: the fragment is outside the mask, whose texture
 * coordinates the reference replaces by zero before sampling
 * (triangles.c:508-513). */
static uint32_t tri_frag(const TriFrag *s, float wn1, float wn2, float wn3, float z, int texOn)
{
    const RVert *v1 = s->v1, *v2 = s->v2, *v3 = s->v3;
    uint32_t frag;
    if (s->smooth) {
        int32_t u1 = ox_cvt_rne(wn1 * 255.0f), u2 = ox_cvt_rne(wn2 * 255.0f), u3 = ox_cvt_rne(wn3 * 255.0f);
        int32_t o[4];
        for (int i = 0; i < 4; i++) {
            uint32_t t = (uint32_t)u1*(uint32_t)ch(s->c1, i) + (uint32_t)u2*(uint32_t)ch(s->c2, i);
            t = t + (uint32_t)u3*(uint32_t)ch(s->c3, i);
            o[i] = (int32_t)((t * 257u) >> 16);
        }
        frag = pack4(o);
    } else {
        float mx = ox_max(wn1, ox_max(wn2, wn3));
        frag = ((mx == wn1) ? s->c1 : 0u) | (((mx == wn2) ? s->c2 : 0u) | ((mx == wn3) ? s->c3 : 0u));
    }
    if (s->tex) {
        float tu = 0.0f, tv = 0.0f;
        if (texOn) {
            tu = v1->texcoord[0]*wn1 + v2->texcoord[0]*wn2;
            tu = tu + v3->texcoord[0]*wn3;
            tv = v1->texcoord[1]*wn1 + v2->texcoord[1]*wn2;
            tv = tv + v3->texcoord[1]*wn3;
            if (s->is3D) { tu = tu * z; tv = tv * z; }
        }
        uint32_t texel = tex_sample(s->tex, tu, tv);
        frag = blend_simd(PF_BLEND_MUL, texel, frag);
    }
    if (s->phong) {
        float N[3], P[3];
        for (int i = 0; i < 3; i++) {
            float a = v1->normal[i]*wn1 + v2->normal[i]*wn2; N[i] = a + v3->normal[i]*wn3;
            float b = v1->position[i]*wn1 + v2->position[i]*wn2; P[i] = b + v3->position[i]*wn3;
        }
        frag = light_phong(s->c, frag, s->fm, s->viewPos, P, N);
    }
    return frag;
}

static void raster_tri(RCtx *c, PFface face, int is3D, const RVert *v1, const RVert *v2,
                       const RVert *v3, const float *viewPos)
{
    int32_t x1 = ox_ftoi(v1->screen[0]), y1 = ox_ftoi(v1->screen[1]);
    int32_t x2 = ox_ftoi(v2->screen[0]), y2 = ox_ftoi(v2->screen[1]);
    int32_t x3 = ox_ftoi(v3->screen[0]), y3 = ox_ftoi(v3->screen[1]);
    float area = (float)(int32_t)((uint32_t)(x2 - x1)*(uint32_t)(y3 - y1) - (uint32_t)(x3 - x1)*(uint32_t)(y2 - y1));
    if ((face == PF_FRONT && area >= 0) || (face == PF_BACK && area <= 0)) return;

    int32_t mnx = x1 < (x2 < x3 ? x2 : x3) ? x1 : (x2 < x3 ? x2 : x3);
    int32_t mny = y1 < (y2 < y3 ? y2 : y3) ? y1 : (y2 < y3 ? y2 : y3);
    int32_t mxx = x1 > (x2 > x3 ? x2 : x3) ? x1 : (x2 > x3 ? x2 : x3);
    int32_t mxy = y1 > (y2 > y3 ? y2 : y3) ? y1 : (y2 > y3 ? y2 : y3);
    uint32_t xMin = (uint32_t)mnx, yMin = (uint32_t)mny, xMax = (uint32_t)mxx, yMax = (uint32_t)mxy;
    if (!is3D) {
#define CLAMPI(v, lo, hi) ((v) < (lo) ? (lo) : ((v) > (hi) ? (hi) : (v)))
        xMin = (uint32_t)CLAMPI((int32_t)xMin, c->vpMin[0], c->vpMax[0]);
        yMin = (uint32_t)CLAMPI((int32_t)yMin, c->vpMin[1], c->vpMax[1]);
        xMax = (uint32_t)CLAMPI((int32_t)xMax, c->vpMin[0], c->vpMax[0]);
        yMax = (uint32_t)CLAMPI((int32_t)yMax, c->vpMin[1], c->vpMax[1]);
    }
    int32_t w1X = y3 - y2, w1Y = x2 - x3;
    int32_t w2X = y1 - y3, w2Y = x3 - x1;
    int32_t w3X = y2 - y1, w3Y = x1 - x2;
    if (face == PF_BACK) { w1X = -w1X; w1Y = -w1Y; w2X = -w2X; w2Y = -w2Y; w3X = -w3X; w3Y = -w3Y; }
    uint32_t w1Row = (xMin - (uint32_t)x2)*(uint32_t)w1X + (uint32_t)w1Y*(yMin - (uint32_t)y2);
    uint32_t w2Row = (xMin - (uint32_t)x3)*(uint32_t)w2X + (uint32_t)w2Y*(yMin - (uint32_t)y3);
    uint32_t w3Row = (xMin - (uint32_t)x1)*(uint32_t)w3X + (uint32_t)w3Y*(yMin - (uint32_t)y1);
    float wInvSum = 1.0f / (float)(int32_t)(w1Row + w2Row + w3Row);

    uint32_t c1 = col_pack(v1->color), c2 = col_pack(v2->color), c3 = col_pack(v3->color);
    const float z1 = v1->homogeneous[2], z2 = v2->homogeneous[2], z3 = v3->homogeneous[2];

    RTex *fbt = (RTex *)c->current->texture;
    float *zb = c->current->zbuffer;
    const uint32_t W = fbt->w, H = fbt->h;

    const int blending = (c->state & PF_BLEND) != 0;
    const int depthTest = (c->state & PF_DEPTH_TEST) != 0;
    RTex *tex = ((c->state & PF_TEXTURE_2D) && c->texture) ? c->texture : NULL;
    const int phong = (c->state & PF_LIGHTING) && c->lightMode == PF_PHONG && c->nActive > 0;
    const RMat *fm = &c->mat[face];
    const int smooth = c->shade == PF_SMOOTH;
    const long area_bb = (long)(yMax - yMin) * (long)(xMax - xMin);   /* (OpenMP threshold) */
    (void)area_bb;
    uint64_t frags = 0;
    const TriFrag sh = { c, is3D, v1, v2, v3, viewPos, c1, c2, c3, tex, phong, fm, smooth };

    if (fb_bgra8(fbt)) {
        /* BGRA / unsigned byte: the SIMD getter and setter shuffle every
         * 4-pixel half of the 8-pixel vector with the bytes of its first
         * pixel (pixel.h:2070-2078, 2916-2921; simd.h:564-583), so each
         * pixel the mask lets through takes the value computed for that
         * first pixel -- its own colour (texture coordinates zeroed when
         * the first pixel is outside the mask), blended with its own
         * destination.  The halves start at xMin + 4k (x steps by 8 from
         * xMin, triangles.c:409); rows are independent. */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4) reduction(+:frags) if (area_bb >= 32*32)
#endif
        for (long yy = (long)yMin; yy <= (long)yMax; yy++) {
            uint32_t y = (uint32_t)yy;
            if (y >= H) continue;   /* memory guard: undefined in the reference */
            for (uint32_t xf = xMin; xf < xMax; xf += 4) {
                int m[4] = { 0, 0, 0, 0 }, any = 0;
                float zl[4] = { 0, 0, 0, 0 };
                float wf[3] = { 0, 0, 0 }, zf = 0.0f;
                for (uint32_t j = 0; j < 4; j++) {
                    const uint32_t x = xf + j;
                    int32_t w1 = (int32_t)(w1Row + (y - yMin)*(uint32_t)w1Y + (x - xMin)*(uint32_t)w1X);
                    int32_t w2 = (int32_t)(w2Row + (y - yMin)*(uint32_t)w2Y + (x - xMin)*(uint32_t)w2X);
                    int32_t w3 = (int32_t)(w3Row + (y - yMin)*(uint32_t)w3Y + (x - xMin)*(uint32_t)w3X);
                    float wn1 = (float)w1 * wInvSum, wn2 = (float)w2 * wInvSum, wn3 = (float)w3 * wInvSum;
                    float zs = z1*wn1 + z2*wn2;
                    zs = zs + z3*wn3;
                    float z = 1.0f / zs;
                    if (j == 0) { wf[0] = wn1; wf[1] = wn2; wf[2] = wn3; zf = z; }
                    if (x >= xMax || (w1 | w2 | w3) <= 0 || x >= W) continue;
                    frags++;
                    if (depthTest && !depth_simd(c->depthFunc, z, zb[(size_t)y * W + x])) continue;
                    m[j] = 1; zl[j] = z; any = 1;
                }
                if (!any) continue;
                uint32_t frag = tri_frag(&sh, wf[0], wf[1], wf[2], zf, m[0]);
                if (blending) frag = blend_simd(c->blend, frag, fb_get_simd(fbt, (size_t)y * W + xf));
                for (uint32_t j = 0; j < 4; j++) {
                    if (!m[j]) continue;
                    const size_t p = (size_t)y * W + xf + j;
                    fb_set_simd(fbt, p, frag);
                    if (c->depthMask) zb[p] = zl[j];
                }
            }
        }
        c->stats.fragments += frags;
        c->stats.rasterized += 1;
        return;
    }

#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4) reduction(+:frags) if (area_bb >= 32*32)
#endif
    for (long yy = (long)yMin; yy <= (long)yMax; yy++) {
        uint32_t y = (uint32_t)yy;
        for (uint32_t x = xMin; x < xMax; x++) {
            int32_t w1 = (int32_t)(w1Row + (y - yMin)*(uint32_t)w1Y + (x - xMin)*(uint32_t)w1X);
            int32_t w2 = (int32_t)(w2Row + (y - yMin)*(uint32_t)w2Y + (x - xMin)*(uint32_t)w2X);
            int32_t w3 = (int32_t)(w3Row + (y - yMin)*(uint32_t)w3Y + (x - xMin)*(uint32_t)w3X);
            if ((w1 | w2 | w3) <= 0) continue;
            if (x >= W || y >= H) continue;   /* memory guard: undefined in the reference */
            frags++;
            float wn1 = (float)w1 * wInvSum, wn2 = (float)w2 * wInvSum, wn3 = (float)w3 * wInvSum;
            float zs = z1*wn1 + z2*wn2;
            zs = zs + z3*wn3;
            float z = 1.0f / zs;
            size_t p = (size_t)y * W + x;
            if (depthTest && !depth_simd(c->depthFunc, z, zb[p])) continue;
            uint32_t frag = tri_frag(&sh, wn1, wn2, wn3, z, 1);
            if (blending) frag = blend_simd(c->blend, frag, fb_get_simd(fbt, p));
            fb_set_simd(fbt, p, frag);
            if (c->depthMask) zb[p] = z;
        }
    }
    c->stats.fragments += frags;
    c->stats.rasterized += 1;
}

/* ------------------------------------------------------------------------ */
/* vertex processing and clipping                                            */
/* ------------------------------------------------------------------------ */

/* pfiHomogeneousToScreen (src/internal/context/context.c:52-65) */
static void to_screen(const RCtx *c, RVert *v)
{
    v->screen[0] = ((float)c->vpPos[0] + (v->homogeneous[0] + 1.0f) * 0.5f * (float)c->vpDim[0]) + 0.5f;
    v->screen[1] = ((float)c->vpPos[1] + (1.0f - v->homogeneous[1]) * 0.5f * (float)c->vpDim[1]) + 0.5f;
}

/* pfiLerpVertex (src/internal/context/context.c:67-90) */
static RVert lerp_vert(const RVert *s, const RVert *e, float t)
{
    RVert r; memset(&r, 0, sizeof r);
    const uint8_t *sc = (const uint8_t *)&s->color, *ec = (const uint8_t *)&e->color;
    uint8_t *rc = (uint8_t *)&r.color;
    uint8_t uT = ox_ftoub(255 * t);
    for (int i = 0; i < 4; i++) {
        r.homogeneous[i] = s->homogeneous[i] + t*(e->homogeneous[i] - s->homogeneous[i]);
        r.position[i] = s->position[i] + t*(e->position[i] - s->position[i]);
        rc[i] = (uint8_t)(sc[i] + (uT*((int32_t)ec[i] - sc[i]))/255);
        if (i < 2) r.texcoord[i] = s->texcoord[i] + t*(e->texcoord[i] - s->texcoord[i]);
        if (i < 3) r.normal[i] = s->normal[i] + t*(e->normal[i] - s->normal[i]);
    }
    return r;
}

/* Process_ClipPolygonW (triangles.c:157-182) */
static int clip_w(RVert *poly, int *n)
{
    RVert in[MAX_POLY]; int nin = *n;
    memcpy(in, poly, (size_t)nin * sizeof(RVert));
    *n = 0;
    const RVert *prev = &in[nin - 1];
    int pd = (prev->homogeneous[3] < CLIP_EPS) ? -1 : 1;
    for (int i = 0; i < nin; i++) {
        int cd = (in[i].homogeneous[3] < CLIP_EPS) ? -1 : 1;
        if (pd * cd < 0)
            poly[(*n)++] = lerp_vert(prev, &in[i], (CLIP_EPS - prev->homogeneous[3]) /
                                     (in[i].homogeneous[3] - prev->homogeneous[3]));
        if (cd > 0) poly[(*n)++] = in[i];
        pd = cd; prev = &in[i];
    }
    return *n > 0;
}

/* Process_ClipPolygonXYZ (triangles.c:184-244) */
static int clip_xyz(RVert *poly, int *n)
{
    for (int ax = 0; ax < 3; ax++) {
        if (*n == 0) return 0;
        RVert in[MAX_POLY]; int nin;
        memcpy(in, poly, (size_t)*n * sizeof(RVert)); nin = *n; *n = 0;
        const RVert *prev = &in[nin - 1];
        int pd = (prev->homogeneous[ax] <= prev->homogeneous[3]) ? 1 : -1;
        for (int i = 0; i < nin; i++) {
            int cd = (in[i].homogeneous[ax] <= in[i].homogeneous[3]) ? 1 : -1;
            if (pd * cd <= 0)
                poly[(*n)++] = lerp_vert(prev, &in[i], (prev->homogeneous[3] - prev->homogeneous[ax]) /
                    ((prev->homogeneous[3] - prev->homogeneous[ax]) - (in[i].homogeneous[3] - in[i].homogeneous[ax])));
            if (cd > 0) poly[(*n)++] = in[i];
            pd = cd; prev = &in[i];
        }
        if (*n == 0) return 0;
        memcpy(in, poly, (size_t)*n * sizeof(RVert)); nin = *n; *n = 0;
        prev = &in[nin - 1];
        pd = (-prev->homogeneous[ax] <= prev->homogeneous[3]) ? 1 : -1;
        for (int i = 0; i < nin; i++) {
            int cd = (-in[i].homogeneous[ax] <= in[i].homogeneous[3]) ? 1 : -1;
            if (pd * cd <= 0)
                poly[(*n)++] = lerp_vert(prev, &in[i], (prev->homogeneous[3] + prev->homogeneous[ax]) /
                    ((prev->homogeneous[3] + prev->homogeneous[ax]) - (in[i].homogeneous[3] + in[i].homogeneous[ax])));
            if (cd > 0) poly[(*n)++] = in[i];
            pd = cd; prev = &in[i];
        }
    }
    return *n > 0;
}

/* Process_ProjectAndClipTriangle (triangles.c:246-280); returns is3D */
static int project_clip(RCtx *c, RVert *poly, int *n)
{
    float ws = 0.0f;
    for (int i = 0; i < *n; i++) {
        memcpy(poly[i].homogeneous, poly[i].position, 16);
        v4_transform(poly[i].homogeneous, poly[i].homogeneous, c->mvp);
        ws += poly[i].homogeneous[3];
    }
    if (fabsf(ws - 3.0f) < CLIP_EPS) {
        for (int i = 0; i < *n; i++) to_screen(c, &poly[i]);
        return 0;
    }
    if (clip_w(poly, n) && clip_xyz(poly, n)) {
        for (int i = 0; i < *n; i++) {
            poly[i].homogeneous[2] = 1.0f / poly[i].homogeneous[2];
            poly[i].texcoord[0] = poly[i].texcoord[0] * poly[i].homogeneous[2];
            poly[i].texcoord[1] = poly[i].texcoord[1] * poly[i].homogeneous[2];
            float invW = 1.0f / poly[i].homogeneous[3];
            poly[i].homogeneous[0] *= invW;
            poly[i].homogeneous[1] *= invW;
            to_screen(c, &poly[i]);
        }
    }
    return 1;
}

/* pfiProcessRasterize_TRIANGLE_IMPL (triangles.c:62-116) */
static void process_triangle(RCtx *c, PFface face, RVert *poly)
{
    int lighting = (c->state & PF_LIGHTING) && c->nActive > 0;
    int n = 3;
    float viewPos[3] = { 0, 0, 0 };
    c->stats.primitives += 1;
    if (lighting) {
        float inv[16]; m_invert(inv, c->view);
        memcpy(viewPos, inv + 12, 12);
        for (int i = 0; i < 3; i++) {
            v3_transform(poly[i].normal, poly[i].normal, c->normal);
            v3_normalize(poly[i].normal);
            poly[i].color = blend_mul_scalar(poly[i].color, c->mat[face].diffuse);
            if (c->lightMode == PF_GOURAUD) {
                float NdotV = v3_dot(poly[i].normal, c->view + 8);
                poly[i].color = light_gouraud(c, &c->mat[(NdotV < 0) ? PF_FRONT : PF_BACK],
                                              poly[i].color, viewPos, poly[i].position, poly[i].normal);
            }
        }
    }
    int is3D = project_clip(c, poly, &n);
    if (n < 3) return;
    for (int i = 0; i < n - 2; i++) raster_tri(c, face, is3D, &poly[0], &poly[i + 1], &poly[i + 2], viewPos);
}

static void tri_from(RCtx *c, PFface face, int a, int b, int d)
{
    RVert poly[MAX_POLY];
    poly[0] = c->vbuf[a]; poly[1] = c->vbuf[b]; poly[2] = c->vbuf[d];
    process_triangle(c, face, poly);
}

static void tri_fan(RCtx *c, PFface face, int n)    /* triangles.c:125-135 */
{
    for (int i = 0; i < n; i++) tri_from(c, face, 0, i + 1, i + 2);
}

static void tri_strip(RCtx *c, PFface face, int n)  /* triangles.c:137-152 */
{
    for (int i = 0; i < n; i++) {
        if (i % 2 == 0) tri_from(c, face, i, i + 1, i + 2);
        else tri_from(c, face, i + 2, i + 1, i);
    }
}

/* ------------------------------------------------------------------------ */
/* points and lines (src/internal/primitives/points.c, lines.c)              */
/* ------------------------------------------------------------------------ */

/* SISD depth tests (src/internal/depth.h:27-74): NOTEQUAL is a real != here */
static int depth_sisd(PFdepthmode f, float src, float dst)
{
    switch (f) {
    case PF_EQUAL: return src == dst;
    case PF_NOTEQUAL: return src != dst;
    case PF_LESS: return src < dst;
    case PF_LEQUAL: return src <= dst;
    case PF_GREATER: return src > dst;
    default: return src >= dst;
    }
}

/* SISD blending (src/internal/blend.h:27-126) */
static uint32_t blend_sisd(PFblendmode m, uint32_t src, uint32_t dst)
{
    int32_t o[4];
    for (int i = 0; i < 4; i++) {
        const int32_t s = (int32_t)ch(src, i), d = (int32_t)ch(dst, i);
        int32_t v;
        switch (m) {
        case PF_BLEND_AVERAGE: v = (s + d) >> 1; break;
        case PF_BLEND_ALPHA: {
            const uint32_t a = ch(src, 3) + 1, ia = 256 - a;
            v = (int32_t)((a * (uint32_t)(i == 3 ? 255 : s) + ia * (uint32_t)d) >> 8);
            break;
        }
        case PF_BLEND_ADD: v = (d + s) < 255 ? (d + s) : 255; break;
        case PF_BLEND_SUB: v = (d - s) > 0 ? (d - s) : 0; break;
        case PF_BLEND_MUL: v = (s * d) / 255; break;
        case PF_BLEND_SCREEN: { int32_t t = ((d * (255 - s)) >> 8) + s; v = t < 255 ? t : 255; break; }
        case PF_BLEND_LIGHTEN: v = s > d ? s : d; break;
        default: v = s < d ? s : d; break;
        }
        o[i] = v & 255;
    }
    return (uint32_t)o[0] | (uint32_t)o[1] << 8 | (uint32_t)o[2] << 16 | (uint32_t)o[3] << 24;
}

/* One pixel of a point or line.  Pixels outside the framebuffer are not
 * drawn (the reference writes them at y*w + x, outside its buffers or
 * wrapped into a neighbouring row). */
static void lp_pixel(RCtx *c, int32_t x, int32_t y, float z, uint32_t col, int test)
{
    RTex *fbt = (RTex *)c->current->texture;
    if (x < 0 || y < 0 || (uint32_t)x >= fbt->w || (uint32_t)y >= fbt->h) return;
    const size_t p = (size_t)y * fbt->w + (size_t)x;
    float *zb = c->current->zbuffer;
    c->stats.fragments++;
    if (test && !depth_sisd(c->depthFunc, z, zb[p])) return;
    if (c->state & PF_BLEND) col = blend_sisd(c->blend, col, fb_get(fbt, p));
    fb_set(fbt, p, col);
    if (c->depthMask) zb[p] = z;
}

/* Process_ProjectPoint (points.c:44-81) */
static int project_point(const RCtx *c, const RVert *v, float *sx, float *sy, float *z)
{
    float h[4];
    v4_transform(h, v->position, c->mvp);
    if (h[3] != 1.0f) {
        for (int i = 0; i < 3; i++) if (h[i] < -h[3] || h[i] > h[3]) return 0;
        const float invW = 1.0f / h[3];
        h[0] = h[0] * invW; h[1] = h[1] * invW;
    }
    *sx = ((float)c->vpPos[0] + (h[0] + 1.0f) * 0.5f * (float)c->vpDim[0]) + 0.5f;
    *sy = ((float)c->vpPos[1] + (1.0f - h[1]) * 0.5f * (float)c->vpDim[1]) + 0.5f;
    *z = h[2];
    return *sx >= (float)c->vpMin[0] && *sy >= (float)c->vpMin[1] && *sx <= (float)c->vpMax[0] && *sy <= (float)c->vpMax[1];
}

/* Rasterize_Point_{DEPTH,NODEPTH} (points.c:85-183) */
static void raster_point(RCtx *c, const RVert *v)
{
    float sx, sy, z;
    if (!project_point(c, v, &sx, &sy, &z)) return;
    const int32_t cx = ox_ftoi(sx), cy = ox_ftoi(sy);
    const uint32_t col = col_pack(v->color);
    const int test = (c->state & PF_DEPTH_TEST) != 0;
    if (c->pointSize <= 1.0f) { lp_pixel(c, cx, cy, z, col, test); return; }
    const float r = c->pointSize * 0.5f, rSq = r * r;
    const int32_t ir = ox_ftoi(r);
    for (int32_t y = -ir; y <= ir; y++)
        for (int32_t x = -ir; x <= ir; x++)
            if ((float)(y * y + x * x) <= rSq) lp_pixel(c, cx + x, cy + y, z, col, test);
}

static void screen_map(const RCtx *c, RVert *v)
{
    v->screen[0] = ((float)c->vpPos[0] + (v->homogeneous[0] + 1.0f) * 0.5f * (float)c->vpDim[0]) + 0.5f;
    v->screen[1] = ((float)c->vpPos[1] + (1.0f - v->homogeneous[1]) * 0.5f * (float)c->vpDim[1]) + 0.5f;
}

/* Helper_EncodeClip2D (lines.c:116-125): 1 left, 2 right, 4 below (y > yMax),
 * 8 above (y < yMin) */
static uint32_t clip_code(const float *sc, int32_t xMin, int32_t yMin, int32_t xMax, int32_t yMax)
{
    uint32_t code = 0;
    if (sc[0] < (float)xMin) code |= 1;
    if (sc[0] > (float)xMax) code |= 2;
    if (sc[1] < (float)yMin) code |= 8;
    if (sc[1] > (float)yMax) code |= 4;
    return code;
}

/* Process_ClipLine2D (lines.c:158-223), Cohen-Sutherland in screen space
 * with the reference's assignments (a point below the viewport moves to
 * its top row and the reverse).  Bounded to 32 rounds (the reference loops
 * until it accepts or rejects). */
static int clip_line_2d(const RCtx *c, RVert *v1, RVert *v2)
{
    const int32_t xMin = c->vpMin[0], yMin = c->vpMin[1], xMax = c->vpMax[0], yMax = c->vpMax[1];
    float m = 0.0f;
    if (v1->screen[0] != v2->screen[0]) m = (v2->screen[1] - v1->screen[1]) / (v2->screen[0] - v1->screen[0]);
    for (int round = 0; round < 32; round++) {
        uint32_t code0 = clip_code(v1->screen, xMin, yMin, xMax, yMax), code1 = clip_code(v2->screen, xMin, yMin, xMax, yMax);
        if ((code0 | code1) == 0) return 1;
        if (code0 & code1) return 0;
        if (code0 == 0) {
            uint32_t t = code0; code0 = code1; code1 = t;
            RVert tv = *v1; *v1 = *v2; *v2 = tv;
        }
        if (code0 & 1) {
            v1->screen[1] = v1->screen[1] + ((float)xMin - v1->screen[0]) * m;
            v1->screen[0] = (float)xMin;
        } else if (code0 & 2) {
            v1->screen[1] = v1->screen[1] + ((float)xMax - v1->screen[0]) * m;
            v1->screen[0] = (float)xMax;
        } else if (code0 & 4) {
            if (m != 0.0f) v1->screen[0] = v1->screen[0] + ((float)yMin - v1->screen[1]) / m;
            v1->screen[1] = (float)yMin;
        } else if (code0 & 8) {
            if (m != 0.0f) v1->screen[0] = v1->screen[0] + ((float)yMax - v1->screen[1]) / m;
            v1->screen[1] = (float)yMax;
        }
    }
    return 0;
}

/* Helper_ClipCoord3D (lines.c:127-150) */
static int clip_coord_3d(float q, float p, float *t1, float *t2)
{
    if (fabsf(p) < CLIP_EPS) return !(q < -CLIP_EPS);
    const float r = q / p;
    if (p < 0) {
        if (r > *t2) return 0;
        if (r > *t1) *t1 = r;
    } else {
        if (r < *t1) return 0;
        if (r < *t2) *t2 = r;
    }
    return 1;
}

/* Process_ClipLine3D (lines.c:225-262), Liang-Barsky in clip space */
static int clip_line_3d(RVert *v1, RVert *v2)
{
    float t1 = 0.0f, t2 = 1.0f, d[4];
    const float *a = v1->homogeneous;
    for (int i = 0; i < 4; i++) d[i] = v2->homogeneous[i] - a[i];
    if (!clip_coord_3d(a[3] - a[0], -d[3] + d[0], &t1, &t2)) return 0;
    if (!clip_coord_3d(a[3] + a[0], -d[3] - d[0], &t1, &t2)) return 0;
    if (!clip_coord_3d(a[3] - a[1], -d[3] + d[1], &t1, &t2)) return 0;
    if (!clip_coord_3d(a[3] + a[1], -d[3] - d[1], &t1, &t2)) return 0;
    if (!clip_coord_3d(a[3] - a[2], -d[3] + d[2], &t1, &t2)) return 0;
    if (!clip_coord_3d(a[3] + a[2], -d[3] - d[2], &t1, &t2)) return 0;
    if (t2 < 1.0f) for (int i = 0; i < 4; i++) v2->homogeneous[i] = v1->homogeneous[i] + d[i] * t2;
    if (t1 > 0.0f) for (int i = 0; i < 4; i++) v1->homogeneous[i] = v1->homogeneous[i] + d[i] * t1;
    return 1;
}

/* Process_ProjectAndClipLine (lines.c:264-300) */
static int project_clip_line(const RCtx *c, RVert *l)
{
    for (int i = 0; i < 2; i++) v4_transform(l[i].homogeneous, l[i].position, c->mvp);
    if (l[0].homogeneous[3] == 1.0f && l[1].homogeneous[3] == 1.0f) {
        screen_map(c, &l[0]); screen_map(c, &l[1]);
        return clip_line_2d(c, &l[0], &l[1]);
    }
    if (!clip_line_3d(&l[0], &l[1])) return 0;
    for (int i = 0; i < 2; i++) {
        const float invW = 1.0f / l[i].homogeneous[3];
        l[i].homogeneous[0] = l[i].homogeneous[0] * invW;
        l[i].homogeneous[1] = l[i].homogeneous[1] * invW;
    }
    screen_map(c, &l[0]); screen_map(c, &l[1]);
    return 1;
}

/* Rasterize_Line_{DEPTH,NODEPTH} (lines.c:304-431): DDA in 16.16 fixed point */
static void raster_line_thin(RCtx *c, const RVert *v1, const RVert *v2, int test)
{
    const int32_t x1 = ox_ftoi(v1->screen[0]), y1 = ox_ftoi(v1->screen[1]);
    const int32_t x2 = ox_ftoi(v2->screen[0]), y2 = ox_ftoi(v2->screen[1]);
    const float z1 = v1->homogeneous[2], z2 = v2->homogeneous[2];
    const PFcolor c1 = v1->color, c2 = v2->color;
    int32_t shortLen = y2 - y1, longLen = x2 - x1;
    int yLonger = 0;
    if (ox_iabs(shortLen) > ox_iabs(longLen)) { int32_t t = shortLen; shortLen = longLen; longLen = t; yLonger = 1; }
    const float invEndVal = 1.0f / (float)longLen;
    const int32_t endVal = longLen;
    int32_t sgnInc = 1;
    if (longLen < 0) { longLen = -longLen; sgnInc = -1; }
    const int32_t decInc = (longLen == 0) ? 0 : (int32_t)((uint32_t)shortLen << 16) / longLen;
    int32_t j = 0;
    for (int32_t i = 0; i != endVal; i += sgnInc, j += decInc) {
        const float t = (float)i * invEndVal;
        const int32_t x = yLonger ? x1 + (j >> 16) : x1 + i;
        const int32_t y = yLonger ? y1 + i : y1 + (j >> 16);
        const float z = z1 + t * (z2 - z1);
        const uint8_t o[4] = { ox_ftoub((float)c1.r + t * (float)(c2.r - c1.r)), ox_ftoub((float)c1.g + t * (float)(c2.g - c1.g)),
                               ox_ftoub((float)c1.b + t * (float)(c2.b - c1.b)), ox_ftoub((float)c1.a + t * (float)(c2.a - c1.a)) };
        lp_pixel(c, x, y, z, (uint32_t)o[0] | (uint32_t)o[1] << 8 | (uint32_t)o[2] << 16 | (uint32_t)o[3] << 24, test);
    }
}

/* pfiProcessRasterize_LINE (lines.c:57-79) and the thick variants
 * (lines.c:433-531): the centre line is always depth-tested */
static void raster_line(RCtx *c, const RVert *a, const RVert *b, int *rejected)
{
    RVert l[2] = { *a, *b };
    if (!project_clip_line(c, l)) { if (rejected) *rejected = 1; return; }
    const int test = (c->state & PF_DEPTH_TEST) != 0;
    if (!(c->lineWidth > 1.5f)) { raster_line_thin(c, &l[0], &l[1], test); return; }
    const int32_t x1 = ox_ftoi(l[0].screen[0]), y1 = ox_ftoi(l[0].screen[1]);
    const int32_t x2 = ox_ftoi(l[1].screen[0]), y2 = ox_ftoi(l[1].screen[1]);
    const int32_t dx = x2 - x1, dy = y2 - y1;
    raster_line_thin(c, &l[0], &l[1], 1);
    const float rs = 1.0f / sqrtf((float)(dx * dx + dy * dy));
    if (dx != 0 && ox_iabs(dy / dx) < 1) {
        const int32_t wy = ox_ftoi((c->lineWidth - 1.0f) * rs * (float)ox_iabs(dx)) >> 1;
        for (int32_t i = 1; i <= wy; i++) {
            RVert t1 = l[0], t2 = l[1];
            t1.screen[1] -= (float)i; t2.screen[1] -= (float)i;
            raster_line_thin(c, &t1, &t2, test);
            t1 = l[0]; t2 = l[1];
            t1.screen[1] += (float)i; t2.screen[1] += (float)i;
            raster_line_thin(c, &t1, &t2, test);
        }
    } else if (dy != 0) {
        const int32_t wx = ox_ftoi((c->lineWidth - 1.0f) * rs * (float)ox_iabs(dy)) >> 1;
        for (int32_t i = 1; i <= wx; i++) {
            RVert t1 = l[0], t2 = l[1];
            t1.screen[0] -= (float)i; t2.screen[0] -= (float)i;
            raster_line_thin(c, &t1, &t2, test);
            t1 = l[0]; t2 = l[1];
            t1.screen[0] += (float)i; t2.screen[0] += (float)i;
            raster_line_thin(c, &t1, &t2, test);
        }
    }
}

/* pfiProcessRasterize_POLY_POINTS / _POLY_LINES (points.c:33-41, lines.c:81-110):
 * the edges stop at the first one clipped away */
static void poly_points(RCtx *c, int n) { for (int i = 0; i < n; i++) raster_point(c, &c->vbuf[i]); }
static void poly_lines(RCtx *c, int n)
{
    for (int i = 0; i < n; i++) {
        int rejected = 0;
        raster_line(c, &c->vbuf[i], &c->vbuf[(i + 1) % n], &rejected);
        if (rejected) return;
    }
}

static void poly_pass(RCtx *c, PFface face, int n)
{
    switch (c->polygonMode[face]) {
    case PF_POINT: poly_points(c, n); break;
    case PF_LINE: poly_lines(c, n); break;
    default: if (n == 3) tri_from(c, face, 0, 1, 2); else tri_fan(c, face, 2); break;
    }
}

/* pfiProcessAndRasterize (src/internal/context/context.c:95-244) */
static void process_and_raster(RCtx *c)
{
    PFface f = (c->state & PF_CULL_FACE) ? (PFface)!c->cullFace : PF_FRONT_AND_BACK;
    switch (c->drawMode) {
    case PF_POINTS: raster_point(c, &c->vbuf[0]); break;
    case PF_LINES: raster_line(c, &c->vbuf[0], &c->vbuf[1], NULL); break;
    case PF_TRIANGLES:
        if (f == PF_FRONT_AND_BACK) { poly_pass(c, PF_FRONT, 3); poly_pass(c, PF_BACK, 3); }
        else poly_pass(c, f, 3);
        break;
    case PF_TRIANGLE_FAN:
        if (f == PF_FRONT_AND_BACK) { tri_fan(c, PF_FRONT, 2); tri_fan(c, PF_BACK, 2); } else tri_fan(c, f, 2);
        break;
    case PF_TRIANGLE_STRIP:
        if (f == PF_FRONT_AND_BACK) { tri_strip(c, PF_FRONT, 2); tri_strip(c, PF_BACK, 2); } else tri_strip(c, f, 2);
        break;
    case PF_QUADS:
        if (f == PF_FRONT_AND_BACK) { poly_pass(c, PF_FRONT, 4); poly_pass(c, PF_BACK, 4); }
        else poly_pass(c, f, 4);
        break;
    case PF_QUAD_FAN:
        if (f == PF_FRONT_AND_BACK) { tri_fan(c, PF_FRONT, 4); tri_fan(c, PF_BACK, 4); } else tri_fan(c, f, 4);
        break;
    case PF_QUAD_STRIP:
        if (f == PF_FRONT_AND_BACK) { tri_strip(c, PF_FRONT, 4); tri_strip(c, PF_BACK, 4); } else tri_strip(c, f, 4);
        break;
    default:
        break;
    }
}

static PFsizei mode_count(PFdrawmode m)    /* context.c:61-74 */
{
    switch (m) {
    case PF_POINTS: return 1; case PF_LINES: return 2; case PF_TRIANGLES: return 3;
    case PF_TRIANGLE_FAN: case PF_TRIANGLE_STRIP: case PF_QUADS: return 4;
    case PF_QUAD_FAN: case PF_QUAD_STRIP: return 6;
    }
    return 0;
}

static void reset_for_next(RCtx *c)        /* context.c:41-59 */
{
    switch (c->drawMode) {
    case PF_TRIANGLE_FAN: case PF_TRIANGLE_STRIP: c->vcount = 1; c->vbuf[0] = c->vbuf[3]; break;
    case PF_QUAD_FAN: case PF_QUAD_STRIP: c->vcount = 2; c->vbuf[0] = c->vbuf[4]; c->vbuf[1] = c->vbuf[5]; break;
    default: c->vcount = 0; break;
    }
}

static void update_matrices(RCtx *c, int withNormal)   /* context.c:96-111 */
{
    if (c->modelUsed) {
        m_mul(c->mvp, c->model, c->view);
        m_mul(c->mvp, c->mvp, c->proj);
        if (withNormal && (c->state & PF_LIGHTING)) { m_invert(c->normal, c->model); m_transpose(c->normal, c->normal); }
    } else {
        m_mul(c->mvp, c->view, c->proj);
        if (withNormal && (c->state & PF_LIGHTING)) m_identity(c->normal);
    }
}

/* ------------------------------------------------------------------------ */
/* API: contexts                                                             */
/* ------------------------------------------------------------------------ */

static int texel_bytes(PFpixelformat f, PFdatatype t);

/* Textures may use any format the reference has a SIMD getter for,
 * framebuffers the formats fb_format_ok accepts. */
static RTex *tex_new(void *pixels, PFsizei w, PFsizei h, PFpixelformat f, PFdatatype t, int sampled)
{
    if (sampled ? !texel_bytes(f, t) : !fb_format_ok(f, t)) {
        if (G) G->err = PF_INVALID_ENUM;
        return NULL;
    }
    RTex *x = (RTex *)calloc(1, sizeof(RTex));
    x->pixels = pixels; x->format = f; x->type = t; x->w = w; x->h = h;
    x->tx = 1.0f / (float)w; x->ty = 1.0f / (float)h;
    x->wrap = PF_REPEAT; x->filter = PF_NEAREST;
    return x;
}

PFcontext pfCreateContext(void *buf, PFsizei w, PFsizei h, PFpixelformat f, PFdatatype t)
{
    RCtx *c = (RCtx *)calloc(1, sizeof(RCtx));
    if (!c) return NULL;
    c->main.texture = tex_new(buf, w, h, f, t, 0);
    if (!c->main.texture) { free(c); return NULL; }
    c->main.zbuffer = (float *)malloc((size_t)w * h * sizeof(float));
    for (size_t i = 0; i < (size_t)w * h; i++) c->main.zbuffer[i] = FLT_MAX;
    c->current = &c->main;
    c->vpPos[0] = c->vpMin[0] = 0; c->vpPos[1] = c->vpMin[1] = 0;
    c->vpDim[0] = w - 1; c->vpMax[0] = (PFint)w - 1;
    c->vpDim[1] = h - 1; c->vpMax[1] = (PFint)h - 1;
    c->blend = PF_BLEND_ALPHA; c->depthFunc = PF_LESS;
    PFcolor cc = { 0, 0, 0, 255 }; c->clearColor = cc; c->clearDepth = FLT_MAX;
    c->polygonMode[0] = c->polygonMode[1] = PF_FILL;
    c->pointSize = 1.0f; c->lineWidth = 1.0f;
    PFcolor white = { 255, 255, 255, 255 }; c->curColor = white;
    for (int i = 0; i < MAX_LIGHTS; i++) {
        RLight *l = &c->lights[i]; memset(l, 0, sizeof *l);
        l->innerCutOff = l->outerCutOff = (float)REF_PI;
        l->attConstant = 1;
        PFcolor amb = { 51, 51, 51, 255 }; l->ambient = amb; l->diffuse = white; l->specular = white;
    }
    RMat m = { white, white, white, { 0, 0, 0, 255 }, 64.0f };
    c->mat[0] = c->mat[1] = m;
    c->colMatFace = PF_FRONT_AND_BACK; c->colMatMode = PF_AMBIENT_AND_DIFFUSE;
    c->matMode = PF_MODELVIEW; c->cur = c->view;
    /* pfmMat4Ortho(-1, 1, -1, 1, -1, 1) (src/pfm.h:2422-2440) */
    memset(c->proj, 0, 64);
    c->proj[0] = 2.0f / 2.0f; c->proj[5] = 2.0f / 2.0f; c->proj[10] = -2.0f / 2.0f;
    c->proj[12] = -(-1.0f + 1.0f) / 2.0f; c->proj[13] = -(1.0f + -1.0f) / 2.0f;
    c->proj[14] = -(1.0f + -1.0f) / 2.0f; c->proj[15] = 1.0f;
    m_identity(c->tex); m_identity(c->normal); m_identity(c->model); m_identity(c->view);
    c->state = PF_CULL_FACE; c->shade = PF_SMOOTH; c->lightMode = PF_GOURAUD; c->cullFace = PF_BACK;
    c->depthMask = PF_TRUE;
    c->rasterPos[3] = 1.0f; c->pixelZoom[0] = c->pixelZoom[1] = 1.0f;          /* context.c:179-180 */
    c->fog.mode = PF_LINEAR; c->fog.density = 1.0f; c->fog.start = 0.0f; c->fog.end = 1.0f;   /* :203-209 */
    return c;
}

void pfDeleteContext(PFcontext ctx)
{
    RCtx *c = (RCtx *)ctx;
    if (!c) return;
    free(c->main.zbuffer); free(c->main.texture); free(c);
    if (G == c) G = NULL;
}

void pfSetMainBuffer(void *buf, PFsizei w, PFsizei h, PFpixelformat f, PFdatatype t)
{
    if (!buf || !w || !h) { G->err = PF_INVALID_VALUE; return; }
    if (!fb_format_ok(f, t)) { G->err = PF_INVALID_ENUM; return; }   /* the main buffer stays as it was */
    RTex *old = (RTex *)G->main.texture;
    if (old->w != w || old->h != h) {
        free(G->main.zbuffer);
        G->main.zbuffer = (float *)malloc((size_t)w * h * sizeof(float));
        for (size_t i = 0; i < (size_t)w * h; i++) G->main.zbuffer[i] = G->clearDepth;
    }
    free(old);
    G->main.texture = tex_new(buf, w, h, f, t, 0);
    G->aux = NULL;
}

void pfSetAuxBuffer(void *aux) { G->aux = aux; }
void pfSwapBuffers(void)
{
    if (!G->aux) { G->err = PF_INVALID_OPERATION; return; }
    RTex *t = (RTex *)G->current->texture;
    void *tmp = t->pixels; t->pixels = G->aux; G->aux = tmp;
}
PFcontext pfGetCurrentContext(void) { return G; }
void pfMakeCurrent(PFcontext ctx) { G = (RCtx *)ctx; }
PFboolean pfIsEnabled(PFstate s) { return (G->state & s) != 0; }
void pfEnable(PFstate s)
{
    G->state |= s;
    if (s & PF_FRAMEBUFFER) G->current = G->bound ? G->bound : &G->main;
}
void pfDisable(PFstate s)
{
    G->state &= ~(PFuint)s;
    if (s & PF_FRAMEBUFFER) G->current = &G->main;
}
PFerrcode pfGetError(void) { PFerrcode e = G->err; G->err = PF_NO_ERROR; return e; }

/* getters (src/getter.c:24-521): the reference's cases; other names set
 * PF_INVALID_ENUM and leave the output untouched.  Point size, line width,
 * raster position and pixel zoom are not modelled by this oracle (the
 * triangle path does not read them) and read as their initial values
 * (context.c:179-180). */
void pfGetBooleanv(PFenum p, PFboolean *v)
{
    switch (p) {
    case PF_TEXTURE_2D: case PF_FRAMEBUFFER: case PF_BLEND: case PF_DEPTH_TEST: case PF_CULL_FACE:
    case PF_NORMALIZE: case PF_LIGHTING: case PF_COLOR_MATERIAL: case PF_VERTEX_ARRAY: case PF_NORMAL_ARRAY:
    case PF_COLOR_ARRAY: case PF_TEXTURE_COORD_ARRAY:
        *v = (G->state & p) != 0; break;
    case PF_VERTEX_ARRAY_TYPE: *v = G->positions.type != 0; break;
    case PF_NORMAL_ARRAY_STRIDE: *v = G->normals.stride != 0; break;
    case PF_NORMAL_ARRAY_TYPE: *v = G->normals.type != 0; break;
    case PF_TEXTURE_COORD_ARRAY_STRIDE: *v = G->texcoords.stride != 0; break;
    case PF_TEXTURE_COORD_ARRAY_TYPE: *v = G->texcoords.type != 0; break;
    case PF_COLOR_ARRAY_SIZE: *v = G->colors.size != 0; break;
    case PF_COLOR_ARRAY_STRIDE: *v = G->colors.stride != 0; break;
    case PF_COLOR_ARRAY_TYPE: *v = G->colors.type != 0; break;
    default: G->err = PF_INVALID_ENUM; break;
    }
}
void pfGetIntegerv(PFenum p, PFint *v)
{
    switch (p) {
    case PF_VIEWPORT: v[0] = G->vpPos[0]; v[1] = G->vpPos[1]; v[2] = (PFint)G->vpDim[0] + 1; v[3] = (PFint)G->vpDim[1] + 1; break;
    case PF_COLOR_CLEAR_VALUE: v[0] = G->clearColor.r; v[1] = G->clearColor.g; v[2] = G->clearColor.b; v[3] = G->clearColor.a; break;
    case PF_CULL_FACE_MODE: v[0] = G->cullFace; break;
    case PF_CURRENT_COLOR: v[0] = G->curColor.r; v[1] = G->curColor.g; v[2] = G->curColor.b; v[3] = G->curColor.a; break;
    case PF_CURRENT_RASTER_POSITION: v[0] = ox_ftoi(G->rasterPos[0]); v[1] = ox_ftoi(G->rasterPos[1]); break;
    case PF_POLYGON_MODE: v[0] = G->polygonMode[0]; v[1] = G->polygonMode[1]; break;
    case PF_MATRIX_MODE: v[0] = G->matMode; break;
    case PF_MAX_PROJECTION_STACK_DEPTH: v[0] = 2; break;
    case PF_MAX_MODELVIEW_STACK_DEPTH: v[0] = 8; break;
    case PF_MAX_TEXTURE_STACK_DEPTH: v[0] = 4; break;
    case PF_SHADE_MODEL: v[0] = G->shade; break;
    case PF_MAX_LIGHTS: v[0] = MAX_LIGHTS; break;
    case PF_VERTEX_ARRAY_SIZE: v[0] = G->positions.size; break;
    case PF_VERTEX_ARRAY_STRIDE: v[0] = (PFint)G->positions.stride; break;
    case PF_VERTEX_ARRAY_TYPE: v[0] = (PFint)G->positions.type; break;
    case PF_NORMAL_ARRAY_STRIDE: v[0] = (PFint)G->normals.stride; break;
    case PF_NORMAL_ARRAY_TYPE: v[0] = (PFint)G->normals.type; break;
    case PF_TEXTURE_COORD_ARRAY_STRIDE: v[0] = (PFint)G->texcoords.stride; break;
    case PF_TEXTURE_COORD_ARRAY_TYPE: v[0] = (PFint)G->texcoords.type; break;
    case PF_COLOR_ARRAY_SIZE: v[0] = G->colors.size; break;
    case PF_COLOR_ARRAY_STRIDE: v[0] = (PFint)G->colors.stride; break;
    case PF_COLOR_ARRAY_TYPE: v[0] = (PFint)G->colors.type; break;
    default: G->err = PF_INVALID_ENUM; break;
    }
}
#define GET_REAL(T, INV)                                                                      \
    switch (p) {                                                                              \
    case PF_COLOR_CLEAR_VALUE: v[0] = G->clearColor.r*(INV); v[1] = G->clearColor.g*(INV);    \
        v[2] = G->clearColor.b*(INV); v[3] = G->clearColor.a*(INV); break;                    \
    case PF_DEPTH_CLEAR_VALUE: v[0] = G->clearDepth; break;                                   \
    case PF_CURRENT_COLOR: v[0] = G->curColor.r*(INV); v[1] = G->curColor.g*(INV);            \
        v[2] = G->curColor.b*(INV); v[3] = G->curColor.a*(INV); break;                        \
    case PF_CURRENT_NORMAL: for (int i = 0; i < 3; i++) v[i] = G->curNormal[i]; break;        \
    case PF_CURRENT_TEXTURE_COORDS: for (int i = 0; i < 2; i++) v[i] = G->curTex[i]; break;   \
    case PF_CURRENT_RASTER_POSITION: v[0] = G->rasterPos[0]; v[1] = G->rasterPos[1]; break;   \
    case PF_POINT_SIZE: v[0] = G->pointSize; break;                                          \
    case PF_LINE_WIDTH: v[0] = G->lineWidth; break;                                          \
    case PF_ZOOM_X: v[0] = G->pixelZoom[0]; break;                                           \
    case PF_ZOOM_Y: v[0] = G->pixelZoom[1]; break;                                           \
    case PF_PROJECTION_MATRIX: for (int i = 0; i < 16; i++) v[i] = G->proj[i]; break;        \
    case PF_MODELVIEW_MATRIX: { mat4 mv; m_mul(mv, G->model, G->view);                       \
        for (int i = 0; i < 16; i++) { v[i] = mv[i]; } break; }                               \
    case PF_TEXTURE_MATRIX: for (int i = 0; i < 16; i++) v[i] = G->tex[i]; break;            \
    default: G->err = PF_INVALID_ENUM; break;                                                 \
    }
void pfGetFloatv(PFenum p, PFfloat *v) { GET_REAL(PFfloat, (PFfloat)(1.0 / 255)) }
void pfGetDoublev(PFenum p, PFdouble *v) { GET_REAL(PFdouble, (1.0 / 255)) }
#undef GET_REAL
void pfGetPointerv(PFenum p, const void **v)
{
    switch (p) {
    case PF_TEXTURE_2D: *v = G->texture; break;
    case PF_FRAMEBUFFER: *v = G->bound; break;
    case PF_BLEND_FUNC: *v = &G->blend; break;
    case PF_DEPTH_FUNC: *v = &G->depthFunc; break;
    default: G->err = PF_INVALID_ENUM; break;
    }
}

/* ------------------------------------------------------------------------ */
/* API: matrices (context.c:392-548)                                         */
/* ------------------------------------------------------------------------ */

void pfMatrixMode(PFmatrixmode m)
{
    switch (m) {
    case PF_PROJECTION: G->cur = G->proj; break;
    case PF_MODELVIEW: G->cur = G->modelUsed ? G->model : G->view; break;
    case PF_TEXTURE: G->cur = G->tex; break;
    default: G->err = PF_INVALID_ENUM; return;
    }
    G->matMode = m;
}
void pfPushMatrix(void)
{
    switch (G->matMode) {
    case PF_PROJECTION:
        if (G->nProj >= 2) { G->err = PF_STACK_OVERFLOW; return; }
        memcpy(G->stackProj[G->nProj++], G->proj, 64); break;
    case PF_MODELVIEW:
        if (G->nMV >= 8) { G->err = PF_STACK_OVERFLOW; return; }
        if (G->modelUsed) memcpy(G->stackMV[G->nMV++], G->model, 64);
        else { G->cur = G->model; G->modelUsed = 1; }
        break;
    case PF_TEXTURE:
        if (G->nTex >= 4) { G->err = PF_STACK_OVERFLOW; return; }
        memcpy(G->stackTex[G->nTex++], G->tex, 64); break;
    }
}
void pfPopMatrix(void)
{
    switch (G->matMode) {
    case PF_PROJECTION:
        if (G->nProj == 0) { G->err = PF_STACK_UNDERFLOW; return; }
        memcpy(G->proj, G->stackProj[--G->nProj], 64); break;
    case PF_MODELVIEW:
        if (G->nMV == 0) {
            if (!G->modelUsed) { G->err = PF_STACK_UNDERFLOW; return; }
            m_identity(G->model); G->modelUsed = 0; G->cur = G->view;
        } else memcpy(G->model, G->stackMV[--G->nMV], 64);
        break;
    case PF_TEXTURE:
        if (G->nTex == 0) { G->err = PF_STACK_UNDERFLOW; return; }
        memcpy(G->tex, G->stackTex[--G->nTex], 64); break;
    }
}
void pfLoadIdentity(void) { m_identity(G->cur); }
void pfTranslatef(PFfloat x, PFfloat y, PFfloat z)
{
    float t[16]; m_identity(t); t[12] = x; t[13] = y; t[14] = z;
    m_mul(G->cur, t, G->cur);
}
void pfRotatef(PFfloat angle, PFfloat x, PFfloat y, PFfloat z)
{
    /* pfmMat4Rotate (src/pfm.h:2227-2262) with angle*DEG2RAD in double then float */
    float a = (float)(angle * REF_DEG2RAD);
    float r[16]; m_identity(r);
    float lsq = x*x + y*y + z*z;
    if (lsq != 1.0f && lsq != 0.0f) { float il = 1.0f / sqrtf(lsq); x *= il; y *= il; z *= il; }
    float s = sinf(a), co = cosf(a), t = 1.0f - co;
    r[0] = x*x*t + co; r[1] = y*x*t + z*s; r[2] = z*x*t - y*s;
    r[4] = x*y*t - z*s; r[5] = y*y*t + co; r[6] = z*y*t + x*s;
    r[8] = x*z*t + y*s; r[9] = y*z*t - x*s; r[10] = z*z*t + co;
    m_mul(G->cur, r, G->cur);
}
void pfScalef(PFfloat x, PFfloat y, PFfloat z)
{
    float s[16]; memset(s, 0, 64); s[0] = x; s[5] = y; s[10] = z; s[15] = 1.0f;
    m_mul(G->cur, s, G->cur);
}
void pfMultMatrixf(const PFfloat *m) { m_mul(G->cur, G->cur, m); }
void pfFrustum(PFfloat l, PFfloat r, PFfloat b, PFfloat t, PFfloat n, PFfloat f)
{
    float m[16]; memset(m, 0, 64);
    float rl = r - l, tb = t - b, fn = f - n;
    m[0] = (n*2.0f)/rl; m[5] = (n*2.0f)/tb; m[8] = (r + l)/rl; m[9] = (t + b)/tb;
    m[10] = -(f + n)/fn; m[11] = -1.0f; m[14] = -(f*n*2.0f)/fn;
    m_mul(G->cur, G->cur, m);
}
void pfOrtho(PFfloat l, PFfloat r, PFfloat b, PFfloat t, PFfloat n, PFfloat f)
{
    float m[16]; memset(m, 0, 64);
    float rl = r - l, tb = t - b, fn = f - n;
    m[0] = 2.0f/rl; m[5] = 2.0f/tb; m[10] = -2.0f/fn;
    m[12] = -(l + r)/rl; m[13] = -(t + b)/tb; m[14] = -(f + n)/fn; m[15] = 1.0f;
    m_mul(G->cur, G->cur, m);
}

/* ------------------------------------------------------------------------ */
/* API: render configuration (context.c:553-797)                             */
/* ------------------------------------------------------------------------ */

void pfViewport(PFint x, PFint y, PFsizei w, PFsizei h)
{
    if (x <= -(PFint)w || y <= -(PFint)h) { G->err = PF_INVALID_OPERATION; return; }
    RTex *mt = (RTex *)G->main.texture;
    G->vpPos[0] = x; G->vpPos[1] = y; G->vpDim[0] = w - 1; G->vpDim[1] = h - 1;
    G->vpMin[0] = x > 0 ? x : 0; G->vpMin[1] = y > 0 ? y : 0;
    PFint ex = x + (PFint)w, ey = y + (PFint)h;
    G->vpMax[0] = ex < (PFint)mt->w - 1 ? ex : (PFint)mt->w - 1;
    G->vpMax[1] = ey < (PFint)mt->h - 1 ? ey : (PFint)mt->h - 1;
}
void pfPolygonMode(PFface f, PFpolygonmode m)
{
    if (!(m == PF_POINT || m == PF_LINE || m == PF_FILL)) { G->err = PF_INVALID_ENUM; return; }
    switch (f) {
    case PF_FRONT: G->polygonMode[0] = m; break;
    case PF_BACK: G->polygonMode[1] = m; break;
    case PF_FRONT_AND_BACK: G->polygonMode[0] = G->polygonMode[1] = m; break;
    default: G->err = PF_INVALID_ENUM; break;
    }
}
void pfShadeModel(PFshademode m) { G->shade = m; }
void pfLightModel(PFlightmode m) { G->lightMode = m; }
void pfLineWidth(PFfloat w) { if (w <= 0.0f) { G->err = PF_INVALID_VALUE; return; } G->lineWidth = w; }   /* context.c:610-626 */
void pfPointSize(PFfloat s) { if (s <= 0.0f) { G->err = PF_INVALID_VALUE; return; } G->pointSize = s; }
void pfCullFace(PFface f) { if (f < PF_FRONT || f > PF_BACK) { G->err = PF_INVALID_ENUM; return; } G->cullFace = f; }
void pfBlendFunc(PFblendmode m) { if (m < PF_BLEND_AVERAGE || m > PF_BLEND_DARKEN) { G->err = PF_INVALID_ENUM; return; } G->blend = m; }
void pfDepthFunc(PFdepthmode m) { if (m < PF_EQUAL || m > PF_GEQUAL) { G->err = PF_INVALID_ENUM; return; } G->depthFunc = m; }
void pfBindFramebuffer(PFframebuffer *fb)
{
    G->bound = fb;
    if (G->state & PF_FRAMEBUFFER) G->current = fb ? fb : &G->main;
}
void pfBindTexture(PFtexture t) { G->texture = (RTex *)t; }

/* pfClear, SIMD build (context.c:680-745): any flag clears colour AND depth;
 * the vector loop starts at pixel 8, so pixels 0..7 keep their values; the
 * tail (size % 8 pixels) is copied from pixel 0. */
void pfClear(PFclearflag flag)
{
    if (!flag) return;
    RTex *t = (RTex *)G->current->texture;
    size_t size = (size_t)t->w * t->h;
    size_t aligned = size - (size % 8);
    float *zb = G->current->zbuffer;
    const uint32_t cc = col_pack(G->clearColor);
    const size_t bpp = (size_t)texel_bytes(t->format, t->type);
    uint8_t *pb = (uint8_t *)t->pixels;
    /* The tail copy steps by pfiGetPixelBytes (pixel.h:3156-3210), components
     * x type size: 6 or 8 bytes for the packed 16-bit types, whose pixels
     * are 2 bytes, so that there it writes past the pixels (outside the
     * buffer) and the tail pixels keep their values. */
    const int packed = t->type == PF_UNSIGNED_SHORT_5_6_5 || t->type == PF_UNSIGNED_SHORT_5_5_5_1 ||
                       t->type == PF_UNSIGNED_SHORT_4_4_4_4;
    for (size_t i = 8; i < aligned; i++) { fb_set_simd(t, i, cc); zb[i] = G->clearDepth; }
    for (size_t i = aligned; i < size; i++) { if (!packed) memcpy(pb + i * bpp, pb, bpp); zb[i] = zb[0]; }
}
void pfClearDepth(PFfloat d) { G->clearDepth = d; }
void pfClearColor(PFubyte r, PFubyte g, PFubyte b, PFubyte a) { PFcolor c = { r, g, b, a }; G->clearColor = c; }
void pfDepthMask(PFboolean f) { G->depthMask = f; }
void pfFinish(void) { }

/* ------------------------------------------------------------------------ */
/* API: lights and materials (context.c:802-1156)                            */
/* ------------------------------------------------------------------------ */

void pfEnableLight(PFsizei l)
{
    if (l >= MAX_LIGHTS) { G->err = PF_INVALID_VALUE; return; }
    for (int i = 0; i < G->nActive; i++) if (G->lightOrder[i] == (int)l) { G->err = PF_INVALID_OPERATION; return; }
    G->lightOrder[G->nActive++] = (int)l;
}
void pfDisableLight(PFsizei l)
{
    if (l >= MAX_LIGHTS) { G->err = PF_INVALID_VALUE; return; }
    for (int i = 0; i < G->nActive; i++) if (G->lightOrder[i] == (int)l) {
        memmove(&G->lightOrder[i], &G->lightOrder[i + 1], (size_t)(G->nActive - i - 1) * sizeof(int));
        G->nActive--; return;
    }
    G->err = PF_INVALID_OPERATION;
}
PFboolean pfIsEnabledLight(PFsizei l)
{
    if (l >= MAX_LIGHTS) { G->err = PF_INVALID_VALUE; return PF_FALSE; }
    for (int i = 0; i < G->nActive; i++) if (G->lightOrder[i] == (int)l) return PF_TRUE;
    return PF_FALSE;
}
static PFcolor f3_to_color(const float *v)
{
    PFcolor c = { ox_ftoub(v[0]*255.0f), ox_ftoub(v[1]*255.0f), ox_ftoub(v[2]*255.0f), 255 };
    return c;
}
static int cutoff_ok(float v) { return (v >= 0 && v <= 90) || v == 180; }
void pfLightf(PFsizei li, PFenum p, PFfloat v)
{
    if (li >= MAX_LIGHTS) { G->err = PF_STACK_OVERFLOW; return; }
    RLight *l = &G->lights[li];
    switch (p) {
    case PF_SPOT_INNER_CUTOFF: if (cutoff_ok(v)) l->innerCutOff = cosf((float)(v * REF_DEG2RAD)); else G->err = PF_INVALID_VALUE; break;
    case PF_SPOT_OUTER_CUTOFF: if (cutoff_ok(v)) l->outerCutOff = cosf((float)(v * REF_DEG2RAD)); else G->err = PF_INVALID_VALUE; break;
    case PF_CONSTANT_ATTENUATION: l->attConstant = v; break;
    case PF_LINEAR_ATTENUATION: l->attLinear = v; break;
    case PF_QUADRATIC_ATTENUATION: l->attQuadratic = v; break;
    default: G->err = PF_INVALID_ENUM; break;
    }
}
void pfLightfv(PFsizei li, PFenum p, const void *value)
{
    if (li >= MAX_LIGHTS) { G->err = PF_STACK_OVERFLOW; return; }
    RLight *l = &G->lights[li];
    const float *v = (const float *)value;
    switch (p) {
    case PF_POSITION: memcpy(l->position, v, 12); break;
    case PF_SPOT_DIRECTION: memcpy(l->direction, v, 12); break;
    case PF_SPOT_INNER_CUTOFF: case PF_SPOT_OUTER_CUTOFF: case PF_CONSTANT_ATTENUATION:
    case PF_LINEAR_ATTENUATION: case PF_QUADRATIC_ATTENUATION: pfLightf(li, p, v[0]); break;
    case PF_AMBIENT: l->ambient = f3_to_color(v); break;
    case PF_DIFFUSE: l->diffuse = f3_to_color(v); break;
    case PF_SPECULAR: l->specular = f3_to_color(v); break;
    default: G->err = PF_INVALID_ENUM; break;
    }
}
static int mat_pair(PFface f, RMat **a, RMat **b)
{
    switch (f) {
    case PF_FRONT: *a = *b = &G->mat[0]; return 1;
    case PF_BACK: *a = *b = &G->mat[1]; return 1;
    case PF_FRONT_AND_BACK: *a = &G->mat[0]; *b = &G->mat[1]; return 1;
    default: G->err = PF_INVALID_ENUM; return 0;
    }
}
static void mat_set(PFface f, PFenum p, const float *v)
{
    RMat *a, *b;
    if (!mat_pair(f, &a, &b)) return;
    PFcolor c = f3_to_color(v);
    switch (p) {
    case PF_AMBIENT: a->ambient = b->ambient = c; break;
    case PF_DIFFUSE: a->diffuse = b->diffuse = c; break;
    case PF_SPECULAR: a->specular = b->specular = c; break;
    case PF_EMISSION: a->emission = b->emission = c; break;
    case PF_SHININESS: a->shininess = b->shininess = v[0]; break;
    case PF_AMBIENT_AND_DIFFUSE: a->ambient = b->ambient = c; a->diffuse = b->diffuse = c; break;
    default: G->err = PF_INVALID_ENUM; break;
    }
}
void pfMaterialf(PFface f, PFenum p, PFfloat v) { float vv[3] = { v, v, v }; mat_set(f, p, vv); }
void pfMaterialfv(PFface f, PFenum p, const void *v) { mat_set(f, p, (const float *)v); }
void pfColorMaterial(PFface f, PFenum m)
{
    if (f > PF_FRONT_AND_BACK) { G->err = PF_INVALID_ENUM; return; }
    if (m < PF_AMBIENT_AND_DIFFUSE || m > PF_EMISSION) { G->err = PF_INVALID_ENUM; return; }
    G->colMatFace = f; G->colMatMode = m;
}

/* ------------------------------------------------------------------------ */
/* API: vertex capture (context.c:1161-1913)                                  */
/* ------------------------------------------------------------------------ */

void pfVertexPointer(PFint size, PFenum type, PFsizei stride, const void *p)
{
    if (size < 2 || size > 4) { G->err = PF_INVALID_VALUE; return; }
    if (!(type == PF_SHORT || type == PF_INT || type == PF_FLOAT || type == PF_DOUBLE)) { G->err = PF_INVALID_ENUM; return; }
    RAttrib a = { p, stride, size, type }; G->positions = a;
}
void pfNormalPointer(PFenum type, PFsizei stride, const void *p)
{
    if (!(type == PF_FLOAT || type == PF_DOUBLE)) { G->err = PF_INVALID_ENUM; return; }
    RAttrib a = { p, stride, 3, type }; G->normals = a;
}
void pfTexCoordPointer(PFenum type, PFsizei stride, const void *p)
{
    if (!(type == PF_FLOAT || type == PF_DOUBLE)) { G->err = PF_INVALID_ENUM; return; }
    RAttrib a = { p, stride, 2, type }; G->texcoords = a;
}
void pfColorPointer(PFint size, PFenum type, PFsizei stride, const void *p)
{
    if (size < 3 || size > 4) { G->err = PF_INVALID_VALUE; return; }
    if (!(type == PF_UNSIGNED_BYTE || type == PF_UNSIGNED_SHORT || type == PF_UNSIGNED_INT ||
          type == PF_FLOAT || type == PF_DOUBLE)) { G->err = PF_INVALID_ENUM; return; }
    RAttrib a = { p, stride, size, type }; G->colors = a;
}

static float attr_f(const RAttrib *a, size_t idx)
{
    switch (a->type) {
    case PF_SHORT: return (float)((const PFshort *)a->buf)[idx];
    case PF_INT: return (float)((const PFint *)a->buf)[idx];
    case PF_FLOAT: return ((const PFfloat *)a->buf)[idx];
    case PF_DOUBLE: return (float)((const PFdouble *)a->buf)[idx];
    }
    return 0.0f;
}

/* Fill one vertex from the enabled arrays, element j (stride ignored, as in
 * context.c:1285 and 1443). */
static void fetch_vertex(RCtx *c, RVert *v, size_t j, int useN, int useT, int useC)
{
    v->position[0] = v->position[1] = v->position[2] = 0.0f; v->position[3] = 1.0f;
    for (int k = 0; k < c->positions.size; k++) v->position[k] = attr_f(&c->positions, j * (size_t)c->positions.size + (size_t)k);
    if (useN) for (int k = 0; k < 3; k++) v->normal[k] = attr_f(&c->normals, j * 3 + (size_t)k);
    if (useT) for (int k = 0; k < 2; k++) v->texcoord[k] = attr_f(&c->texcoords, j * 2 + (size_t)k);
    if (useC) {
        uint8_t *cb = (uint8_t *)&v->color; memset(cb, 0xff, 4);
        for (int k = 0; k < c->colors.size; k++) {
            size_t o = j * (size_t)c->colors.size + (size_t)k;
            switch (c->colors.type) {
            case PF_UNSIGNED_BYTE: cb[k] = ((const PFubyte *)c->colors.buf)[o]; break;
            case PF_UNSIGNED_SHORT: cb[k] = (uint8_t)(((const PFushort *)c->colors.buf)[o] >> 8); break;
            case PF_UNSIGNED_INT: cb[k] = (uint8_t)(((const PFuint *)c->colors.buf)[o] >> 24); break;
            case PF_FLOAT: cb[k] = ox_ftoub(((const PFfloat *)c->colors.buf)[o] * 255); break;
            case PF_DOUBLE: cb[k] = ox_dtoub(((const PFdouble *)c->colors.buf)[o] * 255); break;
            }
        }
    }
}

static void draw_arrays_common(PFdrawmode mode, PFsizei count, const void *idx, PFdatatype itype, PFint first)
{
    RCtx *c = G;
    int useT = (c->state & PF_TEXTURE_COORD_ARRAY) && c->texcoords.buf;
    int useN = (c->state & PF_NORMAL_ARRAY) && c->normals.buf;
    int useC = (c->state & PF_COLOR_ARRAY) && c->colors.buf;
    PFsizei nv = mode_count(mode);
    for (PFsizei i = 0; i < nv && i < 6; i++) { memset(&c->vbuf[i], 0, sizeof(RVert)); c->vbuf[i].color = c->curColor; }
    pfBegin(mode);
    for (PFsizei i = 0; i < count; i++) {
        RVert *v = &c->vbuf[c->vcount++];
        size_t j;
        if (idx) {
            switch (itype) {
            case PF_UNSIGNED_BYTE: j = ((const PFubyte *)idx)[i]; break;
            case PF_UNSIGNED_SHORT: j = ((const PFushort *)idx)[i]; break;
            default: j = ((const PFuint *)idx)[i]; break;
            }
        } else j = (size_t)first + i;
        fetch_vertex(c, v, j, useN, useT, useC);
        if (c->vcount == nv) { process_and_raster(c); reset_for_next(c); }
    }
    pfEnd();
}

void pfDrawElements(PFdrawmode mode, PFsizei count, PFdatatype type, const void *indices)
{
    if (!(type == PF_UNSIGNED_BYTE || type == PF_UNSIGNED_SHORT || type == PF_UNSIGNED_INT)) { G->err = PF_INVALID_ENUM; return; }
    if (!(G->state & PF_VERTEX_ARRAY)) { G->err = PF_INVALID_OPERATION; return; }
    draw_arrays_common(mode, count, indices, type, 0);
}
void pfDrawArrays(PFdrawmode mode, PFint first, PFsizei count)
{
    if (!(G->state & PF_VERTEX_ARRAY)) { G->err = PF_INVALID_OPERATION; return; }
    draw_arrays_common(mode, count, NULL, PF_UNSIGNED_INT, first);
}

static void list_begin(RCtx *c, PFdrawmode mode);
static void list_vertex(RCtx *c, const PFfloat *v);

void pfBegin(PFdrawmode mode)   /* context.c:1580-1603 */
{
    if (G->curList) { list_begin(G, mode); return; }
    if (mode > PF_QUAD_STRIP) { G->err = PF_INVALID_ENUM; return; }
    update_matrices(G, !(mode == PF_POINTS || mode == PF_LINES));
    G->drawMode = mode; G->vcount = 0;
}
void pfEnd(void) { G->vcount = 0; }

void pfVertex4fv(const PFfloat *v)   /* context.c:1655-1685 */
{
    RCtx *c = G;
    if (c->curList) { list_vertex(c, v); return; }
    RVert *x = &c->vbuf[c->vcount++];
    memcpy(x->position, v, 16);
    memcpy(x->normal, c->curNormal, 12);
    memcpy(x->texcoord, c->curTex, 8);
    x->color = c->curColor;
    if (c->vcount == mode_count(c->drawMode)) { process_and_raster(c); reset_for_next(c); }
}
void pfVertex2i(PFint x, PFint y) { float v[4] = { (float)x, (float)y, 0.0f, 1.0f }; pfVertex4fv(v); }
void pfVertex2f(PFfloat x, PFfloat y) { float v[4] = { x, y, 0.0f, 1.0f }; pfVertex4fv(v); }
void pfVertex2fv(const PFfloat *p) { float v[4] = { p[0], p[1], 0.0f, 1.0f }; pfVertex4fv(v); }
void pfVertex3i(PFint x, PFint y, PFint z) { float v[4] = { (float)x, (float)y, (float)z, 1.0f }; pfVertex4fv(v); }
void pfVertex3f(PFfloat x, PFfloat y, PFfloat z) { float v[4] = { x, y, z, 1.0f }; pfVertex4fv(v); }
void pfVertex3fv(const PFfloat *p) { float v[4] = { p[0], p[1], p[2], 1.0f }; pfVertex4fv(v); }
void pfVertex4i(PFint x, PFint y, PFint z, PFint w) { float v[4] = { (float)x, (float)y, (float)z, (float)w }; pfVertex4fv(v); }
void pfVertex4f(PFfloat x, PFfloat y, PFfloat z, PFfloat w) { float v[4] = { x, y, z, w }; pfVertex4fv(v); }

void pfColor(PFcolor col)   /* context.c:1687-1717 */
{
    if (G->state & PF_COLOR_MATERIAL) {
        RMat *m1 = &G->mat[0], *m2 = &G->mat[1];
        if (G->colMatFace == PF_FRONT) m2 = m1; else if (G->colMatFace == PF_BACK) m1 = m2;
        switch (G->colMatMode) {
        case PF_AMBIENT_AND_DIFFUSE: m1->ambient = m2->ambient = col; m1->diffuse = m2->diffuse = col; break;
        case PF_AMBIENT: m1->ambient = m2->ambient = col; break;
        case PF_DIFFUSE: m1->diffuse = m2->diffuse = col; break;
        case PF_SPECULAR: m1->specular = m2->specular = col; break;
        case PF_EMISSION: m1->emission = m2->emission = col; break;
        }
    } else G->curColor = col;
}
void pfColor1ui(PFuint u) { pfColor(col_unpack(u)); }
void pfColor3ub(PFubyte r, PFubyte g, PFubyte b) { PFcolor c = { r, g, b, 255 }; pfColor(c); }
void pfColor3ubv(const PFubyte *v) { pfColor3ub(v[0], v[1], v[2]); }
void pfColor3us(PFushort r, PFushort g, PFushort b) { pfColor3ub((PFubyte)(r >> 8), (PFubyte)(g >> 8), (PFubyte)(b >> 8)); }
void pfColor3usv(const PFushort *v) { pfColor3us(v[0], v[1], v[2]); }
void pfColor3ui(PFuint r, PFuint g, PFuint b) { pfColor3ub((PFubyte)(r >> 24), (PFubyte)(g >> 24), (PFubyte)(b >> 24)); }
void pfColor3uiv(const PFuint *v) { pfColor3ui(v[0], v[1], v[2]); }
void pfColor3f(PFfloat r, PFfloat g, PFfloat b) { pfColor3ub(ox_ftoub(r*255), ox_ftoub(g*255), ox_ftoub(b*255)); }
void pfColor3fv(const PFfloat *v) { pfColor3f(v[0], v[1], v[2]); }
void pfColor4ub(PFubyte r, PFubyte g, PFubyte b, PFubyte a) { PFcolor c = { r, g, b, a }; pfColor(c); }
void pfColor4ubv(const PFubyte *v) { pfColor4ub(v[0], v[1], v[2], v[3]); }
void pfColor4us(PFushort r, PFushort g, PFushort b, PFushort a) { pfColor4ub((PFubyte)(r >> 8), (PFubyte)(g >> 8), (PFubyte)(b >> 8), (PFubyte)(a >> 8)); }
void pfColor4usv(const PFushort *v) { pfColor4us(v[0], v[1], v[2], v[3]); }
void pfColor4ui(PFuint r, PFuint g, PFuint b, PFuint a) { pfColor4ub((PFubyte)(r >> 24), (PFubyte)(g >> 24), (PFubyte)(b >> 24), (PFubyte)(a >> 24)); }
void pfColor4uiv(const PFuint *v) { pfColor4ui(v[0], v[1], v[2], v[3]); }
void pfColor4f(PFfloat r, PFfloat g, PFfloat b, PFfloat a) { pfColor4ub(ox_ftoub(r*255), ox_ftoub(g*255), ox_ftoub(b*255), ox_ftoub(a*255)); }
void pfColor4fv(const PFfloat *v) { pfColor4f(v[0], v[1], v[2], v[3]); }
void pfTexCoord2f(PFfloat u, PFfloat v)   /* context.c:1874-1893: x texture matrix (pfmVec2Transform) */
{
    float *m = G->tex;
    float t0 = m[0]*u + m[4]*v + m[12], t1 = m[1]*u + m[5]*v + m[13];
    G->curTex[0] = t0; G->curTex[1] = t1;
}
void pfTexCoordfv(const PFfloat *v) { pfTexCoord2f(v[0], v[1]); }
void pfNormal3f(PFfloat x, PFfloat y, PFfloat z)
{
    G->curNormal[0] = x; G->curNormal[1] = y; G->curNormal[2] = z;
    if (G->state & PF_NORMALIZE) v3_normalize(G->curNormal);
}
void pfNormal3fv(const PFfloat *v) { pfNormal3f(v[0], v[1], v[2]); }

/* ------------------------------------------------------------------------ */
/* outside the triangle pipeline                                             */
/* ------------------------------------------------------------------------ */
/* (PFsizei)(float) as GCC emits it on x86-64: a 64-bit truncating convert
 * (cvttss2si), low 32 bits kept; 0 for NaN and out of range. */
static inline uint32_t ox_ftou32(float x)
{
    if (!(x > -9.2e18f && x < 9.2e18f)) return 0u;
    return (uint32_t)(int64_t)x;
}

static void put_pixel(RCtx *c, int64_t x, int64_t y, uint32_t col)
{
    RTex *fbt = (RTex *)c->current->texture;
    if (x < 0 || y < 0 || x >= (int64_t)fbt->w || y >= (int64_t)fbt->h) return;
    fb_set(fbt, (size_t)y * fbt->w + (size_t)x, col);
}

/* pfRectf (context.c:1936-1981): the two corners through the MVP to screen
 * (no +0.5), ordered, clamped to the viewport; every pixel of the inclusive
 * rectangle takes the current colour, no depth test, blending or depth
 * write.  Pixels outside the framebuffer are not drawn (the reference writes
 * them at y*w + x). */
void pfRectf(PFfloat x1, PFfloat y1, PFfloat x2, PFfloat y2)
{
    RCtx *c = G;
    update_matrices(c, 0);
    float v1[4] = { x1, y1, 0.0f, 1.0f }, v2[4] = { x2, y2, 0.0f, 1.0f };
    v4_transform(v1, v1, c->mvp);
    v4_transform(v2, v2, c->mvp);
    int32_t iX1 = ox_ftoi((float)c->vpPos[0] + (v1[0] + 1.0f) * 0.5f * (float)c->vpDim[0]);
    int32_t iY1 = ox_ftoi((float)c->vpPos[1] + (1.0f - v1[1]) * 0.5f * (float)c->vpDim[1]);
    int32_t iX2 = ox_ftoi((float)c->vpPos[0] + (v2[0] + 1.0f) * 0.5f * (float)c->vpDim[0]);
    int32_t iY2 = ox_ftoi((float)c->vpPos[1] + (1.0f - v2[1]) * 0.5f * (float)c->vpDim[1]);
    if (iX2 < iX1) { int32_t t = iX1; iX1 = iX2; iX2 = t; }
    if (iY2 < iY1) { int32_t t = iY1; iY1 = iY2; iY2 = t; }
#define ICLAMP(v, lo, hi) ((v) < (lo) ? (lo) : ((v) > (hi) ? (hi) : (v)))
    iX1 = ICLAMP(iX1, c->vpMin[0], c->vpMax[0]); iY1 = ICLAMP(iY1, c->vpMin[1], c->vpMax[1]);
    iX2 = ICLAMP(iX2, c->vpMin[0], c->vpMax[0]); iY2 = ICLAMP(iY2, c->vpMin[1], c->vpMax[1]);
    const uint32_t col = col_pack(c->curColor);
    for (int64_t y = iY1; y <= iY2; y++)
        for (int64_t x = iX1; x <= iX2; x++) put_pixel(c, x, y, col);
}
void pfRects(PFshort x1, PFshort y1, PFshort x2, PFshort y2) { pfRectf((PFfloat)x1, (PFfloat)y1, (PFfloat)x2, (PFfloat)y2); }
void pfRectsv(const PFshort *a, const PFshort *b) { pfRectf((PFfloat)a[0], (PFfloat)a[1], (PFfloat)b[0], (PFfloat)b[1]); }
void pfRectfv(const PFfloat *a, const PFfloat *b) { pfRectf(a[0], a[1], b[0], b[1]); }

/* RGBA8 value of the reference's scalar pixel getter for element o of a
 * buffer (src/internal/pixel.h:410-760), which pfDrawPixels reads with. */
static uint32_t pixel_sisd(PFpixelformat f, PFdatatype t, const void *p, size_t o)
{
    const uint8_t *b = (const uint8_t *)p;
    const uint16_t *h = (const uint16_t *)p;
    const float *fl = (const float *)p;
    uint32_t r = 0, g = 0, bl = 0, a = 255;
    if (t == PF_UNSIGNED_BYTE || t == PF_HALF_FLOAT || t == PF_FLOAT) {
        int n = 1;
        switch (f) {
        case PF_LUMINANCE_ALPHA: n = 2; break;
        case PF_RGB: case PF_BGR: n = 3; break;
        case PF_RGBA: case PF_BGRA: n = 4; break;
        default: n = 1; break;
        }
        uint32_t v[4] = { 0, 0, 0, 0 };
        for (int k = 0; k < n; k++) {
            const size_t i = o * (size_t)n + (size_t)k;
            if (t == PF_UNSIGNED_BYTE) v[k] = b[i];
            else if (t == PF_HALF_FLOAT) v[k] = ox_ftoub(255.0f * half_to_float(h[i]));
            else v[k] = ox_ftoub(255.0f * fl[i]);
        }
        switch (f) {
        case PF_RED: r = v[0]; break;
        case PF_GREEN: g = v[0]; break;
        case PF_BLUE: bl = v[0]; break;
        case PF_ALPHA: r = g = bl = 255; a = v[0]; break;
        case PF_LUMINANCE: r = g = bl = v[0]; break;
        case PF_LUMINANCE_ALPHA: r = g = bl = v[0]; a = v[1]; break;
        case PF_RGB: r = v[0]; g = v[1]; bl = v[2]; break;
        case PF_BGR: r = v[2]; g = v[1]; bl = v[0]; break;
        case PF_RGBA: r = v[0]; g = v[1]; bl = v[2]; a = v[3]; break;
        default: r = v[2]; g = v[1]; bl = v[0]; a = v[3]; break;      /* BGRA */
        }
    } else {
        const uint32_t px = h[o];
        const uint32_t hi5 = ox_ftoub((float)((px & 0xF800u) >> 11) * (255.0f / 31));
        if (t == PF_UNSIGNED_SHORT_5_6_5) {
            const uint32_t mid = ox_ftoub((float)((px & 0x7E0u) >> 5) * (255.0f / 63));
            const uint32_t lo = ox_ftoub((float)(px & 0x1Fu) * (255.0f / 31));
            r = (f == PF_RGB) ? hi5 : lo; g = mid; bl = (f == PF_RGB) ? lo : hi5;
        } else if (t == PF_UNSIGNED_SHORT_5_5_5_1) {
            const uint32_t mid = ox_ftoub((float)((px & 0x7C0u) >> 6) * (255.0f / 31));
            const uint32_t lo = ox_ftoub((float)((px & 0x3Eu) >> 1) * (255.0f / 31));
            r = (f == PF_RGBA) ? hi5 : lo; g = mid; bl = (f == PF_RGBA) ? lo : hi5;
            a = (px & 1u) * 255u;
        } else {                                                      /* 4-4-4-4 */
            const uint32_t c3 = ox_ftoub((float)((px & 0xF000u) >> 12) * (255.0f / 15));
            const uint32_t c2 = ox_ftoub((float)((px & 0xF00u) >> 8) * (255.0f / 15));
            const uint32_t c1 = ox_ftoub((float)((px & 0xF0u) >> 4) * (255.0f / 15));
            a = ox_ftoub((float)(px & 0xFu) * (255.0f / 15));
            r = (f == PF_RGBA) ? c3 : c1; g = c2; bl = (f == PF_RGBA) ? c1 : c3;
        }
    }
    return (r & 255u) | (g & 255u) << 8 | (bl & 255u) << 16 | (a & 255u) << 24;
}

/* pfDrawPixels (context.c:1990-2087): the raster position through the MVP
 * to screen; the destination rectangle [xMin, xMax] x [yMin, yMax] clamped
 * to the viewport; each pixel samples the source at
 * (u (w - 1), v (h - 1)) with u, v the offset over the zoomed size, passes
 * the scalar depth test (if enabled), writes the raster depth and stores the
 * (scalar-)blended colour.  Pixels outside the framebuffer, and source
 * elements outside the source buffer, are neither drawn nor read. */
void pfDrawPixels(PFsizei width, PFsizei height, PFpixelformat format, PFdatatype type, const void *pixels)
{
    RCtx *c = G;
    if (width == 0 || height == 0) { c->err = PF_INVALID_VALUE; return; }
    if (!(format >= PF_RED && format <= PF_BGRA && type >= PF_UNSIGNED_BYTE && type <= PF_DOUBLE)) { c->err = PF_INVALID_ENUM; return; }
    if (!texel_bytes(format, type)) { c->err = PF_INVALID_ENUM; return; }
    update_matrices(c, 0);
    float rp[4];
    v4_transform(rp, c->rasterPos, c->mvp);
    const int32_t xScreen = ox_ftoi((float)c->vpPos[0] + (rp[0] + 1.0f) * 0.5f * (float)c->vpDim[0]);
    const int32_t yScreen = ox_ftoi((float)c->vpPos[1] + (1.0f - rp[1]) * 0.5f * (float)c->vpDim[1]);
    const float zPos = rp[2];
    const int32_t xMin = ICLAMP(xScreen, c->vpMin[0], c->vpMax[0]);
    const int32_t yMin = ICLAMP(yScreen, c->vpMin[1], c->vpMax[1]);
    /* PF_CLAMP of a float against int bounds: the result is a float */
    const float xe = (float)xScreen + (float)width * c->pixelZoom[0];
    const float ye = (float)yScreen + (float)height * c->pixelZoom[1];
    const int32_t xMax = ox_ftoi(xe < (float)c->vpMin[0] ? (float)c->vpMin[0] : (xe > (float)c->vpMax[0] ? (float)c->vpMax[0] : xe));
    const int32_t yMax = ox_ftoi(ye < (float)c->vpMin[1] ? (float)c->vpMin[1] : (ye > (float)c->vpMax[1] ? (float)c->vpMax[1] : ye));
    const float invXLen = 1.0f / ((float)width * c->pixelZoom[0]);
    const float invYLen = 1.0f / ((float)height * c->pixelZoom[1]);
    const uint32_t widthM1 = width - 1, heightM1 = height - 1;
    RTex *dst = (RTex *)c->current->texture;
    float *zb = c->current->zbuffer;
    const int test = (c->state & PF_DEPTH_TEST) != 0;
    const size_t nSrc = (size_t)width * height;
    for (int64_t y = yMin; y <= yMax; y++) {
        const float v = (float)(int32_t)((uint32_t)y - (uint32_t)yScreen) * invYLen;
        const uint32_t ySrc = ox_ftou32(v * (float)heightM1) * width;
        for (int64_t x = xMin; x <= xMax; x++) {
            if (x < 0 || y < 0 || x >= (int64_t)dst->w || y >= (int64_t)dst->h) continue;
            const size_t p = (size_t)y * dst->w + (size_t)x;
            if (test && !depth_sisd(c->depthFunc, zPos, zb[p])) continue;
            const float u = (float)(int32_t)((uint32_t)x - (uint32_t)xScreen) * invXLen;
            const uint32_t src = ySrc + ox_ftou32(u * (float)widthM1);
            if (c->depthMask) zb[p] = zPos;
            uint32_t col = src < nSrc ? pixel_sisd(format, type, pixels, src) : 0u;
            if (c->state & PF_BLEND) col = blend_sisd(c->blend, col, fb_get(dst, p));
            fb_set(dst, p, col);
        }
    }
}

void pfPixelZoom(PFfloat x, PFfloat y) { G->pixelZoom[0] = x; G->pixelZoom[1] = y; }   /* context.c:2089-2093 */
static void raster_pos(float x, float y, float z, float w) { G->rasterPos[0] = x; G->rasterPos[1] = y; G->rasterPos[2] = z; G->rasterPos[3] = w; }
void pfRasterPos2i(PFint x, PFint y) { raster_pos((PFfloat)x, (PFfloat)y, 0.0f, 1.0f); }
void pfRasterPos2f(PFfloat x, PFfloat y) { raster_pos(x, y, 0.0f, 1.0f); }
void pfRasterPos2fv(const PFfloat *v) { raster_pos(v[0], v[1], 0.0f, 1.0f); }
void pfRasterPos3i(PFint x, PFint y, PFint z) { raster_pos((PFfloat)x, (PFfloat)y, (PFfloat)z, 1.0f); }
void pfRasterPos3f(PFfloat x, PFfloat y, PFfloat z) { raster_pos(x, y, z, 1.0f); }
void pfRasterPos3fv(const PFfloat *v) { raster_pos(v[0], v[1], v[2], 1.0f); }
void pfRasterPos4i(PFint x, PFint y, PFint z, PFint w) { raster_pos((PFfloat)x, (PFfloat)y, (PFfloat)z, (PFfloat)w); }
void pfRasterPos4f(PFfloat x, PFfloat y, PFfloat z, PFfloat w) { raster_pos(x, y, z, w); }
void pfRasterPos4fv(const PFfloat *v) { raster_pos(v[0], v[1], v[2], v[3]); }

/* Fog parameters (context.c:2161-2286), with the reference's behaviour: a
 * density sets the mode (truncated), and the vector forms accept any mode
 * and density (their range tests are always true). */
void pfFogi(PFfogparam p, PFint v)
{
    switch (p) {
    case PF_FOG_MODE: if (v >= PF_LINEAR && v <= PF_EXP2) G->fog.mode = (uint32_t)v; else G->err = PF_INVALID_VALUE; break;
    case PF_FOG_DENSITY: if (v == 0 || v == 1) G->fog.mode = (uint32_t)v; else G->err = PF_INVALID_VALUE; break;
    case PF_FOG_START: G->fog.start = (PFfloat)v; break;
    case PF_FOG_END: G->fog.end = (PFfloat)v; break;
    default: G->err = PF_INVALID_ENUM; break;
    }
}
void pfFogf(PFfogparam p, PFfloat v)
{
    switch (p) {
    case PF_FOG_DENSITY: if (v >= 0 && v <= 1) G->fog.mode = ox_ftou32(v); else G->err = PF_INVALID_VALUE; break;
    case PF_FOG_START: G->fog.start = v; break;
    case PF_FOG_END: G->fog.end = v; break;
    default: G->err = PF_INVALID_ENUM; break;
    }
}
void pfFogiv(PFfogparam p, PFint *v)
{
    switch (p) {
    case PF_FOG_MODE: case PF_FOG_DENSITY: G->fog.mode = (uint32_t)*v; break;
    case PF_FOG_START: G->fog.start = (PFfloat)*v; break;
    case PF_FOG_END: G->fog.end = (PFfloat)*v; break;
    case PF_FOG_COLOR: {
        PFcolor fc = { (PFubyte)v[0], (PFubyte)v[1], (PFubyte)v[2], (PFubyte)v[3] };
        G->fog.color = fc;
        break;
    }
    default: G->err = PF_INVALID_ENUM; break;
    }
}
void pfFogfv(PFfogparam p, PFfloat *v)
{
    switch (p) {
    case PF_FOG_DENSITY: if (*v >= 0 || *v <= 1) G->fog.mode = ox_ftou32(*v); else G->err = PF_INVALID_VALUE; break;
    case PF_FOG_START: G->fog.start = *v; break;
    case PF_FOG_END: G->fog.end = *v; break;
    case PF_FOG_COLOR: {
        PFcolor fc = { ox_ftoub(255 * v[0]), ox_ftoub(255 * v[1]), ox_ftoub(255 * v[2]), ox_ftoub(255 * v[3]) };
        G->fog.color = fc;
        break;
    }
    default: G->err = PF_INVALID_ENUM; break;
    }
}

/* pfiBlendAlpha, scalar (src/internal/blend.h:41-52) */
static uint32_t blend_alpha_sisd(uint32_t src, uint32_t dst) { return blend_sisd(PF_BLEND_ALPHA, src, dst); }

/* pfFogProcess (context.c:2288-2351): over the current framebuffer, pixels
 * at or beyond the end take the fog colour (alpha-blended unless opaque),
 * pixels between start and end blend it with alpha t * a, t linear, 1 - e^-d
 * or 1 - 2^-d of the depth past the start. */
void pfFogProcess(void)
{
    RCtx *c = G;
    RTex *t = (RTex *)c->current->texture;
    const float *zb = c->current->zbuffer;
    const float density = c->fog.density, start = c->fog.start, end = c->fog.end;
    const float invLen = 1 / (end - start);
    const uint32_t fc = col_pack(c->fog.color) & 0x00ffffffu, alpha = c->fog.color.a;
    for (size_t o = 0; o < (size_t)t->w * t->h; o++) {
        const float depth = zb[o];
        if (depth >= end) {
            const uint32_t f = fc | alpha << 24;
            fb_set(t, o, alpha == 255 ? f : blend_alpha_sisd(f, fb_get(t, o)));
        } else if (depth > start) {
            float tt = 0;
            switch (c->fog.mode) {
            case PF_LINEAR: tt = (depth - start) * invLen; break;
            case PF_EXP: tt = 1.0f - expf(-density * (depth - start)); break;
            case PF_EXP2: tt = 1.0f - exp2f(-density * (depth - start)); break;
            default: break;
            }
            const uint32_t a = ox_ftoub(tt * (float)alpha);
            fb_set(t, o, blend_alpha_sisd(fc | a << 24, fb_get(t, o)));
        }
    }
}

/* Render lists (src/renderlist.c:6-97, context.c:1580-1685) */
static void call_free(RCall *k) { free(k->pos); free(k->uv); free(k->nrm); free(k->col); memset(k, 0, sizeof *k); }

static void list_begin(RCtx *c, PFdrawmode mode)
{
    RList *l = c->curList;
    if (l->n == l->cap) {
        l->cap = l->cap ? l->cap * 2 : 4;
        l->calls = (RCall *)realloc(l->calls, l->cap * sizeof(RCall));
    }
    RCall *k = &l->calls[l->n++];
    memset(k, 0, sizeof *k);
    k->mode = mode;
    k->mat[0] = c->mat[0]; k->mat[1] = c->mat[1];
    k->texture = c->texture;
}

static void list_vertex(RCtx *c, const PFfloat *v)
{
    RList *l = c->curList;
    if (l->n == 0) return;                       /* the reference indexes call -1 */
    RCall *k = &l->calls[l->n - 1];
    if (k->n == k->cap) {
        k->cap = k->cap ? k->cap * 2 : 8;
        k->pos = realloc(k->pos, k->cap * sizeof *k->pos); k->uv = realloc(k->uv, k->cap * sizeof *k->uv);
        k->nrm = realloc(k->nrm, k->cap * sizeof *k->nrm); k->col = realloc(k->col, k->cap * sizeof *k->col);
    }
    memcpy(k->pos[k->n], v, 16); memcpy(k->uv[k->n], c->curTex, 8); memcpy(k->nrm[k->n], c->curNormal, 12);
    k->col[k->n] = c->curColor;
    k->n++;
}

static void ctx_backup(RCtx *c)   /* pfiMakeContextBackup (internal/context/context.c:26-36) */
{
    c->backup.mat[0] = c->mat[0]; c->backup.mat[1] = c->mat[1];
    memcpy(c->backup.tex, c->curTex, 8); memcpy(c->backup.nrm, c->curNormal, 12);
    c->backup.col = c->curColor; c->backup.texture = c->texture; c->backup.state = c->state;
}
static void ctx_restore(RCtx *c)  /* pfiRestoreContext (:38-48) */
{
    c->mat[0] = c->backup.mat[0]; c->mat[1] = c->backup.mat[1];
    memcpy(c->curTex, c->backup.tex, 8); memcpy(c->curNormal, c->backup.nrm, 12);
    c->curColor = c->backup.col; c->texture = c->backup.texture; c->state = c->backup.state;
}

PFrenderlist pfGenList(void) { return calloc(1, sizeof(RList)); }
void pfDeleteList(PFrenderlist *pl)
{
    if (!pl) return;
    RList *l = (RList *)*pl;
    if (l) {
        for (size_t i = 0; i < l->n; i++) call_free(&l->calls[i]);
        free(l->calls); free(l);
    }
    *pl = NULL;
}
void pfNewList(PFrenderlist pl)
{
    if (!pl) { G->err = PF_INVALID_VALUE; return; }
    RList *l = (RList *)pl;
    for (size_t i = 0; i < l->n; i++) call_free(&l->calls[i]);
    l->n = 0;
    G->curList = l;
    ctx_backup(G);
}
void pfEndList(void)
{
    if (!G->curList) G->err = PF_INVALID_OPERATION;
    G->curList = NULL;
    ctx_restore(G);
}
void pfCallList(const PFrenderlist pl)
{
    const RList *l = (const RList *)pl;
    if (!l) { G->err = PF_INVALID_VALUE; return; }
    ctx_backup(G);
    for (size_t i = 0; i < l->n; i++) {
        const RCall *k = &l->calls[i];
        G->mat[0] = k->mat[0]; G->mat[1] = k->mat[1];
        pfBindTexture(k->texture);
        pfBegin(k->mode);
        for (size_t j = 0; j < k->n; j++) {
            pfColor4ubv((const PFubyte *)&k->col[j]);
            pfTexCoordfv(k->uv[j]);
            pfNormal3fv(k->nrm[j]);
            pfVertex4fv(k->pos[j]);
        }
        pfEnd();
    }
    ctx_restore(G);
}

/* ------------------------------------------------------------------------ */
/* readback, post-process, framebuffers, textures                            */
/* ------------------------------------------------------------------------ */

/* pfmFloatToHalfI (src/pfm.h:108-126): round half up on the dropped bits,
 * flush below 2^-14, infinity from 2^16, all NaNs quiet. */
static uint16_t float_to_half(float x)
{
    const uint32_t ui = ox_fbits(x);
    const int s = (int)((ui >> 16) & 0x8000u);
    const int em = (int)(ui & 0x7fffffffu);
    int h = (em - (112 << 23) + (1 << 12)) >> 13;
    h = (em < (113 << 23)) ? 0 : h;
    h = (em >= (143 << 23)) ? 0x7c00 : h;
    h = (em > (255 << 23)) ? 0x7e00 : h;
    return (uint16_t)(s | h);
}

/* The reference's scalar pixel setter (src/internal/pixel.h:52-405) writing
 * RGBA8 colour col as element o of a buffer of format f / type t. */
#define FTOUB ox_ftoub
static void pixel_set_sisd(PFpixelformat f, PFdatatype t, void *dst, size_t o, uint32_t col)
{
    const float inv = (float)(1.0 / 255);
    const uint32_t r = col & 255u, g = (col >> 8) & 255u, b = (col >> 16) & 255u, a = col >> 24;
    uint8_t *p8 = (uint8_t *)dst;
    uint16_t *p16 = (uint16_t *)dst;
    float *pf = (float *)dst;
    /* PF_COLOR_GARYSCALE (src/internal/pixel.h:69-74) */
    const float gray = (float)r * inv * 0.299f + (float)g * inv * 0.587f + (float)b * inv * 0.114f;
    uint32_t ch = 0;
    switch (f) {
    case PF_RED: ch = r; break;
    case PF_GREEN: ch = g; break;
    case PF_BLUE: ch = b; break;
    case PF_ALPHA: ch = a; break;
    default: break;
    }
    switch (f) {
    case PF_RED: case PF_GREEN: case PF_BLUE: case PF_ALPHA:
        if (t == PF_UNSIGNED_BYTE) p8[o] = (uint8_t)ch;
        else if (t == PF_HALF_FLOAT) p16[o] = float_to_half((float)ch / 255.0f);
        else pf[o] = (float)ch / 255.0f;
        return;
    case PF_LUMINANCE:
        if (t == PF_UNSIGNED_BYTE) p8[o] = FTOUB(255.0f * gray);
        else if (t == PF_HALF_FLOAT) p16[o] = float_to_half(gray);
        else pf[o] = gray;
        return;
    case PF_LUMINANCE_ALPHA:
        if (t == PF_UNSIGNED_BYTE) { p8[2 * o] = FTOUB(255 * gray); p8[2 * o + 1] = (uint8_t)a; }
        else if (t == PF_HALF_FLOAT) { p16[2 * o] = float_to_half(gray); p16[2 * o + 1] = float_to_half((float)a * inv); }
        else { pf[2 * o] = gray; pf[2 * o + 1] = (float)a * inv; }
        return;
    default: break;
    }
    /* PF_COLOR_{RGB,BGR,RGBA,BGRA}_NORMALIZE (pixel.h:36-66): the BGRA one keeps RGBA order */
    const int bgr = (f == PF_BGR);
    float n[4] = { (float)r * inv, (float)g * inv, (float)b * inv, (float)a * inv };
    if (bgr) { n[0] = (float)b * inv; n[2] = (float)r * inv; }
    if (t == PF_UNSIGNED_SHORT_5_6_5) {
        const uint32_t c0 = (uint8_t)roundf(n[0] * 31.0f), c1 = (uint8_t)roundf(n[1] * 63.0f), c2 = (uint8_t)roundf(n[2] * 31.0f);
        p16[o] = (uint16_t)(c0 << 11 | c1 << 5 | c2);
        return;
    }
    if (t == PF_UNSIGNED_SHORT_5_5_5_1) {
        const uint32_t c0 = (uint8_t)roundf(n[0] * 31.0f), c1 = (uint8_t)roundf(n[1] * 31.0f), c2 = (uint8_t)roundf(n[2] * 31.0f);
        const uint32_t al = ((double)n[3] > (double)(float)50 * (1.0 / 255)) ? 1u : 0u;
        p16[o] = (uint16_t)(c0 << 11 | c1 << 6 | c2 << 1 | al);
        return;
    }
    if (t == PF_UNSIGNED_SHORT_4_4_4_4) {
        const uint32_t c0 = (uint8_t)roundf(n[0] * 15.0f), c1 = (uint8_t)roundf(n[1] * 15.0f);
        const uint32_t c2 = (uint8_t)roundf(n[2] * 15.0f), c3 = (uint8_t)roundf(n[3] * 15.0f);
        p16[o] = (uint16_t)(c0 << 12 | c1 << 8 | c2 << 4 | c3);
        return;
    }
    const int k = (f == PF_RGB || f == PF_BGR) ? 3 : 4;
    if (t == PF_UNSIGNED_BYTE) {
        const uint32_t v[4] = { (f == PF_BGR || f == PF_BGRA) ? b : r, g, (f == PF_BGR || f == PF_BGRA) ? r : b, a };
        for (int i = 0; i < k; i++) p8[(size_t)k * o + (size_t)i] = (uint8_t)v[i];
    } else if (t == PF_HALF_FLOAT) {
        for (int i = 0; i < k; i++) p16[(size_t)k * o + (size_t)i] = float_to_half(n[i]);
    } else {
        for (int i = 0; i < k; i++) pf[(size_t)k * o + (size_t)i] = n[i];
    }
}
#undef FTOUB

/* pfReadPixels (context.c:2353-2395): the clamped region, each pixel through
 * the setter of the requested format. */
void pfReadPixels(PFint x, PFint y, PFsizei w, PFsizei h, PFpixelformat f, PFdatatype t, void *pixels)
{
    if (!(f >= PF_RED && f <= PF_BGRA && t >= PF_UNSIGNED_BYTE && t <= PF_DOUBLE)) { G->err = PF_INVALID_ENUM; return; }
    if (!texel_bytes(f, t)) { G->err = PF_INVALID_ENUM; return; }
    RTex *s = (RTex *)G->current->texture;
#define CLAMPR(v, lo, hi) ((v) < (lo) ? (lo) : ((v) > (hi) ? (hi) : (v)))
    PFint xMin = CLAMPR(x, 0, (PFint)s->w - 1), yMin = CLAMPR(y, 0, (PFint)s->h - 1);
    PFint xMax = CLAMPR(x + (PFint)w, 0, (PFint)s->w), yMax = CLAMPR(y + (PFint)h, 0, (PFint)s->h);
    for (PFint yy = yMin; yy < yMax; yy++)
        for (PFint xx = xMin; xx < xMax; xx++)
            pixel_set_sisd(f, t, pixels, (size_t)(yy - yMin) * w + (size_t)(xx - xMin), fb_get(s, (size_t)yy * s->w + (size_t)xx));
}

void pfPostProcess(PFpostprocessfunc fn)   /* context.c:2397-2441 */
{
    RTex *t = (RTex *)G->current->texture;
    const float *zb = G->current->zbuffer;
    for (PFint y = 0; y < (PFint)t->h; y++)
        for (PFint x = 0; x < (PFint)t->w; x++) {
            size_t o = (size_t)y * t->w + (size_t)x;
            fb_set(t, o, col_pack(fn(x, y, zb[o], col_unpack(fb_get(t, o)))));
        }
}

/* Built-in hooks, same definitions as the GPU library's device hooks. */
static PFhookfog g_fog;
static PFcolor hook_fog(PFint x, PFint y, PFfloat depth, PFcolor c)
{
    (void)x; (void)y;
    float d = (depth + g_fog.znear) / (g_fog.zfar + g_fog.znear);
    float f = (g_fog.end - d) / (g_fog.end - g_fog.start);
    f = ox_min(ox_max(f, 0.0f), 1.0f);
    int32_t k = ox_ftoi(f * 255.0f);
    const uint8_t *fc = (const uint8_t *)&g_fog.color;
    uint8_t *cc = (uint8_t *)&c;
    for (int i = 0; i < 4; i++) cc[i] = (uint8_t)((cc[i] * k + fc[i] * (255 - k)) / 255);
    return c;
}
static PFcolor hook_gray(PFint x, PFint y, PFfloat depth, PFcolor c)
{
    (void)x; (void)y; (void)depth;
    uint32_t g = (77u * c.r + 150u * c.g + 29u * c.b) >> 8;
    c.r = c.g = c.b = (uint8_t)g;
    return c;
}
static PFcolor hook_identity(PFint x, PFint y, PFfloat depth, PFcolor c) { (void)x; (void)y; (void)depth; return c; }
/* examples/raylib/raylib_PostProcess.c:7-19 */
static PFcolor hook_dither(PFint x, PFint y, PFfloat depth, PFcolor c)
{
    static const uint8_t m[3][3] = { { 230, 51, 128 }, { 25, 102, 179 }, { 154, 205, 77 } };
    (void)depth;
    const uint8_t dv = m[x % 3][y % 3];
    const uint8_t avg = (uint8_t)((c.r + c.g + c.b) / 3);
    const uint32_t v = (avg >= dv) ? 0xffffffffu : 0u;
    memcpy(&c, &v, 4);
    return c;
}

void pfPostProcessDevice(PFuint hookId, const void *params, PFsizei size)
{
    switch (hookId) {
    case PF_HOOK_IDENTITY: pfPostProcess(hook_identity); break;
    case PF_HOOK_FOG_LINEAR:
        if (!params || size < sizeof(PFhookfog)) { G->err = PF_INVALID_VALUE; return; }
        memcpy(&g_fog, params, sizeof g_fog); pfPostProcess(hook_fog); break;
    case PF_HOOK_GRAYSCALE: pfPostProcess(hook_gray); break;
    case PF_HOOK_DITHER: pfPostProcess(hook_dither); break;
    default: G->err = PF_INVALID_ENUM; break;
    }
}

/* The fog hook as a host callback, for driving the reference's pfPostProcess
 * with the same definition. */
PFcolor pfref_fog_hook(PFint x, PFint y, PFfloat depth, PFcolor c) { return hook_fog(x, y, depth, c); }
void pfref_set_fog(const PFhookfog *f) { g_fog = *f; }
/* The dither hook as a host callback. */
PFcolor pfref_dither_hook(PFint x, PFint y, PFfloat depth, PFcolor c) { return hook_dither(x, y, depth, c); }

void pfGetStats(PFstats *s) { *s = G->stats; }
void pfResetStats(void) { memset(&G->stats, 0, sizeof G->stats); }
PFuint pfGetDeviceStatus(void) { return 0; }
void pfEnableTiming(PFboolean enable) { (void)enable; }

PFframebuffer pfGenFramebuffer(PFsizei w, PFsizei h, PFpixelformat f, PFdatatype t)
{
    PFframebuffer fb = { NULL, NULL };
    if (!fb_format_ok(f, t)) { if (G) G->err = PF_INVALID_ENUM; return fb; }
    void *px = calloc((size_t)w * h, (size_t)texel_bytes(f, t));
    fb.texture = tex_new(px, w, h, f, t, 0);
    fb.zbuffer = (float *)malloc((size_t)w * h * sizeof(float));
    for (size_t i = 0; i < (size_t)w * h; i++) fb.zbuffer[i] = FLT_MAX;
    return fb;
}
void pfDeleteFramebuffer(PFframebuffer *fb)
{
    if (!fb) return;
    if (fb->texture) { free(((RTex *)fb->texture)->pixels); free(fb->texture); }
    free(fb->zbuffer); fb->texture = NULL; fb->zbuffer = NULL;
}
PFboolean pfIsValidFramebuffer(PFframebuffer *fb)
{
    RTex *t = (RTex *)fb->texture;
    return t && fb->zbuffer && t->w > 0 && t->h > 0 && t->pixels;
}
void pfClearFramebuffer(PFframebuffer *fb, PFcolor col, PFfloat d)
{
    RTex *t = (RTex *)fb->texture;
    uint32_t cc = col_pack(col);
    for (size_t i = 0; i < (size_t)t->w * t->h; i++) { fb_set(t, i, cc); fb->zbuffer[i] = d; }
}
PFcolor pfGetFramebufferPixel(const PFframebuffer *fb, PFsizei x, PFsizei y)
{
    const RTex *t = (const RTex *)fb->texture;
    return col_unpack(fb_get(t, (size_t)y * t->w + x));
}
PFfloat pfGetFramebufferDepth(const PFframebuffer *fb, PFsizei x, PFsizei y)
{
    const RTex *t = (const RTex *)fb->texture;
    return fb->zbuffer[(size_t)y * t->w + x];
}
void pfSetFramebufferPixelDepthTest(PFframebuffer *fb, PFsizei x, PFsizei y, PFfloat z, PFcolor col, PFdepthmode m)
{
    if (m > PF_GEQUAL) { if (G) G->err = PF_INVALID_ENUM; return; }
    RTex *t = (RTex *)fb->texture; size_t o = (size_t)y * t->w + x;
    int pass;
    switch (m) {   /* scalar depth functions (src/internal/depth.h:30-70) */
    case PF_EQUAL: pass = z == fb->zbuffer[o]; break;
    case PF_NOTEQUAL: pass = z != fb->zbuffer[o]; break;
    case PF_LESS: pass = z < fb->zbuffer[o]; break;
    case PF_LEQUAL: pass = z <= fb->zbuffer[o]; break;
    case PF_GREATER: pass = z > fb->zbuffer[o]; break;
    default: pass = z >= fb->zbuffer[o]; break;
    }
    if (pass) { fb_set(t, o, col_pack(col)); fb->zbuffer[o] = z; }
}
void pfSetFramebufferPixelDepth(PFframebuffer *fb, PFsizei x, PFsizei y, PFfloat z, PFcolor col)
{
    RTex *t = (RTex *)fb->texture; size_t o = (size_t)y * t->w + x;
    fb_set(t, o, col_pack(col)); fb->zbuffer[o] = z;
}
void pfSetFramebufferPixel(PFframebuffer *fb, PFsizei x, PFsizei y, PFcolor col)
{
    RTex *t = (RTex *)fb->texture;
    fb_set(t, (size_t)y * t->w + x, col_pack(col));
}

PFtexture pfGenTexture(void *pixels, PFsizei w, PFsizei h, PFpixelformat f, PFdatatype t) { return tex_new(pixels, w, h, f, t, 1); }
void pfDeleteTexture(PFtexture *tex, PFboolean freeBuffer)
{
    RTex *t = (RTex *)*tex;
    if (!t) return;
    if (freeBuffer) free(t->pixels);
    free(t); *tex = NULL;
}
PFboolean pfIsValidTexture(const PFtexture tex)
{
    const RTex *t = (const RTex *)tex;
    return t && t->pixels && t->w > 0 && t->h > 0;
}
void pfTextureParameter(PFtexture tex, PFtexturewrap wrap, PFtexturefilter filter)
{
    if (!(wrap <= PF_CLAMP_TO_EDGE && filter <= PF_BILINEAR)) { if (G) G->err = PF_INVALID_ENUM; return; }
    RTex *t = (RTex *)tex; t->wrap = wrap; t->filter = filter;
}
void *pfGetTexturePixels(const PFtexture tex, PFsizei *w, PFsizei *h, PFpixelformat *f, PFdatatype *t)
{
    const RTex *x = (const RTex *)tex;
    if (!x) return NULL;
    if (w) *w = x->w;
    if (h) *h = x->h;
    if (f) *f = x->format;
    if (t) *t = x->type;
    return x->pixels;
}
