// pf_common.cuh -- device arithmetic shared by the pipeline kernels and the
// differentiable path: x86 conversion rules, pfm.h vector arithmetic in the
// reference's operation order, texture coordinate maps and triangle set-up.
// Included inside each translation unit's anonymous namespace.
#pragma once

// ---------------------------------------------------------------------------
// x86 rules
// ---------------------------------------------------------------------------
__device__ __forceinline__ float x86_min(float a, float b) { return (a < b) ? a : b; }   // MINPS
__device__ __forceinline__ float x86_max(float a, float b) { return (a > b) ? a : b; }   // MAXPS

// CVTPS2DQ: round to nearest even, 0x80000000 for NaN / out of range.
__device__ __forceinline__ int32_t x86_cvt_rne(float x)
{
    if (!(x > -2147483648.0f && x < 2147483648.0f)) return INT32_MIN;
    return __float2int_rn(x);
}
// CVTTPS2DQ / CVTTSS2SI: truncation, 0x80000000 for NaN / out of range.
__device__ __forceinline__ int32_t x86_cvt_trunc(float x)
{
    if (!(x > -2147483649.0f && x < 2147483648.0f)) return INT32_MIN;
    return __float2int_rz(x);
}
// (unsigned char)(float) as GCC emits it on x86-64.
__device__ __forceinline__ uint32_t x86_ftoub(float x) { return (uint32_t)x86_cvt_trunc(x) & 255u; }

__device__ __forceinline__ uint32_t chn(uint32_t p, int i) { return (p >> (8 * i)) & 255u; }

// ---------------------------------------------------------------------------
// pfm.h arithmetic in the reference's order
// ---------------------------------------------------------------------------
__device__ __forceinline__ void v4_transform(float *d, const float *v, const float *m)
{
    float t0 = m[0]*v[0] + m[4]*v[1] + m[8]*v[2] + m[12]*v[3];
    float t1 = m[1]*v[0] + m[5]*v[1] + m[9]*v[2] + m[13]*v[3];
    float t2 = m[2]*v[0] + m[6]*v[1] + m[10]*v[2] + m[14]*v[3];
    float t3 = m[3]*v[0] + m[7]*v[1] + m[11]*v[2] + m[15]*v[3];
    d[0] = t0; d[1] = t1; d[2] = t2; d[3] = t3;
}
__device__ __forceinline__ void v3_transform(float *d, const float *v, const float *m)
{
    float t0 = m[0]*v[0] + m[4]*v[1] + m[8]*v[2] + m[12];
    float t1 = m[1]*v[0] + m[5]*v[1] + m[9]*v[2] + m[13];
    float t2 = m[2]*v[0] + m[6]*v[1] + m[10]*v[2] + m[14];
    d[0] = t0; d[1] = t1; d[2] = t2;
}
__device__ __forceinline__ void v3_normalize(float *v)          // pfm.h:1183-1197
{
    float sq = v[0]*v[0] + v[1]*v[1] + v[2]*v[2];
    if (sq == 0.0f) return;
    float inv = __frcp_rn(sqrtf(sq));
    v[0] = v[0] * inv; v[1] = v[1] * inv; v[2] = v[2] * inv;
}
__device__ __forceinline__ float v3_dot(const float *a, const float *b) { return a[0]*b[0] + a[1]*b[1] + a[2]*b[2]; }

// sampler.h:203-258 (SIMD texture maps): texel coordinates of (u, v) in a
// texW x texH texture under wrap mode `wrap` (0 repeat, 1 mirrored repeat,
// 2 clamp to edge).
__device__ __forceinline__ void tex_map_wh(uint32_t texW, uint32_t texH, int32_t wrap, float u, float v,
                                           int32_t &x, int32_t &y)
{
    const float wm1 = (float)(texW - 1), hm1 = (float)(texH - 1);
    if (wrap == 0) {                      // REPEAT
        u = (u - truncf(u)) * wm1;
        v = (v - truncf(v)) * hm1;
        int32_t a = x86_cvt_rne(u), b = x86_cvt_rne(v);
        x = (a < 0) ? (int32_t)(0u - (uint32_t)a) : a;
        y = (b < 0) ? (int32_t)(0u - (uint32_t)b) : b;
    } else if (wrap == 1) {               // MIRRORED_REPEAT; pfiSimdMod_F32 = x - floor(x/2)*2
        u = fabsf(u); v = fabsf(v);
        u = u - floorf(u / 2.0f) * 2.0f;
        v = v - floorf(v / 2.0f) * 2.0f;
        float um = 1.0f - (u - 1.0f), vm = 1.0f - (v - 1.0f);
        u = (u > 1.0f) ? um : u;
        v = (v > 1.0f) ? vm : v;
        u = u * wm1; v = v * hm1;
        x = x86_cvt_rne(u + 0.5f);
        y = x86_cvt_rne(v + 0.5f);
    } else {                              // CLAMP_TO_EDGE
        u = x86_min(x86_max(u, 0.0f), 1.0f) * wm1;
        v = x86_min(x86_max(v, 0.0f), 1.0f) * hm1;
        x = x86_cvt_rne(u + 0.5f);
        y = x86_cvt_rne(v + 0.5f);
    }
}
__device__ __forceinline__ void tex_map(const PFDrawState &S, float u, float v, int32_t &x, int32_t &y)
{
    tex_map_wh(S.texW, S.texH, S.texWrap, u, v, x, y);
}

// ---------------------------------------------------------------------------
// triangle set-up
// ---------------------------------------------------------------------------
struct SVert {                 // a vertex after projection to the screen
    float sx, sy, z, u, v;
    uint32_t c;
    float n[3], p[3];
};

// pfiHomogeneousToScreen (internal/context/context.c:52-65)
__device__ __forceinline__ void to_screen(const PFDrawState &S, float hx, float hy, float &sx, float &sy)
{
    sx = ((float)S.vpPos[0] + (hx + 1.0f) * 0.5f * (float)S.vpDim[0]) + 0.5f;
    sy = ((float)S.vpPos[1] + (1.0f - hy) * 0.5f * (float)S.vpDim[1]) + 0.5f;
}

// The per-fragment operations of a draw state, packed for the tile
// rasterizer: PFS_* bits | depth function << 16 | blend mode << 24.
__device__ __forceinline__ uint32_t raster_state(const PFDrawState &S)
{
    return (S.flags & 0xffffu) | ((uint32_t)S.depthFunc << 16) | ((uint32_t)S.blendMode << 24);
}

// A bound below which no fragment depth of the sub-triangle can fall, for
// PF_LESS (and, one step lower, PF_LEQUAL).  The depth of a covered pixel is
// 1 / ((z1 wN1 + z2 wN2) + z3 wN3) with wN >= 0 summing to 1 within a few
// ulps, so the interpolated term lies in [min z, max z] widened by a
// relative 1e-5; its reciprocal is bounded by the reciprocals of the ends
// when they have one sign.  NaN (never rejects) otherwise.
__device__ __forceinline__ float depth_reject_bound(const PFPrim &P, uint32_t rstate)
{
    const float qnan = __int_as_float(0x7fffffff);
    const int func = (int)((rstate >> 16) & 255u);
    if (!(rstate & PFS_DEPTH_TEST) || (func != 2 && func != 3)) return qnan;
    const float lo = fminf(P.z1, fminf(P.z2, P.z3)), hi = fmaxf(P.z1, fmaxf(P.z2, P.z3));
    if (!(fabsf(lo) < 1e30f && fabsf(hi) < 1e30f)) return qnan;
    float b;
    if (lo > 0.0f) b = __fdiv_rn(1.0f, hi * 1.00001f) * 0.99999f;         // interpolated term <= hi (1 + 1e-5)
    else if (hi < 0.0f) b = __fdiv_rn(1.0f, hi * 0.99999f) * 1.00001f;    // term <= hi (1 - 1e-5) < 0
    else return qnan;
    if (!(fabsf(b) < 1e30f)) return qnan;
    return func == 2 ? b : nextafterf(b, -INFINITY);
}

// Rasterize_Triangle set-up (triangles.c:287-349).  Returns false if culled.
__device__ bool setup_prim(const PFDrawState &S, int face, bool is3D, const SVert &a, const SVert &b,
                           const SVert &c, int stateIdx, PFPrim &P)
{
    int32_t x1 = x86_cvt_trunc(a.sx), y1 = x86_cvt_trunc(a.sy);
    int32_t x2 = x86_cvt_trunc(b.sx), y2 = x86_cvt_trunc(b.sy);
    int32_t x3 = x86_cvt_trunc(c.sx), y3 = x86_cvt_trunc(c.sy);
    float area = (float)(int32_t)((uint32_t)(x2 - x1) * (uint32_t)(y3 - y1) - (uint32_t)(x3 - x1) * (uint32_t)(y2 - y1));
    if ((face == 0 && area >= 0.0f) || (face == 1 && area <= 0.0f)) return false;
    int32_t mnx = min(x1, min(x2, x3)), mny = min(y1, min(y2, y3));
    int32_t mxx = max(x1, max(x2, x3)), mxy = max(y1, max(y2, y3));
    if (!is3D) {
        mnx = min(max(mnx, S.vpMin[0]), S.vpMax[0]); mny = min(max(mny, S.vpMin[1]), S.vpMax[1]);
        mxx = min(max(mxx, S.vpMin[0]), S.vpMax[0]); mxy = min(max(mxy, S.vpMin[1]), S.vpMax[1]);
    }
    uint32_t xMin = (uint32_t)mnx, yMin = (uint32_t)mny;
    int32_t w1X = y3 - y2, w1Y = x2 - x3, w2X = y1 - y3, w2Y = x3 - x1, w3X = y2 - y1, w3Y = x1 - x2;
    if (face == 1) { w1X = -w1X; w1Y = -w1Y; w2X = -w2X; w2Y = -w2Y; w3X = -w3X; w3Y = -w3Y; }
    uint32_t r1 = (xMin - (uint32_t)x2) * (uint32_t)w1X + (uint32_t)w1Y * (yMin - (uint32_t)y2);
    uint32_t r2 = (xMin - (uint32_t)x3) * (uint32_t)w2X + (uint32_t)w2Y * (yMin - (uint32_t)y3);
    uint32_t r3 = (xMin - (uint32_t)x1) * (uint32_t)w3X + (uint32_t)w3Y * (yMin - (uint32_t)y1);
    P.x1 = x1; P.y1 = y1; P.x2 = x2; P.y2 = y2; P.x3 = x3; P.y3 = y3;
    P.xMin = mnx; P.yMin = mny; P.xMax = mxx; P.yMax = mxy;
    P.flags = (uint32_t)face | (is3D ? 2u : 0u) | ((uint32_t)stateIdx << 8);
    P.poolBase = -1;
    P.wInvSum = __frcp_rn((float)(int32_t)(r1 + r2 + r3));
    P.z1 = a.z; P.z2 = b.z; P.z3 = c.z;
    P.c1 = a.c; P.c2 = b.c; P.c3 = c.c;
    P.rstate = raster_state(S);
    P.u1 = a.u; P.v1 = a.v; P.u2 = b.u; P.v2 = b.v; P.u3 = c.u; P.v3 = c.v;
    P.zReject = depth_reject_bound(P, P.rstate);
    // the texture's parameters travel with the record: the rasterizer
    // samples without reading the draw state
    P.src = 0; P.nSrc = 0; P.texTx = 0.0f; P.texTy = 0.0f;
    if (S.flags & PFS_TEXTURE) {
        P.src = (uint64_t)(uintptr_t)S.tex;
        P.texTx = S.texTx; P.texTy = S.texTy;
        P.rstate |= ((uint32_t)S.texWrap & 3u) << PFR_WRAP_SHIFT | (S.texFilter ? (uint32_t)PFR_FILTER : 0u);
        if (S.texW < 65536u && S.texH < 65536u) P.nSrc = S.texW | (S.texH << 16);
        else P.rstate |= PFR_TEX_FROM_STATE;
    }
    return true;
}
