// pf_kernels.cu -- sm_103a kernels of the PixelForge triangle pipeline.
//
//   k_vertex   one thread per vertex: transform, Gouraud lighting
//              (src/internal/primitives/triangles.c:72-104, lighting.c:24-134)
//   k_items    one thread per triangle-face item, in submission order:
//              2D/3D decision, projection, polygon clipping of the rare items
//              that cross a plane (triangles.c:157-280), setup, cull and
//              order-keyed binning into 16x16 tiles (triangles.c:287-339)
//   k_raster   one CTA per tile: restores submission order of the tile's
//              bin, then per chunk of sub-triangles computes coverage with
//              the reference's integer edge functions, shades fragments
//              densely and resolves each pixel's fragments in order (depth
//              test, blend) (triangles.c:398-557); optionally starts from
//              a fused clear
//   k_clear, k_fill, k_hook  framebuffer-wide passes (pfClear,
//              pfClearFramebuffer, device post-process hooks)
//
// Framebuffers of other formats than RGBA / unsigned byte keep their raw
// pixels in HBM; the kernels read and write them through the format's
// getters and setters (pf_pixfmt.h).
//
// Arithmetic parity.  The file is compiled with -fmad=false so that no
// multiply-add is contracted (the reference is built for AVX2 without FMA);
// every floating-point expression keeps the reference's operation order.
// x86 conversion and min/max rules are restated explicitly (see x86_* below).
// Depth and Phong use exact 1/x and 1/sqrt(x) where the reference uses the
// approximate rcp/rsqrt instructions.

#include <cuda_runtime.h>
#include <stdint.h>
#include "pf_layout.h"
#include "pf_device.h"
#include "pf_pixfmt.h"

namespace {

#include "pf_common.cuh"

static_assert((unsigned)PFP_DEPTH_TEST == (unsigned)PFS_DEPTH_TEST && (unsigned)PFP_BLEND == (unsigned)PFS_BLEND &&
              (unsigned)PFP_DEPTH_WRITE == (unsigned)PFS_DEPTH_MASK, "host-set records carry draw-state bits");


// ---------------------------------------------------------------------------
// Gouraud lighting, ubyte arithmetic (lighting.c:24-134), Blinn-Phong
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t min255(int32_t n) { return (uint32_t)(n | ((255 - n) >> 31)) & 255u; }

// powf(x, y) for the Gouraud specular term (lighting.c:114), correctly
// rounded through double precision.  Whole exponents up to 256 (shininess is
// usually one) use binary powering in double -- at most 16 roundings of 2^-53
// each, far below the float rounding step -- instead of the FP64 pow routine,
// which is slow on this part.
__device__ __forceinline__ float pow_gouraud(float x, float y)
{
    if (y >= 1.0f && y <= 256.0f && y == truncf(y)) {
        uint32_t n = (uint32_t)y;
        double b = (double)x, r = 1.0;
        while (n) { if (n & 1u) r *= b; b *= b; n >>= 1; }
        return (float)r;
    }
    return (float)pow((double)x, (double)y);
}

__device__ uint32_t light_gouraud(const PFDrawState &S, const PFDevMaterial &m, uint32_t diffuse,
                                  const float *P, const float *N)
{
    uint32_t R = chn(m.emis, 0), G = chn(m.emis, 1), B = chn(m.emis, 2);
    const uint32_t dR = chn(diffuse, 0), dG = chn(diffuse, 1), dB = chn(diffuse, 2);
    const uint32_t aR = (chn(m.amb, 0) * dR) / 255, aG = (chn(m.amb, 1) * dG) / 255, aB = (chn(m.amb, 2) * dB) / 255;
    float V[3];
    {
        float lsq = 0.0f;
        for (int i = 0; i < 3; i++) { V[i] = S.viewPos[i] - P[i]; lsq += V[i]*V[i]; }
        float inv = __frcp_rn(sqrtf(lsq));
        for (int i = 0; i < 3; i++) V[i] = V[i] * inv;
    }
    const float shin = m.shininess;
    for (int li = 0; li < S.nLights; li++) {
        const PFDevLight &l = S.lights[li];
        uint32_t lR = 0, lG = 0, lB = 0;
        float L[3] = { l.pos[0] - P[0], l.pos[1] - P[1], l.pos[2] - P[2] };
        float dsq = L[0]*L[0] + L[1]*L[1] + L[2]*L[2];
        float dist = 0.0f;
        if (dsq != 0.0f) {
            dist = sqrtf(dsq);
            float inv = __frcp_rn(dist);
            L[0] = L[0] * inv; L[1] = L[1] * inv; L[2] = L[2] * inv;
        }
        uint32_t intensity = 255;
        bool skip = false;
        if ((double)l.inner < 3.14159265358979323846) {
            float nd[3] = { -l.dir[0], -l.dir[1], -l.dir[2] };
            float theta = v3_dot(L, nd);
            float eps = l.inner - l.outer;
            int32_t iv = x86_cvt_trunc(255.0f*(theta - l.outer)/eps);
            intensity = (uint32_t)(iv < 0 ? 0 : (iv > 255 ? 255 : iv));
            if (intensity == 0) skip = true;
        }
        if (!skip) {
            uint32_t att = 255;
            if (l.attL != 0.0f || l.attQ != 0.0f) {
                att = x86_ftoub(255.0f / (l.attC + l.attL*dist + l.attQ*dsq));
                if (att == 0) skip = true;
            }
            if (!skip) {
                uint32_t factor = (intensity * att) / 255;
                int32_t dI = x86_cvt_trunc(255.0f * v3_dot(N, L));
                uint32_t diff = (uint32_t)(dI > 0 ? dI : 0) & 255u;
                lR = min255((int32_t)(lR + (dR * chn(l.diff, 0) * diff) / (255 * 255)));
                lG = min255((int32_t)(lG + (dG * chn(l.diff, 1) * diff) / (255 * 255)));
                lB = min255((int32_t)(lB + (dB * chn(l.diff, 2) * diff) / (255 * 255)));
                float H[3] = { L[0] + V[0], L[1] + V[1], L[2] + V[2] };
                v3_normalize(H);
                float nh = fmaxf(v3_dot(N, H), 0.0f);
                float pw = pow_gouraud(nh, shin);
                uint32_t spec = x86_ftoub(255.0f * pw);
                lR = min255((int32_t)(lR + (chn(m.spec, 0) * chn(l.spec, 0) * spec) / (255 * 255)));
                lG = min255((int32_t)(lG + (chn(m.spec, 1) * chn(l.spec, 1) * spec) / (255 * 255)));
                lB = min255((int32_t)(lB + (chn(m.spec, 2) * chn(l.spec, 2) * spec) / (255 * 255)));
                lR = (lR * factor) / 255; lG = (lG * factor) / 255; lB = (lB * factor) / 255;
            }
        }
        R = min255((int32_t)(R + lR + (aR * chn(l.amb, 0)) / 255));
        G = min255((int32_t)(G + lG + (aG * chn(l.amb, 1)) / 255));
        B = min255((int32_t)(B + lB + (aB * chn(l.amb, 2)) / 255));
    }
    return R | (G << 8) | (B << 16) | (diffuse & 0xff000000u);
}

// scalar pfiBlendMultiplicative (blend.h:77-86)
__device__ __forceinline__ uint32_t blend_mul_scalar(uint32_t s, uint32_t d)
{
    uint32_t r = 0;
    for (int i = 0; i < 4; i++) r |= ((chn(s, i) * chn(d, i)) / 255) << (8 * i);
    return r;
}

// ---------------------------------------------------------------------------
// per-fragment operations, SIMD semantics
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack4(const int32_t *v)
{
    return (uint32_t)v[0] | ((uint32_t)v[1] << 8) | ((uint32_t)v[2] << 16) | ((uint32_t)v[3] << 24);
}

// blend.h:140-277 (SUB adds; channels are ORed without masks when packed)
__device__ uint32_t blend_simd(int mode, uint32_t src, uint32_t dst)
{
    int32_t s[4], d[4], o[4];
    for (int i = 0; i < 4; i++) { s[i] = (int32_t)chn(src, i); d[i] = (int32_t)chn(dst, i); }
    switch (mode) {
    case 0: for (int i = 0; i < 4; i++) o[i] = (s[i] + d[i]) >> 1; break;
    case 1: { int32_t a = s[3] + 1, ia = 256 - a;
              for (int i = 0; i < 3; i++) o[i] = (s[i]*a + d[i]*ia) >> 8;
              o[3] = (255*a + d[3]*ia) >> 8; } break;
    case 2: for (int i = 0; i < 4; i++) { int32_t t = s[i] + d[i]; o[i] = t < 255 ? t : 255; } break;
    case 3: for (int i = 0; i < 4; i++) { int32_t t = s[i] + d[i]; o[i] = t > 0 ? t : 0; } break;
    case 4: for (int i = 0; i < 4; i++) o[i] = (s[i]*d[i]) >> 8; break;
    case 5: for (int i = 0; i < 4; i++) { int32_t t = ((d[i]*(255 - s[i])) >> 8) + s[i]; o[i] = t < 255 ? t : 255; } break;
    case 6: for (int i = 0; i < 4; i++) o[i] = s[i] > d[i] ? s[i] : d[i]; break;
    case 7: for (int i = 0; i < 4; i++) o[i] = s[i] < d[i] ? s[i] : d[i]; break;
    default: return src;
    }
    return pack4(o);
}

// depth.h:80-124 (NOTEQUAL compares equal there)
__device__ __forceinline__ bool depth_simd(int f, float src, float dst)
{
    switch (f) {
    case 0: case 1: return src == dst;
    case 2: return src < dst;
    case 3: return src <= dst;
    case 4: return src > dst;
    default: return src >= dst;
    }
}


// A texture as the rasterizer samples it.
struct TexDesc {
    const uint32_t *tex;
    uint32_t w, h;
    int32_t wrap, filter;
    float tx, ty;
};

// From the set-up record (texture parameters copied there by setup_prim),
// or from the draw state when they did not fit.
__device__ __forceinline__ TexDesc tex_desc(const PFPrim &P, const PFDrawState *states)
{
    TexDesc d;
    if (!(P.rstate & PFR_TEX_FROM_STATE)) {
        d.tex = reinterpret_cast<const uint32_t *>(P.src);
        d.w = P.nSrc & 0xffffu; d.h = P.nSrc >> 16;
        d.wrap = (int32_t)((P.rstate >> PFR_WRAP_SHIFT) & 3u); d.filter = (P.rstate & PFR_FILTER) ? 1 : 0;
        d.tx = P.texTx; d.ty = P.texTy;
    } else {
        const PFDrawState &S = states[P.flags >> 8];
        d.tex = S.tex; d.w = S.texW; d.h = S.texH; d.wrap = S.texWrap; d.filter = S.texFilter;
        d.tx = S.texTx; d.ty = S.texTy;
    }
    return d;
}

// Texel at linear offset y*w + x; offsets outside the texture read as 0
// (the reference reads past its buffer there).
__device__ __forceinline__ uint32_t tex_fetch(const TexDesc &T, int32_t x, int32_t y)
{
    int32_t off = (int32_t)((uint32_t)y * T.w + (uint32_t)x);
    if (off < 0 || (uint32_t)off >= T.w * T.h) return 0u;
    return __ldg(T.tex + off);
}

__device__ __forceinline__ uint32_t lerp_color(uint32_t a, uint32_t b, float t)
{
    const float inv255 = 1.0f / 255.0f;
    int32_t o[4];
    for (int i = 0; i < 4; i++) {
        float af = (float)chn(a, i) * inv255;
        float bf = (float)chn(b, i) * inv255;
        float r = af + t * (bf - af);
        o[i] = __float2int_rn(x86_min(x86_max(r, 0.0f), 1.0f) * 255.0f);   // clamped: in range
    }
    return pack4(o);
}

__device__ uint32_t tex_sample(const TexDesc &T, float u, float v)
{
    int32_t x0, y0;
    tex_map_wh(T.w, T.h, T.wrap, u, v, x0, y0);
    if (T.filter == 0) return tex_fetch(T, x0, y0);
    int32_t x1, y1;
    tex_map_wh(T.w, T.h, T.wrap, u + T.tx, v + T.ty, x1, y1);
    float fx = u * (float)T.w - (float)x0;
    float fy = v * (float)T.h - (float)y0;
    fx = x86_min(x86_max(fx, 0.0f), 1.0f);
    fy = x86_min(x86_max(fy, 0.0f), 1.0f);
    uint32_t c00 = tex_fetch(T, x0, y0), c10 = tex_fetch(T, x1, y0);
    uint32_t c01 = tex_fetch(T, x0, y1), c11 = tex_fetch(T, x1, y1);
    return lerp_color(lerp_color(c00, c10, fx), lerp_color(c01, c11, fx), fy);
}

// Cephes log/exp as adapted for SSE/AVX by J. Pommier and G. Garberoglio
// (zlib licence), the reference's per-fragment power (simd.h:183-300, 1158-1170).
__device__ float cephes_log(float x)
{
    const bool invalid = (x <= 0.0f);
    x = x86_max(x, __uint_as_float(0x00800000u));
    int32_t e_i = (int32_t)(__float_as_uint(x) >> 23);
    x = __uint_as_float((__float_as_uint(x) & ~0x7f800000u) | __float_as_uint(0.5f));
    e_i -= 0x7f;
    float e = (float)e_i;
    e = e + 1.0f;
    const bool lt = (x < 0.707106781186547524f);
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
    return invalid ? __uint_as_float(0xffffffffu) : x;
}

__device__ float cephes_exp(float x)
{
    x = x86_min(x, 88.3762626647949f);
    x = x86_max(x, -88.3762626647949f);
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
    int32_t n = x86_cvt_trunc(fx) + 0x7f;
    return y * __uint_as_float((uint32_t)n << 23);
}

__device__ __forceinline__ void dir_simd(float *d, const float *a, const float *b)   // simd.h:2469-2490
{
    d[0] = a[0] - b[0]; d[1] = a[1] - b[1]; d[2] = a[2] - b[2];
    float lsq = d[0]*d[0] + d[1]*d[1];
    lsq = lsq + d[2]*d[2];
    lsq = x86_max(lsq, 1e-5f);
    float inv = __frcp_rn(sqrtf(lsq));
    d[0] = d[0] * inv; d[1] = d[1] * inv; d[2] = d[2] * inv;
}
__device__ __forceinline__ float dot_simd(const float *a, const float *b)
{
    float d = a[0]*b[0] + a[1]*b[1];
    return d + a[2]*b[2];
}

// pfiSimdLightingProcess (lighting.c:149-258), one lane
__device__ uint32_t light_phong(const PFDrawState &S, uint32_t frag, const PFDevMaterial &m,
                                const float *P, const float *N)
{
    const float inv255 = 1.0f / 255.0f;
    float cd[3], ca[3], cs[3];
    for (int i = 0; i < 3; i++) {
        cd[i] = (float)chn(frag, i) * inv255;
        ca[i] = (float)chn(m.amb, i) * inv255;
        cs[i] = (float)chn(m.spec, i) * inv255;
    }
    for (int i = 0; i < 3; i++) ca[i] = ca[i] * cd[i];
    float V[3]; dir_simd(V, S.viewPos, P);
    float acc[3] = { 0.0f, 0.0f, 0.0f };
    for (int li = 0; li < S.nLights; li++) {
        const PFDevLight &l = S.lights[li];
        float la[3], ld[3], ls[3];
        for (int i = 0; i < 3; i++) {
            la[i] = (float)chn(l.amb, i) * inv255;
            ld[i] = (float)chn(l.diff, i) * inv255;
            ls[i] = (float)chn(l.spec, i) * inv255;
        }
        float L[3]; dir_simd(L, l.pos, P);
        float amb[3], dif[3], spe[3];
        for (int i = 0; i < 3; i++) amb[i] = la[i] * ca[i];
        float diff = x86_max(dot_simd(N, L), 0.0f);
        for (int i = 0; i < 3; i++) { dif[i] = ld[i] * diff; dif[i] = dif[i] * cd[i]; }
        float H[3] = { L[0] + V[0], L[1] + V[1], L[2] + V[2] };
        float hs = H[0]*H[0] + H[1]*H[1];
        hs = hs + H[2]*H[2];
        float hinv = __frcp_rn(sqrtf(hs));
        for (int i = 0; i < 3; i++) H[i] = H[i] * hinv;
        float spec = x86_max(dot_simd(N, H), 0.0f);
        spec = cephes_exp(cephes_log(spec) * m.shininess);
        for (int i = 0; i < 3; i++) { spe[i] = ls[i] * spec; spe[i] = spe[i] * cs[i]; }
        if ((double)l.inner < 3.14159265358979323846) {
            float nd[3] = { -l.dir[0], -l.dir[1], -l.dir[2] };
            float theta = dot_simd(L, nd);
            float eps = l.inner - l.outer;
            float it = (theta - l.outer) / eps;
            it = x86_min(x86_max(it, 0.0f), 1.0f);
            for (int i = 0; i < 3; i++) { dif[i] = dif[i] * it; spe[i] = spe[i] * it; }
        }
        if (l.attL != 0.0f || l.attQ != 0.0f) {
            // pfiVec3DistanceSq_simd reads y for z (simd.h:2423-2442)
            float d0 = l.pos[0] - P[0], d1 = l.pos[1] - P[1], d2 = l.pos[1] - P[1];
            float dsq = d0*d0 + (d1*d1 + d2*d2);
            float dist = sqrtf(dsq);
            float att = __frcp_rn(l.attC + (l.attL*dist + l.attQ*dsq));
            for (int i = 0; i < 3; i++) { amb[i] = amb[i] * att; dif[i] = dif[i] * att; spe[i] = spe[i] * att; }
        }
        for (int i = 0; i < 3; i++) { acc[i] = acc[i] + amb[i]; acc[i] = acc[i] + dif[i]; acc[i] = acc[i] + spe[i]; }
    }
    int32_t o[4] = { 0, 0, 0, 0 };
    for (int i = 0; i < 3; i++) o[i] = __float2int_rn(x86_min(x86_max(acc[i], 0.0f), 1.0f) * 255.0f);
    return pack4(o);
}

// ---------------------------------------------------------------------------
// k_vertex
// ---------------------------------------------------------------------------
__device__ __forceinline__ int seg_of_vertex(const PFSegment *segs, int nSegs, uint32_t g)
{
    int lo = 0, hi = nSegs - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (segs[mid].vtxBase <= g) lo = mid; else hi = mid - 1; }
    return lo;
}
__device__ __forceinline__ int seg_of_item(const PFSegment *segs, int nSegs, uint32_t g)
{
    int lo = 0, hi = nSegs - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (segs[mid].itemBase <= g) lo = mid; else hi = mid - 1; }
    return lo;
}

// One thread per vertex of the batch.  The grid also clears the tile bin
// counters and the per-batch counters for k_items (so no memset launches).
__global__ void k_vertex(const PFSegment *__restrict__ segs, int nSegs, const PFDrawState *__restrict__ states,
                         PFVertexOut *__restrict__ out, uint32_t nVerts, PFDevCounters *cnt,
                         uint32_t *__restrict__ binCount, uint32_t nTiles)
{
    __shared__ int sUniform, sAborted;
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    asm volatile("griddepcontrol.wait;" ::: "memory");   // (no-op unless launched programmatically serialized)
    // thread 0 takes the block's decisions, behind one barrier: the abort
    // (one decision per block) and the segment of the block's vertices when
    // they share one (the usual case; the others search)
    const uint32_t g0 = blockIdx.x * blockDim.x;
    if (threadIdx.x == 0) {
        sAborted = cnt->abortCommand != 0xffffffffu;
        int su = -1;
        if (g0 < nVerts) {
            const int a = seg_of_vertex(segs, nSegs, g0), b = seg_of_vertex(segs, nSegs, min(g0 + blockDim.x, nVerts) - 1);
            su = (a == b) ? a : -1;
        }
        sUniform = su;
    }
    __syncthreads();
    if (sAborted) return;
    for (uint32_t t = g; t < nTiles; t += gridDim.x * blockDim.x) binCount[t] = 0;
    if (g == 0) {
        cnt->clipCount = 0; cnt->batchRasterized = 0; cnt->tileQueue = 0; cnt->sortQueue = 0;
        cnt->tileListCount = 0;
        for (int l = 0; l < PF_HEAVY_LEVELS; l++) cnt->heavyCount[l] = 0;
    }
    if (g >= nVerts) return;
    // the segment and its draw state are read in place (one address for the
    // block: L1 serves it after the first access)
    const int su = sUniform;
    const PFSegment &sg = segs[su >= 0 ? su : seg_of_vertex(segs, nSegs, g)];
    const PFDrawState &S = states[sg.state];
    const uint32_t j = g - sg.vtxBase;
    float pos[4], nrm[3], uv[2];
    uint32_t col;
    if (sg.srcKind == PF_SRC_RECORDS) {
        const PFVertexIn &r = sg.records[j];
        for (int i = 0; i < 4; i++) pos[i] = r.pos[i];
        for (int i = 0; i < 3; i++) nrm[i] = r.normal[i];
        uv[0] = r.uv[0]; uv[1] = r.uv[1];
        col = r.color;
    } else {
        pos[0] = pos[1] = pos[2] = 0.0f; pos[3] = 1.0f;
        for (int k = 0; k < sg.posSize; k++) pos[k] = sg.pos[(size_t)j * sg.posSize + k];
        if (sg.nrm) { for (int k = 0; k < 3; k++) nrm[k] = sg.nrm[(size_t)j * 3 + k]; }
        else { nrm[0] = sg.constNormal[0]; nrm[1] = sg.constNormal[1]; nrm[2] = sg.constNormal[2]; }
        if (sg.uv) { uv[0] = sg.uv[(size_t)j * 2]; uv[1] = sg.uv[(size_t)j * 2 + 1]; }
        else { uv[0] = sg.constUv[0]; uv[1] = sg.constUv[1]; }
        if (sg.col) {
            col = 0xffffffffu;
            for (int k = 0; k < sg.colSize; k++) {
                uint32_t b = sg.col[(size_t)j * sg.colSize + k];
                col = (col & ~(255u << (8 * k))) | (b << (8 * k));
            }
        } else col = sg.constColor;
    }
    PFVertexOut o;
    uint32_t c0 = col, c1 = col;
    float n[3] = { nrm[0], nrm[1], nrm[2] };
    if (S.flags & PFS_LIGHTING) {
        v3_transform(n, nrm, S.normal);
        v3_normalize(n);
        uint32_t base[2] = { blend_mul_scalar(col, S.mat[0].diff), blend_mul_scalar(col, S.mat[1].diff) };
        if (!(S.flags & PFS_PHONG)) {
            float NdotV = v3_dot(n, S.view8);
            const PFDevMaterial &lm = S.mat[(NdotV < 0.0f) ? 0 : 1];
            base[0] = light_gouraud(S, lm, base[0], pos, n);
            base[1] = (S.mat[0].diff == S.mat[1].diff) ? base[0] : light_gouraud(S, lm, base[1], pos, n);
        }
        c0 = base[0]; c1 = base[1];
    }
    v4_transform(o.h, pos, S.mvp);
    o.uv[0] = uv[0]; o.uv[1] = uv[1];
    o.col[0] = c0; o.col[1] = c1;
    o.n[0] = n[0]; o.n[1] = n[1]; o.n[2] = n[2];
    o.p[0] = pos[0]; o.p[1] = pos[1]; o.p[2] = pos[2];
    o.pad[0] = o.pad[1] = 0;
    out[g] = o;
}

// ---------------------------------------------------------------------------
// setup + binning
// ---------------------------------------------------------------------------

struct BinArgs {
    uint32_t *binCount;
    uint32_t *tileList;        // the raster work lists
    uint32_t listStride;
    uint32_t *bins;
    uint32_t cap;
    const PFTarget *targets;
    PFDevCounters *cnt;
    uint32_t command;
};

// Framebuffer geometry a sub-triangle is binned against.
struct TileSpace {
    uint32_t W, H, tilesX, tileBase;
};

__device__ __forceinline__ TileSpace tile_space(const BinArgs &B, int target)
{
    const PFTarget &t = B.targets[target];
    return TileSpace{ t.W, t.H, t.tilesX, t.tileBase };
}


// Tile range of a set-up sub-triangle: pixels x in [xMin, xMax) and y in
// [yMin, yMax], compared as unsigned (the reference's PFsizei loop bounds),
// clipped to the framebuffer.  Returns false when no pixel remains.
__device__ __forceinline__ bool tile_range(const TileSpace &T, const PFPrim &P, uint32_t &tx0, uint32_t &ty0,
                                           uint32_t &ntx, uint32_t &nty)
{
    uint32_t x0 = (uint32_t)P.xMin, x1 = (uint32_t)P.xMax, y0 = (uint32_t)P.yMin, y1 = (uint32_t)P.yMax;
    if (x1 > T.W) x1 = T.W;
    if (y1 >= T.H) y1 = T.H - 1;
    if (x0 >= x1 || y0 > y1) return false;
    tx0 = x0 / PF_TILE; ty0 = y0 / PF_TILE;
    ntx = (x1 - 1) / PF_TILE - tx0 + 1; nty = y1 / PF_TILE - ty0 + 1;
    return true;
}

// A triangle record's edge functions as the binning tests tiles with them:
// w_e(x, y) = x ex_e + y ey_e + c_e (triangles.c:336-349, 398-420), set
// only when every vertex coordinate and the box lie within (-2^13, 2^13)
// and the framebuffer is at most 2^13 pixels a side -- there the edge
// functions of every pixel of the box stay far inside 32 bits, where the
// reference's wrapping arithmetic is exact (on = false otherwise, and for
// points, lines and rectangles, which keep every tile of their box).
struct EdgeTest {
    int32_t ex[3], ey[3], c[3];
    int32_t xMin, xMax, yMin, yMax;
    bool on;
};
__device__ __forceinline__ EdgeTest edge_test(const PFPrim &P, uint32_t W, uint32_t H)
{
    EdgeTest E;
    const int32_t L = 1 << 13;
    const int32_t v[6] = { P.x1, P.y1, P.x2, P.y2, P.x3, P.y3 };
    bool ok = !(P.flags & PFP_KIND) && W <= (uint32_t)L && H <= (uint32_t)L &&
              P.xMin > -L && P.xMin < L && P.xMax > -L && P.xMax < L && P.yMin > -L && P.yMin < L && P.yMax > -L && P.yMax < L;
    for (int k = 0; k < 6; k++) ok = ok && v[k] > -L && v[k] < L;
    const int32_t vx[3] = { P.x2, P.x3, P.x1 }, vy[3] = { P.y2, P.y3, P.y1 };
    const int32_t sgn = (P.flags & 1u) ? -1 : 1;
    const int32_t sx[3] = { P.y3 - P.y2, P.y1 - P.y3, P.y2 - P.y1 }, sy[3] = { P.x2 - P.x3, P.x3 - P.x1, P.x1 - P.x2 };
    for (int e = 0; e < 3; e++) {
        E.ex[e] = ok ? sgn * sx[e] : 0;
        E.ey[e] = ok ? sgn * sy[e] : 0;
        E.c[e] = ok ? -(vx[e] * E.ex[e] + vy[e] * E.ey[e]) : 0;
    }
    E.xMin = P.xMin; E.xMax = P.xMax; E.yMin = P.yMin; E.yMax = P.yMax;
    E.on = ok;
    return E;
}

// Whether the record may cover a pixel of tile (tx, ty): no, when one of
// its edge functions is negative on the whole rectangle where the tile and
// the box meet -- a pixel is covered only when no edge function is negative
// (triangles.c:415-420), and a linear function is largest at a corner.
__device__ __forceinline__ bool tile_touched(const EdgeTest &E, uint32_t tx, uint32_t ty, uint32_t W, uint32_t H)
{
    if (!E.on) return true;
    // the tile's pixels inside the box and the framebuffer (the box was
    // found inside it by tile_range)
    const int32_t x0 = max(E.xMin, (int32_t)(tx * PF_TILE));
    const int32_t x1 = min(min(E.xMax, (int32_t)(tx * PF_TILE + PF_TILE)), (int32_t)W) - 1;
    const int32_t y0 = max(E.yMin, (int32_t)(ty * PF_TILE));
    const int32_t y1 = min(min(E.yMax, (int32_t)(ty * PF_TILE + PF_TILE - 1)), (int32_t)H - 1);
    bool keep = true;
    for (int e = 0; e < 3; e++) {
        const int32_t w00 = x0 * E.ex[e] + y0 * E.ey[e] + E.c[e];
        const int32_t hi = w00 + max((x1 - x0) * E.ex[e], 0) + max((y1 - y0) * E.ey[e], 0);
        keep = keep && hi >= 0;
    }
    return keep;
}

__device__ __forceinline__ void bin_slot(const BinArgs &B, uint32_t t, uint32_t slot, uint32_t key)
{
    if (slot < B.cap) B.bins[(size_t)t * B.cap + slot] = key;
    else {
        atomicMax(&B.cnt->maxBin, slot + 1);
        if (slot == B.cap) {
            atomicOr(&B.cnt->status, (unsigned)PFD_BIN_OVERFLOW);
            atomicMin(&B.cnt->abortCommand, B.command);
        }
    }
}

// Raster work lists: a tile's bin growing from `before` to `before + added`
// entries puts the tile on the list of non-empty tiles (first entry) and on
// the list of each heavy level it reaches (32, 128, 512, 2048 entries),
// which the rasterizer takes first, heaviest level first, so that the
// longest tiles do not start last.
__device__ __forceinline__ uint32_t heavy_level(uint32_t count)
{
    uint32_t l = 0;
    for (uint32_t th = PF_HEAVY_BASE; l < PF_HEAVY_LEVELS && count >= th; th <<= 2) l++;
    return l;                                          // 0: below the first level
}

__device__ __forceinline__ void list_tile(const BinArgs &B, uint32_t t, uint32_t before, uint32_t added)
{
    if (before == 0) B.tileList[atomicAdd(&B.cnt->tileListCount, 1u)] = t;
    for (uint32_t l = heavy_level(before) + 1; l <= heavy_level(before + added); l++)
        B.tileList[l * B.listStride + atomicAdd(&B.cnt->heavyCount[l - 1], 1u)] = t;
}

// Append `key` to the bin of every tile the sub-triangle touches (one
// thread; used by the clipping path).
__device__ void bin_prim(const BinArgs &B, const TileSpace &T, const PFPrim &P, uint32_t key)
{
    uint32_t tx0, ty0, ntx, nty;
    if (!tile_range(T, P, tx0, ty0, ntx, nty)) return;
    const EdgeTest ET = edge_test(P, T.W, T.H);
    for (uint32_t ty = ty0; ty < ty0 + nty; ty++)
        for (uint32_t tx = tx0; tx < tx0 + ntx; tx++) {
            if (!tile_touched(ET, tx, ty, T.W, T.H)) continue;
            const uint32_t t = T.tileBase + ty * T.tilesX + tx;
            const uint32_t slot = atomicAdd(&B.binCount[t], 1u);
            list_tile(B, t, slot, 1u);
            bin_slot(B, t, slot, key);
        }
}

// Warp-cooperative binning: lanes whose sub-triangles touch the same tile
// share one atomic on its counter (neighbouring triangles of a mesh usually
// do); slots within a group follow lane order.  The counters of up to
// BIN_BURST tiles are claimed before any of their slots is written, so that
// the atomics' round trips overlap.  A sub-triangle touching more than
// BIN_WIDE tiles is binned by the whole warp, 32 of its tiles at a time.
// Every lane of the warp must call it (lanes with nothing to bin pass
// has = false).
#define BIN_BURST 4
#define BIN_WIDE 32
__device__ void bin_prim_warp(const BinArgs &B, const TileSpace &T, bool has, const PFPrim &P, uint32_t key)
{
    uint32_t tx0 = 0, ty0 = 0, ntx = 1, nty = 0;
    if (has && !tile_range(T, P, tx0, ty0, ntx, nty)) has = false;
    uint32_t n = has ? ntx * nty : 0;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1;
    // large sub-triangles, one after the other: each lane takes tiles of it,
    // each with its own counter (independent atomics)
    for (uint32_t wide = __ballot_sync(0xffffffffu, n > BIN_WIDE); wide; wide &= wide - 1) {
        const int src = __ffs(wide) - 1;
        const uint32_t wx0 = __shfl_sync(0xffffffffu, tx0, src), wy0 = __shfl_sync(0xffffffffu, ty0, src);
        const uint32_t wnx = __shfl_sync(0xffffffffu, ntx, src), wn = __shfl_sync(0xffffffffu, n, src);
        const uint32_t wkey = __shfl_sync(0xffffffffu, key, src);
        // the tile space of that lane's framebuffer (the lanes of a batch's
        // warp may draw into different ones)
        const uint32_t wbase = __shfl_sync(0xffffffffu, T.tileBase, src), wtx = __shfl_sync(0xffffffffu, T.tilesX, src);
        const uint32_t wW = __shfl_sync(0xffffffffu, T.W, src), wH = __shfl_sync(0xffffffffu, T.H, src);
        EdgeTest wb;
        {
            const EdgeTest mine = edge_test(P, T.W, T.H);
            for (int e = 0; e < 3; e++) {
                wb.ex[e] = __shfl_sync(0xffffffffu, mine.ex[e], src);
                wb.ey[e] = __shfl_sync(0xffffffffu, mine.ey[e], src);
                wb.c[e] = __shfl_sync(0xffffffffu, mine.c[e], src);
            }
            wb.xMin = __shfl_sync(0xffffffffu, mine.xMin, src); wb.xMax = __shfl_sync(0xffffffffu, mine.xMax, src);
            wb.yMin = __shfl_sync(0xffffffffu, mine.yMin, src); wb.yMax = __shfl_sync(0xffffffffu, mine.yMax, src);
            wb.on = __shfl_sync(0xffffffffu, (int)mine.on, src) != 0;
        }
        for (uint32_t i0 = 0; i0 < wn; i0 += 32u * BIN_BURST) {
            uint32_t tt[BIN_BURST], bb[BIN_BURST];
#pragma unroll
            for (int u = 0; u < BIN_BURST; u++) {
                const uint32_t i = i0 + 32u * (uint32_t)u + lane;
                const bool hit = i < wn && tile_touched(wb, wx0 + i % wnx, wy0 + i / wnx, wW, wH);
                tt[u] = hit ? wbase + (wy0 + i / wnx) * wtx + (wx0 + i % wnx) : 0xffffffffu;
                bb[u] = hit ? atomicAdd(&B.binCount[tt[u]], 1u) : 0u;
            }
#pragma unroll
            for (int u = 0; u < BIN_BURST; u++) {
                if (tt[u] == 0xffffffffu) continue;
                list_tile(B, tt[u], bb[u], 1u);
                bin_slot(B, tt[u], bb[u], wkey);
            }
        }
    }
    if (n > BIN_WIDE) n = 0;
    const EdgeTest ET = edge_test(P, T.W, T.H);
    uint32_t most = n;
    for (int o = 16; o > 0; o >>= 1) most = max(most, __shfl_xor_sync(0xffffffffu, most, o));
    for (uint32_t i0 = 0; i0 < most; i0 += BIN_BURST) {
        uint32_t tt[BIN_BURST], gg[BIN_BURST], bb[BIN_BURST];
#pragma unroll
        for (int u = 0; u < BIN_BURST; u++) {
            const uint32_t i = i0 + (uint32_t)u;
            tt[u] = 0xffffffffu; gg[u] = 0; bb[u] = 0;
            if (i >= most) continue;                           // uniform over the warp
            const bool act = i < n && tile_touched(ET, tx0 + i % ntx, ty0 + i / ntx, T.W, T.H);
            const uint32_t t = act ? T.tileBase + (ty0 + i / ntx) * T.tilesX + (tx0 + i % ntx) : 0xffffffffu;
            const uint32_t grp = __match_any_sync(0xffffffffu, t);
            tt[u] = t; gg[u] = grp;
            if (act && lane == (uint32_t)(__ffs(grp) - 1)) bb[u] = atomicAdd(&B.binCount[t], (unsigned)__popc(grp));
        }
#pragma unroll
        for (int u = 0; u < BIN_BURST; u++) {
            const uint32_t i = i0 + (uint32_t)u;
            if (i >= most) continue;
            const uint32_t grp = gg[u], leader = (uint32_t)(__ffs(grp) - 1);
            const uint32_t base = __shfl_sync(0xffffffffu, bb[u], leader);
            if (tt[u] == 0xffffffffu) continue;
            if (lane == leader) list_tile(B, tt[u], base, (uint32_t)__popc(grp));
            bin_slot(B, tt[u], base + __popc(grp & lt), key);
        }
    }
}

__device__ __forceinline__ void store_phong(PFPrimPhong *dst, const SVert &a, const SVert &b, const SVert &c)
{
    PFPrimPhong q;
    for (int i = 0; i < 3; i++) {
        q.n1[i] = a.n[i]; q.n2[i] = b.n[i]; q.n3[i] = c.n[i];
        q.p1[i] = a.p[i]; q.p2[i] = b.p[i]; q.p3[i] = c.p[i];
    }
    q.pad[0] = q.pad[1] = 0.0f;
    *dst = q;
}

__device__ __forceinline__ void item_vertices(const PFSegment &sg, uint32_t k, uint32_t v[3], int &face, unsigned *status)
{
    uint32_t s[3];
    if (sg.itemKind == PF_ITEMS_TRIS) {
        uint32_t tri = (sg.nFaces == 2) ? (k >> 1) : k;
        face = (sg.nFaces == 2) ? (int)(k & 1) : sg.face0;
        s[0] = 3 * tri; s[1] = 3 * tri + 1; s[2] = 3 * tri + 2;
    } else {
        const int4 e = reinterpret_cast<const int4 *>(sg.explicitItems)[k];
        s[0] = (uint32_t)e.x; s[1] = (uint32_t)e.y; s[2] = (uint32_t)e.z; face = e.w;
    }
    for (int m = 0; m < 3; m++) {
        uint32_t j = sg.idx ? __ldg(sg.idx + s[m]) : s[m];
        if (j >= sg.nVerts) {                          // the host sizes nVerts from the indices, except for
            j = sg.nVerts - 1;                         // device indices (pfDrawElementsDevice): clamped, flagged
            atomicOr(status, (unsigned)PFD_BOUNDS);
        }
        v[m] = sg.vtxBase + j;
    }
}

// ---------------------------------------------------------------------------
// polygon clipping (triangles.c:157-280), for the rare items that cross a
// clip plane; called out of line from k_items
// ---------------------------------------------------------------------------
struct CVert { float h[4]; float pos[4]; float n[3]; float uv[2]; uint32_t c; };

// pfiLerpVertex (internal/context/context.c:67-90)
__device__ void lerp_vert(CVert &r, const CVert &s, const CVert &e, float t)
{
    uint32_t uT = x86_ftoub(255.0f * t);
    r.c = 0;
    for (int i = 0; i < 4; i++) {
        r.h[i] = s.h[i] + t*(e.h[i] - s.h[i]);
        r.pos[i] = s.pos[i] + t*(e.pos[i] - s.pos[i]);
        int32_t sc = (int32_t)chn(s.c, i), ec = (int32_t)chn(e.c, i);
        r.c |= ((uint32_t)(sc + ((int32_t)uT * (ec - sc)) / 255) & 255u) << (8 * i);
    }
    r.uv[0] = s.uv[0] + t*(e.uv[0] - s.uv[0]);
    r.uv[1] = s.uv[1] + t*(e.uv[1] - s.uv[1]);
    for (int i = 0; i < 3; i++) r.n[i] = s.n[i] + t*(e.n[i] - s.n[i]);
}

__device__ int clip_plane(CVert *poly, int n, CVert *tmp, int ax, int sign)
{
    // sign 0: w clip (w < eps is outside); sign +1: h[ax] <= w; sign -1: -h[ax] <= w
    for (int i = 0; i < n; i++) tmp[i] = poly[i];
    int m = 0;
    int prev = n - 1;
    auto inside = [&](const CVert &v) -> int {
        if (sign == 0) return (v.h[3] < 1e-5f) ? -1 : 1;
        if (sign > 0) return (v.h[ax] <= v.h[3]) ? 1 : -1;
        return (-v.h[ax] <= v.h[3]) ? 1 : -1;
    };
    int pd = inside(tmp[prev]);
    for (int i = 0; i < n; i++) {
        int cd = inside(tmp[i]);
        if (pd * cd < 0 && m < PF_CLIP_MAXV) {
            const CVert &p = tmp[prev], &c = tmp[i];
            float t;
            if (sign == 0) t = (1e-5f - p.h[3]) / (c.h[3] - p.h[3]);
            else if (sign > 0) t = (p.h[3] - p.h[ax]) / ((p.h[3] - p.h[ax]) - (c.h[3] - c.h[ax]));
            else t = (p.h[3] + p.h[ax]) / ((p.h[3] + p.h[ax]) - (c.h[3] + c.h[ax]));
            lerp_vert(poly[m++], p, c, t);
        }
        if (cd > 0 && m < PF_CLIP_MAXV) poly[m++] = tmp[i];
        pd = cd; prev = i;
    }
    return m;
}

struct ItemOut {
    PFPrim *prims;
    PFPrimPhong *primsPh;
    PFPrim *pool;
    PFPrimPhong *poolPh;
    uint32_t poolCap;
    uint64_t *rowInfo;          // launches with a row-rasterized target: per item, row_info (null otherwise)
    uint64_t *rowGroup;         // and per 32 items (a k_items warp), the rows their records span
};
static_assert(PF_MAX_SUBTRIS <= 16, "an item's sub-triangles are the bits of a 16-bit mask");

// What k_rows needs to know of an item without reading its records: bit s
// (s < 16) set when sub-triangle s has a record that draws something, and
// the first and last framebuffer row of those records (24 bits each, at
// bits 16 and 40; rows are unsigned, as tile_edge reads a box).
__device__ __forceinline__ void row_info_add(uint64_t &info, uint32_t sub, const PFPrim &P)
{
    const uint32_t xMin = (uint32_t)P.xMin, xMax = (uint32_t)P.xMax, lo = (uint32_t)P.yMin, hi = (uint32_t)P.yMax;
    if (xMin >= xMax || lo > hi || hi == 0xffffffffu) return;           // an empty box: nothing drawn
    uint64_t l = min(lo, 0xffffffu), h = min(hi, 0xffffffu);
    if (info & 0xffffu) { l = min(l, (info >> 16) & 0xffffffu); h = max(h, info >> 40); }
    info = (info & 0xffffu) | (1ull << sub) | (l << 16) | (h << 40);
}
// The rows spanned by the records of a warp's 32 items (row_info words w of
// its lanes, 0 past the end): bit 0 set when there is any, the first and
// last row at bits 16 and 40.
__device__ __forceinline__ uint64_t row_group(uint64_t w)
{
    const bool any = (w & 0xffffu) != 0;
    uint32_t lo = any ? (uint32_t)((w >> 16) & 0xffffffu) : 0xffffffu, hi = any ? (uint32_t)(w >> 40) : 0u;
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    return __any_sync(0xffffffffu, any) ? (1ull | (uint64_t)lo << 16 | (uint64_t)hi << 40) : 0ull;
}

// rowInfo[g] of an item whose only record is P (kept) or that has none;
// out of line, so that the set-up path keeps its registers
__device__ __noinline__ void store_row_info(uint64_t *rowInfo, uint32_t g, const PFPrim &P, bool kept)
{
    uint64_t rows = 0;
    if (kept) row_info_add(rows, 0, P);
    rowInfo[g] = rows;
}

__device__ __noinline__ void clip_item(const PFDrawState &S, int stateIdx, const PFVertexOut *const *V, int face,
                                       uint32_t g, const ItemOut &O, const BinArgs &B, const TileSpace &T)
{
    CVert poly[PF_CLIP_MAXV], tmp[PF_CLIP_MAXV];
    if (O.rowInfo) O.rowInfo[g] = 0;
    for (int m = 0; m < 3; m++) {
        const PFVertexOut &o = *V[m];
        for (int i = 0; i < 4; i++) poly[m].h[i] = o.h[i];
        poly[m].pos[0] = o.p[0]; poly[m].pos[1] = o.p[1]; poly[m].pos[2] = o.p[2];
        poly[m].pos[3] = 1.0f;     // object-space w is not read after clipping
        for (int i = 0; i < 3; i++) poly[m].n[i] = o.n[i];
        poly[m].uv[0] = o.uv[0]; poly[m].uv[1] = o.uv[1];
        poly[m].c = o.col[face];
    }
    int n = clip_plane(poly, 3, tmp, 3, 0);
    for (int ax = 0; ax < 3 && n > 0; ax++) {
        n = clip_plane(poly, n, tmp, ax, +1);
        if (n == 0) break;
        n = clip_plane(poly, n, tmp, ax, -1);
    }
    if (n < 3) return;
    SVert s[PF_CLIP_MAXV];
    for (int i = 0; i < n; i++) {
        float hz = __frcp_rn(poly[i].h[2]);
        s[i].u = poly[i].uv[0] * hz; s[i].v = poly[i].uv[1] * hz;
        float invW = __frcp_rn(poly[i].h[3]);
        to_screen(S, poly[i].h[0] * invW, poly[i].h[1] * invW, s[i].sx, s[i].sy);
        s[i].z = hz;
        s[i].c = poly[i].c;
        for (int k = 0; k < 3; k++) { s[i].n[k] = poly[i].n[k]; s[i].p[k] = poly[i].pos[k]; }
    }
    const int nsub = n - 2;
    uint32_t base = 0;
    if (nsub > 1) {
        base = atomicAdd(&B.cnt->clipCount, (unsigned)(nsub - 1));
        if (base + (uint32_t)(nsub - 1) > O.poolCap) {
            atomicOr(&B.cnt->status, (unsigned)PFD_CLIP_OVERFLOW);
            atomicMin(&B.cnt->abortCommand, B.command);
            return;
        }
    }
    PFPrim first;
    bool firstSet = false;
    uint64_t rows = 0;
    for (int i = 0; i < nsub; i++) {
        PFPrim P;
        if (!setup_prim(S, face, true, s[0], s[i + 1], s[i + 2], stateIdx, P)) continue;
        row_info_add(rows, (uint32_t)i, P);
        atomicAdd(&B.cnt->batchRasterized, 1ull);
        if (i == 0) { first = P; firstSet = true; }
        else {
            O.pool[base + i - 1] = P;
            if (S.flags & PFS_PHONG) store_phong(&O.poolPh[base + i - 1], s[0], s[i + 1], s[i + 2]);
        }
        bin_prim(B, T, P, (g << PF_SUB_BITS) | (uint32_t)i);
    }
    // prims[g] carries the pool base of sub-triangles >= 1 even when
    // sub-triangle 0 was culled.
    if (!firstSet) { first.flags = 0; first.xMin = 1; first.xMax = 0; }
    first.poolBase = (int32_t)base;
    O.prims[g] = first;
    if (O.rowInfo) O.rowInfo[g] = rows;
    if (firstSet && (S.flags & PFS_PHONG)) store_phong(&O.primsPh[g], s[0], s[1], s[2]);
}

// ---------------------------------------------------------------------------
// k_items: one thread per triangle-face item, in submission order
// ---------------------------------------------------------------------------
// Project, clip if needed and set up item g.  Returns true when its
// unclipped sub-triangle survived culling and must be binned by the caller
// (clipped items bin their sub-triangles themselves).
__device__ __forceinline__ bool item_setup(const PFSegment &sg, const PFDrawState *sState,
                                           const PFDrawState *__restrict__ states,
                                           const PFVertexOut *__restrict__ vout, uint32_t g, const ItemOut &O,
                                           const BinArgs &B, const TileSpace &T, PFPrim &P)
{
    const PFDrawState &S = sState ? *sState : states[sg.state];
    const uint32_t k = g - sg.itemBase + sg.itemSkip;
    if (sg.itemKind == PF_ITEMS_EXPLICIT && reinterpret_cast<const int4 *>(sg.explicitItems)[k].w < 0) {
        // a point or a line set up on the host: its record, under this draw state
        const uint32_t r = (uint32_t)reinterpret_cast<const int4 *>(sg.explicitItems)[k].x;
        P = static_cast<const PFPrim *>(sg.prebuilt)[r];
        P.flags = (P.flags & 0xffu) | ((uint32_t)sg.state << 8);
        // its own depth test, blending and depth write stand in for the
        // state's (a thick line's centre is always tested; pfRectf does none)
        P.rstate = (raster_state(S) & ~(uint32_t)PFP_OPS) | (P.flags & PFP_OPS);
        P.zReject = __int_as_float(0x7fffffff);
        O.prims[g] = P;
        if (O.rowInfo) store_row_info(O.rowInfo, g, P, true);
        return true;
    }
    uint32_t vi[3]; int face;
    item_vertices(sg, k, vi, face, &B.cnt->status);
    const PFVertexOut *V[3] = { &vout[vi[0]], &vout[vi[1]], &vout[vi[2]] };
    float4 hv[3];
    for (int m = 0; m < 3; m++) hv[m] = *reinterpret_cast<const float4 *>(V[m]->h);
    float ws = 0.0f;
    for (int m = 0; m < 3; m++) ws += hv[m].w;
    const bool is2D = fabsf(ws - 3.0f) < 1e-5f;
    if (!is2D) {
        bool inside = true;
        for (int m = 0; m < 3; m++) {
            const float4 h = hv[m];
            inside = inside && !(h.w < 1e-5f) && (h.x <= h.w) && (-h.x <= h.w) && (h.y <= h.w) && (-h.y <= h.w) &&
                     (h.z <= h.w) && (-h.z <= h.w);
        }
        if (!inside) { clip_item(S, sg.state, V, face, g, O, B, T); return false; }
    }
    SVert s[3];
    for (int m = 0; m < 3; m++) {
        const PFVertexOut &o = *V[m];
        const float4 h = hv[m];
        const float2 uv = *reinterpret_cast<const float2 *>(o.uv);
        if (is2D) {
            to_screen(S, h.x, h.y, s[m].sx, s[m].sy);
            s[m].z = h.z; s[m].u = uv.x; s[m].v = uv.y;
        } else {
            float hz = __frcp_rn(h.z);
            s[m].u = uv.x * hz; s[m].v = uv.y * hz;
            float invW = __frcp_rn(h.w);
            to_screen(S, h.x * invW, h.y * invW, s[m].sx, s[m].sy);
            s[m].z = hz;
        }
        s[m].c = o.col[face];
        if (S.flags & PFS_PHONG)
            for (int i = 0; i < 3; i++) { s[m].n[i] = o.n[i]; s[m].p[i] = o.p[i]; }
    }
    const bool kept = setup_prim(S, face, !is2D, s[0], s[1], s[2], sg.state, P);
    if (O.rowInfo) store_row_info(O.rowInfo, g, P, kept);
    if (!kept) return false;
    O.prims[g] = P;
    if (S.flags & PFS_PHONG) store_phong(&O.primsPh[g], s[0], s[1], s[2]);
    return true;
}
__global__ void __launch_bounds__(128, 6) k_items(const PFSegment *__restrict__ segs, int nSegs, const PFDrawState *__restrict__ states,
                        const PFVertexOut *__restrict__ vout, uint32_t nItems, ItemOut O, BinArgs B)
{
    __shared__ int sUniform, sAborted;
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    asm volatile("griddepcontrol.wait;" ::: "memory");   // k_vertex is done
    // Thread 0 takes the block's decisions, behind one barrier: whether an
    // overflow in this launch has flagged the abort (other blocks set it
    // while this one runs; a thread that returned alone would leave the rest
    // of the block with unset shared state), and the segment of the block's
    // items when they share one (the usual case; the others search).
    const uint32_t g0 = blockIdx.x * blockDim.x;
    if (threadIdx.x == 0) {
        sAborted = B.cnt->abortCommand != 0xffffffffu;
        const int a = seg_of_item(segs, nSegs, g0), b = seg_of_item(segs, nSegs, min(g0 + blockDim.x, nItems) - 1);
        sUniform = (a == b) ? a : -1;
    }
    __syncthreads();
    if (sAborted) return;
    const int su = sUniform;
    // every lane stays to the end: binning below is warp-cooperative
    PFPrim P;
    bool kept = false;
    TileSpace T{ 0, 0, 0, 0 };
    if (g < nItems) {
        // the segment and its draw state are read in place (one address for
        // the block: L1 serves it after the first access)
        const PFSegment &sg = segs[su >= 0 ? su : seg_of_item(segs, nSegs, g)];
        T = tile_space(B, sg.target);
        kept = item_setup(sg, nullptr, states, vout, g, O, B, T, P);
    }
    // one counter update per warp, its result unused (a reduction in L2, no
    // round trip, no block barrier)
    const unsigned wk = __popc(__ballot_sync(0xffffffffu, kept));
    if ((threadIdx.x & 31) == 0 && wk) atomicAdd(&B.cnt->batchRasterized, (unsigned long long)wk);
    if (O.rowInfo) {                                   // the warp's summary for k_rows
        const uint64_t grp = row_group(g < nItems ? O.rowInfo[g] : 0ull);
        if ((threadIdx.x & 31) == 0) O.rowGroup[g >> 5] = grp;
    }
    bin_prim_warp(B, T, kept, P, g << PF_SUB_BITS);
}

// ---------------------------------------------------------------------------
// k_binsort and k_raster
//
// k_items appends a tile's bin entries (order keys item << 4 | sub-triangle)
// in atomic order.  k_binsort puts every bin that reached REG_SORT_MAX
// entries back into submission order, in place (one CTA per bin); shorter
// bins are sorted by the rasterizing warp itself, in registers.
//
// k_raster: one warp per 8x8 tile, two pixels per lane, warps independent
// of each other (a CTA only groups four of them).  A warp takes a tile from
// the work queue and walks its bin in batches of 32 sub-triangles in
// submission order:
//   1. every lane loads one record of the batch into the warp's shared
//      memory and derives its edge functions at the tile origin and its
//      bounding box clipped to the tile;
//   2. each lane walks the batch in order at its own two pixels: coverage
//      with the reference's integer edge functions, depth, depth test and
//      depth write (triangles.c:398-438) -- which leaves, per pixel, the
//      fragments that passed (bit k of a 32-bit mask: the record's place in
//      the batch);
//   3. the passing fragments are listed pixel by pixel in submission order
//      and shaded densely over the warp (texture, Gouraud / Phong colour:
//      the source colour does not depend on the destination);
//   4. every pixel blends its listed fragments in order into its colour,
//      held in registers with its depth for the whole tile.
// ---------------------------------------------------------------------------
// k_raster's CTAs group 2, 4 or 8 independent warps (the block shape, a
// tuning knob); each warp owns one tile at a time
#define QCHN 32                     // records per batch (bit k of a pixel's 32-bit masks)
// work-queue entries of a half tile: the tile index with one of these set
#define TILE_TOP 0x40000000u
#define TILE_BOTTOM 0x60000000u
#define TILE_HALF_MASK 0x60000000u
#define QFW 128                     // fragment window of a warp
#define SORT_THREADS 256
#define REG_SORT_MAX 128            // bins shorter than this are sorted by the raster warp (four keys a lane)
#define REG_SORT_LEVEL 2            // the heavy-level list of bins that reached REG_SORT_MAX entries

static_assert(PF_TILE == 8 && PF_TILE_PIXELS == 64, "a warp owns a tile: two pixels per lane");
static_assert(REG_SORT_MAX == (PF_HEAVY_BASE << (2 * (REG_SORT_LEVEL - 1))), "k_binsort takes one heavy-level list");

struct RasterArgs {
    const uint32_t *binCount;
    const uint32_t *tileList;
    uint32_t listStride;
    uint32_t *bins;
    uint32_t cap;
    const PFPrim *prims;
    const PFPrimPhong *primsPh;
    const PFPrim *pool;
    const PFPrimPhong *poolPh;
    const PFDrawState *states;
    const PFTarget *targets;
    int nTargets;
    uint32_t totalTiles;
    PFDevCounters *cnt;
    uint32_t command;
    int anyPhong;
};

// A batch record in shared memory, padded to 144 bytes: lane i's record
// starts 4 banks after lane i-1's, so 16-byte accesses of the records of 8
// lanes touch all 32 banks once (with 128 bytes they would all start in
// bank 0).
struct __align__(16) SPrim {
    PFPrim p;
    const PFPrimPhong *ph;     // its per-fragment lighting record (read when a fragment is shaded)
    uint64_t pad;
};

// A batch record's coverage view, three 16-byte words: edge functions at the
// tile origin and their x / y steps, the box clipped to the tile
// (x0 | width << 4 | y0 << 8 | height << 12) with the record's kind above
// (bits 16-17), the raster state and the depth-test rejection bound.
struct __align__(16) QEdge {
    int32_t e0[3], ex0;
    int32_t ex1, ex2, ey0, ey1;
    int32_t ey2;
    uint32_t box, rstate;
    float zReject;             // every covered fragment fails the depth test when zReject >= depth (NaN: never)
};

// Shared memory of one warp.
struct QWarp {
    SPrim rec[QCHN];
    QEdge edge[QCHN];
    uint32_t keys[REG_SORT_MAX];   // a short bin's keys in submission order (sorted in registers)
    uint16_t fdesc[QFW];       // listed fragments: tile pixel << 5 | record
    uint32_t fc[QFW];          // their colour
};

// Edge set-up of a record (its first three 16-byte words: x1 y1 x2 y2 |
// x3 y3 xMin yMin | xMax yMax flags -) for the tile at (ox, oy) of a W x H
// framebuffer (triangles.c:336-349, 398-420: the integer edge functions,
// stepped from the tile origin).
__device__ __forceinline__ void tile_edge(const int4 q0, const int4 q1, const int4 q2, uint32_t rstate, float zReject,
                                          uint32_t ox, uint32_t oy, uint32_t W, uint32_t H, QEdge &E)
{
    const int32_t X1 = q0.x, Y1 = q0.y, X2 = q0.z, Y2 = q0.w, X3 = q1.x, Y3 = q1.y;
    const uint32_t xMin = (uint32_t)q1.z, yMin = (uint32_t)q1.w, xMax = (uint32_t)q2.x, yMax = (uint32_t)q2.y;
    const uint32_t flags = (uint32_t)q2.z, face = flags & 1u;
    int32_t sx[3] = { Y3 - Y2, Y1 - Y3, Y2 - Y1 };
    int32_t sy[3] = { X2 - X3, X3 - X1, X1 - X2 };
    const int32_t rx[3] = { X2, X3, X1 }, ry[3] = { Y2, Y3, Y1 };
    int32_t e0[3];
    for (int e = 0; e < 3; e++) {
        if (face) { sx[e] = -sx[e]; sy[e] = -sy[e]; }
        e0[e] = (int32_t)((ox - (uint32_t)rx[e]) * (uint32_t)sx[e] + (oy - (uint32_t)ry[e]) * (uint32_t)sy[e]);
    }
    // pixels x in [xMin, xMax), y in [yMin, yMax] (unsigned), inside the tile and the framebuffer
    const uint32_t x0 = max(xMin, ox), x1 = min(min(xMax, ox + PF_TILE), W);
    const uint32_t y0 = max(yMin, oy);
    uint32_t y1e = min(min(yMax + 1u, oy + PF_TILE), H);
    if (yMax == 0xffffffffu) y1e = 0;                  // yMax + 1 wrapped
    const bool empty = (x0 >= x1) || (y0 >= y1e) || (xMin >= xMax) || (yMin > yMax);
    const uint32_t bx0 = empty ? 0 : x0 - ox, by0 = empty ? 0 : y0 - oy;
    const uint32_t bw = empty ? 0 : x1 - x0, bh = empty ? 0 : y1e - y0;
    E.e0[0] = e0[0]; E.e0[1] = e0[1]; E.e0[2] = e0[2];
    E.ex0 = sx[0]; E.ex1 = sx[1]; E.ex2 = sx[2];
    E.ey0 = sy[0]; E.ey1 = sy[1]; E.ey2 = sy[2];
    E.box = bx0 | (bw << 4) | (by0 << 8) | (bh << 12) | (((flags & PFP_KIND) >> 6) << 16);
    E.rstate = rstate;
    E.zReject = zReject;
}

// Normalised weights and depth of a covered fragment at tile pixel (X, Y)
// (triangles.c:421-438).
__device__ __forceinline__ float tile_depth(const QEdge &E, const PFPrim &P, uint32_t X, uint32_t Y, float *wn)
{
    const int32_t w1 = (int32_t)((uint32_t)E.e0[0] + X * (uint32_t)E.ex0 + Y * (uint32_t)E.ey0);
    const int32_t w2 = (int32_t)((uint32_t)E.e0[1] + X * (uint32_t)E.ex1 + Y * (uint32_t)E.ey1);
    const int32_t w3 = (int32_t)((uint32_t)E.e0[2] + X * (uint32_t)E.ex2 + Y * (uint32_t)E.ey2);
    wn[0] = (float)w1 * P.wInvSum; wn[1] = (float)w2 * P.wInvSum; wn[2] = (float)w3 * P.wInvSum;
    float zs = P.z1 * wn[0] + P.z2 * wn[1];
    zs = zs + P.z3 * wn[2];
    return __frcp_rn(zs);          // 1 / zs, correctly rounded
}

// Source colour of one fragment (triangles.c:500-521): colour interpolation,
// texturing, per-fragment lighting.  Independent of the destination pixel.
// texOn false: a pixel outside the mask, whose texture coordinates the
// reference replaces by zero before sampling (triangles.c:508-513);
// anyWeights: the pixel may lie outside the triangle (weights outside
// [0, 1]), so the weight conversions follow CVTPS2DQ out of range too.
__device__ __forceinline__ uint32_t shade_fragment(const PFPrim &P, const PFPrimPhong *Q, const PFDrawState *states,
                                                   float wn1, float wn2, float wn3, float z,
                                                   bool texOn = true, bool anyWeights = false)
{
    const uint32_t fl = P.rstate;
    uint32_t frag;
    if (fl & PFS_SMOOTH) {
        // covered pixels have weights in [0, 1]: the conversions are in range
        const float s1 = wn1 * 255.0f, s2 = wn2 * 255.0f, s3 = wn3 * 255.0f;
        const uint32_t u1 = anyWeights ? pff_cvt_rne(s1) : (uint32_t)__float2int_rn(s1);
        const uint32_t u2 = anyWeights ? pff_cvt_rne(s2) : (uint32_t)__float2int_rn(s2);
        const uint32_t u3 = anyWeights ? pff_cvt_rne(s3) : (uint32_t)__float2int_rn(s3);
        int32_t o[4];
        for (int i = 0; i < 4; i++) {
            uint32_t s = u1 * chn(P.c1, i) + u2 * chn(P.c2, i);
            s = s + u3 * chn(P.c3, i);
            o[i] = (int32_t)((s * 257u) >> 16);
        }
        frag = pack4(o);
    } else {
        const float mx = x86_max(wn1, x86_max(wn2, wn3));
        frag = ((mx == wn1) ? P.c1 : 0u) | (((mx == wn2) ? P.c2 : 0u) | ((mx == wn3) ? P.c3 : 0u));
    }
    if (fl & PFS_TEXTURE) {
        float tu = 0.0f, tv = 0.0f;
        if (texOn) {
            tu = P.u1 * wn1 + P.u2 * wn2;
            tu = tu + P.u3 * wn3;
            tv = P.v1 * wn1 + P.v2 * wn2;
            tv = tv + P.v3 * wn3;
            if (P.flags & 2) { tu = tu * z; tv = tv * z; }
        }
        frag = blend_simd(4, tex_sample(tex_desc(P, states), tu, tv), frag);
    }
    if (fl & PFS_PHONG) {
        const PFDrawState &S = states[P.flags >> 8];
        PFPrimPhong q;                                  // (80 bytes, five 16-byte loads)
        for (int i = 0; i < 5; i++) reinterpret_cast<float4 *>(&q)[i] = __ldg(reinterpret_cast<const float4 *>(Q) + i);
        float N[3], Pp[3];
        for (int i = 0; i < 3; i++) {
            float t0 = q.n1[i] * wn1 + q.n2[i] * wn2; N[i] = t0 + q.n3[i] * wn3;
            float t1 = q.p1[i] * wn1 + q.p2[i] * wn2; Pp[i] = t1 + q.p3[i] * wn3;
        }
        frag = light_phong(S, frag, S.mat[P.flags & 1], Pp, N);
    }
    return frag;
}

// ---------------------------------------------------------------------------
// points and lines (src/internal/primitives/points.c, lines.c), set up on
// the host into PFPrim records:
//   line   x1, y1 first pixel; x2 endVal (signed pixel count along the long
//          axis); y2 decInc (16.16 step of the short axis); x3 sgnInc;
//          wInvSum 1 / endVal; z1, z2 and c1, c2 at the ends
//   point  x1, y1 centre; x2 radius in pixels (-1: the single centre
//          pixel); wInvSum the squared radius; z1, c1
// Pixels are absolute framebuffer coordinates.  These run out of line: the
// triangle path stays free of their registers.
// ---------------------------------------------------------------------------
__device__ __noinline__ bool lp_covers(const PFPrim &P, int32_t X, int32_t Y)
{
    if ((P.flags & PFP_KIND) == PFP_BLIT) return true;          // every pixel of its box
    if ((P.flags & PFP_KIND) == PFP_POINT) {                     // points.c:106-183
        const int32_t dx = X - P.x1, dy = Y - P.y1;
        if (P.x2 < 0) return dx == 0 && dy == 0;
        if (dx < -P.x2 || dx > P.x2 || dy < -P.x2 || dy > P.x2) return false;
        return (float)(dy * dy + dx * dx) <= P.wInvSum;
    }
    // lines.c:304-431: step i of the DDA lands on long-axis coordinate a1 + i
    const bool yl = (P.flags & PFP_Y_LONGER) != 0;
    const int32_t a = yl ? Y : X, b = yl ? X : Y, a1 = yl ? P.y1 : P.x1, b1 = yl ? P.x1 : P.y1;
    const uint32_t k = ((uint32_t)a - (uint32_t)a1) * (uint32_t)P.x3;          // steps taken
    const uint32_t steps = P.x2 < 0 ? 0u - (uint32_t)P.x2 : (uint32_t)P.x2;
    if (k >= steps) return false;
    const int32_t j = (int32_t)(k * (uint32_t)P.y2);
    return (uint32_t)b == (uint32_t)b1 + (uint32_t)(j >> 16);
}

// Interpolation parameter of a line pixel: t = i / endVal (lines.c:366).
__device__ __forceinline__ float lp_t(const PFPrim &P, int32_t X, int32_t Y)
{
    const bool yl = (P.flags & PFP_Y_LONGER) != 0;
    const int32_t i = (int32_t)((uint32_t)(yl ? Y : X) - (uint32_t)(yl ? P.y1 : P.x1));
    return (float)i * P.wInvSum;
}

// (PFsizei)(float) as the reference's x86-64 build converts it: a 64-bit
// truncating conversion whose low 32 bits are kept; 0 for NaN / out of range.
__device__ __forceinline__ uint32_t x86_ftou32(float x)
{
    if (!(x > -9.2e18f && x < 9.2e18f)) return 0u;
    return (uint32_t)(unsigned long long)__float2ll_rz(x);
}

// A pfRectf record's colour, or the pfDrawPixels source pixel that lands on
// (X, Y) (context.c:2044-2082): x1, y1 the raster position on screen, x2 the
// image width, y2 / x3 width - 1 / height - 1, wInvSum / z2 the inverse
// zoomed width / height.  Elements past the image read as 0.
__device__ __forceinline__ uint32_t blit_color(const PFPrim &P, int32_t X, int32_t Y)
{
    if (!P.src) return P.c1;
    const float v = (float)(int32_t)((uint32_t)Y - (uint32_t)P.y1) * P.z2;
    const uint32_t ySrc = x86_ftou32(v * (float)(uint32_t)P.x3) * (uint32_t)P.x2;
    const float u = (float)(int32_t)((uint32_t)X - (uint32_t)P.x1) * P.wInvSum;
    const uint32_t o = ySrc + x86_ftou32(u * (float)(uint32_t)P.y2);
    return o < P.nSrc ? __ldg(reinterpret_cast<const uint32_t *>(P.src) + o) : 0u;
}

__device__ __noinline__ float lp_depth(const PFPrim &P, int32_t X, int32_t Y)
{
    if ((P.flags & PFP_KIND) != PFP_LINE) return P.z1;
    const float t = lp_t(P, X, Y);
    return P.z1 + t * (P.z2 - P.z1);
}

// pfiColorLerpSmooth (src/internal/color.h): (PFubyte)(a + t (b - a)) per channel
__device__ __noinline__ uint32_t lp_color(const PFPrim &P, int32_t X, int32_t Y)
{
    if ((P.flags & PFP_KIND) == PFP_POINT) return P.c1;
    if ((P.flags & PFP_KIND) == PFP_BLIT) return blit_color(P, X, Y);
    const float t = lp_t(P, X, Y);
    int32_t o[4];
    for (int i = 0; i < 4; i++) {
        const int32_t a = (int32_t)chn(P.c1, i), b = (int32_t)chn(P.c2, i);
        o[i] = x86_cvt_trunc((float)a + t * (float)(b - a)) & 255;
    }
    return pack4(o);
}

// Scalar depth test of points and lines (src/internal/depth.h:27-74):
// NOTEQUAL is a real !=.
__device__ __forceinline__ bool depth_sisd(int f, float src, float dst)
{
    switch (f) {
    case 0: return src == dst;                                   // EQUAL
    case 1: return src != dst;                                   // NOTEQUAL
    case 2: return src < dst;                                    // LESS
    case 3: return src <= dst;                                   // LEQUAL
    case 4: return src > dst;                                    // GREATER
    default: return src >= dst;                                  // GEQUAL
    }
}

// Scalar blending of points and lines (src/internal/blend.h:27-126): SUB
// subtracts, MUL divides by 255, ALPHA weighs with a + 1.
__device__ __noinline__ uint32_t blend_sisd(int mode, uint32_t src, uint32_t dst)
{
    int32_t o[4];
    for (int i = 0; i < 4; i++) {
        const int32_t s = (int32_t)chn(src, i), d = (int32_t)chn(dst, i);
        int32_t v;
        switch (mode) {
        case 0: v = (s + d) >> 1; break;                         // AVERAGE
        case 1: {                                                // ALPHA
            const uint32_t al = chn(src, 3) + 1u, ia = 256u - al;
            v = (int32_t)((al * (uint32_t)(i == 3 ? 255 : s) + ia * (uint32_t)d) >> 8);
            break;
        }
        case 2: v = min(d + s, 255); break;                      // ADD
        case 3: v = max(d - s, 0); break;                        // SUB
        case 4: v = (s * d) / 255; break;                        // MUL
        case 5: v = min(((d * (255 - s)) >> 8) + s, 255); break; // SCREEN
        case 6: v = max(s, d); break;                            // LIGHTEN
        default: v = min(s, d); break;                           // DARKEN
        }
        o[i] = v & 255;
    }
    return pack4(o);
}

// The colour of the pixel a k_raster thread owns, as the framebuffer holds
// it.  RGBA / unsigned byte: the packed colour, whose getters and setters
// are the identity.  Other formats: the raw pixel, read for blending through
// the SIMD getter (triangles) or the scalar one (points, lines, rectangles,
// images) and written through the matching setter.
template <bool GEN> struct FbPixel;
template <> struct FbPixel<false> {
    uint32_t c;
    __device__ __forceinline__ void load(const PFTarget &T, size_t i) { c = ((const uint32_t *)T.color)[i]; }
    __device__ __forceinline__ void clear(const PFTarget &T) { c = T.clearRaw[0]; }
    __device__ __forceinline__ void store(const PFTarget &T, size_t i) const { ((uint32_t *)T.color)[i] = c; }
    __device__ __forceinline__ uint32_t get(bool) const { return c; }
    __device__ __forceinline__ void set(bool, uint32_t v) { c = v; }
};
template <> struct FbPixel<true> {
    uint32_t r[4];
    uint32_t f;
    __device__ __forceinline__ void load(const PFTarget &T, size_t i) { f = T.fmt; pff_load(f, T.color, i, r); }
    __device__ __forceinline__ void clear(const PFTarget &T)
    {
        f = T.fmt; r[0] = T.clearRaw[0]; r[1] = T.clearRaw[1]; r[2] = T.clearRaw[2]; r[3] = T.clearRaw[3];
    }
    __device__ __forceinline__ void store(const PFTarget &T, size_t i) const { pff_store(f, T.color, i, r); }
    __device__ __forceinline__ uint32_t get(bool scalar) const { return scalar ? pff_get_sisd(f, r) : pff_get_simd(f, r); }
    __device__ __forceinline__ void set(bool scalar, uint32_t v) { if (scalar) pff_set_sisd(f, v, r); else pff_set_simd(f, v, r); }
};

// k_binsort: one CTA per bin that reached REG_SORT_MAX entries (a
// heavy-level list), taken from a queue: its keys are put back into
// submission order in place by a merge sort in shared memory.  A bin is a
// concatenation of runs that are each in order already (a warp of k_items
// appends its lanes' entries of a tile in lane order): each warp first
// sorts 32-key chunks in registers, then chunks are merged pairwise, level
// by level -- a key's place in the merged run is its place in its own run
// plus the number of smaller keys in the partner run, found by binary
// search.  Keys are unique (item << PF_SUB_BITS | sub-triangle, below 2^31);
// the padding to a whole chunk is unique too (2^31 + place), so every level
// is a permutation.
__device__ __forceinline__ uint32_t warp_sort32(uint32_t key)
{
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t k = 2; k <= 32; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            const uint32_t o = __shfl_xor_sync(0xffffffffu, key, (int)j);
            const bool asc = (lane & k) == 0, low = (lane & j) == 0;
            key = (asc == low) ? min(key, o) : max(key, o);
        }
    return key;
}

__global__ void __launch_bounds__(SORT_THREADS) k_binsort(RasterArgs a)
{
    extern __shared__ uint32_t sbuf[];                // two buffers of a bin's keys (merge source and target)
    __shared__ uint32_t sTile;
    asm volatile("griddepcontrol.wait;" ::: "memory");   // k_items is done
    if (a.cnt->abortCommand <= a.command) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t nList = min(a.cnt->heavyCount[REG_SORT_LEVEL - 1], a.totalTiles);
    uint32_t capPad = 32; while (capPad < a.cap) capPad <<= 1;   // each buffer's room
    // a CTA's first entry is its index in the grid, the counter hands out
    // the entries after those (no atomics at all when no bin needs sorting)
    for (uint32_t first = 1;; first = 0) {
        if (tid == 0) {
            const uint32_t q = first ? blockIdx.x : (blockIdx.x < nList ? gridDim.x + atomicAdd(&a.cnt->sortQueue, 1u) : nList);
            sTile = q < nList ? __ldg(a.tileList + (size_t)REG_SORT_LEVEL * a.listStride + q) : 0xffffffffu;
        }
        __syncthreads();
        const uint32_t t = sTile;
        if (t == 0xffffffffu) break;
        const uint32_t n = min(__ldg(a.binCount + t), a.cap);
        const uint32_t nPad = (n + 31u) & ~31u;
        uint32_t *bin = a.bins + (size_t)t * a.cap;
        // 1. chunks of 32 keys sorted in registers (padding 2^31 + place);
        //    whether the bin is in order already
        int unsorted = 0;
        for (uint32_t c = (uint32_t)warp * 32u; c < nPad; c += SORT_THREADS) {
            const uint32_t i = c + (uint32_t)lane;
            const uint32_t key = i < n ? bin[i] : 0x80000000u + i;
            const uint32_t prev = __shfl_up_sync(0xffffffffu, key, 1);
            unsorted |= (lane > 0 && prev > key) || (lane == 0 && c > 0 && i < n && bin[i - 1] > key);
            sbuf[i] = warp_sort32(key);
        }
        if (__syncthreads_or(unsorted)) {
            // 2. merge levels: runs of w keys, pairwise, into the other buffer
            uint32_t *src = sbuf, *dst = sbuf + capPad;
            for (uint32_t w = 32; w < nPad; w <<= 1) {
                for (uint32_t i = tid; i < nPad; i += SORT_THREADS) {
                    const uint32_t run = i / w, s0 = run * w;
                    const uint32_t oStart = (run & 1u) ? s0 - w : s0 + w;      // the partner run
                    const uint32_t oLen = oStart < nPad ? min(w, nPad - oStart) : 0u;
                    const uint32_t key = src[i];
                    uint32_t lo = 0, hi = oLen;                                  // partner keys below key
                    while (lo < hi) { const uint32_t mid = (lo + hi) >> 1; if (src[oStart + mid] < key) lo = mid + 1; else hi = mid; }
                    dst[(run & ~1u) * w + (i - s0) + lo] = key;
                }
                __syncthreads();
                uint32_t *tmp = src; src = dst; dst = tmp;
            }
            for (uint32_t i = tid; i < n; i += SORT_THREADS) bin[i] = src[i];
        }
        __syncthreads();                               // sTile and the buffers are free
    }
}

// List this lane's fragments (bit 32 s + k of m: record k at its pixel of
// slot s), in order, as entries off, off + 1, ... of the warp's fragment
// list, as far as they fall in the window [b0, bEnd).
__device__ __forceinline__ void tile_list(unsigned long long m, uint32_t off, uint32_t b0, uint32_t bEnd,
                                          uint16_t *fdesc)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t cnt = __popcll(m);
    if (!cnt || off >= bEnd || off + cnt <= b0) return;
    uint32_t f = off;
    for (unsigned long long mm = m; mm && f < bEnd; mm &= mm - 1, f++) {
        if (f < b0) continue;
        const uint32_t b = (uint32_t)(__ffsll(mm) - 1);
        fdesc[f - b0] = (uint16_t)(((lane + 32u * (b >> 5)) << 5) | (b & 31u));
    }
}

// 32x32 bit matrix held one row a lane (bit j of lane k) -> one column a
// lane: lane j gets bit k = bit j of lane k.  Five exchange steps, each
// swapping the off-diagonal s x s blocks between lanes k and k ^ s.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t masks[5] = { 0x0000ffffu, 0x00ff00ffu, 0x0f0f0f0fu, 0x33333333u, 0x55555555u };
#pragma unroll
    for (int i = 0; i < 5; i++) {
        const uint32_t s = 16u >> i, m = masks[i];
        const uint32_t y = __shfl_xor_sync(0xffffffffu, x, (int)s);
        x = (lane & s) ? ((x & ~m) | ((y >> s) & m)) : ((x & m) | ((y << s) & ~m));
    }
    return x;
}

// Warp-wide exclusive prefix sum of v; total gets the sum over the warp.
__device__ __forceinline__ uint32_t warp_offsets(uint32_t v, uint32_t &total)
{
    const int lane = threadIdx.x & 31;
    uint32_t s = v;
    for (int o = 1; o < 32; o <<= 1) { const uint32_t t = __shfl_up_sync(0xffffffffu, s, o); if (lane >= o) s += t; }
    total = __shfl_sync(0xffffffffu, s, 31);
    return s - v;
}

template <bool GEN, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, 24 / WARPS) k_raster(RasterArgs a)
{
    extern __shared__ __align__(16) unsigned char rsmem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    QWarp &Q = reinterpret_cast<QWarp *>(rsmem)[warp];

    asm volatile("griddepcontrol.wait;" ::: "memory");   // k_binsort is done
    if (a.cnt->abortCommand <= a.command) return;
    // the batch completed set-up without overflow: its sub-triangles count
    if (blockIdx.x == 0 && tid == 0) atomicAdd(&a.cnt->rasterized, a.cnt->batchRasterized);
    const uint32_t lx = (uint32_t)lane & 7u, ly = (uint32_t)lane >> 3;     // my pixels: (lx, ly) and (lx, ly + 4)
    unsigned long long frags = 0;

    // persistent: warps take tiles from a shared work queue -- the tiles the
    // binning listed as non-empty, those of the heaviest level first, then
    // of each lighter level, then the rest (a tile is rasterized from the
    // first list it is on and skipped on the later ones); then the groups of
    // 32 tiles whose empty bins only get their fused clear, if any, one tile
    // a lane
    uint32_t levelEnd[PF_HEAVY_LEVELS + 1];           // queue index past level l's entries, heaviest first
    uint32_t nQueue = 0;
    // A heavy level with few tiles against the grid's warps sets the end of
    // the launch (its tiles start first but run longest): each of its tiles
    // is then two work items, its top and bottom halves, each a warp with
    // one pixel a lane, which take about half as long.  Where heavy tiles
    // are many the launch is bound by the total work, which halves would
    // only add to (each half walks the whole bin).
    uint32_t splitLevels = 0;
    for (int l = PF_HEAVY_LEVELS; l >= 1; l--) {
        const uint32_t c = min(a.cnt->heavyCount[l - 1], a.totalTiles);
        const bool split = 4u * c <= gridDim.x * (uint32_t)WARPS;
        splitLevels |= split ? 1u << l : 0u;
        nQueue += split ? 2u * c : c;
        levelEnd[l] = nQueue;
    }
    nQueue += min(a.cnt->tileListCount, a.totalTiles);
    levelEnd[0] = nQueue;
    const uint32_t nClear = (a.totalTiles + 31u) / 32u;
    // each warp's first entry is its own index in the grid; the counter
    // hands out the entries after those (3,648 warps claiming their first
    // entry with one atomic each would serialise at the start)
    const uint32_t gridWarps = gridDim.x * (uint32_t)WARPS;
    uint32_t claim = blockIdx.x * (uint32_t)WARPS + (uint32_t)warp;
    for (;;) {
    uint32_t next = 0xffffffffu, nextCount = 0;
    if (lane == 0) {
        const uint32_t q = claim;
        if (q < nQueue + nClear) {
            claim = gridWarps + atomicAdd(&a.cnt->tileQueue, 1u);
            if (q >= nQueue) next = 0x80000000u | (q - nQueue);      // a group of tiles to clear
            else {
                uint32_t level = PF_HEAVY_LEVELS, begin = 0;
                while (q >= levelEnd[level]) { begin = levelEnd[level]; level--; }
                const uint32_t e = q - begin;
                const bool split = (splitLevels >> level) & 1u;
                next = __ldg(a.tileList + (size_t)level * a.listStride + (split ? e >> 1 : e));
                nextCount = __ldg(a.binCount + next);
                if (heavy_level(nextCount) != level) next = 0xfffffffeu;   // rasterized from an earlier list
                else if (split) next |= (e & 1u) ? TILE_BOTTOM : TILE_TOP;
            }
        }
    }
    const uint32_t gt = __shfl_sync(0xffffffffu, next, 0);
    const uint32_t gtCount = __shfl_sync(0xffffffffu, nextCount, 0);   // (its bin count, read for the check)
    if (gt == 0xffffffffu) break;
    if (gt == 0xfffffffeu) continue;
    if (gt & 0x80000000u) {
        // the fused clear of the empty tiles of group gt: one tile a lane,
        // each row of RGBA8 pixels and depths as two 16-byte stores
        const uint32_t t = 32u * (gt & 0x7fffffffu) + (uint32_t)lane;
        if (t < a.totalTiles && __ldg(a.binCount + t) == 0) {
            int clo = 0, chi = a.nTargets - 1;
            while (clo < chi) { int mid = (clo + chi + 1) >> 1; if (a.targets[mid].tileBase <= t) clo = mid; else chi = mid - 1; }
            const PFTarget &C = a.targets[clo];
            if (C.clearMode != 0 && !(GEN && C.fmt == PFF_BGRA8)) {     // (k_rows clears those)
                const uint32_t tile = t - C.tileBase;
                const uint32_t cx = (tile % C.tilesX) * PF_TILE, cy = (tile / C.tilesX) * PF_TILE;
                const uint32_t xe = min(cx + PF_TILE, C.W);
                for (uint32_t py = cy; py < min(cy + PF_TILE, C.H); py++) {
                    const size_t row = (size_t)py * C.W;
                    if (!GEN && xe == cx + 8u && ((row + cx) & 3u) == 0 && !(C.clearMode == 1 && row + cx < 8) &&
                        (((uintptr_t)C.color | (uintptr_t)C.depth) & 15u) == 0) {
                        const uint32_t cr = C.clearRaw[0];
                        const float cd = C.clearDepth;
                        uint4 *cp = reinterpret_cast<uint4 *>((uint32_t *)C.color + row + cx);
                        float4 *dp = reinterpret_cast<float4 *>(C.depth + row + cx);
                        cp[0] = make_uint4(cr, cr, cr, cr); cp[1] = make_uint4(cr, cr, cr, cr);
                        dp[0] = make_float4(cd, cd, cd, cd); dp[1] = make_float4(cd, cd, cd, cd);
                        continue;
                    }
                    for (uint32_t px = cx; px < xe; px++) {
                        const size_t pidx = row + px;
                        if (C.clearMode == 1 && pidx < 8) continue;  // pfClear keeps pixels 0..7
                        if (GEN) pff_store(C.fmt, C.color, pidx, C.clearRaw);
                        else ((uint32_t *)C.color)[pidx] = C.clearRaw[0];
                        C.depth[pidx] = C.clearDepth;
                    }
                }
            }
        }
        continue;
    }
    // whole tile: my pixels are rows ly and ly + 4; half tile: row ly of
    // the top half or ly + 4 of the bottom half only
    const uint32_t gtile = gt & ~TILE_HALF_MASK;
    const bool whole = (gt & TILE_HALF_MASK) == 0;
    const uint32_t rowA = ly + ((gt & TILE_HALF_MASK) == TILE_BOTTOM ? 4u : 0u);
    int tlo = 0, thi = a.nTargets - 1;
    while (tlo < thi) { int mid = (tlo + thi + 1) >> 1; if (a.targets[mid].tileBase <= gtile) tlo = mid; else thi = mid - 1; }
    const PFTarget &T = a.targets[tlo];
    if (GEN && T.fmt == PFF_BGRA8) continue;                 // rasterized by k_rows
    const uint32_t tile = gtile - T.tileBase;
    const uint32_t n = min(gtCount, a.cap);
    if (n == 0 && T.clearMode == 0) continue;
    const uint32_t ox = (tile % T.tilesX) * PF_TILE, oy = (tile / T.tilesX) * PF_TILE;
    const uint32_t W = T.W, H = T.H;

    FbPixel<GEN> col0{}, col1{};
    float dep0 = 0.0f, dep1 = 0.0f;
    const uint32_t X0 = ox + lx, Y0 = oy + rowA, Y1 = Y0 + 4u;
    const bool in0 = X0 < W && Y0 < H, in1 = whole && X0 < W && Y1 < H;
    const size_t pidx0 = (size_t)Y0 * W + X0, pidx1 = (size_t)Y1 * W + X0;
    {
        auto init = [&](FbPixel<GEN> &c, float &d, bool in, size_t pi) {
            if (!in) return;
            if (T.clearMode == 2 || (T.clearMode == 1 && pi >= 8)) { c.clear(T); d = T.clearDepth; }
            else { c.load(T, pi); d = T.depth[pi]; }
        };
        init(col0, dep0, in0, pidx0);
        init(col1, dep1, in1, pidx1);
    }

    // a bin shorter than REG_SORT_MAX is put into submission order here, in
    // registers: a bitonic network over 32, 64 or 128 places, place
    // 32 r + lane in key r of the lane; longer bins were sorted by k_binsort
    const uint32_t *bin = a.bins + (size_t)gtile * a.cap;
    const bool regSort = n < REG_SORT_MAX;
    uint32_t sk[4] = { 0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu };
    if (regSort) {
        const uint32_t nk = n <= 32 ? 1u : n <= 64 ? 2u : 4u;    // keys a lane sorts: a power-of-two network
        for (uint32_t r = 0; r < 4; r++)
            if (32 * r + (uint32_t)lane < n) sk[r] = __ldg(bin + 32 * r + lane);
        // keys binned by one warp of k_items arrive in order: check first
        bool ordered = true;
#pragma unroll
        for (uint32_t r = 0; r < 4; r++) {
            if (r >= nk) break;                               // uniform over the warp
            const uint32_t o = __shfl_down_sync(0xffffffffu, sk[r], 1);
            const uint32_t b = __shfl_sync(0xffffffffu, sk[r < 3 ? r + 1 : 3], 0);
            ordered = ordered && (lane < 31 ? sk[r] <= o : (r + 1 < nk ? sk[r] <= b : true));
        }
        if (!__all_sync(0xffffffffu, ordered))
        for (uint32_t k = 2; k <= 32 * nk; k <<= 1)
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                if (j >= 32) {
                    // partners are keys of the same lane: places i and i + j
                    const uint32_t dr = j >> 5;
#pragma unroll
                    for (uint32_t r = 0; r < 4; r++) {
                        if (r >= nk) break;
                        if (r & dr) continue;
                        const uint32_t i = 32 * r + (uint32_t)lane;
                        const uint32_t x = sk[r], y = sk[r + dr];
                        const bool asc = (i & k) == 0;
                        sk[r] = asc ? min(x, y) : max(x, y);
                        sk[r + dr] = asc ? max(x, y) : min(x, y);
                    }
                } else {
#pragma unroll
                    for (uint32_t r = 0; r < 4; r++) {
                        if (r >= nk) break;                       // uniform over the warp
                        const uint32_t i = 32 * r + (uint32_t)lane;
                        const uint32_t o = __shfl_xor_sync(0xffffffffu, sk[r], j);
                        sk[r] = (((i & k) == 0) == ((i & j) == 0)) ? min(sk[r], o) : max(sk[r], o);
                    }
                }
            }
        // (kept in shared memory for the batches: the registers are free)
        for (uint32_t r = 0; r < 4; r++) Q.keys[32 * r + (uint32_t)lane] = sk[r];
        __syncwarp();
    }

    for (uint32_t c0 = 0; c0 < n; c0 += QCHN) {
        const uint32_t cn = min((uint32_t)QCHN, n - c0);
        // 1. my record: load, stage, derive its tile set-up and coverage
        uint32_t kind = 0;
        unsigned long long covMask = 0;
        if ((uint32_t)lane < cn) {
            uint32_t key;
            if (!regSort) key = __ldg(bin + c0 + lane);
            else key = Q.keys[c0 + (uint32_t)lane];
            const uint32_t item = key >> PF_SUB_BITS, sub = key & ((1u << PF_SUB_BITS) - 1);
            const PFPrim *src = &a.prims[item];
            uint32_t pi = item;
            if (sub != 0) { pi = (uint32_t)__ldg(&a.prims[item].poolBase) + sub - 1; src = &a.pool[pi]; }
            const int4 *s4 = reinterpret_cast<const int4 *>(src);
            int4 r[8];
            for (int i = 0; i < 8; i++) r[i] = __ldg(s4 + i);
            int4 *d4 = reinterpret_cast<int4 *>(&Q.rec[lane].p);
            for (int i = 0; i < 8; i++) d4[i] = r[i];
            Q.rec[lane].ph = a.anyPhong ? (sub != 0 ? &a.poolPh[pi] : &a.primsPh[item]) : nullptr;
            QEdge E;
            tile_edge(r[0], r[1], r[2], (uint32_t)r[4].w, __int_as_float(r[6].z), ox, oy, W, H, E);
            Q.edge[lane] = E;
            kind = (uint32_t)r[2].z & PFP_KIND;
            // my record's coverage of the tile, bit 8 y + x: the pixels of its
            // box that pass the integer edge test (triangles.c:398-424) or,
            // for a point, line or rectangle, its own rule
            const uint32_t bx0 = E.box & 15u, bw = (E.box >> 4) & 15u, by0 = (E.box >> 8) & 15u, bh = (E.box >> 12) & 15u;
            if (kind == 0) {
                for (uint32_t y = by0; y < by0 + bh; y++) {
                    uint32_t w1 = (uint32_t)E.e0[0] + bx0 * (uint32_t)E.ex0 + y * (uint32_t)E.ey0;
                    uint32_t w2 = (uint32_t)E.e0[1] + bx0 * (uint32_t)E.ex1 + y * (uint32_t)E.ey1;
                    uint32_t w3 = (uint32_t)E.e0[2] + bx0 * (uint32_t)E.ex2 + y * (uint32_t)E.ey2;
                    uint32_t row = 0;
                    for (uint32_t x = 0; x < bw; x++) {
                        row |= ((int32_t)(w1 | w2 | w3) > 0 ? 1u : 0u) << x;
                        w1 += (uint32_t)E.ex0; w2 += (uint32_t)E.ex1; w3 += (uint32_t)E.ex2;
                    }
                    covMask |= (unsigned long long)(row << bx0) << (8u * y);
                }
            } else {
                const PFPrim &P = Q.rec[lane].p;
                for (uint32_t y = by0; y < by0 + bh; y++)
                    for (uint32_t x = bx0; x < bx0 + bw; x++)
                        if (lp_covers(P, (int32_t)(ox + x), (int32_t)(oy + y))) covMask |= 1ull << (8u * y + x);
            }
        }
        const bool anyLP = __any_sync(0xffffffffu, kind != 0);
        __syncwarp();
        // 2a. coverage per pixel: bit k of cm0 / cm1 -- record k covers my
        //     pixel of slot 0 / 1 -- the records' masks transposed over the
        //     warp (rows 0-3 of the tile are bits 0-31: bit 8 y + x is lane
        //     8 y + x's pixel of slot 0; rows 4-7 its pixel of slot 1)
        const uint32_t cmLo = warp_transpose32((uint32_t)covMask);
        const uint32_t cmHi = warp_transpose32((uint32_t)(covMask >> 32));
        const uint32_t cm0 = (rowA == ly) ? cmLo : cmHi, cm1 = whole ? cmHi : 0u;
        // 2b. depth: each of my pixels walks its covering records in
        //     submission order -- depth (the correctly rounded reciprocal),
        //     the depth-test rejection bound, the depth test and write
        uint32_t vis0 = 0, vis1 = 0;                    // bit k: record k passed at my pixel of slot 0 / 1
        uint32_t cov = 0;
        auto depth_walk = [&](uint32_t cm, float &d, uint32_t &vis, uint32_t row, uint32_t Y) {
            for (; cm; cm &= cm - 1) {
                const uint32_t k = (uint32_t)(__ffs(cm) - 1);
                const int4 *e4 = reinterpret_cast<const int4 *>(&Q.edge[k]);
                const int4 q2 = e4[2];
                const uint32_t box = (uint32_t)q2.y, rs = (uint32_t)q2.z;
                const int func = (int)((rs >> 16) & 255u);
                float z;
                if (((box >> 16) & 3u) == 0) {
                    cov++;
                    if (__int_as_float(q2.w) >= d) continue;  // every fragment of it fails the depth test
                    const int4 q0 = e4[0], q1 = e4[1];
                    const uint32_t w1 = (uint32_t)q0.x + lx * (uint32_t)q0.w + row * (uint32_t)q1.z;
                    const uint32_t w2 = (uint32_t)q0.y + lx * (uint32_t)q1.x + row * (uint32_t)q1.w;
                    const uint32_t w3 = (uint32_t)q0.z + lx * (uint32_t)q1.y + row * (uint32_t)q2.x;
                    const float4 zq = reinterpret_cast<const float4 *>(&Q.rec[k].p)[3];     // wInvSum z1 z2 z3
                    const float wn1 = (float)(int32_t)w1 * zq.x, wn2 = (float)(int32_t)w2 * zq.x;
                    const float wn3 = (float)(int32_t)w3 * zq.x;
                    float zs = zq.y * wn1 + zq.z * wn2;
                    zs = zs + zq.w * wn3;
                    z = __frcp_rn(zs);
                    if ((rs & PFS_DEPTH_TEST) && !depth_simd(func, z, d)) continue;
                } else {
                    // a point, line or rectangle set up on the host: its own
                    // depth, the scalar depth test (rectangles are not fragments)
                    const PFPrim &P = Q.rec[k].p;
                    if (((box >> 16) & 3u) != (PFP_BLIT >> 6)) cov++;
                    z = lp_depth(P, (int32_t)X0, (int32_t)Y);
                    if ((rs & PFS_DEPTH_TEST) && !depth_sisd(func, z, d)) continue;
                }
                vis |= 1u << k;
                if (rs & PFS_DEPTH_MASK) d = z;
            }
        };
        depth_walk(cm0, dep0, vis0, rowA, Y0);
        depth_walk(cm1, dep1, vis1, ly + 4u, Y1);
        frags += cov;
        // 3+4. shade the fragments that passed, densely over the warp, and
        //      blend each pixel's in submission order
        uint32_t totalv;
        const uint32_t cntv = __popc(vis0) + __popc(vis1);
        const uint32_t offv = warp_offsets(cntv, totalv);
        for (uint32_t b0 = 0; b0 < totalv; b0 += QFW) {
            const uint32_t bEnd = min(totalv, b0 + QFW);
            tile_list(vis0 | ((unsigned long long)vis1 << 32), offv, b0, bEnd, Q.fdesc);
            __syncwarp();
            for (uint32_t f = b0 + (uint32_t)lane; f < bEnd; f += 32) {
                const uint32_t d = Q.fdesc[f - b0], p = d >> 5, k = d & 31u;
                const uint32_t X = p & 7u, Y = (p >> 3) + (rowA - ly);     // (a bottom half's slot 0 is row ly + 4)
                const PFPrim &P = Q.rec[k].p;
                if (anyLP && (P.flags & PFP_KIND)) {
                    Q.fc[f - b0] = lp_color(P, (int32_t)(ox + X), (int32_t)(oy + Y));
                    continue;
                }
                float wn[3];
                const float z = tile_depth(Q.edge[k], P, X, Y, wn);
                Q.fc[f - b0] = shade_fragment(P, Q.rec[k].ph, a.states, wn[0], wn[1], wn[2], z);
            }
            __syncwarp();
            if (cntv && offv < bEnd && offv + cntv > b0) {
                uint32_t f = offv;
                auto blend = [&](FbPixel<GEN> &c, uint32_t mm) {
                    for (; mm && f < bEnd; mm &= mm - 1, f++) {
                        if (f < b0) continue;
                        const uint32_t k = (uint32_t)(__ffs(mm) - 1);
                        const uint32_t rs = Q.edge[k].rstate;
                        const bool lpk = anyLP && (Q.rec[k].p.flags & PFP_KIND);
                        uint32_t frag = Q.fc[f - b0];
                        if (rs & PFS_BLEND)
                            frag = lpk ? blend_sisd((int)(rs >> 24), frag, c.get(true))
                                       : blend_simd((int)(rs >> 24), frag, c.get(false));
                        c.set(lpk, frag);
                    }
                };
                blend(col0, vis0);
                blend(col1, vis1);
            }
            __syncwarp();                                  // the window's lists are free
        }
        __syncwarp();                                      // the batch's records are free
    }
    if (in0) { col0.store(T, pidx0); T.depth[pidx0] = dep0; }
    if (in1) { col1.store(T, pidx1); T.depth[pidx1] = dep1; }
    }   // tile loop

    // fragment counter: one atomic per CTA (same-address atomics serialise)
    __shared__ unsigned long long sFrags;
    if (tid == 0) sFrags = 0;
    __syncthreads();
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o);
    if (lane == 0 && frags) atomicAdd(&sFrags, frags);
    __syncthreads();
    if (tid == 0 && sFrags) atomicAdd(&a.cnt->fragments, sFrags);
}

// ---------------------------------------------------------------------------
// k_rows: targets of BGRA / unsigned-byte format, band by band in
// submission order.
//
// The reference writes such a framebuffer through a SIMD getter and setter
// that shuffle each 4-pixel half of the 8-pixel vector with the bytes of
// the half's first pixel (pixel.h:2070-2078, 2916-2921; simd.h:564-583):
// every pixel of a half that a triangle's mask lets through takes the value
// computed at the half's first pixel -- that pixel's own colour (texture
// coordinates zero when it is outside the mask, triangles.c:508-513)
// blended with that pixel's destination.  The halves start at xMin + 4k of
// the triangle's box (x steps by 8 from xMin, triangles.c:409), so a half's
// first pixel may lie in the tile to the left, whose colour when the
// triangle is drawn depends on everything drawn there before it: the tiles
// of a row are not independent.  Rows are.  A warp owns one row of such a
// target for the whole launch and walks the launch's items in submission
// order -- four 8-byte summaries a lane at a time (row_info: the records an
// item has and the rows they span), so that items off the row cost a
// coalesced load -- drawing each record whose box meets the row: its
// 4-pixel halves are spread over the lanes, each lane drawing its half
// alone, and the warp moves to the next record when all are done.  Points,
// lines and rectangles use the scalar getter and setter (a plain R / B
// swap, pixel.h:356-363, 703-707), pixel by pixel.
// ---------------------------------------------------------------------------
#define ROW_WARPS 4

// One record over row y of a BGRA / unsigned-byte target of width W whose
// colour and depth the row pointers crow / drow hold (in global or shared
// memory), the part of lane `lane`; returns the covered pixels it counted.
__device__ __noinline__ uint32_t row_record(const PFPrim &P, const PFPrimPhong *ph, const PFDrawState *states,
                                            uint32_t *crow, float *drow, uint32_t W, uint32_t y, uint32_t lane)
{
    // the row and columns as tile_edge clips a box: y in [yMin, yMax], x in
    // [xMin, xMax), inside the framebuffer (unsigned)
    const uint32_t xMin = (uint32_t)P.xMin, xMax = (uint32_t)P.xMax, yMin = (uint32_t)P.yMin, yMax = (uint32_t)P.yMax;
    const uint32_t xEnd = min(xMax, W);
    if (xMin >= xEnd || y < yMin || y > yMax) return 0;
    const uint32_t nH = (xEnd - xMin + 3u) / 4u;
    const uint32_t kind = P.flags & PFP_KIND, rs = P.rstate;
    const int func = (int)((rs >> 16) & 255u), mode = (int)(rs >> 24);
    // edge functions at pixel (x, y): (x - rx) sx + (y - ry) sy, 32-bit
    // wrapping (triangles.c:336-349, 398-420)
    int32_t sx[3] = { P.y3 - P.y2, P.y1 - P.y3, P.y2 - P.y1 };
    int32_t sy[3] = { P.x2 - P.x3, P.x3 - P.x1, P.x1 - P.x2 };
    const int32_t rx[3] = { P.x2, P.x3, P.x1 }, ry[3] = { P.y2, P.y3, P.y1 };
    if (P.flags & 1u)
        for (int e = 0; e < 3; e++) { sx[e] = -sx[e]; sy[e] = -sy[e]; }
    uint32_t cov = 0;
    for (uint32_t t = lane; t < nH; t += 32) {
        const uint32_t xf = xMin + 4u * t;
        if (kind == 0) {
            bool m[4] = { false, false, false, false }, any = false;
            float zl[4] = { 0.0f, 0.0f, 0.0f, 0.0f }, wf[3] = { 0.0f, 0.0f, 0.0f }, zf = 0.0f;
            for (uint32_t j = 0; j < 4; j++) {
                const uint32_t x = xf + j;
                uint32_t w[3];
                for (int e = 0; e < 3; e++)
                    w[e] = (x - (uint32_t)rx[e]) * (uint32_t)sx[e] + (y - (uint32_t)ry[e]) * (uint32_t)sy[e];
                const float wn1 = (float)(int32_t)w[0] * P.wInvSum, wn2 = (float)(int32_t)w[1] * P.wInvSum;
                const float wn3 = (float)(int32_t)w[2] * P.wInvSum;
                float zs = P.z1 * wn1 + P.z2 * wn2;
                zs = zs + P.z3 * wn3;
                const float z = __frcp_rn(zs);
                if (j == 0) { wf[0] = wn1; wf[1] = wn2; wf[2] = wn3; zf = z; }
                if (x >= xEnd || (int32_t)(w[0] | w[1] | w[2]) <= 0) continue;
                cov++;
                if ((rs & PFS_DEPTH_TEST) && !depth_simd(func, z, drow[x])) continue;
                m[j] = true; zl[j] = z; any = true;
            }
            if (!any) continue;
            // the half's value: its first pixel's colour and destination
            uint32_t frag = shade_fragment(P, ph, states, wf[0], wf[1], wf[2], zf, m[0], true);
            if (rs & PFS_BLEND) frag = blend_simd(mode, frag, pff_swap_rb(crow[xf]));
            const uint32_t out = pff_swap_rb(frag);
            for (uint32_t j = 0; j < 4; j++) {
                if (!m[j]) continue;
                crow[xf + j] = out;
                if (rs & PFS_DEPTH_MASK) drow[xf + j] = zl[j];
            }
        } else {
            for (uint32_t j = 0; j < 4; j++) {
                const uint32_t x = xf + j;
                if (x >= xEnd || !lp_covers(P, (int32_t)x, (int32_t)y)) continue;
                if (kind != PFP_BLIT) cov++;
                const float z = lp_depth(P, (int32_t)x, (int32_t)y);
                if ((rs & PFS_DEPTH_TEST) && !depth_sisd(func, z, drow[x])) continue;
                uint32_t c = lp_color(P, (int32_t)x, (int32_t)y);
                if (rs & PFS_BLEND) c = blend_sisd(mode, c, pff_swap_rb(crow[x]));
                crow[x] = pff_swap_rb(c);
                if (rs & PFS_DEPTH_MASK) drow[x] = z;
            }
        }
    }
    return cov;
}

// SMEM: the warp keeps its row's colour and depth in shared memory while it
// draws (rows up to ROW_SMEM_MAX_W pixels), else it draws in place.
#define ROW_SMEM_MAX_W 2048
template <bool SMEM>
__global__ void __launch_bounds__(ROW_WARPS * 32) k_rows(RasterArgs a, const PFSegment *__restrict__ segs, int nSegs,
                                                         const uint64_t *__restrict__ rowInfo,
                                                         const uint64_t *__restrict__ rowGroup, uint32_t nRows)
{
    extern __shared__ __align__(16) unsigned char rowSmem[];
    __shared__ __align__(16) PFPrim sRec[ROW_WARPS];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    asm volatile("griddepcontrol.wait;" ::: "memory");   // k_raster is done
    if (a.cnt->abortCommand <= a.command) return;
    // my row: row y of the BGRA / unsigned-byte targets, in target order
    uint32_t y = blockIdx.x * ROW_WARPS + warp;
    if (y >= nRows) return;
    int t = 0;
    for (; t < a.nTargets; t++) {
        if (a.targets[t].fmt != PFF_BGRA8) continue;
        if (y < a.targets[t].H) break;
        y -= a.targets[t].H;
    }
    if (t >= a.nTargets) return;
    const PFTarget &T = a.targets[t];
    const uint32_t W = T.W;
    uint32_t *gcol = static_cast<uint32_t *>(T.color) + (size_t)y * W;
    float *gdep = T.depth + (size_t)y * W;
    uint32_t *crow = gcol;
    float *drow = gdep;
    if (SMEM) {
        crow = reinterpret_cast<uint32_t *>(rowSmem) + (size_t)warp * 2 * ROW_SMEM_MAX_W;
        drow = reinterpret_cast<float *>(crow + ROW_SMEM_MAX_W);
    }
    // the row as the draws find it: the fused clear (pfClear keeps pixels
    // 0..7), or the framebuffer's contents
    for (uint32_t x = lane; x < W; x += 32) {
        const bool clr = T.clearMode == 2 || (T.clearMode == 1 && (size_t)y * W + x >= 8);
        if (clr) { crow[x] = T.clearRaw[0]; drow[x] = T.clearDepth; }
        else if (SMEM) { crow[x] = gcol[x]; drow[x] = gdep[x]; }
    }
    __syncwarp();
    PFPrim &R = sRec[warp];
    unsigned long long frags = 0;
    for (int si = 0; si < nSegs; si++) {
        if (segs[si].target != t) continue;
        const uint32_t gBegin = segs[si].itemBase, gEnd = gBegin + segs[si].nItems;
        if (gBegin >= gEnd) continue;
        // groups of 32 items (one summary word each, 32 groups a step), then
        // the items of the groups that reach the row, in order
        const uint32_t cEnd = ((gEnd - 1) >> 5) + 1;
        for (uint32_t cb = gBegin >> 5; cb < cEnd; cb += 32) {
            const uint32_t c = cb + lane;
            const uint64_t sg = c < cEnd ? __ldg(rowGroup + c) : 0ull;
            const bool ghit = (sg & 1u) && ((sg >> 16) & 0xffffffu) <= y && (sg >> 40) >= y;
            for (uint32_t gneed = __ballot_sync(0xffffffffu, ghit); gneed; gneed &= gneed - 1) {
                const uint32_t gb = (cb + (uint32_t)(__ffs(gneed) - 1)) << 5;
                const uint32_t g = gb + lane;
                const uint64_t w = (g >= gBegin && g < gEnd) ? __ldg(rowInfo + g) : 0ull;
                const bool hit = (w & 0xffffu) && ((w >> 16) & 0xffffffu) <= y && (w >> 40) >= y;
                for (uint32_t need = __ballot_sync(0xffffffffu, hit); need; need &= need - 1) {
                    const int src = __ffs(need) - 1;
                    const uint32_t gi = gb + (uint32_t)src;
                    const uint32_t subs = (uint32_t)__shfl_sync(0xffffffffu, (uint32_t)w, src) & 0xffffu;
                    const int32_t pb = (subs & ~1u) ? __ldg(&a.prims[gi].poolBase) : 0;
                    for (uint32_t mm = subs; mm; mm &= mm - 1) {
                        const uint32_t sub = (uint32_t)(__ffs(mm) - 1);
                        const uint32_t pi = sub ? (uint32_t)pb + sub - 1 : gi;
                        const PFPrim *rec = sub ? &a.pool[pi] : &a.prims[gi];
                        if (lane < 8) reinterpret_cast<int4 *>(&R)[lane] = __ldg(reinterpret_cast<const int4 *>(rec) + lane);
                        __syncwarp();
                        const PFPrimPhong *ph = a.anyPhong ? (sub ? &a.poolPh[pi] : &a.primsPh[gi]) : nullptr;
                        frags += row_record(R, ph, a.states, crow, drow, W, y, lane);
                        __syncwarp();              // the record's pixels are written; R is free
                    }
                }
            }
        }
    }
    if (SMEM)
        for (uint32_t x = lane; x < W; x += 32) { gcol[x] = crow[x]; gdep[x] = drow[x]; }
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_down_sync(0xffffffffu, frags, o);
    if (lane == 0 && frags) atomicAdd(&a.cnt->fragments, frags);
}

// ---------------------------------------------------------------------------
// framebuffer-wide passes
// ---------------------------------------------------------------------------
// pfClear, SIMD build (context.c:680-745): pixels [8, n - n%8) take the clear
// value (as the SIMD setter stores it), the tail copies pixel 0's bytes,
// pixels 0..7 are left as they are.  For the packed 16-bit formats the
// reference steps the tail copy by components x 2 bytes (pixel.h:3156-3210),
// past the pixels: their tail keeps its colour (the depth tail is copied).
__global__ void k_clear(void *color, uint32_t fmt, float *depth, size_t n, uint4 cc, float cd,
                        const PFDevCounters *cnt, uint32_t command)
{
    if (cnt->abortCommand <= command) return;
    const size_t aligned = n - (n % 8);
    const uint32_t craw[4] = { cc.x, cc.y, cc.z, cc.w };
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        // the vector loop starts at pixel 8; the tail starts at `aligned`,
        // which is 0 below 8 pixels (then every pixel takes pixel 0's value)
        if (i < aligned ? i < 8 : i == 0) continue;
        if (fmt == PFF_RGBA8) {
            uint32_t *c32 = (uint32_t *)color;
            if (i < aligned) c32[i] = cc.x; else c32[i] = c32[0];
        } else if (i < aligned) pff_store(fmt, color, i, craw);
        else if (pff_bytes(fmt) != 2) { uint32_t r[4]; pff_load(fmt, color, 0, r); pff_store(fmt, color, i, r); }
        depth[i] = (i < aligned) ? cd : depth[0];
    }
}

// pfClearFramebuffer (framebuffer.c:89-102): every pixel, through the
// scalar setter.
__global__ void k_fill(void *color, uint32_t fmt, float *depth, size_t n, uint4 cc, float cd,
                       const PFDevCounters *cnt, uint32_t command)
{
    if (cnt->abortCommand <= command) return;
    const uint32_t craw[4] = { cc.x, cc.y, cc.z, cc.w };
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if (fmt == PFF_RGBA8) ((uint32_t *)color)[i] = cc.x;
        else pff_store(fmt, color, i, craw);
        depth[i] = cd;
    }
}

// Post-process hooks (pfPostProcess, context.c:2397-2441) and pfFogProcess
// (context.c:2288-2351), through the scalar getter and setter.  The hooks
// rewrite every pixel; the fog writes only the pixels past its start.
__global__ void k_hook(void *color, uint32_t fmt, const float *depth, size_t n, int hook, PFHookParams hp,
                       const PFDevCounters *cnt, uint32_t command)
{
    if (cnt->abortCommand <= command) return;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint32_t raw[4];
        pff_load(fmt, color, i, raw);
        uint32_t c = pff_get_sisd(fmt, raw);
        bool write = true;
        if (hook == 1) {          // linear fog on depth
            float d = (depth[i] + hp.znear) / (hp.zfar + hp.znear);
            float f = (hp.end - d) / (hp.end - hp.start);
            f = x86_min(x86_max(f, 0.0f), 1.0f);
            uint32_t k = (uint32_t)x86_cvt_trunc(f * 255.0f);
            uint32_t r = 0;
            for (int ch = 0; ch < 4; ch++) r |= (((chn(c, ch) * k + chn(hp.color, ch) * (255u - k)) / 255u) & 255u) << (8 * ch);
            c = r;
        } else if (hook == 3) {   // pfFogProcess (context.c:2288-2351)
            const float d = depth[i];
            write = d > hp.start;
            const uint32_t alpha = hp.color >> 24, fc = hp.color & 0x00ffffffu;
            if (d >= hp.end) {
                const uint32_t f = fc | (alpha << 24);
                c = alpha == 255u ? f : blend_sisd(1, f, c);
            } else if (d > hp.start) {
                float t = 0.0f;
                const float invLen = __frcp_rn(hp.end - hp.start);
                if (hp.mode == 0) t = (d - hp.start) * invLen;
                else if (hp.mode == 1) t = 1.0f - (float)exp((double)(-hp.density * (d - hp.start)));
                else if (hp.mode == 2) t = 1.0f - (float)exp2((double)(-hp.density * (d - hp.start)));
                const uint32_t a = (uint32_t)x86_cvt_trunc(t * (float)alpha) & 255u;
                c = blend_sisd(1, fc | (a << 24), c);
            }
        } else if (hook == 2) {   // grayscale
            uint32_t gy = (77u * chn(c, 0) + 150u * chn(c, 1) + 29u * chn(c, 2)) >> 8;
            c = gy | (gy << 8) | (gy << 16) | (c & 0xff000000u);
        } else if (hook == 4) {   // ordered 3x3 dither (examples/raylib/raylib_PostProcess.c:7-19)
            const uint32_t x = (uint32_t)(i % hp.width), y = (uint32_t)(i / hp.width);
            // the matrix {{230, 51, 128}, {25, 102, 179}, {154, 205, 77}}, row
            // x % 3, column y % 3: its first eight bytes packed low to high
            const uint32_t m = x % 3u * 3u + y % 3u;
            const uint32_t dv = m < 8u ? (uint32_t)((0xCD9AB366198033E6ull >> (8u * m)) & 255u) : 77u;
            const uint32_t avg = (chn(c, 0) + chn(c, 1) + chn(c, 2)) / 3u;
            c = (avg >= dv) ? 0xffffffffu : 0u;
        }
        if (write) {
            pff_set_sisd(fmt, c, raw);
            pff_store(fmt, color, i, raw);
        }
    }
}

// The largest of n u32 indices (already on the device, 16-byte aligned):
// per-warp maxima folded into *out with one atomic per warp.
__global__ void k_max_u32(const uint32_t *src, size_t n, unsigned *out)
{
    const size_t n4 = n / 4;
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    unsigned m = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += stride) {
        const uint4 v = __ldg(s4 + i);
        m = max(m, max(max(v.x, v.y), max(v.z, v.w)));
    }
    for (size_t i = n4 * 4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += stride) m = max(m, __ldg(src + i));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers (called by pf_host.cpp)
// ---------------------------------------------------------------------------
static inline unsigned grid_for(size_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

// The three pipeline kernels are launched with programmatic stream
// serialization: a kernel's CTAs may be scheduled as the previous kernel's
// last CTAs exit (no early trigger is issued, so every CTA of the previous
// grid has left its SM by then), and each kernel starts with
// griddepcontrol.wait, which returns once the previous grid has completed
// and its memory is visible.  What this hides is the launch gap between
// the kernels of a frame.
template <typename... KArgs, typename... Args>
static cudaError_t launch_serialized(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem,
                                     cudaStream_t st, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

int pfd_sm_count(void)
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            sms = 152;
        }
    }
    return sms;
}

// k_vertex starts a launch's chain: its predecessors in the stream are the
// uploads, the counter reset and the wait for the draw-time copies, so it
// is launched without programmatic serialization (its griddepcontrol.wait
// then returns at once).
cudaError_t pfd_launch_vertex(const PFBatchLaunch &L, cudaStream_t st)
{
    const uint32_t nTiles = L.totalTiles;
    const size_t work = L.nVerts > nTiles ? L.nVerts : nTiles;
    k_vertex<<<grid_for(work, 128), 128, 0, st>>>(L.segs, L.nSegs, L.states, L.vout, L.nVerts, L.cnt, L.binCount, nTiles);
    return cudaGetLastError();
}

cudaError_t pfd_launch_items(const PFBatchLaunch &L, cudaStream_t st)
{
    if (L.nItems == 0) return cudaSuccess;
    BinArgs B{ L.binCount, L.tileList, L.listStride, L.bins, L.cap, L.targets, L.cnt, L.command };
    ItemOut O{ L.prims, L.primsPh, L.pool, L.poolPh, L.poolCap, L.rowCount ? L.rowInfo : nullptr, L.rowGroup };
    return launch_serialized(k_items, grid_for(L.nItems, 128), 128, 0, st, L.segs, L.nSegs, L.states,
                             (const PFVertexOut *)L.vout, L.nItems, O, B);
}

// Dynamic shared memory of k_raster: the warps' batch buffers (a record's
// per-fragment lighting data is read through L1 when a fragment is shaded,
// not staged: the CTAs' shared memory would bound how many fit on an SM).
static size_t raster_smem(int warps)
{
    return (size_t)warps * sizeof(QWarp);
}

static RasterArgs raster_args(const PFBatchLaunch &L)
{
    return RasterArgs{ L.binCount, L.tileList, L.listStride, L.bins, L.cap, L.prims, L.primsPh, L.pool, L.poolPh, L.states,
                       L.targets, L.nTargets, L.totalTiles, L.cnt, L.command, L.anyPhong };
}

// Persistent grid of `kernel`: as many CTAs as fit on the GPU at once, at
// most `perSM` per SM (0: as many as fit), at most `units`.
static cudaError_t persistent_grid(const void *kernel, int block, size_t smem, int perSM, uint32_t units, uint32_t &grid)
{
    int fit = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kernel, block, smem);
    if (e != cudaSuccess) return e;
    uint32_t per = (uint32_t)(fit > 0 ? fit : 1);
    if (perSM > 0) per = min(per, (uint32_t)perSM);
    grid = max(1u, min(units, (uint32_t)pfd_sm_count() * per));
    return cudaSuccess;
}

cudaError_t pfd_launch_binsort(const PFBatchLaunch &L, cudaStream_t st)
{
    if (L.totalTiles == 0) return cudaSuccess;
    uint32_t N = 32; while (N < L.cap) N <<= 1;
    const size_t smem = 2 * (size_t)N * sizeof(uint32_t);             // merge source and target
    cudaError_t e = cudaFuncSetAttribute(k_binsort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    uint32_t grid = 0;
    if (e == cudaSuccess) e = persistent_grid((const void *)k_binsort, SORT_THREADS, smem, 0, L.totalTiles, grid);
    if (e != cudaSuccess) return e;
    return launch_serialized(k_binsort, grid, SORT_THREADS, smem, st, raster_args(L));
}

cudaError_t pfd_launch_raster(const PFBatchLaunch &L, cudaStream_t st)
{
    if (L.totalTiles == 0) return cudaSuccess;
    const int warps = (L.rasterWarps == 2 || L.rasterWarps == 8) ? L.rasterWarps : 4;
    const size_t smem = raster_smem(warps);
    void (*kernel)(RasterArgs) =
        L.generic ? (warps == 2 ? k_raster<true, 2> : warps == 8 ? k_raster<true, 8> : k_raster<true, 4>)
                  : (warps == 2 ? k_raster<false, 2> : warps == 8 ? k_raster<false, 8> : k_raster<false, 4>);
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)     // the CTAs' shared memory, not L1, bounds how many fit on an SM
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    uint32_t grid = 0;
    if (e == cudaSuccess) e = persistent_grid((const void *)kernel, warps * 32, smem, L.rasterCtasPerSM,
                                              (L.totalTiles + (uint32_t)warps - 1) / (uint32_t)warps, grid);
    if (e != cudaSuccess) return e;
    e = launch_serialized(kernel, grid, (unsigned)(warps * 32), smem, st, raster_args(L));
    if (e != cudaSuccess || L.rowCount == 0 || !L.rowInfo || !L.rowGroup) return e;
    const unsigned rowGrid = (L.rowCount + ROW_WARPS - 1) / ROW_WARPS;
    if (L.rowMaxW <= ROW_SMEM_MAX_W) {
        const size_t rsm = (size_t)ROW_WARPS * 2 * ROW_SMEM_MAX_W * 4;          // colour and depth rows
        e = cudaFuncSetAttribute(k_rows<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm);
        if (e != cudaSuccess) return e;
        return launch_serialized(k_rows<true>, rowGrid, ROW_WARPS * 32, rsm, st, raster_args(L), L.segs, L.nSegs,
                                 (const uint64_t *)L.rowInfo, (const uint64_t *)L.rowGroup, L.rowCount);
    }
    return launch_serialized(k_rows<false>, rowGrid, ROW_WARPS * 32, 0, st, raster_args(L), L.segs, L.nSegs,
                             (const uint64_t *)L.rowInfo, (const uint64_t *)L.rowGroup, L.rowCount);
}

cudaError_t pfd_launch_clear(void *color, uint32_t fmt, float *depth, size_t n, const uint32_t cc[4], float cd, bool all,
                             const PFDevCounters *cnt, uint32_t command, cudaStream_t st)
{
    unsigned grid = (unsigned)min((size_t)152 * 8, (n + 255) / 256);
    if (grid == 0) return cudaSuccess;
    const uint4 c4 = make_uint4(cc[0], cc[1], cc[2], cc[3]);
    if (all) k_fill<<<grid, 256, 0, st>>>(color, fmt, depth, n, c4, cd, cnt, command);
    else k_clear<<<grid, 256, 0, st>>>(color, fmt, depth, n, c4, cd, cnt, command);
    return cudaGetLastError();
}

cudaError_t pfd_launch_hook(void *color, uint32_t fmt, const float *depth, size_t n, int hook, const PFHookParams &hp,
                            const PFDevCounters *cnt, uint32_t command, cudaStream_t st)
{
    unsigned grid = (unsigned)min((size_t)152 * 8, (n + 255) / 256);
    if (grid == 0) return cudaSuccess;
    k_hook<<<grid, 256, 0, st>>>(color, fmt, depth, n, hook, hp, cnt, command);
    return cudaGetLastError();
}

cudaError_t pfd_max_u32(const uint32_t *d, size_t n, unsigned *dWord, unsigned *hWord, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(dWord, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    if (n) {
        const unsigned grid = (unsigned)min((size_t)pfd_sm_count() * 2, (n / 4 + 255) / 256 + 1);
        k_max_u32<<<grid, 256, 0, st>>>(d, n, dWord);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaMemcpyAsync(hWord, dWord, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
}


