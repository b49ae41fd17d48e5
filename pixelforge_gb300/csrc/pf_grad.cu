// pf_grad.cu -- differentiable float relaxation of the triangle pipeline
// (the pfgrad* entry points of include/pixelforge_grad.h).
//
// Scene set-up (once per mesh and set of views):
//   k_gsetup    one thread per (view, triangle, face) item, in the reference's
//               order (triangle-major, FRONT pass before BACK): projection,
//               2D/3D decision and the reference's integer set-up and cull --
//               the same device code as the pipeline's k_items -- and a count
//               of the 16x16 tiles each set-up triangle overlaps
//   k_gscan     exclusive scan of the tile counts (one CTA)
//   k_gfill     item numbers into the tile lists (atomic slots)
//   k_gsort     per tile: restores item order (bitonic sort in shared memory)
// Every evaluation:
//   k_glight          one thread per (view, vertex): Gouraud Blinn-Phong in float
//   k_gforward        one CTA per tile: coverage and depth test exactly as the
//                     reference, then float shading and alpha-over in item order
//   k_gadjoint        one CTA per tile: replays the tile to find, per pixel, its
//                     visible fragments and the colour under each, then walks
//                     them back to front, scattering texel gradients (vector
//                     atomics, pairs of adjacent lanes on one texel combined
//                     first) and vertex-colour gradients (shared-memory
//                     accumulation per tile)
//   k_glight_adjoint  one thread per (vertex, 8 views): back through the
//                     Gouraud Blinn-Phong formula; scalar gradients reduced per CTA
//   k_gfinish         light-direction normalisation adjoint
//
// The file is compiled with -fmad=false: coverage, depth and texel addressing
// use the same separately rounded arithmetic as the u8 pipeline.

#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>
#include <math.h>
#include <string.h>
#include <new>
#include "pf_layout.h"
#include "pixelforge_grad.h"

namespace {

#include "pf_common.cuh"

constexpr int GTILE = 16;
constexpr int GTHREADS = GTILE * GTILE;
constexpr int GCH = 32;            // triangles staged per chunk (adjoint)
constexpr int RING = 4;            // visible fragments walked back per pixel per replay
constexpr int NACC = 256;          // tile lists up to this length accumulate vertex gradients in shared memory
constexpr uint32_t GP_VALID = 1u << 31;

struct GPrim {                     // set-up triangle of one view
    int32_t x1, y1, x2, y2, x3, y3;
    int32_t xMin, yMin, xMax, yMax;  // pixels x in [xMin, xMax), y in [yMin, yMax] (unsigned compares)
    float wInvSum;
    uint32_t flags;                // bit0 face (1 = BACK), bit1 3D path, bit31 valid
    uint32_t v[3];                 // vertex indices
    float z[3];                    // depth terms: 1/z_clip on the 3D path, z on the 2D path
    float su[3], sv[3];            // texture coordinates, times 1/z_clip on the 3D path
};
static_assert(sizeof(GPrim) == 96, "GPrim is six 16-byte words");

struct GTex {
    const float4 *tex;
    uint32_t w, h;
    int32_t wrap, filter;
    float tx, ty;
};

struct GView {
    uint32_t W, H, tilesX, tilesPerView;
    uint32_t nv;
    float bg[3];
    float clearDepth;
};

// ---------------------------------------------------------------------------
// set-up and binning
// ---------------------------------------------------------------------------
struct SetupArgs {
    const float *pos, *uv;
    const uint32_t *idx;
    uint32_t nv, nt, nViews, nFaces;
    int32_t face0;
    const float *mvp;              // nViews x 16
    const PFDrawState *S;          // viewport of the views
    GView view;
    GPrim *prims;
    uint32_t *tileCount;
    uint32_t *status;              // [0] items needing clipping, [1] valid prims
};

__device__ __forceinline__ bool gtile_range(const GView &V, const GPrim &P, uint32_t &tx0, uint32_t &ty0,
                                            uint32_t &ntx, uint32_t &nty)
{
    uint32_t x0 = (uint32_t)P.xMin, x1 = (uint32_t)P.xMax, y0 = (uint32_t)P.yMin, y1 = (uint32_t)P.yMax;
    if (x1 > V.W) x1 = V.W;
    if (y1 >= V.H) y1 = V.H - 1;
    if (x0 >= x1 || y0 > y1) return false;
    tx0 = x0 / GTILE; ty0 = y0 / GTILE;
    ntx = (x1 - 1) / GTILE - tx0 + 1; nty = y1 / GTILE - ty0 + 1;
    return true;
}

__global__ void k_gsetup(SetupArgs a)
{
    const uint32_t perView = a.nt * a.nFaces;
    const uint64_t total = (uint64_t)perView * a.nViews;
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const uint32_t view = (uint32_t)(g / perView), r = (uint32_t)(g % perView);
    const uint32_t tri = r / a.nFaces;
    const int face = (a.nFaces == 2) ? (int)(r & 1u) : a.face0;
    GPrim &out = a.prims[g];
    out.flags = 0;
    const float *M = a.mvp + 16 * (size_t)view;
    uint32_t vi[3];
    float4 hv[3];
    for (int m = 0; m < 3; m++) {
        vi[m] = min(a.idx[3 * (size_t)tri + m], a.nv - 1);
        const float p[4] = { a.pos[3 * (size_t)vi[m]], a.pos[3 * (size_t)vi[m] + 1], a.pos[3 * (size_t)vi[m] + 2], 1.0f };
        float h[4];
        v4_transform(h, p, M);
        hv[m] = make_float4(h[0], h[1], h[2], h[3]);
    }
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
        if (!inside) { atomicAdd(&a.status[0], 1u); return; }
    }
    const PFDrawState &S = *a.S;
    SVert s[3];
    for (int m = 0; m < 3; m++) {
        const float4 h = hv[m];
        const float u = a.uv[2 * (size_t)vi[m]], v = a.uv[2 * (size_t)vi[m] + 1];
        if (is2D) {
            to_screen(S, h.x, h.y, s[m].sx, s[m].sy);
            s[m].z = h.z; s[m].u = u; s[m].v = v;
        } else {
            const float hz = 1.0f / h.z;
            s[m].u = u * hz; s[m].v = v * hz;
            const float invW = 1.0f / h.w;
            to_screen(S, h.x * invW, h.y * invW, s[m].sx, s[m].sy);
            s[m].z = hz;
        }
        s[m].c = 0;
    }
    PFPrim P;
    if (!setup_prim(S, face, !is2D, s[0], s[1], s[2], 0, P)) return;
    GPrim q;
    q.x1 = P.x1; q.y1 = P.y1; q.x2 = P.x2; q.y2 = P.y2; q.x3 = P.x3; q.y3 = P.y3;
    q.xMin = P.xMin; q.yMin = P.yMin; q.xMax = P.xMax; q.yMax = P.yMax;
    q.wInvSum = P.wInvSum;
    q.flags = (uint32_t)face | (is2D ? 0u : 2u);
    for (int m = 0; m < 3; m++) { q.v[m] = vi[m]; q.z[m] = s[m].z; q.su[m] = s[m].u; q.sv[m] = s[m].v; }
    uint32_t tx0, ty0, ntx, nty;
    if (!gtile_range(a.view, q, tx0, ty0, ntx, nty)) { out = q; return; }
    q.flags |= GP_VALID;
    out = q;
    atomicAdd(&a.status[1], 1u);
    const uint32_t base = view * a.view.tilesPerView;
    for (uint32_t ty = ty0; ty < ty0 + nty; ty++)
        for (uint32_t tx = tx0; tx < tx0 + ntx; tx++) atomicAdd(&a.tileCount[base + ty * a.view.tilesX + tx], 1u);
}

// Exclusive scan of n counts into off[0..n]; info[0] = longest list.
__global__ void __launch_bounds__(1024) k_gscan(const uint32_t *cnt, uint32_t *off, uint32_t n, uint32_t *info)
{
    __shared__ uint32_t warpSum[32];
    __shared__ uint32_t carry;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) carry = 0;
    uint32_t mx = 0;
    for (uint32_t b = 0; b < n; b += 1024) {
        __syncthreads();
        const uint32_t i = b + tid;
        const uint32_t v = i < n ? cnt[i] : 0u;
        mx = max(mx, v);
        uint32_t s = v;
        for (int o = 1; o < 32; o <<= 1) { uint32_t t = __shfl_up_sync(0xffffffffu, s, o); if (lane >= o) s += t; }
        if (lane == 31) warpSum[warp] = s;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = warpSum[lane];
            for (int o = 1; o < 32; o <<= 1) { uint32_t t = __shfl_up_sync(0xffffffffu, w, o); if (lane >= o) w += t; }
            warpSum[lane] = w;
        }
        __syncthreads();
        const uint32_t excl = carry + (warp ? warpSum[warp - 1] : 0u) + s - v;
        if (i < n) off[i] = excl;
        __syncthreads();
        if (tid == 1023) carry = excl + v;
    }
    __syncthreads();
    if (tid == 0) off[n] = carry;
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) atomicMax(&info[0], mx);
}

__global__ void k_gfill(const GPrim *prims, uint64_t total, GView V, uint32_t perView, const uint32_t *off,
                        uint32_t *fillCount, uint32_t *list)
{
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const GPrim &P = prims[g];
    if (!(P.flags & GP_VALID)) return;
    uint32_t tx0, ty0, ntx, nty;
    if (!gtile_range(V, P, tx0, ty0, ntx, nty)) return;
    const uint32_t base = (uint32_t)(g / perView) * V.tilesPerView;
    for (uint32_t ty = ty0; ty < ty0 + nty; ty++)
        for (uint32_t tx = tx0; tx < tx0 + ntx; tx++) {
            const uint32_t t = base + ty * V.tilesX + tx;
            list[off[t] + atomicAdd(&fillCount[t], 1u)] = (uint32_t)g;
        }
}

// Sorts each tile's list ascending (item order).  Lists are at most `cap`
// long (a power of two, checked by the host).
__global__ void k_gsort(const uint32_t *off, uint32_t *list, uint32_t cap)
{
    extern __shared__ uint32_t sk[];
    const uint32_t t = blockIdx.x;
    const uint32_t beg = off[t], n = off[t + 1] - beg;
    if (n < 2) return;
    uint32_t *L = list + beg;
    int unsorted = 0;
    for (uint32_t i = threadIdx.x; i + 1 < n; i += blockDim.x) unsorted |= (L[i] > L[i + 1]);
    if (!__syncthreads_or(unsorted)) return;
    uint32_t N = 1; while (N < n) N <<= 1;
    if (N > cap) return;
    for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) sk[i] = i < n ? L[i] : 0xffffffffu;
    __syncthreads();
    for (uint32_t k = 2; k <= N; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) {
                const uint32_t ixj = i ^ j;
                if (ixj > i) {
                    const uint32_t x = sk[i], y = sk[ixj];
                    const bool up = (i & k) == 0;
                    if ((x > y) == up) { sk[i] = y; sk[ixj] = x; }
                }
            }
            __syncthreads();
        }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) L[i] = sk[i];
}

// ---------------------------------------------------------------------------
// vertex lighting (float relaxation of lighting.c:24-134, one directional
// light, Blinn half vector)
// ---------------------------------------------------------------------------
struct LightArgs {
    const float *pos, *nrm, *col, *alpha;
    const float *material;         // diffuse, specular, shininess
    const float *light;            // direction towards the light
    const float *eye;              // nViews x 3
    uint32_t nv, nViews;
    float ambient;
};

struct VertexTerms {
    float N[3], L[3], H[3];
    float hlen;                    // |L + V|
    float nl, nh, spec;
};

__device__ __forceinline__ void vertex_terms(const LightArgs &a, uint32_t v, uint32_t view, const float *Ldir,
                                             VertexTerms &t)
{
    float N[3] = { a.nrm[3 * (size_t)v], a.nrm[3 * (size_t)v + 1], a.nrm[3 * (size_t)v + 2] };
    v3_normalize(N);
    const float *E = a.eye + 3 * (size_t)view;
    float V[3] = { E[0] - a.pos[3 * (size_t)v], E[1] - a.pos[3 * (size_t)v + 1], E[2] - a.pos[3 * (size_t)v + 2] };
    v3_normalize(V);
    float Hu[3] = { Ldir[0] + V[0], Ldir[1] + V[1], Ldir[2] + V[2] };
    const float hl = sqrtf(Hu[0] * Hu[0] + Hu[1] * Hu[1] + Hu[2] * Hu[2]);
    const float ih = hl > 0.0f ? 1.0f / hl : 0.0f;
    for (int i = 0; i < 3; i++) { t.N[i] = N[i]; t.L[i] = Ldir[i]; t.H[i] = Hu[i] * ih; }
    t.hlen = hl;
    t.nl = v3_dot(t.N, t.L);
    t.nh = v3_dot(t.N, t.H);
    const float shin = a.material[2];
    t.spec = t.nh > 0.0f ? powf(t.nh, shin) : 0.0f;
}

__device__ __forceinline__ void light_dir(const float *l, float *L, float &len)
{
    len = sqrtf(l[0] * l[0] + l[1] * l[1] + l[2] * l[2]);
    const float inv = len > 0.0f ? 1.0f / len : 0.0f;
    L[0] = l[0] * inv; L[1] = l[1] * inv; L[2] = l[2] * inv;
}

__global__ void k_glight(LightArgs a, float4 *lit)
{
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (uint64_t)a.nv * a.nViews) return;
    const uint32_t view = (uint32_t)(g / a.nv), v = (uint32_t)(g % a.nv);
    float L[3], llen;
    light_dir(a.light, L, llen);
    VertexTerms t;
    vertex_terms(a, v, view, L, t);
    const float kd = a.material[0], ks = a.material[1];
    const float diff = fmaxf(t.nl, 0.0f);
    float o[3];
    for (int c = 0; c < 3; c++) {
        const float D = a.col[3 * (size_t)v + c] * kd;
        o[c] = fminf(D * (a.ambient + diff) + ks * t.spec, 1.0f);
    }
    lit[g] = make_float4(o[0], o[1], o[2], a.alpha[v]);
}

// ---------------------------------------------------------------------------
// fragments
// ---------------------------------------------------------------------------
struct FragIn {                    // a covered pixel of a set-up triangle
    float wn[3];                   // screen-space weights
    float z;                       // interpolated depth
};

// Edge functions of pixel (px, py): the reference's row start and steps
// (triangles.c:331-349, 404-424), in 32-bit wrap-around arithmetic, so the
// values equal the reference's whatever the stepping order.
__device__ __forceinline__ bool cover(const GPrim &P, uint32_t px, uint32_t py, FragIn &f)
{
    if (!(px >= (uint32_t)P.xMin && px < (uint32_t)P.xMax && py >= (uint32_t)P.yMin && py <= (uint32_t)P.yMax))
        return false;
    int32_t w1X = P.y3 - P.y2, w1Y = P.x2 - P.x3, w2X = P.y1 - P.y3, w2Y = P.x3 - P.x1, w3X = P.y2 - P.y1,
            w3Y = P.x1 - P.x2;
    if (P.flags & 1u) { w1X = -w1X; w1Y = -w1Y; w2X = -w2X; w2Y = -w2Y; w3X = -w3X; w3Y = -w3Y; }
    const int32_t w1 = (int32_t)((px - (uint32_t)P.x2) * (uint32_t)w1X + (uint32_t)w1Y * (py - (uint32_t)P.y2));
    const int32_t w2 = (int32_t)((px - (uint32_t)P.x3) * (uint32_t)w2X + (uint32_t)w2Y * (py - (uint32_t)P.y3));
    const int32_t w3 = (int32_t)((px - (uint32_t)P.x1) * (uint32_t)w3X + (uint32_t)w3Y * (py - (uint32_t)P.y1));
    if (!((w1 | w2 | w3) > 0)) return false;
    f.wn[0] = (float)w1 * P.wInvSum; f.wn[1] = (float)w2 * P.wInvSum; f.wn[2] = (float)w3 * P.wInvSum;
    float zs = P.z[0] * f.wn[0] + P.z[1] * f.wn[1];
    zs = zs + P.z[2] * f.wn[2];
    f.z = 1.0f / zs;
    return true;
}

struct Taps {                      // texel offsets (-1: none) and weights of a texture sample
    int32_t off[4];
    float w[4];
};

__device__ __forceinline__ int32_t texel_off(const GTex &T, int32_t x, int32_t y)
{
    const int32_t off = (int32_t)((uint32_t)y * T.w + (uint32_t)x);
    return (off < 0 || (uint32_t)off >= T.w * T.h) ? -1 : off;
}

__device__ __forceinline__ float4 texel(const GTex &T, int32_t off)
{
    return off < 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : __ldg(T.tex + off);
}

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t)
{
    return make_float4(a.x + t * (b.x - a.x), a.y + t * (b.y - a.y), a.z + t * (b.z - a.z), a.w + t * (b.w - a.w));
}

// Texture sample with the reference's addressing (sampler.h:203-430):
// nearest, or bilinear from x0 = map(u), x1 = map(u + 1/w) and
// fx = clamp(u*w - x0, 0, 1).
__device__ __forceinline__ float4 sample(const GTex &T, float u, float v, Taps &tp)
{
    int32_t x0, y0;
    tex_map_wh(T.w, T.h, T.wrap, u, v, x0, y0);
    if (T.filter == 0) {
        tp.off[0] = texel_off(T, x0, y0); tp.w[0] = 1.0f;
        tp.off[1] = tp.off[2] = tp.off[3] = -1; tp.w[1] = tp.w[2] = tp.w[3] = 0.0f;
        return texel(T, tp.off[0]);
    }
    int32_t x1, y1;
    tex_map_wh(T.w, T.h, T.wrap, u + T.tx, v + T.ty, x1, y1);
    float fx = u * (float)T.w - (float)x0;
    float fy = v * (float)T.h - (float)y0;
    fx = x86_min(x86_max(fx, 0.0f), 1.0f);
    fy = x86_min(x86_max(fy, 0.0f), 1.0f);
    tp.off[0] = texel_off(T, x0, y0); tp.off[1] = texel_off(T, x1, y0);
    tp.off[2] = texel_off(T, x0, y1); tp.off[3] = texel_off(T, x1, y1);
    tp.w[0] = (1.0f - fx) * (1.0f - fy); tp.w[1] = fx * (1.0f - fy);
    tp.w[2] = (1.0f - fx) * fy;          tp.w[3] = fx * fy;
    const float4 r0 = lerp4(texel(T, tp.off[0]), texel(T, tp.off[1]), fx);
    const float4 r1 = lerp4(texel(T, tp.off[2]), texel(T, tp.off[3]), fx);
    return lerp4(r0, r1, fy);
}

struct Shade {
    float4 c;                      // interpolated lit colour (rgb) and alpha
    float4 t;                      // texel
    float src[3], a;               // fragment colour and opacity
    Taps tp;
};

__device__ __forceinline__ void shade(const GPrim &P, const FragIn &f, const float4 *lit, const GTex &T, Shade &s)
{
    const float4 l1 = lit[P.v[0]], l2 = lit[P.v[1]], l3 = lit[P.v[2]];
    s.c.x = (f.wn[0] * l1.x + f.wn[1] * l2.x) + f.wn[2] * l3.x;
    s.c.y = (f.wn[0] * l1.y + f.wn[1] * l2.y) + f.wn[2] * l3.y;
    s.c.z = (f.wn[0] * l1.z + f.wn[1] * l2.z) + f.wn[2] * l3.z;
    s.c.w = (f.wn[0] * l1.w + f.wn[1] * l2.w) + f.wn[2] * l3.w;
    float tu = P.su[0] * f.wn[0] + P.su[1] * f.wn[1];
    tu = tu + P.su[2] * f.wn[2];
    float tv = P.sv[0] * f.wn[0] + P.sv[1] * f.wn[1];
    tv = tv + P.sv[2] * f.wn[2];
    if (P.flags & 2u) { tu = tu * f.z; tv = tv * f.z; }
    s.t = sample(T, tu, tv, s.tp);
    s.src[0] = s.t.x * s.c.x; s.src[1] = s.t.y * s.c.y; s.src[2] = s.t.z * s.c.z;
    s.a = s.t.w * s.c.w;
}

struct RasterArgsG {
    const GPrim *prims;
    const uint32_t *off, *list;
    const float4 *lit;             // nViews x nv
    GTex T;
    GView V;
    float *image;                  // nViews x H x W x 3
    const float *dImage;
    float4 *dTex;
    float4 *dLit;                  // nViews x nv
};

__device__ __forceinline__ GPrim load_prim(const RasterArgsG &a, uint32_t i)
{
    GPrim P;
    const int4 *src = reinterpret_cast<const int4 *>(a.prims + __ldg(a.list + i));
    int4 *dst = reinterpret_cast<int4 *>(&P);
    for (int w = 0; w < 6; w++) dst[w] = __ldg(src + w);
    return P;
}

// A warp covers two pixel rows of its tile (y0, y0 + 1); triangles whose
// rows [yMin, yMax] miss both are skipped by the whole warp.
__device__ __forceinline__ bool misses_rows(const GPrim &P, uint32_t y0)
{
    return (uint32_t)P.yMin > y0 + 1 || (uint32_t)P.yMax < y0;
}

// Each warp walks the tile's list on its own (the list is read through L1,
// the same addresses for all lanes): no block-wide barriers.
__global__ void __launch_bounds__(GTHREADS) k_gforward(RasterArgsG a)
{
    const uint32_t gt = blockIdx.x;
    const uint32_t view = gt / a.V.tilesPerView, tile = gt % a.V.tilesPerView;
    const uint32_t px = (tile % a.V.tilesX) * GTILE + threadIdx.x % GTILE;
    const uint32_t py = (tile / a.V.tilesX) * GTILE + threadIdx.x / GTILE;
    const uint32_t y0 = py & ~1u;
    const bool inside = px < a.V.W && py < a.V.H;
    const float4 *lit = a.lit + (size_t)view * a.V.nv;
    float C[3] = { a.V.bg[0], a.V.bg[1], a.V.bg[2] };
    float D = a.V.clearDepth;
    const uint32_t beg = a.off[gt], n = a.off[gt + 1] - beg;
    for (uint32_t k = 0; k < n; k++) {
        const GPrim P = load_prim(a, beg + k);
        if (misses_rows(P, y0) || !inside) continue;
        FragIn f;
        if (!cover(P, px, py, f)) continue;
        if (!(f.z < D)) continue;                  // PF_LESS, depth written
        D = f.z;
        Shade s;
        shade(P, f, lit, a.T, s);
        for (int c = 0; c < 3; c++) C[c] = s.a * s.src[c] + (1.0f - s.a) * C[c];
    }
    if (inside) {
        float *o = a.image + (((size_t)view * a.V.H + py) * a.V.W + px) * 3;
        o[0] = C[0]; o[1] = C[1]; o[2] = C[2];
    }
}

__device__ __forceinline__ void add4(float4 *p, float4 v) { atomicAdd(p, v); }

__device__ __forceinline__ void stage_chunk(const RasterArgsG &a, uint32_t beg, uint32_t c0, uint32_t cn, GPrim *sp)
{
    for (uint32_t w = threadIdx.x; w < cn * 6; w += GTHREADS) {
        const uint32_t k = w / 6, part = w % 6;
        const uint32_t pi = __ldg(a.list + beg + c0 + k);
        reinterpret_cast<int4 *>(&sp[k])[part] = __ldg(reinterpret_cast<const int4 *>(a.prims + pi) + part);
    }
}

__global__ void __launch_bounds__(GTHREADS) k_gadjoint(RasterArgsG a)
{
    __shared__ GPrim sp[GCH];
    __shared__ uint32_t rpos[RING][GTHREADS];        // list position of the visible fragment
    __shared__ float rc[RING][3][GTHREADS];          // colour under it
    __shared__ float sacc[NACC][12];                 // per list position: d(lit) of its 3 vertices
    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t gt = blockIdx.x;
    const uint32_t view = gt / a.V.tilesPerView, tile = gt % a.V.tilesPerView;
    const uint32_t px = (tile % a.V.tilesX) * GTILE + tid % GTILE;
    const uint32_t py = (tile / a.V.tilesX) * GTILE + tid / GTILE;
    const bool inside = px < a.V.W && py < a.V.H;
    const float4 *lit = a.lit + (size_t)view * a.V.nv;
    float4 *dLit = a.dLit + (size_t)view * a.V.nv;
    const uint32_t beg = a.off[gt], n = a.off[gt + 1] - beg;
    if (n == 0) return;
    const bool useAcc = n <= (uint32_t)NACC;
    if (useAcc)
        for (uint32_t i = tid; i < n * 12; i += GTHREADS) (&sacc[0][0])[i] = 0.0f;

    float g[3] = { 0.f, 0.f, 0.f };
    if (inside) {
        const float *gi = a.dImage + (((size_t)view * a.V.H + py) * a.V.W + px) * 3;
        g[0] = gi[0]; g[1] = gi[1]; g[2] = gi[2];
    }
    uint32_t hi = 0xffffffffu;       // visible fragments at or above this index are done
    for (;;) {
        // replay: visible fragments below `hi`, the last RING of them recorded
        float C[3] = { a.V.bg[0], a.V.bg[1], a.V.bg[2] };
        float D = a.V.clearDepth;
        uint32_t j = 0;
        for (uint32_t c0 = 0; c0 < n; c0 += GCH) {
            const uint32_t cn = min((uint32_t)GCH, n - c0);
            __syncthreads();
            stage_chunk(a, beg, c0, cn, sp);
            __syncthreads();
            if (!inside || j >= hi) continue;
            for (uint32_t k = 0; k < cn && j < hi; k++) {
                FragIn f;
                if (!cover(sp[k], px, py, f)) continue;
                if (!(f.z < D)) continue;
                D = f.z;
                Shade s;
                shade(sp[k], f, lit, a.T, s);
                const uint32_t slot = j % RING;
                rpos[slot][tid] = c0 + k;
                rc[slot][0][tid] = C[0]; rc[slot][1][tid] = C[1]; rc[slot][2][tid] = C[2];
                for (int c = 0; c < 3; c++) C[c] = s.a * s.src[c] + (1.0f - s.a) * C[c];
                j++;
            }
        }
        if (hi == 0xffffffffu) hi = j;
        const uint32_t lo = hi > (uint32_t)RING ? hi - RING : 0u;
        // walk back over [lo, hi), warp-synchronously
        uint32_t steps = hi - lo;
        for (int o = 16; o > 0; o >>= 1) steps = max(steps, __shfl_xor_sync(0xffffffffu, steps, o));
        for (uint32_t st = 0; st < steps; st++) {
            const bool act = st < hi - lo;
            const uint32_t jj = hi - 1 - st;
            Shade s;
            FragIn f;
            uint32_t q = 0;
            GPrim P;
            float4 dt = make_float4(0.f, 0.f, 0.f, 0.f);
            float dc[4] = { 0.f, 0.f, 0.f, 0.f };
            if (act) {
                const uint32_t slot = jj % RING;
                q = rpos[slot][tid];
                P = a.prims[__ldg(a.list + beg + q)];
                cover(P, px, py, f);
                shade(P, f, lit, a.T, s);
                const float Cp[3] = { rc[slot][0][tid], rc[slot][1][tid], rc[slot][2][tid] };
                float ds[3], da = 0.0f;
                for (int c = 0; c < 3; c++) { ds[c] = g[c] * s.a; da += g[c] * (s.src[c] - Cp[c]); }
                for (int c = 0; c < 3; c++) g[c] = g[c] * (1.0f - s.a);
                dt = make_float4(ds[0] * s.c.x, ds[1] * s.c.y, ds[2] * s.c.z, da * s.c.w);
                dc[0] = ds[0] * s.t.x; dc[1] = ds[1] * s.t.y; dc[2] = ds[2] * s.t.z; dc[3] = da * s.t.w;
            }
            // texel gradients: lanes hitting the same texel add up first
            const int ntap = a.T.filter == 0 ? 1 : 4;
            for (int k = 0; k < ntap; k++) {
                const int32_t off = act ? s.tp.off[k] : -1;
                const float w = act ? s.tp.w[k] : 0.0f;
                const float4 v = make_float4(dt.x * w, dt.y * w, dt.z * w, dt.w * w);
                // horizontally adjacent pixels (lanes 2i, 2i+1) that read the
                // same texel send one atomic
                const int32_t po = __shfl_xor_sync(0xffffffffu, off, 1);
                const float4 pv = make_float4(__shfl_xor_sync(0xffffffffu, v.x, 1), __shfl_xor_sync(0xffffffffu, v.y, 1),
                                              __shfl_xor_sync(0xffffffffu, v.z, 1), __shfl_xor_sync(0xffffffffu, v.w, 1));
                if (off >= 0) {
                    if (po != off) add4(a.dTex + off, v);
                    else if ((lane & 1) == 0) add4(a.dTex + off, make_float4(v.x + pv.x, v.y + pv.y, v.z + pv.z, v.w + pv.w));
                }
            }
            if (act) {
                if (useAcc) {
                    // the 12 accumulators of list position q in an order
                    // rotated by lane, so that neighbouring lanes of the same
                    // triangle add to different words in each step
                    const uint32_t r = (uint32_t)lane % 12u;
                    for (uint32_t i = 0; i < 12; i++) {
                        uint32_t sl = i + r;
                        sl = sl >= 12u ? sl - 12u : sl;
                        const uint32_t m = sl >> 2, c = sl & 3u;
                        const float w = m == 0 ? f.wn[0] : (m == 1 ? f.wn[1] : f.wn[2]);
                        const float d = c == 0 ? dc[0] : (c == 1 ? dc[1] : (c == 2 ? dc[2] : dc[3]));
                        atomicAdd(&sacc[q][sl], d * w);
                    }
                } else {
                    for (int m = 0; m < 3; m++) {
                        const float w = f.wn[m];
                        add4(dLit + P.v[m], make_float4(dc[0] * w, dc[1] * w, dc[2] * w, dc[3] * w));
                    }
                }
            }
        }
        hi = lo;
        if (!__syncthreads_or(hi > 0)) break;
    }
    if (useAcc) {
        __syncthreads();
        for (uint32_t e = tid; e < n * 3; e += GTHREADS) {
            const uint32_t q = e / 3, m = e % 3;
            const float4 d = make_float4(sacc[q][4 * m], sacc[q][4 * m + 1], sacc[q][4 * m + 2], sacc[q][4 * m + 3]);
            if (d.x != 0.0f || d.y != 0.0f || d.z != 0.0f || d.w != 0.0f) {
                const uint32_t pi = __ldg(a.list + beg + q);
                add4(dLit + a.prims[pi].v[m], d);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// vertex adjoint
// ---------------------------------------------------------------------------
// One thread per (vertex, group of GVIEWS views).  Per-vertex gradients are
// added into dCol/dAlpha (zeroed first); acc: [0] d diffuse, [1] d specular,
// [2] d shininess, [3..5] d L (unit light direction), reduced per CTA.
constexpr uint32_t GVIEWS = 8;

__global__ void __launch_bounds__(256) k_glight_adjoint(LightArgs a, const float4 *dLit, float *dCol, float *dAlpha,
                                                         float *acc)
{
    const uint32_t groups = (a.nViews + GVIEWS - 1) / GVIEWS;
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = g < (uint64_t)a.nv * groups;
    const uint32_t v = valid ? (uint32_t)(g % a.nv) : 0u;
    const uint32_t v0 = valid ? (uint32_t)(g / a.nv) * GVIEWS : a.nViews;
    float L[3], llen;
    light_dir(a.light, L, llen);
    const float kd = a.material[0], ks = a.material[1], shin = a.material[2];
    float part[6] = { 0.f, 0.f, 0.f, 0.f, 0.f, 0.f };
    if (valid) {
        const float C[3] = { a.col[3 * (size_t)v], a.col[3 * (size_t)v + 1], a.col[3 * (size_t)v + 2] };
        float dC[3] = { 0.f, 0.f, 0.f }, dA = 0.0f;
        const uint32_t vEnd = min(v0 + GVIEWS, a.nViews);
        for (uint32_t view = v0; view < vEnd; view++) {
            const float4 g4 = dLit[(size_t)view * a.nv + v];
            dA += g4.w;
            if (g4.x == 0.0f && g4.y == 0.0f && g4.z == 0.0f) continue;
            VertexTerms t;
            vertex_terms(a, v, view, L, t);
            const float diff = fmaxf(t.nl, 0.0f);
            const float gin[3] = { g4.x, g4.y, g4.z };
            float gdiff = 0.0f, gspec = 0.0f;
            for (int c = 0; c < 3; c++) {
                const float D = C[c] * kd;
                const float pre = D * (a.ambient + diff) + ks * t.spec;
                const float gc = pre < 1.0f ? gin[c] : 0.0f;
                dC[c] += gc * kd * (a.ambient + diff);
                part[0] += gc * C[c] * (a.ambient + diff);
                gdiff += gc * D;
                part[1] += gc * t.spec;
                gspec += gc * ks;
            }
            if (t.nl > 0.0f)
                for (int i = 0; i < 3; i++) part[3 + i] += gdiff * t.N[i];
            if (t.nh > 0.0f && t.spec > 0.0f) {
                part[2] += gspec * t.spec * logf(t.nh);
                const float gx = gspec * shin * powf(t.nh, shin - 1.0f);
                // H = (L + V) / |L + V|: dH = (I - H H^T) dHu / |L + V|
                float gH[3] = { gx * t.N[0], gx * t.N[1], gx * t.N[2] };
                const float hg = v3_dot(t.H, gH);
                for (int i = 0; i < 3; i++) part[3 + i] += (gH[i] - t.H[i] * hg) / t.hlen;
            }
        }
        if (groups == 1) {
            for (int c = 0; c < 3; c++) dCol[3 * (size_t)v + c] = dC[c];
            dAlpha[v] = dA;
        } else {
            for (int c = 0; c < 3; c++) if (dC[c] != 0.0f) atomicAdd(&dCol[3 * (size_t)v + c], dC[c]);
            if (dA != 0.0f) atomicAdd(&dAlpha[v], dA);
        }
    }
    __shared__ float red[8][6];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = 0; i < 6; i++) {
        float x = part[i];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[warp][i] = x;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        float x = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) x += red[w][threadIdx.x];
        if (x != 0.0f) atomicAdd(&acc[threadIdx.x], x);
    }
}

// d light = (I - L L^T) dL / |light|
__global__ void k_gfinish(const float *light, const float *acc, float *dMaterial, float *dLight)
{
    float L[3], len;
    light_dir(light, L, len);
    dMaterial[0] = acc[0]; dMaterial[1] = acc[1]; dMaterial[2] = acc[2];
    const float gl[3] = { acc[3], acc[4], acc[5] };
    const float d = v3_dot(L, gl);
    for (int i = 0; i < 3; i++) dLight[i] = len > 0.0f ? (gl[i] - L[i] * d) / len : 0.0f;
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct PFgradScene_ {
    PFgradSceneDesc desc{};
    uint32_t nFaces = 1;
    int32_t face0 = 0;
    GView V{};
    uint64_t nItems = 0;
    uint32_t nTiles = 0;
    PFgradInfo info{};
    // device
    PFDrawState *state = nullptr;
    float *mvp = nullptr, *eye = nullptr;
    GPrim *prims = nullptr;
    uint32_t *off = nullptr, *list = nullptr, *work = nullptr;   // work: tile counts, then status words
    float4 *lit = nullptr, *dLit = nullptr;
    float *acc = nullptr;
};

namespace {

void scene_free(PFgradScene_ *s)
{
    cudaFree(s->state); cudaFree(s->mvp); cudaFree(s->eye); cudaFree(s->prims); cudaFree(s->off);
    cudaFree(s->list); cudaFree(s->work); cudaFree(s->lit); cudaFree(s->dLit); cudaFree(s->acc);
}

inline unsigned blocks(uint64_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

LightArgs light_args(const PFgradScene_ *s, const PFgradParams *p)
{
    LightArgs a;
    a.pos = s->desc.positions; a.nrm = s->desc.normals; a.col = p->colors; a.alpha = p->alphas;
    a.material = p->material; a.light = p->light; a.eye = s->eye;
    a.nv = s->desc.nVertices; a.nViews = s->desc.nViews; a.ambient = s->desc.ambient;
    return a;
}

RasterArgsG raster_args(const PFgradScene_ *s, const PFgradParams *p)
{
    RasterArgsG a;
    a.prims = s->prims; a.off = s->off; a.list = s->list; a.lit = s->lit;
    a.T.tex = reinterpret_cast<const float4 *>(p->texture);
    a.T.w = s->desc.texWidth; a.T.h = s->desc.texHeight;
    a.T.wrap = s->desc.texWrap; a.T.filter = s->desc.texFilter;
    a.T.tx = 1.0f / (float)s->desc.texWidth; a.T.ty = 1.0f / (float)s->desc.texHeight;
    a.V = s->V;
    a.image = nullptr; a.dImage = nullptr; a.dTex = nullptr; a.dLit = nullptr;
    return a;
}

bool params_ok(const PFgradParams *p)
{
    return p && p->texture && p->colors && p->alphas && p->material && p->light;
}

}  // namespace

#define PFG_CHECK(x) do { if ((x) != cudaSuccess) { cudaGetLastError(); goto fail; } } while (0)

extern "C" int pfgradSceneCreate(PFgradScene *out, const PFgradSceneDesc *d, void *stream)
{
    if (!out || !d) return PFGRAD_ERR_INVALID;
    *out = nullptr;
    if (!d->positions || !d->normals || !d->texcoords || !d->indices || !d->mvp || !d->eye) return PFGRAD_ERR_INVALID;
    if (d->nVertices == 0 || d->nViews == 0 || d->width == 0 || d->height == 0 || d->width > 16384 ||
        d->height > 16384 || d->texWidth == 0 || d->texHeight == 0 || d->texFilter < 0 || d->texFilter > 1 ||
        d->texWrap < 0 || d->texWrap > 2 || d->cullFace < -1 || d->cullFace > 1)
        return PFGRAD_ERR_INVALID;
    cudaStream_t st = (cudaStream_t)stream;
    PFgradScene_ *s = new (std::nothrow) PFgradScene_();
    if (!s) return PFGRAD_ERR_CUDA;
    s->desc = *d;
    s->nFaces = d->cullFace < 0 ? 2u : 1u;
    s->face0 = d->cullFace < 0 ? 0 : (d->cullFace == 1 ? 0 : 1);   // culling BACK draws FRONT and the reverse
    const uint32_t tilesX = (d->width + GTILE - 1) / GTILE, tilesY = (d->height + GTILE - 1) / GTILE;
    s->V = GView{ d->width, d->height, tilesX, tilesX * tilesY, d->nVertices,
                  { d->background[0], d->background[1], d->background[2] }, d->clearDepth };
    s->nItems = (uint64_t)d->nTriangles * s->nFaces * d->nViews;
    const uint64_t nTiles64 = (uint64_t)tilesX * tilesY * d->nViews;
    if (nTiles64 >= 0x7fffffffu || s->nItems >= 0xffffffffu) { delete s; return PFGRAD_ERR_INVALID; }
    s->nTiles = (uint32_t)nTiles64;
    int rc = PFGRAD_ERR_CUDA;
    uint32_t host[3] = { 0, 0, 0 };
    {
        PFDrawState S;
        memset(&S, 0, sizeof(S));
        S.vpPos[0] = 0; S.vpPos[1] = 0;
        S.vpDim[0] = (int32_t)d->width - 1; S.vpDim[1] = (int32_t)d->height - 1;
        S.vpMin[0] = 0; S.vpMin[1] = 0;
        S.vpMax[0] = (int32_t)d->width - 1; S.vpMax[1] = (int32_t)d->height - 1;
        const size_t nv = d->nVertices, nV = d->nViews;
        PFG_CHECK(cudaMalloc(&s->state, sizeof(PFDrawState)));
        PFG_CHECK(cudaMalloc(&s->mvp, nV * 16 * sizeof(float)));
        PFG_CHECK(cudaMalloc(&s->eye, nV * 3 * sizeof(float)));
        PFG_CHECK(cudaMalloc(&s->prims, (s->nItems ? s->nItems : 1) * sizeof(GPrim)));
        PFG_CHECK(cudaMalloc(&s->off, ((size_t)s->nTiles + 1) * sizeof(uint32_t)));
        PFG_CHECK(cudaMalloc(&s->work, ((size_t)s->nTiles + 4) * sizeof(uint32_t)));
        PFG_CHECK(cudaMalloc(&s->lit, nv * nV * sizeof(float4)));
        PFG_CHECK(cudaMalloc(&s->dLit, nv * nV * sizeof(float4)));
        PFG_CHECK(cudaMalloc(&s->acc, 8 * sizeof(float)));
        PFG_CHECK(cudaMemcpyAsync(s->state, &S, sizeof(S), cudaMemcpyHostToDevice, st));
        PFG_CHECK(cudaMemcpyAsync(s->mvp, d->mvp, nV * 16 * sizeof(float), cudaMemcpyHostToDevice, st));
        PFG_CHECK(cudaMemcpyAsync(s->eye, d->eye, nV * 3 * sizeof(float), cudaMemcpyHostToDevice, st));
        uint32_t *cnt = s->work, *status = s->work + s->nTiles;     // status: clipped items, valid prims, longest list
        PFG_CHECK(cudaMemsetAsync(s->work, 0, ((size_t)s->nTiles + 4) * sizeof(uint32_t), st));
        if (s->nItems) {
            SetupArgs a{ d->positions, d->texcoords, d->indices, d->nVertices, d->nTriangles, d->nViews, s->nFaces,
                         s->face0, s->mvp, s->state, s->V, s->prims, cnt, status };
            k_gsetup<<<blocks(s->nItems, 128), 128, 0, st>>>(a);
            PFG_CHECK(cudaGetLastError());
        }
        k_gscan<<<1, 1024, 0, st>>>(cnt, s->off, s->nTiles, status + 2);
        PFG_CHECK(cudaGetLastError());
        PFG_CHECK(cudaMemcpyAsync(host, status, 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        uint32_t total = 0;
        PFG_CHECK(cudaMemcpyAsync(&total, s->off + s->nTiles, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        PFG_CHECK(cudaStreamSynchronize(st));
        if (host[0]) { rc = PFGRAD_ERR_CLIP; goto fail; }
        if (host[2] > PFGRAD_MAX_TILE_PRIMS) { rc = PFGRAD_ERR_CAPACITY; goto fail; }
        PFG_CHECK(cudaMalloc(&s->list, (total ? total : 1) * sizeof(uint32_t)));
        if (total) {
            PFG_CHECK(cudaMemsetAsync(cnt, 0, (size_t)s->nTiles * sizeof(uint32_t), st));
            k_gfill<<<blocks(s->nItems, 256), 256, 0, st>>>(s->prims, s->nItems, s->V,
                                                            d->nTriangles * s->nFaces, s->off, cnt, s->list);
            PFG_CHECK(cudaGetLastError());
            uint32_t cap = 2; while (cap < host[2]) cap <<= 1;
            const size_t smem = (size_t)cap * sizeof(uint32_t);
            PFG_CHECK(cudaFuncSetAttribute(k_gsort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k_gsort<<<s->nTiles, 256, smem, st>>>(s->off, s->list, cap);
            PFG_CHECK(cudaGetLastError());
        }
        PFG_CHECK(cudaStreamSynchronize(st));
        s->info.primitives = host[1];
        s->info.tileEntries = total;
        s->info.maxTilePrims = host[2];
        s->info.tiles = s->nTiles;
    }
    *out = s;
    return 0;
fail:
    scene_free(s);
    delete s;
    return rc;
}

extern "C" int pfgradSceneDestroy(PFgradScene s)
{
    if (!s) return PFGRAD_ERR_INVALID;
    scene_free(s);
    delete s;
    return 0;
}

extern "C" int pfgradSceneInfo(PFgradScene s, PFgradInfo *info)
{
    if (!s || !info) return PFGRAD_ERR_INVALID;
    *info = s->info;
    return 0;
}

extern "C" int pfgradForward(PFgradScene s, const PFgradParams *p, float *image, void *stream)
{
    if (!s || !params_ok(p) || !image) return PFGRAD_ERR_INVALID;
    cudaStream_t st = (cudaStream_t)stream;
    const LightArgs la = light_args(s, p);
    k_glight<<<blocks((uint64_t)s->desc.nVertices * s->desc.nViews, 256), 256, 0, st>>>(la, s->lit);
    RasterArgsG ra = raster_args(s, p);
    ra.image = image;
    k_gforward<<<s->nTiles, GTHREADS, 0, st>>>(ra);
    if (cudaGetLastError() != cudaSuccess) return PFGRAD_ERR_CUDA;
    return 0;
}

extern "C" int pfgradBackward(PFgradScene s, const PFgradParams *p, const float *dImage, const PFgradGrads *g,
                              void *stream)
{
    if (!s || !params_ok(p) || !dImage || !g || !g->texture || !g->colors || !g->alphas || !g->material || !g->light)
        return PFGRAD_ERR_INVALID;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t nv = s->desc.nVertices, nV = s->desc.nViews;
    if (cudaMemsetAsync(g->texture, 0, (size_t)s->desc.texWidth * s->desc.texHeight * sizeof(float4), st) != cudaSuccess ||
        cudaMemsetAsync(s->dLit, 0, nv * nV * sizeof(float4), st) != cudaSuccess ||
        cudaMemsetAsync(s->acc, 0, 8 * sizeof(float), st) != cudaSuccess ||
        cudaMemsetAsync(g->colors, 0, nv * 3 * sizeof(float), st) != cudaSuccess ||
        cudaMemsetAsync(g->alphas, 0, nv * sizeof(float), st) != cudaSuccess) {
        cudaGetLastError();
        return PFGRAD_ERR_CUDA;
    }
    const LightArgs la = light_args(s, p);
    k_glight<<<blocks((uint64_t)nv * nV, 256), 256, 0, st>>>(la, s->lit);
    RasterArgsG ra = raster_args(s, p);
    ra.dImage = dImage;
    ra.dTex = reinterpret_cast<float4 *>(g->texture);
    ra.dLit = s->dLit;
    k_gadjoint<<<s->nTiles, GTHREADS, 0, st>>>(ra);
    const uint64_t groups = (nV + GVIEWS - 1) / GVIEWS;
    k_glight_adjoint<<<blocks(nv * groups, 256), 256, 0, st>>>(la, s->dLit, g->colors, g->alphas, s->acc);
    k_gfinish<<<1, 1, 0, st>>>(p->light, s->acc, g->material, g->light);
    if (cudaGetLastError() != cudaSuccess) return PFGRAD_ERR_CUDA;
    return 0;
}
