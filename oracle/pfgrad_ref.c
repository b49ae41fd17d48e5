/*
 * pfgrad_ref.c -- CPU ORACLE of the differentiable rendering path
 * (include/pixelforge_grad.h): FP64 forward, FP64 adjoint and the loss
 * restricted to the pixels that depend on one parameter (for central finite
 * differences).
 *
 * TEST INFRASTRUCTURE ONLY.  tests/ load it (the gradient and visibility checks);
 * the product never does.
 *
 * Visibility is computed once, in single precision with the reference's
 * operation order (the Makefile builds this file with -ffp-contract=off):
 *   projection      pfmVec4Transform (src/pfm.h:1996-2006)
 *   2D/3D decision  |w1 + w2 + w3 - 3| < 1e-5 (src/internal/primitives/triangles.c:246-280)
 *   screen map      pfiHomogeneousToScreen (src/internal/context/context.c:52-65),
 *                   z <- 1/z_clip and uv <- uv/z_clip on the 3D path (triangles.c:262-275)
 *   set-up, cull    triangles.c:287-349 (integer edge functions, face by the
 *                   sign of the integer area)
 *   coverage        (w1 | w2 | w3) > 0, x in [xMin, xMax), y in [yMin, yMax] (triangles.c:398-424)
 *   weights, depth  wN = (float)w * wInvSum; z = 1 / ((z1 wN1 + z2 wN2) + z3 wN3) (triangles.c:426-438),
 *                   the exact reciprocal where the reference uses rcp_ps
 *   depth test      PF_LESS with the depth written (src/internal/depth.h:80-124)
 *   texel address   sampler.h:203-430 (nearest, or bilinear x0 = map(u), x1 = map(u + 1/w),
 *                   fx = clamp(u w - x0, 0, 1)); offsets outside the texture read 0
 * and each pixel's list of visible fragments (those passing the depth test,
 * in submission order) is kept with its weights, texel offsets and lerp
 * factors.  The shading of those fragments is then a function of the
 * parameters evaluated in double precision:
 *   lit   = min(C kd (ambient + max(N.L, 0)) + ks max(N.H, 0)^shininess, 1)   (lighting.c:24-134)
 *   c     = (wN1 lit1 + wN2 lit2) + wN3 lit3,  alpha likewise
 *   t     = texel or lerp(lerp(t00, t10, fx), lerp(t01, t11, fx), fy)
 *   src   = t.rgb c,  a = t.a alpha,  dst = a src + (1 - a) dst               (blend.h:140-213)
 * Parameter vector layout (double): texture (texH x texW x 4) | colours
 * (nv x 3) | alphas (nv) | diffuse, specular, shininess | light (3).
 * Loss = scale * sum over pixels and RGB of (image - target)^2.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "pfref_internal.h"

#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    uint32_t v[3];
    float wn[3];
    int32_t off[4];              /* texel offsets, -1 when outside the texture */
    float fx, fy;
    float z;                     /* depth written by the fragment */
} GFrag;

typedef struct {
    int nv, nt, nViews, W, H, cull, texW, texH, filter, wrap;
    float ambient, clearDepth;
    double bg[3];
    float *pos, *nrm;            /* copies, nv x 3 */
    float *eye;                  /* nViews x 3 */
    int64_t *pixStart;           /* nViews*H*W + 1 */
    GFrag *frags;
    int64_t nFrags;
} GScene;

typedef struct { int32_t x1, y1, x2, y2, x3, y3, xMin, yMin, xMax, yMax; float wInvSum; float z[3], su[3], sv[3];
                 int face, is3D; uint32_t v[3]; } SPrim;

static void v4_transform(float *d, const float *v, const float *m)
{
    float t[4] = {
        m[0]*v[0] + m[4]*v[1] + m[8]*v[2] + m[12]*v[3],
        m[1]*v[0] + m[5]*v[1] + m[9]*v[2] + m[13]*v[3],
        m[2]*v[0] + m[6]*v[1] + m[10]*v[2] + m[14]*v[3],
        m[3]*v[0] + m[7]*v[1] + m[11]*v[2] + m[15]*v[3] };
    memcpy(d, t, 16);
}

static void tex_map(int w, int h, int wrap, float u, float v, int32_t *x, int32_t *y)
{
    if (wrap == 0) {
        u = (u - truncf(u)) * (float)(w - 1);
        v = (v - truncf(v)) * (float)(h - 1);
        *x = ox_iabs(ox_cvt_rne(u));
        *y = ox_iabs(ox_cvt_rne(v));
    } else if (wrap == 1) {
        u = fabsf(u); v = fabsf(v);
        u = u - floorf(u / 2.0f) * 2.0f;
        v = v - floorf(v / 2.0f) * 2.0f;
        float um = 1.0f - (u - 1.0f), vm = 1.0f - (v - 1.0f);
        u = (u > 1.0f) ? um : u;
        v = (v > 1.0f) ? vm : v;
        *x = ox_cvt_rne(u * (float)(w - 1) + 0.5f);
        *y = ox_cvt_rne(v * (float)(h - 1) + 0.5f);
    } else {
        *x = ox_cvt_rne(ox_min(ox_max(u, 0.0f), 1.0f) * (float)(w - 1) + 0.5f);
        *y = ox_cvt_rne(ox_min(ox_max(v, 0.0f), 1.0f) * (float)(h - 1) + 0.5f);
    }
}

static int32_t texel_off(const GScene *s, int32_t x, int32_t y)
{
    int64_t off = (int64_t)(int32_t)((uint32_t)y * (uint32_t)s->texW + (uint32_t)x);
    return (off < 0 || off >= (int64_t)s->texW * s->texH) ? -1 : (int32_t)off;
}

/* Set-up of one (triangle, face) item of one view; 0 when culled, clipped
 * away or needing clipping (*clip set). */
static int setup(const GScene *s, const float *pos, const float *uv, const uint32_t *idx, const float *M,
                 int tri, int face, SPrim *P, int *clip)
{
    float h[3][4];
    for (int m = 0; m < 3; m++) {
        uint32_t vi = idx[3 * tri + m];
        if (vi >= (uint32_t)s->nv) vi = (uint32_t)s->nv - 1;
        P->v[m] = vi;
        const float p[4] = { pos[3 * vi], pos[3 * vi + 1], pos[3 * vi + 2], 1.0f };
        v4_transform(h[m], p, M);
    }
    float ws = 0.0f;
    for (int m = 0; m < 3; m++) ws += h[m][3];
    const int is2D = fabsf(ws - 3.0f) < 1e-5f;
    if (!is2D) {
        for (int m = 0; m < 3; m++) {
            const float *q = h[m];
            if (q[3] < 1e-5f || !(q[0] <= q[3]) || !(-q[0] <= q[3]) || !(q[1] <= q[3]) || !(-q[1] <= q[3]) ||
                !(q[2] <= q[3]) || !(-q[2] <= q[3])) { *clip = 1; return 0; }
        }
    }
    float sx[3], sy[3];
    const float dimX = (float)(s->W - 1), dimY = (float)(s->H - 1);
    for (int m = 0; m < 3; m++) {
        float hx = h[m][0], hy = h[m][1];
        const float u = uv[2 * P->v[m]], v = uv[2 * P->v[m] + 1];
        if (is2D) {
            P->z[m] = h[m][2]; P->su[m] = u; P->sv[m] = v;
        } else {
            const float hz = 1.0f / h[m][2];
            P->su[m] = u * hz; P->sv[m] = v * hz;
            const float invW = 1.0f / h[m][3];
            hx = hx * invW; hy = hy * invW;
            P->z[m] = hz;
        }
        sx[m] = (0.0f + (hx + 1.0f) * 0.5f * dimX) + 0.5f;
        sy[m] = (0.0f + (1.0f - hy) * 0.5f * dimY) + 0.5f;
    }
    const int32_t x1 = ox_cvt_trunc(sx[0]), y1 = ox_cvt_trunc(sy[0]);
    const int32_t x2 = ox_cvt_trunc(sx[1]), y2 = ox_cvt_trunc(sy[1]);
    const int32_t x3 = ox_cvt_trunc(sx[2]), y3 = ox_cvt_trunc(sy[2]);
    const float area = (float)(int32_t)((uint32_t)(x2 - x1) * (uint32_t)(y3 - y1) - (uint32_t)(x3 - x1) * (uint32_t)(y2 - y1));
    if ((face == 0 && area >= 0.0f) || (face == 1 && area <= 0.0f)) return 0;
    int32_t mnx = x1 < x2 ? x1 : x2; mnx = mnx < x3 ? mnx : x3;
    int32_t mny = y1 < y2 ? y1 : y2; mny = mny < y3 ? mny : y3;
    int32_t mxx = x1 > x2 ? x1 : x2; mxx = mxx > x3 ? mxx : x3;
    int32_t mxy = y1 > y2 ? y1 : y2; mxy = mxy > y3 ? mxy : y3;
    if (is2D) {
#define CL(v, lo, hi) ((v) < (lo) ? (lo) : ((v) > (hi) ? (hi) : (v)))
        mnx = CL(mnx, 0, s->W - 1); mny = CL(mny, 0, s->H - 1);
        mxx = CL(mxx, 0, s->W - 1); mxy = CL(mxy, 0, s->H - 1);
#undef CL
    }
    int32_t w1X = y3 - y2, w1Y = x2 - x3, w2X = y1 - y3, w2Y = x3 - x1, w3X = y2 - y1, w3Y = x1 - x2;
    if (face == 1) { w1X = -w1X; w1Y = -w1Y; w2X = -w2X; w2Y = -w2Y; w3X = -w3X; w3Y = -w3Y; }
    const uint32_t xMin = (uint32_t)mnx, yMin = (uint32_t)mny;
    const uint32_t r1 = (xMin - (uint32_t)x2) * (uint32_t)w1X + (uint32_t)w1Y * (yMin - (uint32_t)y2);
    const uint32_t r2 = (xMin - (uint32_t)x3) * (uint32_t)w2X + (uint32_t)w2Y * (yMin - (uint32_t)y3);
    const uint32_t r3 = (xMin - (uint32_t)x1) * (uint32_t)w3X + (uint32_t)w3Y * (yMin - (uint32_t)y1);
    P->x1 = x1; P->y1 = y1; P->x2 = x2; P->y2 = y2; P->x3 = x3; P->y3 = y3;
    P->xMin = mnx; P->yMin = mny; P->xMax = mxx; P->yMax = mxy;
    P->wInvSum = 1.0f / (float)(int32_t)(r1 + r2 + r3);
    P->face = face; P->is3D = !is2D;
    return 1;
}

/* Coverage, weights and depth of pixel (px, py). */
static int cover(const SPrim *P, uint32_t px, uint32_t py, float wn[3], float *z)
{
    if (!(px >= (uint32_t)P->xMin && px < (uint32_t)P->xMax && py >= (uint32_t)P->yMin && py <= (uint32_t)P->yMax))
        return 0;
    int32_t w1X = P->y3 - P->y2, w1Y = P->x2 - P->x3, w2X = P->y1 - P->y3, w2Y = P->x3 - P->x1,
            w3X = P->y2 - P->y1, w3Y = P->x1 - P->x2;
    if (P->face) { w1X = -w1X; w1Y = -w1Y; w2X = -w2X; w2Y = -w2Y; w3X = -w3X; w3Y = -w3Y; }
    const int32_t w1 = (int32_t)((px - (uint32_t)P->x2) * (uint32_t)w1X + (uint32_t)w1Y * (py - (uint32_t)P->y2));
    const int32_t w2 = (int32_t)((px - (uint32_t)P->x3) * (uint32_t)w2X + (uint32_t)w2Y * (py - (uint32_t)P->y3));
    const int32_t w3 = (int32_t)((px - (uint32_t)P->x1) * (uint32_t)w3X + (uint32_t)w3Y * (py - (uint32_t)P->y1));
    if ((w1 | w2 | w3) <= 0) return 0;
    wn[0] = (float)w1 * P->wInvSum; wn[1] = (float)w2 * P->wInvSum; wn[2] = (float)w3 * P->wInvSum;
    float zs = P->z[0] * wn[0] + P->z[1] * wn[1];
    zs = zs + P->z[2] * wn[2];
    *z = 1.0f / zs;
    return 1;
}

static void fill_taps(const GScene *s, const SPrim *P, const float wn[3], float z, GFrag *f)
{
    float tu = P->su[0] * wn[0] + P->su[1] * wn[1];
    tu = tu + P->su[2] * wn[2];
    float tv = P->sv[0] * wn[0] + P->sv[1] * wn[1];
    tv = tv + P->sv[2] * wn[2];
    if (P->is3D) { tu = tu * z; tv = tv * z; }
    int32_t x0, y0;
    tex_map(s->texW, s->texH, s->wrap, tu, tv, &x0, &y0);
    f->off[0] = texel_off(s, x0, y0);
    if (s->filter == 0) { f->off[1] = f->off[2] = f->off[3] = -1; f->fx = f->fy = 0.0f; return; }
    int32_t x1, y1;
    tex_map(s->texW, s->texH, s->wrap, tu + 1.0f / (float)s->texW, tv + 1.0f / (float)s->texH, &x1, &y1);
    float fx = tu * (float)s->texW - (float)x0;
    float fy = tv * (float)s->texH - (float)y0;
    f->fx = ox_min(ox_max(fx, 0.0f), 1.0f);
    f->fy = ox_min(ox_max(fy, 0.0f), 1.0f);
    f->off[1] = texel_off(s, x1, y0);
    f->off[2] = texel_off(s, x0, y1);
    f->off[3] = texel_off(s, x1, y1);
}

void pgref_destroy(void *h)
{
    GScene *s = (GScene *)h;
    if (!s) return;
    free(s->pos); free(s->nrm); free(s->eye); free(s->pixStart); free(s->frags);
    free(s);
}

/* Returns NULL on a bad argument, when a triangle needs clipping (*status = 5)
 * or when memory runs out (*status = 3). */
void *pgref_create(const float *pos, const float *nrm, const float *uv, const uint32_t *idx, int nv, int nt,
                   const float *mvp, const float *eye, int nViews, int W, int H, int cull, int texW, int texH,
                   int filter, int wrap, float ambient, const float *bg, float clearDepth, int *status)
{
    *status = 2;
    if (nv <= 0 || nt < 0 || nViews <= 0 || W <= 0 || H <= 0 || texW <= 0 || texH <= 0) return NULL;
    GScene *s = (GScene *)calloc(1, sizeof(GScene));
    if (!s) { *status = 3; return NULL; }
    s->nv = nv; s->nt = nt; s->nViews = nViews; s->W = W; s->H = H; s->cull = cull;
    s->texW = texW; s->texH = texH; s->filter = filter; s->wrap = wrap;
    s->ambient = ambient; s->clearDepth = clearDepth;
    for (int i = 0; i < 3; i++) s->bg[i] = bg[i];
    s->pos = (float *)malloc(sizeof(float) * 3 * nv);
    s->nrm = (float *)malloc(sizeof(float) * 3 * nv);
    s->eye = (float *)malloc(sizeof(float) * 3 * nViews);
    const int64_t npix = (int64_t)nViews * W * H;
    s->pixStart = (int64_t *)calloc((size_t)npix + 1, sizeof(int64_t));
    if (!s->pos || !s->nrm || !s->eye || !s->pixStart) { pgref_destroy(s); *status = 3; return NULL; }
    memcpy(s->pos, pos, sizeof(float) * 3 * nv);
    memcpy(s->nrm, nrm, sizeof(float) * 3 * nv);
    memcpy(s->eye, eye, sizeof(float) * 3 * nViews);
    const int nFaces = cull < 0 ? 2 : 1;
    const int face0 = cull == 1 ? 0 : 1;
    /* pass 1: set-up per view, visible-fragment count per pixel; pass 2: lists */
    SPrim *prims = (SPrim *)malloc(sizeof(SPrim) * ((size_t)nt * nFaces + 1) * (size_t)nViews);
    int *valid = (int *)malloc(sizeof(int) * ((size_t)nt * nFaces + 1) * (size_t)nViews);
    if (!prims || !valid) { free(prims); free(valid); pgref_destroy(s); *status = 3; return NULL; }
    int clip = 0;
    const size_t per = (size_t)nt * nFaces;
#pragma omp parallel for reduction(|:clip) schedule(dynamic, 1)
    for (int vw = 0; vw < nViews; vw++)
        for (size_t it = 0; it < per; it++) {
            const int tri = (int)(it / nFaces), face = nFaces == 2 ? (int)(it & 1) : face0;
            int c = 0;
            valid[vw * per + it] = setup(s, pos, uv, idx, mvp + 16 * vw, tri, face, &prims[vw * per + it], &c);
            clip |= c;
        }
    if (clip) { free(prims); free(valid); pgref_destroy(s); *status = 5; return NULL; }
    for (int pass = 0; pass < 2; pass++) {
#pragma omp parallel for schedule(dynamic, 1)
        for (int vw = 0; vw < nViews; vw++) {
            float *depth = (float *)malloc(sizeof(float) * (size_t)W * H);
            int64_t *cur = (int64_t *)malloc(sizeof(int64_t) * (size_t)W * H);
            for (int64_t i = 0; i < (int64_t)W * H; i++) depth[i] = clearDepth;
            int64_t *start = s->pixStart + (int64_t)vw * W * H;
            if (pass == 1) for (int64_t i = 0; i < (int64_t)W * H; i++) cur[i] = start[i];
            else for (int64_t i = 0; i < (int64_t)W * H; i++) cur[i] = 0;
            for (size_t it = 0; it < per; it++) {
                if (!valid[vw * per + it]) continue;
                const SPrim *P = &prims[vw * per + it];
                uint32_t x0 = (uint32_t)P->xMin, x1 = (uint32_t)P->xMax, y0 = (uint32_t)P->yMin, y1 = (uint32_t)P->yMax;
                if (x1 > (uint32_t)W) x1 = (uint32_t)W;
                if (y1 >= (uint32_t)H) y1 = (uint32_t)H - 1;
                if (x0 >= x1 || y0 > y1) continue;
                for (uint32_t y = y0; y <= y1; y++)
                    for (uint32_t x = x0; x < x1; x++) {
                        float wn[3], z;
                        if (!cover(P, x, y, wn, &z)) continue;
                        const int64_t p = (int64_t)y * W + x;
                        if (!(z < depth[p])) continue;
                        depth[p] = z;
                        if (pass == 0) { cur[p]++; continue; }
                        GFrag *f = &s->frags[cur[p]++];
                        for (int m = 0; m < 3; m++) { f->v[m] = P->v[m]; f->wn[m] = wn[m]; }
                        f->z = z;
                        fill_taps(s, P, wn, z, f);
                    }
            }
            if (pass == 0) for (int64_t i = 0; i < (int64_t)W * H; i++) start[i] = cur[i];   /* counts for now */
            free(depth); free(cur);
        }
        if (pass == 0) {
            int64_t acc = 0;
            for (int64_t i = 0; i < npix; i++) { int64_t c = s->pixStart[i]; s->pixStart[i] = acc; acc += c; }
            s->pixStart[npix] = acc;
            s->nFrags = acc;
            s->frags = (GFrag *)malloc(sizeof(GFrag) * (size_t)(acc ? acc : 1));
            if (!s->frags) { free(prims); free(valid); pgref_destroy(s); *status = 3; return NULL; }
        }
    }
    free(prims); free(valid);
    *status = 0;
    return s;
}

int64_t pgref_fragments(void *h) { return ((GScene *)h)->nFrags; }

/* visible-fragment count of each pixel (nViews*H*W int32) */
void pgref_fragment_counts(void *h, int32_t *out)
{
    GScene *s = (GScene *)h;
    const int64_t npix = (int64_t)s->nViews * s->W * s->H;
    for (int64_t i = 0; i < npix; i++) out[i] = (int32_t)(s->pixStart[i + 1] - s->pixStart[i]);
}

/* final depth buffer of each view (nViews*H*W floats): the depth of the last
 * visible fragment, or the clear value */
void pgref_depth(void *h, float *out)
{
    GScene *s = (GScene *)h;
    const int64_t npix = (int64_t)s->nViews * s->W * s->H;
    for (int64_t i = 0; i < npix; i++)
        out[i] = s->pixStart[i + 1] > s->pixStart[i] ? s->frags[s->pixStart[i + 1] - 1].z : s->clearDepth;
}

/* ------------------------------------------------------------------------ */
/* FP64 shading                                                              */
/* ------------------------------------------------------------------------ */
typedef struct { const double *tex, *col, *alpha, *mat, *light; } Par;

static Par par_of(const GScene *s, const double *p)
{
    Par r;
    r.tex = p;
    r.col = r.tex + (size_t)s->texW * s->texH * 4;
    r.alpha = r.col + 3 * (size_t)s->nv;
    r.mat = r.alpha + s->nv;
    r.light = r.mat + 3;
    return r;
}

typedef struct { double N[3], L[3], H[3], hlen, nl, nh, spec, llen; } VT;

static void vterms(const GScene *s, const Par *P, int vw, int v, VT *t)
{
    double N[3] = { s->nrm[3 * v], s->nrm[3 * v + 1], s->nrm[3 * v + 2] };
    double nn = sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
    if (nn > 0) for (int i = 0; i < 3; i++) N[i] /= nn;
    double V[3];
    for (int i = 0; i < 3; i++) V[i] = (double)s->eye[3 * vw + i] - (double)s->pos[3 * v + i];
    double vn = sqrt(V[0] * V[0] + V[1] * V[1] + V[2] * V[2]);
    if (vn > 0) for (int i = 0; i < 3; i++) V[i] /= vn;
    t->llen = sqrt(P->light[0] * P->light[0] + P->light[1] * P->light[1] + P->light[2] * P->light[2]);
    for (int i = 0; i < 3; i++) t->L[i] = t->llen > 0 ? P->light[i] / t->llen : 0.0;
    double Hu[3];
    for (int i = 0; i < 3; i++) Hu[i] = t->L[i] + V[i];
    t->hlen = sqrt(Hu[0] * Hu[0] + Hu[1] * Hu[1] + Hu[2] * Hu[2]);
    for (int i = 0; i < 3; i++) { t->N[i] = N[i]; t->H[i] = t->hlen > 0 ? Hu[i] / t->hlen : 0.0; }
    t->nl = N[0] * t->L[0] + N[1] * t->L[1] + N[2] * t->L[2];
    t->nh = N[0] * t->H[0] + N[1] * t->H[1] + N[2] * t->H[2];
    t->spec = t->nh > 0 ? pow(t->nh, P->mat[2]) : 0.0;
}

static void lit_of(const GScene *s, const Par *P, int vw, int v, double o[4])
{
    VT t;
    vterms(s, P, vw, v, &t);
    const double diff = t.nl > 0 ? t.nl : 0.0;
    for (int c = 0; c < 3; c++) {
        const double x = P->col[3 * v + c] * P->mat[0] * (s->ambient + diff) + P->mat[1] * t.spec;
        o[c] = x < 1.0 ? x : 1.0;
    }
    o[3] = P->alpha[v];
}

static void texel4(const GScene *s, const Par *P, int32_t off, double t[4])
{
    for (int c = 0; c < 4; c++) t[c] = off < 0 ? 0.0 : P->tex[4 * (size_t)off + c];
}

/* fragment colour: src (rgb), a; intermediates for the adjoint */
typedef struct { double c[4], t[4], src[3], a; double tw[4]; } FS;

static void frag_shade(const GScene *s, const Par *P, const double *lit, const GFrag *f, FS *o)
{
    for (int k = 0; k < 4; k++) {
        const double *l1 = lit + 4 * (size_t)f->v[0], *l2 = lit + 4 * (size_t)f->v[1], *l3 = lit + 4 * (size_t)f->v[2];
        o->c[k] = (f->wn[0] * l1[k] + f->wn[1] * l2[k]) + f->wn[2] * l3[k];
    }
    if (s->filter == 0) {
        texel4(s, P, f->off[0], o->t);
        o->tw[0] = 1.0; o->tw[1] = o->tw[2] = o->tw[3] = 0.0;
    } else {
        double t00[4], t10[4], t01[4], t11[4];
        texel4(s, P, f->off[0], t00); texel4(s, P, f->off[1], t10);
        texel4(s, P, f->off[2], t01); texel4(s, P, f->off[3], t11);
        const double fx = f->fx, fy = f->fy;
        for (int k = 0; k < 4; k++) {
            const double r0 = t00[k] + fx * (t10[k] - t00[k]);
            const double r1 = t01[k] + fx * (t11[k] - t01[k]);
            o->t[k] = r0 + fy * (r1 - r0);
        }
        o->tw[0] = (1 - fx) * (1 - fy); o->tw[1] = fx * (1 - fy); o->tw[2] = (1 - fx) * fy; o->tw[3] = fx * fy;
    }
    for (int k = 0; k < 3; k++) o->src[k] = o->t[k] * o->c[k];
    o->a = o->t[3] * o->c[3];
}

static double *lit_all(const GScene *s, const Par *P)
{
    double *lit = (double *)malloc(sizeof(double) * 4 * (size_t)s->nv * s->nViews);
    if (!lit) return NULL;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)s->nv * s->nViews; i++)
        lit_of(s, P, (int)(i / s->nv), (int)(i % s->nv), lit + 4 * i);
    return lit;
}

/* Pixel value and loss term. */
static double pixel(const GScene *s, const Par *P, const double *litAll, int64_t p, const float *target, double *img)
{
    const int vw = (int)(p / ((int64_t)s->W * s->H));
    const double *lit = litAll + 4 * (size_t)s->nv * vw;
    double C[3] = { s->bg[0], s->bg[1], s->bg[2] };
    for (int64_t k = s->pixStart[p]; k < s->pixStart[p + 1]; k++) {
        FS o;
        frag_shade(s, P, lit, &s->frags[k], &o);
        for (int c = 0; c < 3; c++) C[c] = o.a * o.src[c] + (1.0 - o.a) * C[c];
    }
    double l = 0.0;
    for (int c = 0; c < 3; c++) {
        if (img) img[3 * p + c] = C[c];
        const double d = C[c] - (target ? (double)target[3 * p + c] : 0.0);
        l += d * d;
    }
    return l;
}

/* Loss = scale * sum (image - target)^2; image (nViews*H*W*3) optional. */
double pgref_forward(void *h, const double *params, const float *target, double scale, double *image)
{
    GScene *s = (GScene *)h;
    Par P = par_of(s, params);
    double *lit = lit_all(s, &P);
    if (!lit) return NAN;
    const int64_t npix = (int64_t)s->nViews * s->W * s->H;
    double L = 0.0;
#pragma omp parallel for reduction(+:L) schedule(static, 4096)
    for (int64_t p = 0; p < npix; p++) L += pixel(s, &P, lit, p, target, image);
    free(lit);
    return L * scale;
}

static int pixel_depends(const GScene *s, int64_t p, int64_t q)
{
    const int64_t nTex = (int64_t)s->texW * s->texH * 4;
    for (int64_t k = s->pixStart[p]; k < s->pixStart[p + 1]; k++) {
        const GFrag *f = &s->frags[k];
        if (q < nTex) {
            const int32_t off = (int32_t)(q / 4);
            for (int t = 0; t < 4; t++) if (f->off[t] == off) return 1;
        } else {
            const int64_t r = q - nTex;
            const int v = r < 3 * (int64_t)s->nv ? (int)(r / 3) : (int)(r - 3 * (int64_t)s->nv);
            if (f->v[0] == (uint32_t)v || f->v[1] == (uint32_t)v || f->v[2] == (uint32_t)v) return 1;
        }
    }
    return 0;
}

/* Loss over the pixels whose value can depend on parameter q (all pixels for
 * the material and light parameters); differences of it equal differences of
 * the full loss, without the rounding noise of the untouched pixels. */
double pgref_loss_local(void *h, const double *params, const float *target, double scale, int64_t q)
{
    GScene *s = (GScene *)h;
    const int64_t nLocal = (int64_t)s->texW * s->texH * 4 + 4 * (int64_t)s->nv;
    if (q >= nLocal) return pgref_forward(h, params, target, scale, NULL);
    Par P = par_of(s, params);
    double *lit = lit_all(s, &P);
    if (!lit) return NAN;
    const int64_t npix = (int64_t)s->nViews * s->W * s->H;
    double L = 0.0;
#pragma omp parallel for reduction(+:L) schedule(static, 4096)
    for (int64_t p = 0; p < npix; p++)
        if (pixel_depends(s, p, q)) L += pixel(s, &P, lit, p, target, NULL);
    free(lit);
    return L * scale;
}

/* Gradient of the loss (scale * sum (image - target)^2) into grad (same
 * layout as params). */
int pgref_backward(void *h, const double *params, const float *target, double scale, double *grad)
{
    GScene *s = (GScene *)h;
    Par P = par_of(s, params);
    const int64_t nParams = (int64_t)s->texW * s->texH * 4 + 4 * (int64_t)s->nv + 6;
    memset(grad, 0, sizeof(double) * (size_t)nParams);
    double *lit = lit_all(s, &P);
    double *dlit = (double *)calloc(4 * (size_t)s->nv * s->nViews, sizeof(double));
    if (!lit || !dlit) { free(lit); free(dlit); return -3; }
    double *gtex = grad;
    const int64_t npix = (int64_t)s->nViews * s->W * s->H;
    /* pixels, serially (scatter), fragments walked back to front */
    for (int64_t p = 0; p < npix; p++) {
        const int64_t b = s->pixStart[p], e = s->pixStart[p + 1];
        if (b == e) continue;
        const int vw = (int)(p / ((int64_t)s->W * s->H));
        const double *litv = lit + 4 * (size_t)s->nv * vw;
        double *dlv = dlit + 4 * (size_t)s->nv * vw;
        double under[64][3];
        FS fs[64];
        const int64_t n = e - b;
        double C[3] = { s->bg[0], s->bg[1], s->bg[2] };
        double *U = n <= 64 ? &under[0][0] : (double *)malloc(sizeof(double) * 3 * (size_t)n);
        FS *F = n <= 64 ? fs : (FS *)malloc(sizeof(FS) * (size_t)n);
        for (int64_t k = 0; k < n; k++) {
            frag_shade(s, &P, litv, &s->frags[b + k], &F[k]);
            for (int c = 0; c < 3; c++) { U[3 * k + c] = C[c]; C[c] = F[k].a * F[k].src[c] + (1.0 - F[k].a) * C[c]; }
        }
        double g[3];
        for (int c = 0; c < 3; c++) g[c] = 2.0 * scale * (C[c] - (double)target[3 * p + c]);
        for (int64_t k = n - 1; k >= 0; k--) {
            const FS *o = &F[k];
            const GFrag *f = &s->frags[b + k];
            double ds[3], da = 0.0;
            for (int c = 0; c < 3; c++) { ds[c] = g[c] * o->a; da += g[c] * (o->src[c] - U[3 * k + c]); }
            for (int c = 0; c < 3; c++) g[c] *= (1.0 - o->a);
            const double dt[4] = { ds[0] * o->c[0], ds[1] * o->c[1], ds[2] * o->c[2], da * o->c[3] };
            const double dc[4] = { ds[0] * o->t[0], ds[1] * o->t[1], ds[2] * o->t[2], da * o->t[3] };
            const int ntap = s->filter == 0 ? 1 : 4;
            for (int t = 0; t < ntap; t++)
                if (f->off[t] >= 0)
                    for (int c = 0; c < 4; c++) gtex[4 * (size_t)f->off[t] + c] += o->tw[t] * dt[c];
            for (int m = 0; m < 3; m++)
                for (int c = 0; c < 4; c++) dlv[4 * (size_t)f->v[m] + c] += f->wn[m] * dc[c];
        }
        if (n > 64) { free(U); free(F); }
    }
    /* vertex lighting adjoint */
    double *gcol = grad + (size_t)s->texW * s->texH * 4, *galpha = gcol + 3 * (size_t)s->nv, *gmat = galpha + s->nv;
    double *glight = gmat + 3;
    double gL[3] = { 0, 0, 0 }, llen = 0.0, Lu[3] = { 0, 0, 0 };
    const double kd = P.mat[0], ks = P.mat[1], shin = P.mat[2];
    for (int vw = 0; vw < s->nViews; vw++)
        for (int v = 0; v < s->nv; v++) {
            const double *g4 = dlit + 4 * ((size_t)s->nv * vw + v);
            galpha[v] += g4[3];
            VT t;
            vterms(s, &P, vw, v, &t);
            llen = t.llen; for (int i = 0; i < 3; i++) Lu[i] = t.L[i];
            const double diff = t.nl > 0 ? t.nl : 0.0;
            double gdiff = 0.0, gspec = 0.0;
            for (int c = 0; c < 3; c++) {
                const double C = P.col[3 * v + c], D = C * kd;
                const double pre = D * (s->ambient + diff) + ks * t.spec;
                const double gc = pre < 1.0 ? g4[c] : 0.0;
                gcol[3 * v + c] += gc * kd * (s->ambient + diff);
                gmat[0] += gc * C * (s->ambient + diff);
                gdiff += gc * D;
                gmat[1] += gc * t.spec;
                gspec += gc * ks;
            }
            if (t.nl > 0) for (int i = 0; i < 3; i++) gL[i] += gdiff * t.N[i];
            if (t.nh > 0 && t.spec > 0) {
                gmat[2] += gspec * t.spec * log(t.nh);
                const double gx = gspec * shin * pow(t.nh, shin - 1.0);
                double gH[3] = { gx * t.N[0], gx * t.N[1], gx * t.N[2] };
                const double hg = t.H[0] * gH[0] + t.H[1] * gH[1] + t.H[2] * gH[2];
                for (int i = 0; i < 3; i++) gL[i] += (gH[i] - t.H[i] * hg) / t.hlen;
            }
        }
    const double d = Lu[0] * gL[0] + Lu[1] * gL[1] + Lu[2] * gL[2];
    for (int i = 0; i < 3; i++) glight[i] = llen > 0 ? (gL[i] - Lu[i] * d) / llen : 0.0;
    free(lit); free(dlit);
    return 0;
}
