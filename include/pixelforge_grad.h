/*
 * pixelforge_grad.h -- differentiable rendering extension of the PixelForge
 * triangle pipeline (libpixelforge_gb300.so).
 *
 * The reference has no differentiable path; this interface adds one over the
 * same triangle pipeline.  A scene is a fixed triangle mesh seen from a set
 * of views (one framebuffer per view, all of the same size).  Coverage and
 * the depth-test outcome of every fragment are computed exactly as the
 * reference computes them (integer edge functions and set-up of
 * src/internal/primitives/triangles.c:287-438, projection of
 * src/internal/context/context.c:52-65 and triangles.c:246-280) and are held
 * fixed; the shading of the visible fragments is a floating-point relaxation
 * of the reference's formulas, differentiable in the parameters:
 *
 *   vertex lighting (Gouraud, Blinn-Phong; lighting.c:24-134 with one
 *   directional light, material ambient x light ambient = `ambient`):
 *       D   = colour_v * diffuse                      (BlendMultiplicative)
 *       L   = light / |light|,  V = normalize(eye - p_v),  H = normalize(L + V)
 *       lit = min(D * (ambient + max(N.L, 0)) + specular * max(N.H, 0)^shininess, 1)
 *   fragment (triangles.c:404-527), screen-space weights wN_i = w_i * wInvSum:
 *       c   = (wN1 lit_1 + wN2 lit_2) + wN3 lit_3,   alpha = same of alpha_v
 *       uv  = perspective-correct texture coordinate as in the reference
 *       t   = texture sample, nearest or bilinear with the reference's texel
 *             addressing (sampler.h:203-430), lerps a + f (b - a) in float
 *       src = t.rgb * c,   a = t.a * alpha                        (blend.h:200-213)
 *       dst = a * src + (1 - a) * dst                             (alpha-over, blend.h:140-160)
 *
 * pfgradForward writes the RGB image of every view; pfgradBackward takes
 * dLoss/dImage and writes dLoss/dParameters.  The backward pass recomputes
 * fragments tile by tile (no per-pixel fragment lists are stored between the
 * calls).  All buffers passed to forward/backward are device pointers; calls
 * are asynchronous on `stream` (a cudaStream_t, or NULL for the default
 * stream).
 *
 * Return codes: 0 success, PFGRAD_ERR_* below.
 */
#ifndef PIXELFORGE_GRAD_H
#define PIXELFORGE_GRAD_H

#include <stdint.h>

#ifndef PFGRAD_API
#   if defined(__GNUC__)
#       define PFGRAD_API __attribute__((visibility("default")))
#   else
#       define PFGRAD_API
#   endif
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define PFGRAD_ERR_INVALID   (-2)   /* bad argument */
#define PFGRAD_ERR_CUDA      (-3)   /* a CUDA call failed (no device, out of memory, ...) */
#define PFGRAD_ERR_CAPACITY  (-4)   /* a screen tile holds more than PFGRAD_MAX_TILE_PRIMS triangles */
#define PFGRAD_ERR_CLIP      (-5)   /* a triangle crosses the view volume: clipping is not differentiated */

#define PFGRAD_MAX_TILE_PRIMS 16384

typedef struct PFgradScene_ *PFgradScene;

typedef struct {
    const float *positions;     /* device, nVertices x 3 (object space; the model matrix is the identity) */
    const float *normals;       /* device, nVertices x 3 */
    const float *texcoords;     /* device, nVertices x 2 */
    const uint32_t *indices;    /* device, nTriangles x 3 */
    uint32_t nVertices, nTriangles;
    const float *mvp;           /* host, nViews x 16: model-view-projection of each view, the
                                   row-vector layout of pfMultMatrixf (h = p * M) */
    const float *eye;           /* host, nViews x 3: camera position (the viewPos of lighting) */
    uint32_t nViews, width, height;
    int32_t cullFace;           /* -1: no culling (both faces, FRONT pass first), else the face culled:
                                   0 PF_FRONT, 1 PF_BACK (the reference default) */
    uint32_t texWidth, texHeight;
    int32_t texFilter;          /* 0 PF_NEAREST, 1 PF_BILINEAR */
    int32_t texWrap;            /* 0 PF_REPEAT, 1 PF_MIRRORED_REPEAT, 2 PF_CLAMP_TO_EDGE */
    float ambient;              /* material ambient x light ambient */
    float background[3];        /* clear colour, RGB in [0, 1] */
    float clearDepth;           /* depth buffer clear value (the reference's initial value is FLT_MAX) */
} PFgradSceneDesc;

typedef struct {
    const float *texture;       /* device, texHeight x texWidth x 4 (RGBA) */
    const float *colors;        /* device, nVertices x 3 */
    const float *alphas;        /* device, nVertices */
    const float *material;      /* device, 3: diffuse, specular, shininess */
    const float *light;         /* device, 3: direction towards the light */
} PFgradParams;

typedef struct {
    float *texture, *colors, *alphas, *material, *light;   /* device, shaped as PFgradParams; overwritten */
} PFgradGrads;

typedef struct {
    uint64_t primitives;        /* triangles (per view) that survived culling and cover a tile */
    uint64_t tileEntries;       /* (triangle, tile) pairs */
    uint32_t maxTilePrims;      /* longest tile list */
    uint32_t tiles;             /* tiles of all views */
} PFgradInfo;

/* Projects, sets up, culls and bins the mesh for every view (synchronous). */
PFGRAD_API int pfgradSceneCreate(PFgradScene *scene, const PFgradSceneDesc *desc, void *stream);
PFGRAD_API int pfgradSceneDestroy(PFgradScene scene);
PFGRAD_API int pfgradSceneInfo(PFgradScene scene, PFgradInfo *info);

/* image: device, nViews x height x width x 3 floats. */
PFGRAD_API int pfgradForward(PFgradScene scene, const PFgradParams *params, float *image, void *stream);

/* dImage: device, shaped as image.  Every gradient buffer is overwritten. */
PFGRAD_API int pfgradBackward(PFgradScene scene, const PFgradParams *params, const float *dImage,
                   const PFgradGrads *grads, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PIXELFORGE_GRAD_H */
