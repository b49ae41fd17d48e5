/*
 * pf_layout.h -- data laid out in HBM by the host front end and read by the
 * kernels.  Plain structs, shared by pf_host.cpp and pf_kernels.cu.
 *
 * One flush uploads a single staging block (draw states, segment table,
 * vertex records / raw vertex arrays, index arrays, explicit item lists and
 * texture snapshots) with one host-to-device copy; every pointer below is an
 * address inside that device block or inside a persistent framebuffer
 * allocation.
 */
#ifndef PF_LAYOUT_H
#define PF_LAYOUT_H

#include <stdint.h>

/* Records read and written whole by the kernels are 16-byte aligned, so
 * that copies of them compile to 128-bit loads and stores. */
#define PF_ALIGN16 __attribute__((aligned(16)))

#define PF_MAX_LIGHTS      8
#define PF_TILE            8           /* tile edge in pixels (one warp per tile) */
#define PF_TILE_PIXELS     (PF_TILE * PF_TILE)
#define PF_MAX_SUBTRIS     10          /* fan of a triangle clipped by 7 planes */
#define PF_CLIP_MAXV       12          /* polygon capacity during clipping */
#define PF_SUB_BITS        4           /* bin key = item << 4 | sub-triangle */
#define PF_HEAVY_LEVELS    4           /* bin sizes from which a tile is rasterized early: */
#define PF_HEAVY_BASE      32          /* 32, 128, 512, 2048 entries (x4 per level) */

/* draw-state flag bits */
enum {
    PFS_LIGHTING   = 1u << 0,   /* lighting prologue (lighting on and >= 1 light) */
    PFS_PHONG      = 1u << 1,   /* per-fragment lighting */
    PFS_TEXTURE    = 1u << 2,
    PFS_BLEND      = 1u << 3,
    PFS_DEPTH_TEST = 1u << 4,
    PFS_DEPTH_MASK = 1u << 5,
    PFS_SMOOTH     = 1u << 6
};

typedef struct {
    float pos[3];
    float dir[3];
    float inner, outer;
    float attC, attL, attQ;
    uint32_t amb, diff, spec;     /* packed RGBA8 */
} PFDevLight;                     /* 56 bytes */

typedef struct {
    uint32_t amb, diff, spec, emis;
    float shininess;
} PFDevMaterial;                  /* 20 bytes */

/* Everything one draw needs, snapshotted when the draw was recorded. */
typedef struct {
    float mvp[16];
    float normal[16];
    float view8[3];               /* matView[8..10]: the NdotV axis (triangles.c:96) */
    float viewPos[3];             /* translation of inverse(matView) (triangles.c:84-86) */
    uint32_t flags;
    int32_t blendMode, depthFunc;
    int32_t vpPos[2];
    uint32_t vpDim[2];
    int32_t vpMin[2], vpMax[2];
    int32_t nLights;
    PFDevLight lights[PF_MAX_LIGHTS];
    PFDevMaterial mat[2];
    const uint32_t *tex;          /* device texels, RGBA8 */
    uint32_t texW, texH;
    int32_t texWrap, texFilter;
    float texTx, texTy;
} PFDrawState;

/* Vertex record for immediate mode and for converted vertex arrays. */
typedef struct PF_ALIGN16 {
    float pos[4];
    float normal[3];
    float uv[2];
    uint32_t color;
    uint32_t pad[2];
} PFVertexIn;                     /* 48 bytes */

/* A run of primitives sharing one draw state (one draw call, or the part of
 * a pfBegin/pfEnd block between two state changes). */
enum { PF_SRC_RECORDS = 0, PF_SRC_ARRAYS = 1 };
enum { PF_ITEMS_TRIS = 0, PF_ITEMS_EXPLICIT = 1 };

typedef struct {
    int32_t state;
    int32_t srcKind;
    uint32_t vtxBase;             /* first transformed vertex of this segment */
    uint32_t nVerts;
    uint32_t itemBase;            /* first item (global order number in the batch) */
    uint32_t nItems;
    /* vertex source */
    const PFVertexIn *records;    /* PF_SRC_RECORDS */
    const float *pos;             /* PF_SRC_ARRAYS: float positions, posSize per vertex */
    const float *nrm;             /* float3 or NULL (constant normal) */
    const float *uv;              /* float2 or NULL (constant texcoord) */
    const uint8_t *col;           /* u8 x colSize or NULL (constant colour) */
    int32_t posSize, colSize;
    float constNormal[3];
    float constUv[2];
    uint32_t constColor;
    /* primitive source */
    int32_t itemKind;
    const uint32_t *idx;          /* element indices (u32) or NULL (sequential) */
    const int32_t *explicitItems; /* PF_ITEMS_EXPLICIT: int4 {s0, s1, s2, face} */
    int32_t nFaces;               /* PF_ITEMS_TRIS: 1 or 2 */
    int32_t face0;                /* PF_ITEMS_TRIS with nFaces == 1 */
    int32_t target;               /* framebuffer of this segment (index into the batch's targets) */
    uint32_t itemSkip;            /* items of the draw before this segment's first (a draw split into passes) */
    const void *prebuilt;         /* PFPrim records of points and lines set up on the host: an explicit
                                     item {i, 0, 0, -1} stands for record i */
} PFSegment;                      /* 144 bytes */

/* A framebuffer rendered by a batch.  Its tiles are numbered
 * tileBase .. tileBase + tilesX*tilesY - 1 in the batch's bin arrays. */
typedef struct {
    void *color;                  /* pixels of format fmt (pf_pixfmt.h) */
    float *depth;
    uint32_t W, H;
    uint32_t tilesX, tilesY;
    uint32_t tileBase;
    int32_t clearMode;            /* 0 keep, 1 fused pfClear (pixels 0..7 kept), 2 fused full fill */
    uint32_t clearRaw[4];         /* the clear colour as stored: SIMD setter (pfClear), scalar (fill) */
    float clearDepth;
    uint32_t fmt;                 /* PFF_* framebuffer format */
} PFTarget;                       /* 64 bytes */

/* Transformed vertex. */
typedef struct PF_ALIGN16 {
    float h[4];                   /* clip-space position */
    float uv[2];
    uint32_t col[2];              /* lit colour for PF_FRONT, PF_BACK */
    float n[3];                   /* transformed normal (lighting) */
    float p[3];                   /* object-space position */
    uint32_t pad[2];
} PFVertexOut;                    /* 64 bytes */

/* PFPrim.flags bits: bit0 face (1 = BACK), bit1 3D path, bits 6-7 the kind
 * of record, bits 8.. the draw state.  Records other than triangles are set
 * up on the host (pf_host.cpp: lp_point, lp_thin_line, pfRectf,
 * pfDrawPixels) and carry their own per-fragment operations in bits 3-5,
 * which stand in for the draw state's (same bit positions as PFS_*). */
enum {
    PFP_Y_LONGER = 1u << 2,       /* lines: y is the long axis */
    PFP_BLEND = 1u << 3,          /* blend (scalar rules) */
    PFP_DEPTH_TEST = 1u << 4,     /* depth-test (scalar rules) */
    PFP_DEPTH_WRITE = 1u << 5,    /* write depth */
    PFP_OPS = PFP_BLEND | PFP_DEPTH_TEST | PFP_DEPTH_WRITE,
    PFP_LINE = 1u << 6,           /* a thin line of the reference's 16.16 DDA */
    PFP_POINT = 2u << 6,          /* a point: one pixel or a disc */
    PFP_BLIT = 3u << 6,           /* a rectangle: pfRectf colour or pfDrawPixels image */
    PFP_KIND = 3u << 6
};

/* Set-up sub-triangle, as read by the tile rasterizer. */
typedef struct PF_ALIGN16 {
    int32_t x1, y1, x2, y2;
    int32_t x3, y3, xMin, yMin;
    int32_t xMax, yMax;           /* x in [xMin, xMax), y in [yMin, yMax] */
    uint32_t flags;               /* bit0 face (1 = BACK), bit1 is3D, bits 8.. state */
    int32_t poolBase;             /* clipped items: pool index of sub-triangle 1 */
    float wInvSum, z1, z2, z3;
    uint32_t c1, c2, c3;
    uint32_t rstate;              /* the state's PFS_* bits | depth function << 16 | blend mode << 24,
                                     with a host-set record's own operations in place of the state's */
    float u1, v1, u2, v2;
    float u3, v3;
    float zReject;                /* depth-test rejection bound (k_raster's dense path); NaN: none */
    float texTx;                  /* textured triangles: 1 / texture width (the bilinear step) */
    uint64_t src;                 /* textured triangles: the texels; PFP_BLIT: the RGBA8 image, 0 for a colour */
    uint32_t nSrc;                /* textured triangles: width | height << 16; PFP_BLIT: pixels in the image */
    float texTy;                  /* textured triangles: 1 / texture height */
} PFPrim;                         /* 128 bytes */

/* PFPrim.rstate bits above the state's PFS_* flags: the texture's wrap mode
 * and filter, and whether its parameters must be read from the draw state
 * (a side of 65536 texels or more does not fit nSrc). */
enum {
    PFR_WRAP_SHIFT = 8,
    PFR_FILTER = 1u << 10,
    PFR_TEX_FROM_STATE = 1u << 11
};

typedef struct PF_ALIGN16 {
    float n1[3], n2[3], n3[3];
    float p1[3], p2[3], p3[3];
    float pad[2];
} PFPrimPhong;                    /* 80 bytes */

/* Device status word bits (also returned by pfGetDeviceStatus). */
enum {
    PFD_BIN_OVERFLOW = 1u << 0,   /* a tile bin exceeded the capacity of this pass */
    PFD_CLIP_OVERFLOW = 1u << 1,  /* the clipped sub-triangle pool was too small */
    PFD_BOUNDS = 1u << 2          /* an index outside the uploaded vertex range was clamped */
};

/* Counters kept on the device per context. */
typedef struct {
    unsigned long long fragments;
    unsigned long long rasterized;
    unsigned int status;          /* PFD_* */
    unsigned int abortCommand;    /* first command index that overflowed, or ~0 */
    unsigned int maxBin;          /* largest tile bin count seen */
    unsigned int clipCount;       /* clipped sub-triangles allocated */
    unsigned long long batchRasterized;   /* sub-triangles set up by the current batch */
    unsigned int tileQueue;       /* next entry of the current batch's raster work list */
    unsigned int sortQueue;       /* next entry of the current batch's bin-sort list */
    unsigned int tileListCount;   /* tiles with a non-empty bin, listed by the binning */
    unsigned int heavyCount[PF_HEAVY_LEVELS];   /* tiles whose bin reached 32 << 2 l entries */
} PFDevCounters;

#endif /* PF_LAYOUT_H */
