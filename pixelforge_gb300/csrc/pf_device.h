/*
 * pf_device.h -- launchers of the device pipeline (pf_kernels.cu), called by
 * the host front end (pf_host.cpp).  Internal to libpixelforge_gb300.so.
 */
#ifndef PF_DEVICE_H
#define PF_DEVICE_H

#include <cuda_runtime.h>
#include <stdint.h>
#include "pf_layout.h"

struct PFHookParams {
    float znear, zfar, start, end;
    uint32_t color;
    uint32_t mode;                /* pfFogProcess: PF_LINEAR, PF_EXP, PF_EXP2 (others: no fog term) */
    float density;
    uint32_t width;               /* framebuffer width (hooks that depend on the pixel's column and row) */
};

/* Device pointers and sizes of one raster batch (a run of draw segments on
 * one framebuffer). */
struct PFBatchLaunch {
    const PFSegment *segs;
    int nSegs;
    const PFDrawState *states;
    PFVertexOut *vout;
    uint32_t nVerts;
    uint32_t nItems;
    PFPrim *prims;            /* nItems records (sub-triangle 0 of each item) */
    PFPrimPhong *primsPh;
    PFPrim *pool;             /* clipped sub-triangles >= 1 */
    PFPrimPhong *poolPh;
    uint32_t poolCap;
    uint32_t *binCount;       /* totalTiles */
    uint32_t *tileList;       /* 1 + PF_HEAVY_LEVELS lists of listStride entries: the tiles with a
                                 non-empty bin, then those whose bin reached each heavy level */
    uint32_t listStride;
    uint32_t *bins;           /* totalTiles * cap */
    uint32_t cap;
    const PFTarget *targets;  /* device */
    int nTargets;
    uint32_t totalTiles;
    int rasterCtasPerSM;      /* persistent raster grid: SMs x this, at most as many as fit (0: as many as fit) */
    int rasterWarps;          /* warps (tiles in flight) per raster CTA: 2, 4 (default) or 8 */
    int anyPhong;             /* some state of the launch lights per fragment */
    int generic;              /* some target is not RGBA / unsigned byte */
    uint32_t rowCount;        /* rows of the BGRA / unsigned-byte targets (k_rows, after k_raster),
                                 0 when there are none */
    uint64_t *rowInfo;        /* rowCount > 0: nItems summaries of the items' records (row_info) */
    uint64_t *rowGroup;       /* and (nItems + 31) / 32 summaries of 32 items each */
    uint32_t rowMaxW;         /* widest of those targets */
    PFDevCounters *cnt;
    uint32_t command;
};

/* k_vertex also zeroes the tile bin counters and the batch counters. */
cudaError_t pfd_launch_vertex(const PFBatchLaunch &L, cudaStream_t st);
cudaError_t pfd_launch_items(const PFBatchLaunch &L, cudaStream_t st);
/* Bins that reached 128 entries put back into submission order (k_items
 * appends in atomic order; shorter bins are sorted by the raster). */
cudaError_t pfd_launch_binsort(const PFBatchLaunch &L, cudaStream_t st);
/* Persistent tile raster over every tile of every target; each target's
 * clearMode says how its tiles start (see PFTarget).  BGRA / unsigned-byte
 * targets are rasterized row by row by a second kernel (rowCount). */
cudaError_t pfd_launch_raster(const PFBatchLaunch &L, cudaStream_t st);
/* Number of SMs of the current device (cached). */
int pfd_sm_count(void);
/* The largest of n u32 values at d (device, 16-byte aligned) into the
 * page-locked *hWord, through the device word *dWord; complete once st is. */
cudaError_t pfd_max_u32(const uint32_t *d, size_t n, unsigned *dWord, unsigned *hWord, cudaStream_t st);
/* pfClear (all = false) or pfClearFramebuffer (all = true) of a framebuffer
 * of format fmt (PFF_*); cc is the clear colour as stored. */
cudaError_t pfd_launch_clear(void *color, uint32_t fmt, float *depth, size_t n, const uint32_t cc[4], float cd, bool all,
                             const PFDevCounters *cnt, uint32_t command, cudaStream_t st);
cudaError_t pfd_launch_hook(void *color, uint32_t fmt, const float *depth, size_t n, int hook, const PFHookParams &hp,
                            const PFDevCounters *cnt, uint32_t command, cudaStream_t st);

#endif /* PF_DEVICE_H */
