// pf_noalloc.cu -- pfgbDrawTrianglesStatic: the triangle pipeline without any
// allocation.
//
// Some callers cannot allocate device memory.  A real-time renderer must not
// call cudaMalloc on its frame path, because an allocation can block and
// synchronise the whole device; an engine or plugin host that owns all
// device memory through its own pool only lends out pre-allocated buffers.
// For them this entry point renders a soup of smooth-coloured triangles
// straight into device colour and depth buffers the caller owns, with the
// same kernels as the pf* API (k_vertex, k_items, k_raster), and keeps every
// intermediate -- transformed vertices, set-up sub-triangles, tile bins,
// counters -- in one file-scope __device__ array of fixed size.
//
// That array exists once per GPU that loads the library and stays allocated
// until the process exits.  Every call uses it, so two calls that run at the
// same time on the GPU (on different streams, or from different threads)
// race on it and corrupt each other's results; issue calls one after another
// on one stream.  A call leaves its intermediates in the array; everything a
// call needs zeroed (bin counters, device counters) it clears itself.  The
// call reads the device counters back and waits for its stream before it
// returns.

#include <cuda_runtime.h>
#include <cstdio>
#include <cstring>

#include "pixelforge.h"
#include "pf_layout.h"
#include "pf_device.h"

namespace {

constexpr uint32_t kMaxTris = PFGB_STATIC_MAX_TRIANGLES;
constexpr uint32_t kMaxW = PFGB_STATIC_MAX_WIDTH, kMaxH = PFGB_STATIC_MAX_HEIGHT;
constexpr uint32_t kMaxTiles = ((kMaxW + PF_TILE - 1) / PF_TILE) * ((kMaxH + PF_TILE - 1) / PF_TILE);
constexpr uint32_t kBinCap = PFGB_STATIC_BIN_CAPACITY;
// culling off sets up every triangle twice (FRONT then BACK face items)
constexpr uint32_t kMaxItems = 2 * kMaxTris;
constexpr uint32_t kPoolCap = PFGB_STATIC_CLIP_CAPACITY;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffState = 0;
constexpr size_t kOffSeg = align256(kOffState + sizeof(PFDrawState));
constexpr size_t kOffCnt = align256(kOffSeg + sizeof(PFSegment));
constexpr size_t kOffTarget = align256(kOffCnt + sizeof(PFDevCounters));
constexpr size_t kOffVout = align256(kOffTarget + sizeof(PFTarget));
constexpr size_t kOffPrims = align256(kOffVout + sizeof(PFVertexOut) * 3 * (size_t)kMaxTris);
constexpr size_t kOffPool = align256(kOffPrims + sizeof(PFPrim) * (size_t)kMaxItems);
constexpr size_t kOffPh = align256(kOffPool + sizeof(PFPrim) * (size_t)kPoolCap);
// bin counters, then the raster's work lists (the non-empty tiles and those
// of each heavy level), listStride entries each
constexpr uint32_t kListStride = (kMaxTiles + 31) & ~31u;
constexpr size_t kOffBinCount = align256(kOffPh + sizeof(PFPrimPhong));
constexpr size_t kOffBins = align256(kOffBinCount + sizeof(uint32_t) * (size_t)kListStride * (2 + PF_HEAVY_LEVELS));
constexpr size_t kScratchBytes = align256(kOffBins + sizeof(uint32_t) * (size_t)kMaxTiles * kBinCap);
static_assert(kScratchBytes == PFGB_STATIC_SCRATCH_BYTES, "header states the scratch size");

// The scratch.  In host code this name is only a stand-in for the device
// symbol: its address must come from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
static unsigned char *g_scratch_ptr[kMaxDevices];   // device address per device ordinal

// Look up the scratch's device address for the current device (once per
// device, with that device current).
static int scratch_for_current_device(unsigned char **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) { cudaGetLastError(); return PFGB_STATIC_E_CUDA; }
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) {
            std::fprintf(stderr, "pfgbDrawTrianglesStatic: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            cudaGetLastError();
            return PFGB_STATIC_E_CUDA;
        }
        g_scratch_ptr[dev] = (unsigned char *)p;
    }
    *out = g_scratch_ptr[dev];
    return 0;
}

}  // namespace

extern "C" int pfgbDrawTrianglesStatic(const float *positions, const uint32_t *colors, uint32_t ntris,
                                       const float *mvp, uint32_t *color, float *depth,
                                       uint32_t width, uint32_t height, int depthFunc, int cullMode, void *stream)
{
    if (ntris > kMaxTris || width == 0 || height == 0 || width > kMaxW || height > kMaxH) {
        std::fprintf(stderr, "pfgbDrawTrianglesStatic: %u triangles at %ux%u exceed the limits "
                     "(%u triangles, %ux%u pixels)\n", ntris, width, height, kMaxTris, kMaxW, kMaxH);
        return PFGB_STATIC_E_TOO_LARGE;
    }
    if (!positions || !colors || !mvp || !color || !depth || depthFunc < -1 || depthFunc > 5 ||
        cullMode < 0 || cullMode > 2)
        return PFGB_STATIC_E_INVALID;
    unsigned char *s = nullptr;
    int rc = scratch_for_current_device(&s);
    if (rc) return rc;
    if (ntris == 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;

    // draw state: what pfBegin(PF_TRIANGLES) would snapshot with the given
    // MVP, smooth shading, no lighting/texture/blend, the full-framebuffer
    // viewport and the given depth test (depth writes on)
    PFDrawState S;
    std::memset(&S, 0, sizeof S);
    std::memcpy(S.mvp, mvp, 64);
    for (int i = 0; i < 16; i++) S.normal[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    S.flags = PFS_SMOOTH | PFS_DEPTH_MASK | (depthFunc >= 0 ? PFS_DEPTH_TEST : 0u);
    S.depthFunc = depthFunc >= 0 ? depthFunc : PF_LESS;
    S.blendMode = PF_BLEND_ALPHA;
    S.vpDim[0] = width - 1; S.vpDim[1] = height - 1;
    S.vpMax[0] = (int32_t)width - 1; S.vpMax[1] = (int32_t)height - 1;
    PFSegment G;
    std::memset(&G, 0, sizeof G);
    G.state = 0; G.srcKind = PF_SRC_ARRAYS; G.vtxBase = 0; G.nVerts = 3 * ntris;
    G.itemBase = 0;
    G.pos = positions; G.posSize = 3;
    G.col = (const uint8_t *)colors; G.colSize = 4;
    G.itemKind = PF_ITEMS_TRIS;
    // face passes (internal/context/context.c:104-138): culling off renders
    // FRONT then BACK; culling a face renders the other one
    G.nFaces = (cullMode == 0) ? 2 : 1;
    G.face0 = (cullMode == 2) ? PF_BACK : PF_FRONT;
    G.nItems = ntris * (uint32_t)G.nFaces;
    PFDevCounters C;
    std::memset(&C, 0, sizeof C);
    C.abortCommand = 0xffffffffu;
    PFTarget T;
    std::memset(&T, 0, sizeof T);
    T.color = color; T.depth = depth; T.W = width; T.H = height;
    T.tilesX = (width + PF_TILE - 1) / PF_TILE; T.tilesY = (height + PF_TILE - 1) / PF_TILE;
    T.tileBase = 0; T.clearMode = 0;

    // pageable sources: these copies return once the data left the stack
    cudaError_t e = cudaMemcpyAsync(s + kOffState, &S, sizeof S, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s + kOffSeg, &G, sizeof G, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s + kOffCnt, &C, sizeof C, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s + kOffTarget, &T, sizeof T, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) { cudaGetLastError(); return PFGB_STATIC_E_CUDA; }

    PFBatchLaunch L{};
    L.segs = (const PFSegment *)(s + kOffSeg); L.nSegs = 1;
    L.states = (const PFDrawState *)(s + kOffState);
    L.vout = (PFVertexOut *)(s + kOffVout); L.nVerts = G.nVerts; L.nItems = G.nItems;
    L.prims = (PFPrim *)(s + kOffPrims); L.primsPh = (PFPrimPhong *)(s + kOffPh);
    L.pool = (PFPrim *)(s + kOffPool); L.poolPh = (PFPrimPhong *)(s + kOffPh); L.poolCap = kPoolCap;
    L.binCount = (uint32_t *)(s + kOffBinCount); L.bins = (uint32_t *)(s + kOffBins); L.cap = kBinCap;
    L.listStride = kListStride; L.tileList = L.binCount + kListStride;
    L.targets = (const PFTarget *)(s + kOffTarget); L.nTargets = 1; L.totalTiles = T.tilesX * T.tilesY;
    L.rasterCtasPerSM = 0; L.rasterWarps = 4;
    L.cnt = (PFDevCounters *)(s + kOffCnt); L.command = 0;
    e = pfd_launch_vertex(L, st);
    if (e == cudaSuccess) e = pfd_launch_items(L, st);
    if (e == cudaSuccess) e = pfd_launch_binsort(L, st);
    if (e == cudaSuccess) e = pfd_launch_raster(L, st);
    if (e != cudaSuccess) { cudaGetLastError(); return PFGB_STATIC_E_CUDA; }
    // the counters say whether a tile bin or the clip pool overflowed
    e = cudaMemcpyAsync(&C, s + kOffCnt, sizeof C, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { cudaGetLastError(); return PFGB_STATIC_E_CUDA; }
    if (C.abortCommand != 0xffffffffu) return PFGB_STATIC_E_CAPACITY;
    return 0;
}
