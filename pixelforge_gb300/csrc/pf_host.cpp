// pf_host.cpp -- host front end of libpixelforge_gb300.so.
//
// Implements the PixelForge C API (include/pixelforge.h) on top of the
// device pipeline in pf_kernels.cu.  The state machine (matrices, lights,
// materials, vertex capture, error codes) follows the reference's
// src/context.c; what changes is *when* primitives are rasterized.  The
// reference processes each primitive synchronously inside pfVertex /
// pfDrawElements; here every draw is recorded -- its state snapshotted into
// a PFDrawState, its vertices and indices copied into one pinned staging
// block -- and the whole recording is rendered by the GPU at an observation
// point (pfFinish, pfReadPixels, pfPostProcess, ...).  The recorded order of
// primitives, face passes and clears is the reference's order, and the tile
// rasterizer applies fragments per pixel in that order.
//
// Built with -ffp-contract=off: the matrix arithmetic must round exactly as
// the reference's (src/pfm.h) does.

#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pixelforge.h"
#include "pf_layout.h"
#include "pf_device.h"
#include "pf_pixfmt.h"

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kDeg2Rad = kPi / 180.0;
constexpr uint32_t kCapMax = 16384;       // largest tile bin the rasterizer sorts in shared memory

// ---------------------------------------------------------------------------
// matrix arithmetic in the order of src/pfm.h
// ---------------------------------------------------------------------------
using Mat = float[16];

void m_identity(float *d) { std::memset(d, 0, 64); d[0] = d[5] = d[10] = d[15] = 1.0f; }

void m_mul(float *dst, const float *l, const float *r)               // pfm.h:2176-2199
{
    float res[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            float s = 0.0f;
            for (int k = 0; k < 4; k++) s += l[i * 4 + k] * r[k * 4 + j];
            res[i * 4 + j] = s;
        }
    std::memcpy(dst, res, 64);
}

void m_invert(float *dst, const float *s)                            // pfm.h:2082-2121
{
    float a00 = s[0], a01 = s[1], a02 = s[2], a03 = s[3], a10 = s[4], a11 = s[5], a12 = s[6], a13 = s[7];
    float a20 = s[8], a21 = s[9], a22 = s[10], a23 = s[11], a30 = s[12], a31 = s[13], a32 = s[14], a33 = s[15];
    float b00 = a00*a11 - a01*a10, b01 = a00*a12 - a02*a10, b02 = a00*a13 - a03*a10;
    float b03 = a01*a12 - a02*a11, b04 = a01*a13 - a03*a11, b05 = a02*a13 - a03*a12;
    float b06 = a20*a31 - a21*a30, b07 = a20*a32 - a22*a30, b08 = a20*a33 - a23*a30;
    float b09 = a21*a32 - a22*a31, b10 = a21*a33 - a23*a31, b11 = a22*a33 - a23*a32;
    float inv = 1.0f/(b00*b11 - b01*b10 + b02*b09 + b03*b08 - b04*b07 + b05*b06);
    float d[16] = {
        (a11*b11 - a12*b10 + a13*b09)*inv, (-a01*b11 + a02*b10 - a03*b09)*inv,
        (a31*b05 - a32*b04 + a33*b03)*inv, (-a21*b05 + a22*b04 - a23*b03)*inv,
        (-a10*b11 + a12*b08 - a13*b07)*inv, (a00*b11 - a02*b08 + a03*b07)*inv,
        (-a30*b05 + a32*b02 - a33*b01)*inv, (a20*b05 - a22*b02 + a23*b01)*inv,
        (a10*b10 - a11*b08 + a13*b06)*inv, (-a00*b10 + a01*b08 - a03*b06)*inv,
        (a30*b04 - a31*b02 + a33*b00)*inv, (-a20*b04 + a21*b02 - a23*b00)*inv,
        (-a10*b09 + a11*b07 - a12*b06)*inv, (a00*b09 - a01*b07 + a02*b06)*inv,
        (-a30*b03 + a31*b01 - a32*b00)*inv, (a20*b03 - a21*b01 + a22*b00)*inv };
    std::memcpy(dst, d, 64);
}

void m_transpose(float *dst, const float *s)
{
    float r[16];
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) r[i * 4 + j] = s[j * 4 + i];
    std::memcpy(dst, r, 64);
}

void v3_normalize(float *v)                                         // pfm.h:1183-1197
{
    float sq = v[0]*v[0] + v[1]*v[1] + v[2]*v[2];
    if (sq == 0.0f) return;
    float inv = 1.0f / std::sqrt(sq);
    for (int i = 0; i < 3; i++) v[i] = v[i] * inv;
}

// (PFubyte)(float) as the reference's x86-64 build converts it: truncate to
// int32 (0x80000000 out of range), keep the low 8 bits.
inline uint8_t ftoub(float x)
{
    if (!(x > -2147483649.0f && x < 2147483648.0f)) return 0;
    return (uint8_t)(uint32_t)(int32_t)x;
}
inline uint8_t dtoub(double x)
{
    if (!(x > -2147483649.0 && x < 2147483648.0)) return 0;
    return (uint8_t)(uint32_t)(int32_t)x;
}
inline uint32_t pack(PFcolor c) { uint32_t u; std::memcpy(&u, &c, 4); return u; }
inline PFcolor unpack(uint32_t u) { PFcolor c; std::memcpy(&c, &u, 4); return c; }

// ---------------------------------------------------------------------------
// objects
// ---------------------------------------------------------------------------
struct Tex {
    void *pixels;
    PFsizei w, h;
    PFpixelformat format;
    PFdatatype type;
    float tx, ty;
    int wrap, filter;
    bool ownsPinned;     // colour of a pfGenFramebuffer framebuffer (pinned host memory)
    bool depthPinned;    // its depth buffer is pinned host memory (else malloc)
    bool isMain;         // a context's main framebuffer (its depth is internal)
    uint32_t drawUses = 0;         // draw-time snapshots taken of the texels
    bool hostRegistered = false;   // the texels were page-locked by the library (cudaHostRegister)
    bool device = false;           // pfGenTextureDevice: the texels are device memory, read at the flush
};

struct Light {
    float position[3] = { 0, 0, 0 }, direction[3] = { 0, 0, 0 };
    float inner = (float)kPi, outer = (float)kPi;
    float attC = 1, attL = 0, attQ = 0;
    PFcolor ambient{ 51, 51, 51, 255 }, diffuse{ 255, 255, 255, 255 }, specular{ 255, 255, 255, 255 };
};

struct Material {
    PFcolor ambient{ 255, 255, 255, 255 }, diffuse{ 255, 255, 255, 255 };
    PFcolor specular{ 255, 255, 255, 255 }, emission{ 0, 0, 0, 255 };
    float shininess = 64.0f;
};

struct Attrib {
    const void *buf = nullptr;
    PFsizei stride = 0;
    PFint size = 0;
    PFenum type = 0;
    bool dev = false;          // buf is device memory (pf*PointerDevice): read at the flush, not copied
};

// Device mirror of one framebuffer (main or pfGenFramebuffer).
struct FBMirror {
    Tex *tex = nullptr;
    float *hostDepth = nullptr;
    bool depthUserVisible = false;     // pfGenFramebuffer: zbuffer is a public host pointer
    void *dColor = nullptr;            // pixels of format fmt
    uint32_t fmt = PFF_RGBA8;
    size_t bpp = 4;
    float *dDepth = nullptr;
    size_t w = 0, h = 0;
    bool depthOnDevice = false;        // device depth already holds the authoritative copy
    void *registered = nullptr;        // host colour registered with cudaHostRegister
    size_t registeredBytes = 0;
};

enum CmdKind { CMD_CLEAR, CMD_FILL, CMD_DRAW, CMD_HOOK };
struct Cmd {
    CmdKind kind;
    PFframebuffer *fb;
    uint32_t color;
    float depth;
    int hook;
    PFHookParams hp;
    int segBegin, segEnd;              // CMD_DRAW: segments [segBegin, segEnd)
};

// The clear colour of a CMD_CLEAR (pfClear: the SIMD setter,
// context.c:700-710) or CMD_FILL (pfClearFramebuffer: the scalar setter,
// framebuffer.c:89-102) as a framebuffer of format fmt stores it.
void clear_raw(uint32_t fmt, const Cmd &cmd, uint32_t raw[4])
{
    if (cmd.kind == CMD_FILL) pff_set_sisd(fmt, cmd.color, raw);
    else pff_set_simd(fmt, cmd.color, raw);
}

// Segment as recorded on the host: references instead of pointers.  A
// reference is -1 (none), an offset >= 0 into the staging block, or the
// negated address (< -1) of a device copy made at record time (upload()).
struct SegRec {
    PFSegment seg;                     // pointer fields left null until the flush
    PFframebuffer *fb = nullptr;       // framebuffer the segment draws into
    int64_t recordsOff = -1, posOff = -1, nrmOff = -1, uvOff = -1, colOff = -1, idxOff = -1, itemsOff = -1;
    std::vector<int32_t> explicitItems;   // immediate / non-triangle modes, grown while recording
    std::vector<PFVertexIn> records;       // immediate mode vertices
    std::vector<PFPrim> prebuilt;          // points, lines and rectangles set up on the host
    std::vector<std::pair<uint32_t, int64_t>> blitSrc;   // pfDrawPixels records: record, staged image
    int64_t prebuiltOff = -1;
};

struct StateRec {
    PFDrawState st;
    int64_t texOff = -1;
};

// Pinned host staging block, bump-allocated, uploaded with one copy per flush.
struct Staging {
    uint8_t *base = nullptr;
    size_t cap = 0, used = 0;
    bool pinned = false;
    void reserve(size_t need)
    {
        if (need <= cap) return;
        size_t nc = std::max(need, cap ? cap * 2 : (size_t)64 << 20);
        uint8_t *nb = nullptr;
        bool np = cudaMallocHost((void **)&nb, nc) == cudaSuccess;
        if (!np) { cudaGetLastError(); nb = (uint8_t *)std::malloc(nc); }
        if (base && used) std::memcpy(nb, base, used);
        release();
        base = nb; cap = nc; pinned = np;
    }
    void release()
    {
        if (!base) return;
        if (pinned) cudaFreeHost(base); else std::free(base);
        base = nullptr; cap = 0;
    }
    int64_t alloc(size_t bytes)
    {
        size_t off = (used + 255) & ~(size_t)255;
        reserve(off + bytes);
        used = off + bytes;
        return (int64_t)off;
    }
};

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    bool ensure(size_t bytes)
    {
        if (bytes <= cap) return true;
        if (p) cudaFree(p);
        size_t nc = std::max(bytes, cap + cap / 2);
        nc = (nc + 4095) & ~(size_t)4095;
        if (cudaMalloc(&p, nc) != cudaSuccess) { cudaGetLastError(); p = nullptr; cap = 0; return false; }
        cap = nc;
        return true;
    }
    void release() { if (p) cudaFree(p); p = nullptr; cap = 0; }
};

// Recording and device state of one renderer.  Every context owns one; a
// batch (pfgbBatchBegin .. pfgbBatchEnd) owns one that all contexts made
// current during the batch record into, so that the whole batch renders with
// one launch of each pipeline kernel.
struct Renderer {
    // recording
    Staging staging;
    std::vector<StateRec> states;
    std::vector<SegRec> segs;
    std::vector<Cmd> cmds;
    struct SnapKey { const void *p; size_t bytes; int64_t off; int64_t maxU32; };   // maxU32: largest u32 element, -1 unknown
    std::vector<SnapKey> snaps;
    struct Conversion { int64_t rawOff, off; PFpixelformat format; PFdatatype type; };
    std::vector<Conversion> conversions;   // RGBA8 copies of textures of other formats in this recording          // dedup of texture / array snapshots in this recording

    // caller arrays copied to the device at record time (upload()): device
    // chunks reused from one recording to the next
    struct UpChunk { void *p; size_t cap; };
    std::vector<UpChunk> up;
    size_t upChunk = 0, upOff = 0, upBytes = 0;
    // page-locked host chunks that pageable caller arrays are copied into
    // (by the worker pool) for their DMA: the GPU never reads pageable memory
    std::vector<UpChunk> hostUp;
    size_t hostChunk = 0, hostOff = 0;
    // uploads of this recording from pageable memory, for reuse by a later
    // draw that references the same unchanged array
    struct UpSnap { const void *p; size_t bytes; const uint8_t *copy; int64_t ref; int64_t maxU32; };
    std::vector<UpSnap> upSnaps;
    cudaStream_t upStream = nullptr;
    cudaEvent_t upDone = nullptr;
    // copies from page-locked caller memory (a pinned texture): DMAs on their
    // own stream, under way while the call takes its other copies, waited
    // for when the outermost API call that took them returns (CopyScope)
    cudaStream_t pinStream = nullptr;
    bool pinPending = false;
    int copyScope = 0;
    unsigned *dMax = nullptr, *hMax = nullptr;   // largest uploaded index: device word, page-locked result

    // device
    bool devInit = false, devOk = false;
    cudaStream_t stream = nullptr;
    DevBuf arena, vout, prims, primsPh, pool, poolPh, binCount, bins, counters;
    DevBuf rowInfo, rowGroup;               // per item and per 32 items, their records' rows (BGRA8 targets)
    uint32_t cap = 256, poolCap = 4096;
    int rasterCtasPerSM = 0;                // 0: as many raster CTAs per SM as fit
    int rasterWarps = 4;                    // warps per raster CTA
    PFDevCounters *hostCounters = nullptr;
    PFstats stats{};
    PFuint devStatus = 0;
    bool timing = false;
    cudaEvent_t evStart = nullptr, evEnd = nullptr;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> rasterEv;   // per raster launch, reused

    // the device work of the last successful flush, for graph replay
    struct Op { int kind; int cmd; PFBatchLaunch L; size_t n; void *color; uint32_t fmt; float *depth;
                uint32_t cc[4]; float cd; bool all; int hook; PFHookParams hp; };
    std::vector<Op> lastOps;
    std::vector<void *> splitMem;        // device segments/targets of draw groups split by the last flush
    cudaGraphExec_t graph = nullptr;
    bool graphValid = false;
};

// A render list (src/renderlist.c): per pfBegin while recording, the draw
// mode, both materials and the texture, and per vertex its position,
// texcoord, normal and colour as they were current.
struct RenderCall {
    PFdrawmode mode;
    Material mat[2];
    Tex *texture;
    std::vector<float> pos, uv, nrm;
    std::vector<PFcolor> col;
};
struct RenderList { std::vector<RenderCall> calls; };

struct Ctx {
    PFframebuffer mainFB{ nullptr, nullptr };
    PFframebuffer *current = nullptr;
    PFframebuffer *bound = nullptr;
    Tex *texture = nullptr;
    void *aux = nullptr;

    PFint vpPos[2]{ 0, 0 }; PFsizei vpDim[2]{ 0, 0 }; PFint vpMin[2]{ 0, 0 }; PFint vpMax[2]{ 0, 0 };
    Attrib positions, normals, colors, texcoords;

    // immediate-mode capture: the reference's 6-slot vertex buffer (context.c:1658-1685)
    PFVertexIn slots[6];
    PFsizei vcount = 0;
    float curNormal[3]{ 0, 0, 0 }; float curTex[2]{ 0, 0 }; PFcolor curColor{ 255, 255, 255, 255 };

    PFcolor clearColor{ 0, 0, 0, 255 }; float clearDepth = FLT_MAX;
    PFdrawmode drawMode = PF_POINTS;
    PFpolygonmode polygonMode[2]{ PF_FILL, PF_FILL };
    Material mat[2];
    PFface colMatFace = PF_FRONT_AND_BACK; PFenum colMatMode = PF_AMBIENT_AND_DIFFUSE;
    Light lights[PF_MAX_LIGHTS];
    std::vector<int> activeLights;       // insertion order, as the reference's linked list

    Mat proj, tex, model, view, mvp, normal;
    Mat stackProj[2], stackMV[8], stackTex[4];
    PFsizei nProj = 0, nMV = 0, nTex = 0;
    PFmatrixmode matMode = PF_MODELVIEW; bool modelUsed = false;
    float *cur = nullptr;

    PFshademode shade = PF_SMOOTH; PFlightmode lightMode = PF_GOURAUD; PFface cullFace = PF_BACK;
    PFblendmode blend = PF_BLEND_ALPHA; PFdepthmode depthFunc = PF_LESS;
    PFerrcode err = PF_NO_ERROR; PFuint state = PF_CULL_FACE;
    bool depthMask = true;
    PFfloat pointSize = 1.0f, lineWidth = 1.0f;
    float rasterPos[4]{ 0.0f, 0.0f, 0.0f, 1.0f }; float pixelZoom[2]{ 1.0f, 1.0f };   // context.c:179-180
    struct { uint32_t mode = PF_LINEAR; float density = 1.0f, start = 0.0f, end = 1.0f; PFcolor color{ 0, 0, 0, 0 }; } fog;
    RenderList *curList = nullptr;          // render list being recorded
    struct { Material mat[2]; float tex[2]; float nrm[3]; PFcolor col; Tex *texture; PFuint state; } backup{};

    bool stateDirty = true;
    int openImmSeg = -1;                 // immediate-mode segment accepting primitives (index in rend->segs)
    Renderer own;
    Renderer *rend = &own;
};

struct Batch {
    Renderer r;
    std::vector<Ctx *> members;
    bool open = false;
};

thread_local Ctx *G = nullptr;
thread_local Batch *gBatch = nullptr;     // batch being recorded on this thread

// Device copies of every framebuffer, shared by all renderers (a framebuffer
// has one device copy whichever renderer draws into it).
std::mutex gMirrorMutex;
std::unordered_map<const void *, FBMirror> gMirrors;

void set_err(PFerrcode e) { if (G) G->err = e; }

void report_device_failure(const char *what, cudaError_t e)
{
    static bool once = false;
    if (!once) {
        std::fprintf(stderr, "pixelforge_gb300: %s failed: %s -- nothing is rendered without a CUDA device\n",
                     what, cudaGetErrorString(e));
        once = true;
    }
}

// ---------------------------------------------------------------------------
// texel formats.  The device samples RGBA8; a texture in another format is
// converted when it is snapshotted, texel by texel, to the value the
// reference's SIMD pixel getter returns for it (src/internal/pixel.h:
// 2253-3097), including its reads: a single-channel unsigned-byte getter takes
// the top byte of a 32-bit load (the texel three places further on), the
// luminance-alpha one the next texel's pair, half and float channels scale by
// 255 and round to nearest even without clamping, and the BGR half/float
// getters return the channels in memory order.  Bytes past the end of the
// caller's buffer read 0.  BGRA / unsigned byte uses the per-texel swizzle
// (the reference's shuffle mask repeats the first texel of each half vector,
// src/internal/simd.h:564-583).
// ---------------------------------------------------------------------------
int texel_bytes(PFpixelformat f, PFdatatype t)
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

struct TexelSrc {
    const uint8_t *p;
    int64_t n;                  // bytes
    uint32_t byte(int64_t b) const { return (b >= 0 && b < n) ? p[b] : 0u; }
    uint32_t word(int64_t b) const { return byte(b) | byte(b + 1) << 8 | byte(b + 2) << 16 | byte(b + 3) << 24; }
};

// pfmHalfToFloat (src/pfm.h:129-161): denormals flush to zero
inline float half_to_float(uint32_t h)
{
    const uint32_t sgn = (h & 0x8000u) << 16;
    const int32_t em = (int32_t)(h & 0x7fffu);
    int32_t r = (int32_t)((uint32_t)(em + (112 << 10)) << 13);
    r = (em < (1 << 10)) ? 0 : r;
    r += (em >= (31 << 10)) ? (112 << 23) : 0;
    const uint32_t u = sgn | (uint32_t)r;
    float f; std::memcpy(&f, &u, 4);
    return f;
}
// CVTPS2DQ: round to nearest even, 0x80000000 for NaN or out of range
inline uint32_t cvt_rne_u(float x)
{
    if (!(x > -2147483648.0f && x < 2147483648.0f)) return 0x80000000u;
    return (uint32_t)(int32_t)std::nearbyint(x);
}

uint32_t texel_rgba8(PFpixelformat f, PFdatatype t, const TexelSrc &s, int64_t o)
{
    auto h8 = [&](int64_t i) { return cvt_rne_u(half_to_float(s.word(2 * i) & 0xffffu) * 255.0f); };
    auto f8 = [&](int64_t i) { const uint32_t u = s.word(4 * i); float x; std::memcpy(&x, &u, 4); return cvt_rne_u(x * 255.0f); };
    switch (t) {
    case PF_UNSIGNED_BYTE:
        switch (f) {
        case PF_RED: return (s.word(o) >> 24) | 0xff000000u;
        case PF_GREEN: return ((s.word(o) >> 24) << 8) | 0xff000000u;
        case PF_BLUE: return ((s.word(o) >> 24) << 16) | 0xff000000u;
        case PF_ALPHA: return s.word(o) << 24;
        case PF_LUMINANCE: { const uint32_t v = s.word(o) >> 24; return v | v << 8 | v << 16 | 0xff000000u; }
        case PF_LUMINANCE_ALPHA: { const uint32_t w = s.word(2 * o), l = (w >> 16) & 255u; return l | l << 8 | l << 16 | (w & 0xff000000u); }
        case PF_RGB: return (s.word(3 * o) & 0xffffffu) | 0xff000000u;
        case PF_BGR: { const uint32_t w = s.word(3 * o); return ((w >> 16) & 255u) | (w & 0xff00u) | (w & 255u) << 16 | 0xff000000u; }
        case PF_RGBA: return s.word(4 * o);
        case PF_BGRA: { const uint32_t w = s.word(4 * o); return ((w >> 16) & 255u) | (w & 0xff00u) | (w & 255u) << 16 | (w & 0xff000000u); }
        default: return 0;
        }
    case PF_HALF_FLOAT:
    case PF_FLOAT: {
        auto c8 = [&](int64_t i) { return t == PF_HALF_FLOAT ? h8(i) : f8(i); };
        switch (f) {
        case PF_RED: return c8(o) | 0xff000000u;
        case PF_GREEN: return c8(o) << 8 | 0xff000000u;
        case PF_BLUE: return c8(o) << 16 | 0xff000000u;
        case PF_ALPHA: return c8(o) << 24;
        case PF_LUMINANCE: { const uint32_t v = c8(o); return 0xff000000u | v << 16 | v << 8 | v; }
        case PF_LUMINANCE_ALPHA: { const uint32_t v = c8(2 * o), a = c8(2 * o + 1); return a << 24 | v << 16 | v << 8 | v; }
        case PF_RGB: case PF_BGR: return 0xff000000u | c8(3 * o + 2) << 16 | c8(3 * o + 1) << 8 | c8(3 * o);
        case PF_RGBA: return c8(4 * o + 3) << 24 | c8(4 * o + 2) << 16 | c8(4 * o + 1) << 8 | c8(4 * o);
        case PF_BGRA: return c8(4 * o + 3) << 24 | c8(4 * o) << 16 | c8(4 * o + 1) << 8 | c8(4 * o + 2);
        default: return 0;
        }
    }
    case PF_UNSIGNED_SHORT_5_6_5: {
        const uint32_t w = s.word(2 * o);
        const uint32_t hi = ((w & 0xf800u) >> 11) << 3, g = ((w & 0x07e0u) >> 5) << 2, lo = (w & 0x1fu) << 3;
        return (f == PF_RGB) ? (0xff000000u | lo << 16 | g << 8 | hi) : (0xff000000u | hi << 16 | g << 8 | lo);
    }
    case PF_UNSIGNED_SHORT_5_5_5_1: {
        const uint32_t w = s.word(2 * o);
        const uint32_t c0 = ((w >> 11) & 0x1fu) * 8u, c1 = ((w >> 6) & 0x1fu) * 8u, c2 = ((w >> 1) & 0x1fu) * 8u, a = (w & 1u) * 255u;
        return (f == PF_RGBA) ? (a << 24 | c2 << 16 | c1 << 8 | c0) : (a << 24 | c0 << 16 | c1 << 8 | c2);
    }
    case PF_UNSIGNED_SHORT_4_4_4_4: {
        const uint32_t w = s.word(2 * o);
        const uint32_t c0 = ((w >> 12) & 0xfu) * 17u, c1 = ((w >> 8) & 0xfu) * 17u, c2 = ((w >> 4) & 0xfu) * 17u, a = (w & 0xfu) * 17u;
        return (f == PF_RGBA) ? (a << 24 | c2 << 16 | c1 << 8 | c0) : (a << 24 | c0 << 16 | c1 << 8 | c2);
    }
    default: return 0;
    }
}

// The PFF_* code of a framebuffer format, -1 for the formats a framebuffer
// may not have: those for which one pixel's result would depend on other
// pixels or on its SIMD lane in the reference -- single-channel and
// luminance(-alpha) unsigned byte (their SIMD getters read the texel three
// places on, or the next texel, src/internal/pixel.h:2253-2420),
// single-channel and luminance half / float (their SIMD setters rewrite,
// requantised, the pixels of the vector that the mask leaves out,
// pixel.h:905-970, 1219-1490).  BGRA unsigned byte, whose SIMD setter
// writes a half vector with its first pixel's value, is rasterized row by
// row (k_rows).
int fb_code(PFpixelformat f, PFdatatype t)
{
    switch (t) {
    case PF_UNSIGNED_BYTE:
        return f == PF_RGBA ? PFF_RGBA8 : f == PF_RGB ? PFF_RGB8 : f == PF_BGR ? PFF_BGR8 : f == PF_BGRA ? PFF_BGRA8 : -1;
    case PF_UNSIGNED_SHORT_5_6_5: return f == PF_RGB ? PFF_RGB565 : f == PF_BGR ? PFF_BGR565 : -1;
    case PF_UNSIGNED_SHORT_5_5_5_1: return f == PF_RGBA ? PFF_RGBA5551 : f == PF_BGRA ? PFF_BGRA5551 : -1;
    case PF_UNSIGNED_SHORT_4_4_4_4: return f == PF_RGBA ? PFF_RGBA4444 : f == PF_BGRA ? PFF_BGRA4444 : -1;
    case PF_HALF_FLOAT:
        switch (f) {
        case PF_LUMINANCE_ALPHA: return PFF_LA16F;
        case PF_RGB: return PFF_RGB16F;
        case PF_BGR: return PFF_BGR16F;
        case PF_RGBA: return PFF_RGBA16F;
        case PF_BGRA: return PFF_BGRA16F;
        default: return -1;
        }
    case PF_FLOAT:
        switch (f) {
        case PF_LUMINANCE_ALPHA: return PFF_LA32F;
        case PF_RGB: return PFF_RGB32F;
        case PF_BGR: return PFF_BGR32F;
        case PF_RGBA: return PFF_RGBA32F;
        case PF_BGRA: return PFF_BGRA32F;
        default: return -1;
        }
    default: return -1;
    }
}

// Textures may use any format the reference has a SIMD getter for,
// framebuffers the formats fb_code accepts.
Tex *tex_new(void *pixels, PFsizei w, PFsizei h, PFpixelformat f, PFdatatype t, bool sampled)
{
    if (sampled ? !texel_bytes(f, t) : fb_code(f, t) < 0) { set_err(PF_INVALID_ENUM); return nullptr; }
    Tex *x = new Tex();
    x->pixels = pixels; x->w = w; x->h = h; x->format = f; x->type = t;
    x->tx = 1.0f / (float)w; x->ty = 1.0f / (float)h;
    x->wrap = PF_REPEAT; x->filter = PF_NEAREST; x->ownsPinned = false; x->depthPinned = false; x->isMain = false;
    return x;
}

// ---------------------------------------------------------------------------
// host worker pool: large snapshots (vertex arrays, indices, textures) are
// copied and compared by several threads, the caller taking a share.
// A drawing call makes several such loops of a few microseconds each, so
// dispatch must cost less than the work: items are claimed from one atomic
// word that also carries the loop's generation and size, completions are
// counted atomically, and an idle worker spins on the word for a while
// (kSpinUs) before it sleeps on a condition variable.
// ---------------------------------------------------------------------------
class Pool {
public:
    static Pool &get() { static Pool p; return p; }
    int workers() const { return (int)threads_.size() + 1; }
    // run fn(i) for i in [0, n); returns when all are done
    void run(int n, const std::function<void(int)> &fn)
    {
        if (n <= 1 || threads_.empty() || n > (int)kMaxItems) { for (int i = 0; i < n; i++) fn(i); return; }
        std::lock_guard<std::mutex> one(runMutex_);      // one parallel loop at a time
        // every item of the previous loop is done, so no worker still reads fn_
        fn_ = &fn;
        done_.store(0, std::memory_order_relaxed);
        gen_ = (gen_ + 1) & kGenMask;
        claim_.store(pack(gen_, (uint64_t)n, 0), std::memory_order_seq_cst);
        wake_one();                                      // a woken worker wakes the next
        work(gen_);
        while (done_.load(std::memory_order_acquire) != n) std::this_thread::yield();
    }
    ~Pool()
    {
        stop_.store(true);
        { std::lock_guard<std::mutex> lk(m_); }
        cv_.notify_all();
        for (auto &t : threads_) t.join();
    }
private:
    // claim word: generation (24 bits) | items (20 bits) | next item (20 bits)
    static constexpr uint64_t kGenMask = (1u << 24) - 1, kMaxItems = (1u << 20) - 1;
    static constexpr int kSpinUs = 1000;          // about a frame's flush: the next draw finds the workers awake
    static uint64_t pack(uint64_t g, uint64_t n, uint64_t next) { return (g << 40) | (n << 20) | next; }
    static uint64_t gen_of(uint64_t c) { return c >> 40; }

    Pool()
    {
        // all cores but the caller's: the copies into staging are bound by
        // per-core memory bandwidth
        unsigned hw = std::thread::hardware_concurrency();
        int n = (int)std::min(15u, hw > 1 ? hw - 1 : 0u);
        for (int i = 0; i < n; i++) threads_.emplace_back([this] { loop(); });
    }
    // claim and run items of loop `g` until none is left (or a newer loop began)
    void work(uint64_t g)
    {
        for (;;) {
            uint64_t c = claim_.load(std::memory_order_acquire);
            int item = -1;
            while (gen_of(c) == g && (c & kMaxItems) < ((c >> 20) & kMaxItems)) {
                if (claim_.compare_exchange_weak(c, c + 1, std::memory_order_acq_rel)) { item = (int)(c & kMaxItems); break; }
            }
            if (item < 0) return;
            (*fn_)(item);
            done_.fetch_add(1, std::memory_order_release);
        }
    }
    void wake_one()
    {
        if (sleepers_.load(std::memory_order_seq_cst) > 0) {
            std::lock_guard<std::mutex> lk(m_);
            cv_.notify_one();
        }
    }
    void loop()
    {
        uint64_t seen = 0;
        for (;;) {
            // spin for a new loop, then sleep
            const auto t0 = std::chrono::steady_clock::now();
            uint64_t g = gen_of(claim_.load(std::memory_order_acquire));
            for (int k = 0; g == seen && !stop_.load(std::memory_order_relaxed); k++) {
                if ((k & 255) == 255) {
                    if (std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(kSpinUs)) break;
                    std::this_thread::yield();
                }
                g = gen_of(claim_.load(std::memory_order_acquire));
            }
            if (g == seen && !stop_.load()) {
                sleepers_.fetch_add(1, std::memory_order_seq_cst);
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return stop_.load() || gen_of(claim_.load(std::memory_order_seq_cst)) != seen; });
                sleepers_.fetch_sub(1, std::memory_order_relaxed);
                lk.unlock();
                const uint64_t c = claim_.load(std::memory_order_acquire);
                g = gen_of(c);
                if ((c & kMaxItems) < ((c >> 20) & kMaxItems)) wake_one();   // items left: pass the wake on
            }
            if (stop_.load()) return;
            seen = g;
            work(g);
        }
    }
    std::vector<std::thread> threads_;
    std::mutex m_, runMutex_;
    std::condition_variable cv_;
    const std::function<void(int)> *fn_ = nullptr;
    std::atomic<uint64_t> claim_{ 0 };
    std::atomic<int> done_{ 0 };
    std::atomic<int> sleepers_{ 0 };
    std::atomic<bool> stop_{ false };
    uint64_t gen_ = 0;
};

constexpr size_t kParallelChunk = (size_t)1 << 16;     // 64 KiB

void par_memcpy(void *dst, const void *src, size_t bytes)
{
    if (bytes < 2 * kParallelChunk) { std::memcpy(dst, src, bytes); return; }
    const int n = (int)((bytes + kParallelChunk - 1) / kParallelChunk);
    Pool::get().run(n, [&](int i) {
        size_t o = (size_t)i * kParallelChunk, len = std::min(kParallelChunk, bytes - o);
        std::memcpy((uint8_t *)dst + o, (const uint8_t *)src + o, len);
    });
}

bool par_equal(const void *a, const void *b, size_t bytes)
{
    if (bytes < 2 * kParallelChunk) return std::memcmp(a, b, bytes) == 0;
    const int n = (int)((bytes + kParallelChunk - 1) / kParallelChunk);
    std::atomic<bool> diff{ false };
    Pool::get().run(n, [&](int i) {
        if (diff.load(std::memory_order_relaxed)) return;
        size_t o = (size_t)i * kParallelChunk, len = std::min(kParallelChunk, bytes - o);
        if (std::memcmp((const uint8_t *)a + o, (const uint8_t *)b + o, len) != 0) diff.store(true);
    });
    return !diff.load();
}

// Largest of `count` u32 values.
uint32_t par_max_u32(const uint32_t *src, size_t count)
{
    const size_t chunk = kParallelChunk / 4;
    const int n = (int)((count + chunk - 1) / chunk);
    std::vector<uint32_t> mx((size_t)std::max(n, 1), 0u);
    Pool::get().run(n, [&](int i) {
        size_t o = (size_t)i * chunk, len = std::min(chunk, count - o);
        uint32_t m = 0;
        for (size_t k = 0; k < len; k++) { uint32_t v = src[o + k]; m = v > m ? v : m; }
        mx[(size_t)i] = m;
    });
    uint32_t m = 0;
    for (uint32_t v : mx) m = std::max(m, v);
    return m;
}

// u32 indices: copy and return the largest
uint32_t par_copy_max_u32(uint32_t *dst, const uint32_t *src, size_t count)
{
    const size_t chunk = kParallelChunk / 4;
    const int n = (int)((count + chunk - 1) / chunk);
    std::vector<uint32_t> mx((size_t)std::max(n, 1), 0u);
    Pool::get().run(n, [&](int i) {
        size_t o = (size_t)i * chunk, len = std::min(chunk, count - o);
        const uint32_t *s = src + o;
        uint32_t *d = dst + o;
        uint32_t m0 = 0, m1 = 0, m2 = 0, m3 = 0;
        size_t k = 0;
        for (; k + 4 <= len; k += 4) {
            const uint32_t a = s[k], b = s[k + 1], c = s[k + 2], e = s[k + 3];
            d[k] = a; d[k + 1] = b; d[k + 2] = c; d[k + 3] = e;
            m0 = std::max(m0, a); m1 = std::max(m1, b); m2 = std::max(m2, c); m3 = std::max(m3, e);
        }
        for (; k < len; k++) { d[k] = s[k]; m0 = std::max(m0, s[k]); }
        mx[(size_t)i] = std::max(std::max(m0, m1), std::max(m2, m3));
    });
    uint32_t m = 0;
    for (uint32_t v : mx) m = std::max(m, v);
    return m;
}

// ---------------------------------------------------------------------------
// recording
// ---------------------------------------------------------------------------
bool device_init(Renderer *r);

inline int64_t dev_ref(const void *p) { return -(int64_t)(uintptr_t)p; }

#ifndef PF_UPLOAD_MIN_BYTES
#define PF_UPLOAD_MIN_BYTES ((size_t)64 << 10)
#endif
constexpr size_t kUploadMin = PF_UPLOAD_MIN_BYTES;        // smaller arrays go through staging
constexpr size_t kUploadBudget = (size_t)8 << 30;        // per recording; beyond it, staging with de-duplication
constexpr size_t kUploadChunk = (size_t)64 << 20;

// Room for `bytes` in the upload chunks, or nullptr (the caller takes the
// staging path); upload_commit takes it.
uint8_t *upload_room(Renderer *r, size_t bytes)
{
    if (r->upBytes + bytes > kUploadBudget) return nullptr;
    if (r->upBytes == 0) {               // a new recording: the last flush's device data is overwritten
        r->lastOps.clear();
        r->graphValid = false;
    }
    const size_t need = (bytes + 255) & ~(size_t)255;
    while (r->upChunk < r->up.size() && r->upOff + need > r->up[r->upChunk].cap) { r->upChunk++; r->upOff = 0; }
    if (r->upChunk == r->up.size()) {
        Renderer::UpChunk c{ nullptr, std::max(kUploadChunk, need) };
        if (cudaMalloc(&c.p, c.cap) != cudaSuccess) { cudaGetLastError(); return nullptr; }
        r->up.push_back(c);
        r->upOff = 0;
    }
    return (uint8_t *)r->up[r->upChunk].p + r->upOff;
}
void upload_commit(Renderer *r, size_t bytes)
{
    r->upOff += (bytes + 255) & ~(size_t)255;
    r->upBytes += bytes;
}
bool is_pageable(const void *p)
{
    cudaPointerAttributes attr{};
    const bool pageable = cudaPointerGetAttributes(&attr, p) == cudaSuccess && attr.type == cudaMemoryTypeUnregistered;
    cudaGetLastError();
    return pageable;
}

// Room for `bytes` in the page-locked host chunks (kept from one recording
// to the next; a new chunk at least doubles what the renderer holds).
uint8_t *host_room(Renderer *r, size_t bytes)
{
    const size_t need = (bytes + 255) & ~(size_t)255;
    while (r->hostChunk < r->hostUp.size() && r->hostOff + need > r->hostUp[r->hostChunk].cap) {
        r->hostChunk++; r->hostOff = 0;
    }
    if (r->hostChunk == r->hostUp.size()) {
        size_t held = 0;
        for (auto &c : r->hostUp) held += c.cap;
        Renderer::UpChunk c{ nullptr, std::max(std::max(need, held), (size_t)4 << 20) };
        if (cudaMallocHost(&c.p, c.cap) != cudaSuccess) { cudaGetLastError(); return nullptr; }
        r->hostUp.push_back(c);
        r->hostOff = 0;
    }
    uint8_t *h = (uint8_t *)r->hostUp[r->hostChunk].p + r->hostOff;
    r->hostOff += need;
    return h;
}

// Copy `bytes` of caller memory to the device now (large arrays; the caller
// may change them once the drawing call returns).  Pageable memory is
// copied by the worker pool into a page-locked host chunk (u32 arrays: their
// largest element found in the same pass, into *maxU32) and sent from
// there by an asynchronous DMA; a later draw of the same recording that
// references the same unchanged array reuses that copy.  Page-locked and
// device memory is copied by a DMA straight from where it lies, waited for
// before the drawing call returns.  Returns the device reference, or -1
// (the caller takes the staging path).
int64_t upload(Renderer *r, const void *p, size_t bytes, int64_t *maxU32 = nullptr)
{
    if (bytes < kUploadMin || !device_init(r)) return -1;
    const bool pageable = is_pageable(p);
    if (pageable)
        for (const auto &u : r->upSnaps)
            if (u.p == p && u.bytes == bytes && (!maxU32 || u.maxU32 >= 0) && par_equal(u.copy, p, bytes)) {
                if (maxU32) *maxU32 = u.maxU32;
                return u.ref;
            }
    uint8_t *dst = upload_room(r, bytes);
    if (!dst) return -1;
    if (pageable) {
        uint8_t *h = host_room(r, bytes);
        if (!h) return -1;
        int64_t mx = -1;
        if (maxU32) mx = (int64_t)par_copy_max_u32((uint32_t *)h, (const uint32_t *)p, bytes / 4);
        else par_memcpy(h, p, bytes);
        if (cudaMemcpyAsync(dst, h, bytes, cudaMemcpyHostToDevice, r->upStream) != cudaSuccess) { cudaGetLastError(); return -1; }
        if (maxU32) *maxU32 = mx;
        r->upSnaps.push_back({ p, bytes, h, dev_ref(dst), mx });
    } else {
        if (cudaMemcpyAsync(dst, p, bytes, cudaMemcpyDefault, r->pinStream) != cudaSuccess) { cudaGetLastError(); return -1; }
        // (an index maximum is then reduced on the device, on the upload
        // stream: the copy must have landed)
        if (r->copyScope > 0 && !maxU32) r->pinPending = true;      // waited for as the API call returns
        else cudaStreamSynchronize(r->pinStream);
    }
    upload_commit(r, bytes);
    return dev_ref(dst);
}

// Scope of an API call that takes snapshots of caller memory: copies from
// page-locked memory started inside it are complete when the outermost
// scope ends (before the call returns to the caller, who may then change
// the memory).
void settle_pinned(Renderer *r)
{
    if (!r->pinPending) return;
    if (cudaStreamSynchronize(r->pinStream) != cudaSuccess) cudaGetLastError();
    r->pinPending = false;
}
struct CopyScope {
    Renderer *r;
    explicit CopyScope(Renderer *rr) : r(rr) { r->copyScope++; }
    ~CopyScope() { if (--r->copyScope == 0) settle_pinned(r); }
    CopyScope(const CopyScope &) = delete;
    CopyScope &operator=(const CopyScope &) = delete;
};

// Copy `bytes` of caller memory for the device: uploaded now (large arrays;
// device_ok), or into staging, reusing an identical snapshot taken earlier
// in the same recording.
int64_t snapshot(Renderer *r, const void *p, size_t bytes, bool device_ok = true)
{
    if (device_ok) {
        const int64_t ref = upload(r, p, bytes);
        if (ref != -1) return ref;
    }
    for (auto &s : r->snaps)
        if (s.p == p && s.bytes == bytes && par_equal(r->staging.base + s.off, p, bytes)) return s.off;
    int64_t off = r->staging.alloc(bytes);
    par_memcpy(r->staging.base + off, p, bytes);
    r->snaps.push_back({ p, bytes, off, -1 });
    return off;
}
int64_t snapshot(Ctx *c, const void *p, size_t bytes) { return snapshot(c->rend, p, bytes); }

// The largest of `count` indices uploaded to d, reduced on the device (a
// few microseconds after the copy lands; a host scan of the caller's array
// takes several times longer).  False if the device could not do it.
// The device word and page-locked word that return an index maximum.
bool max_words(Renderer *r)
{
    if (!r->dMax) {
        unsigned *d = nullptr;
        if (cudaMalloc((void **)&d, sizeof(unsigned)) != cudaSuccess) { cudaGetLastError(); return false; }
        r->dMax = d;
    }
    if (!r->hMax) {
        unsigned *h = nullptr;
        if (cudaMallocHost((void **)&h, sizeof(unsigned)) != cudaSuccess) { cudaGetLastError(); return false; }
        r->hMax = h;
    }
    return true;
}

bool device_max_u32(Renderer *r, const uint32_t *d, size_t count, uint32_t &mx)
{
    if (!max_words(r)) return false;
    if (pfd_max_u32(d, count, r->dMax, r->hMax, r->upStream) != cudaSuccess || cudaStreamSynchronize(r->upStream) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    r->stats.kernel_launches += 1; r->stats.copy_launches += 1;
    mx = *r->hMax;
    return true;
}

// Snapshot of `count` u32 indices and their largest value (kept with the
// snapshot, so a draw that repeats the indices compares instead of copying).
int64_t snapshot_u32(Renderer *r, const uint32_t *p, size_t count, uint32_t &mx)
{
    const size_t bytes = count * 4;
    if (bytes >= kUploadMin) {
        int64_t hm = -1;
        const int64_t ref = upload(r, p, bytes, &hm);
        if (ref != -1) {
            if (hm >= 0) mx = (uint32_t)hm;                  // found while copying
            else if (!device_max_u32(r, (const uint32_t *)(uintptr_t)(-ref), count, mx)) mx = par_max_u32(p, count);
            return ref;
        }
    }
    for (auto &s : r->snaps)
        if (s.p == p && s.bytes == bytes && s.maxU32 >= 0 && par_equal(r->staging.base + s.off, p, bytes)) {
            mx = (uint32_t)s.maxU32;
            return s.off;
        }
    const int64_t off = r->staging.alloc(bytes);
    mx = par_copy_max_u32((uint32_t *)(r->staging.base + off), p, count);
    r->snaps.push_back({ p, bytes, off, (int64_t)mx });
    return off;
}

// RGBA8 snapshot of a texture: its own bytes, or the converted texels of
// another format (from a snapshot of its bytes, converted once per recording).
// A texture drawn with a second time and large enough that its draw-time
// copy pays for page-locking: its texels are registered with the driver
// (until pfDeleteTexture), so that every later snapshot is a DMA rather
// than a copy through the driver's pageable staging.
constexpr size_t kPinTextureMin = (size_t)1 << 20;
void pin_texture(Renderer *r, Tex *t, size_t bytes)
{
    if (t->hostRegistered || t->ownsPinned || ++t->drawUses < 2 || bytes < kPinTextureMin || !device_init(r)) return;
    if (!is_pageable(t->pixels)) return;                          // page-locked by someone else already
    // registering pins the pages (the kernel may move them first): no copy
    // of this or a neighbouring array may still be reading them
    if (cudaDeviceSynchronize() != cudaSuccess) { cudaGetLastError(); return; }
    if (cudaHostRegister(t->pixels, bytes, cudaHostRegisterDefault) == cudaSuccess) t->hostRegistered = true;
    else cudaGetLastError();
}

int64_t snapshot_texture(Renderer *r, const Tex *t)
{
    if (t->device) return -(int64_t)(uintptr_t)t->pixels;      // the caller's device texels, as they are
    const size_t n = (size_t)t->w * t->h;
    if (t->format == PF_RGBA && t->type == PF_UNSIGNED_BYTE) {
        pin_texture(r, const_cast<Tex *>(t), n * 4);
        return snapshot(r, t->pixels, n * 4);
    }
    const int64_t raw = snapshot(r, t->pixels, n * (size_t)texel_bytes(t->format, t->type), false);   // read here
    for (auto &cv : r->conversions)
        if (cv.rawOff == raw && cv.format == t->format && cv.type == t->type) return cv.off;
    const int64_t off = r->staging.alloc(n * 4);
    const TexelSrc src{ r->staging.base + raw, (int64_t)(n * (size_t)texel_bytes(t->format, t->type)) };
    uint32_t *dst = (uint32_t *)(r->staging.base + off);
    const size_t chunk = 1 << 16;
    const int parts = (int)((n + chunk - 1) / chunk);
    auto work = [&](int i) {
        const size_t b = (size_t)i * chunk, e = std::min(n, b + chunk);
        for (size_t k = b; k < e; k++) dst[k] = texel_rgba8(t->format, t->type, src, (int64_t)k);
    };
    if (parts > 1) Pool::get().run(parts, work); else work(0);
    r->conversions.push_back({ raw, off, t->format, t->type });
    return off;
}

void update_matrices(Ctx *c, bool withNormal)                      // context.c:96-111
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

// Snapshot the state every primitive of the next segment is processed with.
int snapshot_state(Ctx *c)
{
    StateRec r;
    PFDrawState &s = r.st;
    std::memset(&s, 0, sizeof s);
    std::memcpy(s.mvp, c->mvp, 64);
    std::memcpy(s.normal, c->normal, 64);
    const bool lighting = (c->state & PF_LIGHTING) && !c->activeLights.empty();
    if (lighting) {
        float inv[16]; m_invert(inv, c->view);                        // triangles.c:84-86
        s.viewPos[0] = inv[12]; s.viewPos[1] = inv[13]; s.viewPos[2] = inv[14];
    }
    s.view8[0] = c->view[8]; s.view8[1] = c->view[9]; s.view8[2] = c->view[10];
    uint32_t fl = 0;
    if (lighting) fl |= PFS_LIGHTING;
    if (lighting && c->lightMode == PF_PHONG) fl |= PFS_PHONG;
    Tex *t = ((c->state & PF_TEXTURE_2D) && c->texture) ? c->texture : nullptr;
    if (t) {
        fl |= PFS_TEXTURE;
        r.texOff = snapshot_texture(c->rend, t);
        s.texW = t->w; s.texH = t->h; s.texWrap = t->wrap; s.texFilter = t->filter; s.texTx = t->tx; s.texTy = t->ty;
    }
    if (c->state & PF_BLEND) fl |= PFS_BLEND;
    if (c->state & PF_DEPTH_TEST) fl |= PFS_DEPTH_TEST;
    if (c->depthMask) fl |= PFS_DEPTH_MASK;
    if (c->shade == PF_SMOOTH) fl |= PFS_SMOOTH;
    s.flags = fl;
    s.blendMode = c->blend; s.depthFunc = c->depthFunc;
    for (int i = 0; i < 2; i++) {
        s.vpPos[i] = c->vpPos[i]; s.vpDim[i] = c->vpDim[i]; s.vpMin[i] = c->vpMin[i]; s.vpMax[i] = c->vpMax[i];
    }
    s.nLights = lighting ? (int)c->activeLights.size() : 0;
    for (int i = 0; i < s.nLights; i++) {
        const Light &l = c->lights[c->activeLights[i]];
        PFDevLight &d = s.lights[i];
        std::memcpy(d.pos, l.position, 12); std::memcpy(d.dir, l.direction, 12);
        d.inner = l.inner; d.outer = l.outer; d.attC = l.attC; d.attL = l.attL; d.attQ = l.attQ;
        d.amb = pack(l.ambient); d.diff = pack(l.diffuse); d.spec = pack(l.specular);
    }
    for (int f = 0; f < 2; f++) {
        s.mat[f].amb = pack(c->mat[f].ambient); s.mat[f].diff = pack(c->mat[f].diffuse);
        s.mat[f].spec = pack(c->mat[f].specular); s.mat[f].emis = pack(c->mat[f].emission);
        s.mat[f].shininess = c->mat[f].shininess;
    }
    c->rend->states.push_back(r);
    return (int)c->rend->states.size() - 1;
}

// Face passes of one primitive (internal/context/context.c:95-244): the
// faces, in order, and the polygon mode of each (PF_FILL outside
// PF_TRIANGLES / PF_QUADS, the only modes with a polygon-mode switch).
int face_passes(const Ctx *c, PFdrawmode mode, int faces[2], PFpolygonmode pm[2])
{
    const bool cull = (c->state & PF_CULL_FACE) != 0;
    const PFface f = cull ? (PFface)!c->cullFace : PF_FRONT_AND_BACK;
    const bool usesPolyMode = (mode == PF_TRIANGLES || mode == PF_QUADS);
    int n = 0;
    if (f == PF_FRONT_AND_BACK) { faces[n++] = PF_FRONT; faces[n++] = PF_BACK; }
    else faces[n++] = f;
    for (int k = 0; k < n; k++) pm[k] = usesPolyMode ? c->polygonMode[faces[k]] : PF_FILL;
    return n;
}

// Filled faces of a primitive drawn by the device's vertex path alone.
int fill_faces(const Ctx *c, PFdrawmode mode, int faces[2], bool &allFill)
{
    PFpolygonmode pm[2];
    const int n = face_passes(c, mode, faces, pm);
    allFill = mode != PF_POINTS && mode != PF_LINES;
    for (int k = 0; k < n; k++) allFill = allFill && pm[k] == PF_FILL;
    return n;
}

// Items of one completed primitive of `mode` whose vertices are the slot
// sequence positions s[0..count).  Order: the reference's per-face loops
// (triangles.c:118-152 and internal/context/context.c:104-243).
void emit_items(std::vector<int32_t> &out, PFdrawmode mode, const uint32_t *s, const int *faces, int nf)
{
    auto tri = [&](int a, int b, int d, int face) {
        out.push_back((int32_t)s[a]); out.push_back((int32_t)s[b]); out.push_back((int32_t)s[d]); out.push_back(face);
    };
    auto fan = [&](int face, int n) { for (int i = 0; i < n; i++) tri(0, i + 1, i + 2, face); };
    auto strip = [&](int face, int n) {
        for (int i = 0; i < n; i++) { if (i % 2 == 0) tri(i, i + 1, i + 2, face); else tri(i + 2, i + 1, i, face); }
    };
    for (int k = 0; k < nf; k++) {
        switch (mode) {
        case PF_TRIANGLES: tri(0, 1, 2, faces[k]); break;
        case PF_TRIANGLE_FAN: case PF_QUADS: fan(faces[k], 2); break;
        case PF_TRIANGLE_STRIP: strip(faces[k], 2); break;
        case PF_QUAD_FAN: fan(faces[k], 4); break;
        case PF_QUAD_STRIP: strip(faces[k], 4); break;
        default: break;
        }
    }
}

PFsizei mode_count(PFdrawmode m)                                    // context.c:61-74
{
    switch (m) {
    case PF_POINTS: return 1; case PF_LINES: return 2; case PF_TRIANGLES: return 3;
    case PF_TRIANGLE_FAN: case PF_TRIANGLE_STRIP: case PF_QUADS: return 4;
    case PF_QUAD_FAN: case PF_QUAD_STRIP: return 6;
    }
    return 0;
}

// After a primitive: which slots carry over (context.c:41-59); returns the
// new vertex count and moves slot indices in `slot` accordingly.
template <typename T> PFsizei reset_for_next(PFdrawmode mode, T *slot)
{
    switch (mode) {
    case PF_TRIANGLE_FAN: case PF_TRIANGLE_STRIP: slot[0] = slot[3]; return 1;
    case PF_QUAD_FAN: case PF_QUAD_STRIP: slot[0] = slot[4]; slot[1] = slot[5]; return 2;
    default: return 0;
    }
}

// Append a DRAW of segment `si` to the command list, merging with the
// previous DRAW when it targets the same framebuffer.
void push_draw(Renderer *r, PFframebuffer *fb, int si)
{
    if (!r->cmds.empty() && r->cmds.back().kind == CMD_DRAW && r->cmds.back().fb == fb && r->cmds.back().segEnd == si) {
        r->cmds.back().segEnd = si + 1;
        return;
    }
    Cmd cmd{};
    cmd.kind = CMD_DRAW; cmd.fb = fb; cmd.segBegin = si; cmd.segEnd = si + 1;
    r->cmds.push_back(cmd);
}

int new_segment(Ctx *c, int srcKind, int itemKind)
{
    Renderer *r = c->rend;
    CopyScope scope(r);
    SegRec rec;
    std::memset(&rec.seg, 0, sizeof rec.seg);
    rec.seg.state = snapshot_state(c);
    rec.seg.srcKind = srcKind;
    rec.seg.itemKind = itemKind;
    rec.fb = c->current;
    r->segs.push_back(std::move(rec));
    int si = (int)r->segs.size() - 1;
    push_draw(r, c->current, si);
    c->stateDirty = false;
    return si;
}

void push_cmd(Ctx *c, const Cmd &cmd)
{
    c->rend->cmds.push_back(cmd);
    c->openImmSeg = -1;
}

// ---------------------------------------------------------------------------
// points and lines (src/internal/primitives/points.c, lines.c)
//
// Their set-up runs here, on the host, when the primitive is recorded: the
// projection, the reference's two line clippers and the 16.16 DDA
// parameters, all in the reference's operation order (this file is built
// without contraction of multiply-adds).  Each point, thin line and offset
// line of a thick line becomes one PFPrim record (fields as k_raster's
// lp_covers reads them) and one explicit item {record, 0, 0, -1} in
// submission order; the tile rasterizer covers, depth-tests (scalar rules)
// and blends (scalar rules) their pixels in order with the triangles'.
// Pixels outside the framebuffer are not drawn (the reference writes them
// at y*w + x, outside its buffers or wrapped into a neighbouring row).
// ---------------------------------------------------------------------------
struct LPVert { float pos[4]; float h[4]; float sx, sy; uint32_t col; };

inline int32_t ftoi_x86(float x)                // cvttss2si: 0x80000000 out of range
{
    if (!(x > -2147483649.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int32_t)x;
}
inline int32_t iabs32(int32_t v) { return v < 0 ? (int32_t)(0u - (uint32_t)v) : v; }
inline int32_t isub32(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }

void v4_transform(float *dst, const float *v, const float *m)      // pfm.h:1996-2006
{
    const float t[4] = {
        m[0]*v[0] + m[4]*v[1] + m[8]*v[2] + m[12]*v[3],
        m[1]*v[0] + m[5]*v[1] + m[9]*v[2] + m[13]*v[3],
        m[2]*v[0] + m[6]*v[1] + m[10]*v[2] + m[14]*v[3],
        m[3]*v[0] + m[7]*v[1] + m[11]*v[2] + m[15]*v[3] };
    std::memcpy(dst, t, 16);
}

// Where set-up records of one recording go.
struct LPOut {
    std::vector<PFPrim> &prims;
    std::vector<int32_t> &items;
    int32_t W, H;                               // framebuffer the records draw into
};

// Append record P with pixels in the inclusive box [x0, x1] x [y0, y1]
// (clipped to the framebuffer; nothing is appended when no pixel remains).
int64_t lp_emit(LPOut &o, PFPrim &P, int64_t x0, int64_t x1, int64_t y0, int64_t y1)
{
    x0 = std::max<int64_t>(x0, 0); y0 = std::max<int64_t>(y0, 0);
    x1 = std::min<int64_t>(x1, (int64_t)o.W - 1); y1 = std::min<int64_t>(y1, (int64_t)o.H - 1);
    if (x0 > x1 || y0 > y1) return -1;
    P.xMin = (int32_t)x0; P.xMax = (int32_t)(x1 + 1); P.yMin = (int32_t)y0; P.yMax = (int32_t)y1;
    P.poolBase = 0;
    const int32_t item[4] = { (int32_t)o.prims.size(), 0, 0, -1 };
    o.items.insert(o.items.end(), item, item + 4);
    o.prims.push_back(P);
    return (int64_t)o.prims.size() - 1;
}

// Per-fragment operations of a point or line record: its depth test, and
// blending and depth write as the state has them.
uint32_t lp_ops(const Ctx *c, bool test)
{
    return (test ? (uint32_t)PFP_DEPTH_TEST : 0u) | ((c->state & PF_BLEND) ? (uint32_t)PFP_BLEND : 0u) |
           (c->depthMask ? (uint32_t)PFP_DEPTH_WRITE : 0u);
}

void screen_map(const Ctx *c, LPVert &v)                           // lines.c:272-298
{
    v.sx = ((float)c->vpPos[0] + (v.h[0] + 1.0f) * 0.5f * (float)c->vpDim[0]) + 0.5f;
    v.sy = ((float)c->vpPos[1] + (1.0f - v.h[1]) * 0.5f * (float)c->vpDim[1]) + 0.5f;
}

// Rasterize_Point_{DEPTH,NODEPTH} after Process_ProjectPoint (points.c:44-183)
void lp_point(const Ctx *c, LPOut &o, const LPVert &v)
{
    float h[4];
    v4_transform(h, v.pos, c->mvp);
    if (h[3] != 1.0f) {
        for (int i = 0; i < 3; i++) if (h[i] < -h[3] || h[i] > h[3]) return;
        const float invW = 1.0f / h[3];
        h[0] = h[0] * invW; h[1] = h[1] * invW;
    }
    const float sx = ((float)c->vpPos[0] + (h[0] + 1.0f) * 0.5f * (float)c->vpDim[0]) + 0.5f;
    const float sy = ((float)c->vpPos[1] + (1.0f - h[1]) * 0.5f * (float)c->vpDim[1]) + 0.5f;
    if (!(sx >= (float)c->vpMin[0] && sy >= (float)c->vpMin[1] && sx <= (float)c->vpMax[0] && sy <= (float)c->vpMax[1]))
        return;
    PFPrim P;
    std::memset(&P, 0, sizeof P);
    P.x1 = ftoi_x86(sx); P.y1 = ftoi_x86(sy);
    P.flags = PFP_POINT | lp_ops(c, (c->state & PF_DEPTH_TEST) != 0);
    P.z1 = h[2];
    P.c1 = v.col;
    int32_t ir = 0;
    if (c->pointSize <= 1.0f) P.x2 = -1;
    else {
        const float rad = c->pointSize * 0.5f;
        ir = ftoi_x86(rad);
        if (ir < 0) return;                     // the reference's loop runs no step
        P.x2 = ir;
        P.wInvSum = rad * rad;
    }
    lp_emit(o, P, (int64_t)P.x1 - ir, (int64_t)P.x1 + ir, (int64_t)P.y1 - ir, (int64_t)P.y1 + ir);
}

// Helper_EncodeClip2D (lines.c:116-125): 1 left, 2 right, 4 y > yMax, 8 y < yMin
uint32_t clip_code(float x, float y, const Ctx *c)
{
    uint32_t code = 0;
    if (x < (float)c->vpMin[0]) code |= 1;
    if (x > (float)c->vpMax[0]) code |= 2;
    if (y < (float)c->vpMin[1]) code |= 8;
    if (y > (float)c->vpMax[1]) code |= 4;
    return code;
}

// Process_ClipLine2D (lines.c:158-223): Cohen-Sutherland in screen space with
// the reference's assignments (an end beyond the bottom edge moves to the
// top row, and the reverse).  Bounded to 32 rounds; the reference loops
// until it accepts or rejects.
bool clip_line_2d(const Ctx *c, LPVert &v1, LPVert &v2)
{
    const float xMin = (float)c->vpMin[0], yMin = (float)c->vpMin[1], xMax = (float)c->vpMax[0], yMax = (float)c->vpMax[1];
    float m = 0.0f;
    if (v1.sx != v2.sx) m = (v2.sy - v1.sy) / (v2.sx - v1.sx);
    for (int round = 0; round < 32; round++) {
        uint32_t code0 = clip_code(v1.sx, v1.sy, c), code1 = clip_code(v2.sx, v2.sy, c);
        if ((code0 | code1) == 0) return true;
        if (code0 & code1) return false;
        if (code0 == 0) { std::swap(code0, code1); std::swap(v1, v2); }
        if (code0 & 1) { v1.sy = v1.sy + (xMin - v1.sx) * m; v1.sx = xMin; }
        else if (code0 & 2) { v1.sy = v1.sy + (xMax - v1.sx) * m; v1.sx = xMax; }
        else if (code0 & 4) { if (m != 0.0f) v1.sx = v1.sx + (yMin - v1.sy) / m; v1.sy = yMin; }
        else if (code0 & 8) { if (m != 0.0f) v1.sx = v1.sx + (yMax - v1.sy) / m; v1.sy = yMax; }
    }
    return false;
}

bool clip_coord_3d(float q, float p, float &t1, float &t2)           // lines.c:127-150
{
    if (std::fabs(p) < 1e-5f) return !(q < -1e-5f);
    const float r = q / p;
    if (p < 0) { if (r > t2) return false; if (r > t1) t1 = r; }
    else { if (r < t1) return false; if (r < t2) t2 = r; }
    return true;
}

// Process_ClipLine3D (lines.c:225-262): Liang-Barsky in clip space
bool clip_line_3d(LPVert &v1, LPVert &v2)
{
    float t1 = 0.0f, t2 = 1.0f, d[4];
    const float *a = v1.h;
    for (int i = 0; i < 4; i++) d[i] = v2.h[i] - a[i];
    if (!clip_coord_3d(a[3] - a[0], -d[3] + d[0], t1, t2)) return false;
    if (!clip_coord_3d(a[3] + a[0], -d[3] - d[0], t1, t2)) return false;
    if (!clip_coord_3d(a[3] - a[1], -d[3] + d[1], t1, t2)) return false;
    if (!clip_coord_3d(a[3] + a[1], -d[3] - d[1], t1, t2)) return false;
    if (!clip_coord_3d(a[3] - a[2], -d[3] + d[2], t1, t2)) return false;
    if (!clip_coord_3d(a[3] + a[2], -d[3] - d[2], t1, t2)) return false;
    if (t2 < 1.0f) for (int i = 0; i < 4; i++) v2.h[i] = v1.h[i] + d[i] * t2;
    if (t1 > 0.0f) for (int i = 0; i < 4; i++) v1.h[i] = v1.h[i] + d[i] * t1;
    return true;
}

// Process_ProjectAndClipLine (lines.c:264-300)
bool project_clip_line(const Ctx *c, LPVert *l)
{
    for (int i = 0; i < 2; i++) v4_transform(l[i].h, l[i].pos, c->mvp);
    if (l[0].h[3] == 1.0f && l[1].h[3] == 1.0f) {
        screen_map(c, l[0]); screen_map(c, l[1]);
        return clip_line_2d(c, l[0], l[1]);
    }
    if (!clip_line_3d(l[0], l[1])) return false;
    for (int i = 0; i < 2; i++) {
        const float invW = 1.0f / l[i].h[3];
        l[i].h[0] = l[i].h[0] * invW; l[i].h[1] = l[i].h[1] * invW;
    }
    screen_map(c, l[0]); screen_map(c, l[1]);
    return true;
}

// Rasterize_Line_{DEPTH,NODEPTH} (lines.c:304-431): one record holding the
// DDA's start, step count, 16.16 short-axis step and direction.
void lp_thin_line(LPOut &o, float sx1, float sy1, float sx2, float sy2, const LPVert &a, const LPVert &b, uint32_t ops)
{
    const int32_t x1 = ftoi_x86(sx1), y1 = ftoi_x86(sy1), x2 = ftoi_x86(sx2), y2 = ftoi_x86(sy2);
    int32_t shortLen = isub32(y2, y1), longLen = isub32(x2, x1);
    bool yLonger = false;
    if (iabs32(shortLen) > iabs32(longLen)) { std::swap(shortLen, longLen); yLonger = true; }
    if (longLen == 0) return;                   // the loop runs no step
    const float invEndVal = 1.0f / (float)longLen;
    const int32_t endVal = longLen;
    int32_t sgnInc = 1;
    if (longLen < 0) { longLen = iabs32(longLen); sgnInc = -1; }
    if (longLen < 0 || longLen > (1 << 30)) return;   // only from unrepresentable coordinates
    const int32_t decInc = (int32_t)((uint32_t)shortLen << 16) / longLen;
    PFPrim P;
    std::memset(&P, 0, sizeof P);
    P.x1 = x1; P.y1 = y1; P.x2 = endVal; P.y2 = decInc; P.x3 = sgnInc;
    P.flags = (uint32_t)PFP_LINE | ops | (yLonger ? (uint32_t)PFP_Y_LONGER : 0u);
    P.wInvSum = invEndVal;
    P.z1 = a.h[2]; P.z2 = b.h[2];
    P.c1 = a.col; P.c2 = b.col;
    // long axis: a1 + i for i = 0, sgnInc, ..., endVal - sgnInc; short axis:
    // b1 + (k decInc >> 16), monotone in the step k unless k decInc wraps
    const int64_t a1 = yLonger ? y1 : x1, b1 = yLonger ? x1 : y1;
    const int64_t aEnd = a1 + (int64_t)endVal - sgnInc;
    const int64_t jl = (int64_t)(longLen - 1) * decInc;
    int64_t bLo, bHi;
    if (jl >= INT32_MIN && jl <= INT32_MAX) {
        const int64_t bEnd = b1 + ((int32_t)jl >> 16);
        bLo = std::min(b1, bEnd); bHi = std::max(b1, bEnd);
    } else { bLo = INT32_MIN; bHi = INT32_MAX; }
    const int64_t aLo = std::min(a1, aEnd), aHi = std::max(a1, aEnd);
    if (yLonger) lp_emit(o, P, bLo, bHi, aLo, aHi);
    else lp_emit(o, P, aLo, aHi, bLo, bHi);
}

// pfiProcessRasterize_LINE (lines.c:57-79) and its thick variants
// (lines.c:433-531): the centre line is always depth-tested, offset copies
// follow it one pixel further out each side in turn.  Returns false when
// the line was clipped away.
bool lp_line(const Ctx *c, LPOut &o, const LPVert &va, const LPVert &vb)
{
    LPVert l[2] = { va, vb };
    if (!project_clip_line(c, l)) return false;
    const uint32_t test = lp_ops(c, (c->state & PF_DEPTH_TEST) != 0);
    if (!(c->lineWidth > 1.5f)) { lp_thin_line(o, l[0].sx, l[0].sy, l[1].sx, l[1].sy, l[0], l[1], test); return true; }
    const int32_t x1 = ftoi_x86(l[0].sx), y1 = ftoi_x86(l[0].sy), x2 = ftoi_x86(l[1].sx), y2 = ftoi_x86(l[1].sy);
    const int32_t dx = isub32(x2, x1), dy = isub32(y2, y1);
    lp_thin_line(o, l[0].sx, l[0].sy, l[1].sx, l[1].sy, l[0], l[1], lp_ops(c, true));
    const float rs = 1.0f / std::sqrt((float)(int32_t)((uint32_t)dx * (uint32_t)dx + (uint32_t)dy * (uint32_t)dy));
    if (dx != 0 && iabs32((dx == -1 && dy == INT32_MIN) ? dy : dy / dx) < 1) {
        const int32_t wy = ftoi_x86((c->lineWidth - 1.0f) * rs * (float)iabs32(dx)) >> 1;
        for (int32_t i = 1; i <= wy; i++) {
            lp_thin_line(o, l[0].sx, l[0].sy - (float)i, l[1].sx, l[1].sy - (float)i, l[0], l[1], test);
            lp_thin_line(o, l[0].sx, l[0].sy + (float)i, l[1].sx, l[1].sy + (float)i, l[0], l[1], test);
        }
    } else if (dy != 0) {
        const int32_t wx = ftoi_x86((c->lineWidth - 1.0f) * rs * (float)iabs32(dy)) >> 1;
        for (int32_t i = 1; i <= wx; i++) {
            lp_thin_line(o, l[0].sx - (float)i, l[0].sy, l[1].sx - (float)i, l[1].sy, l[0], l[1], test);
            lp_thin_line(o, l[0].sx + (float)i, l[0].sy, l[1].sx + (float)i, l[1].sy, l[0], l[1], test);
        }
    }
    return true;
}

LPVert lp_vert(const PFVertexIn &v)
{
    LPVert r;
    std::memcpy(r.pos, v.pos, 16);
    std::memset(r.h, 0, 16);
    r.sx = r.sy = 0.0f;
    r.col = v.color;
    return r;
}

// The immediate-mode segment accepting records under the current state.  A
// segment stays open only while it is the renderer's last one (another
// context of a batch may have appended since).
SegRec &open_segment(Ctx *c)
{
    Renderer *r = c->rend;
    if (c->openImmSeg < 0 || c->stateDirty || c->openImmSeg != (int)r->segs.size() - 1)
        c->openImmSeg = new_segment(c, PF_SRC_RECORDS, PF_ITEMS_EXPLICIT);
    return r->segs[c->openImmSeg];
}

// A completed primitive of `mode` over the vertices `slots` (immediate mode,
// or vertex arrays assembled on the host): triangle faces become items over
// vertex records, points and lines (the modes and the PF_POINT / PF_LINE
// polygon modes) become set-up records; all in the reference's order
// (internal/context/context.c:95-244, points.c:33-41, lines.c:81-110).
void record_primitive(Ctx *c, PFdrawmode mode, const PFVertexIn *slots)
{
    const PFsizei n = mode_count(mode);
    int faces[2]; PFpolygonmode pm[2];
    const int nf = (mode == PF_POINTS || mode == PF_LINES) ? 0 : face_passes(c, mode, faces, pm);
    SegRec &rec = open_segment(c);
    const Tex *fbt = (const Tex *)c->current->texture;
    LPOut o{ rec.prebuilt, rec.explicitItems, (int32_t)fbt->w, (int32_t)fbt->h };
    if (mode == PF_POINTS) { lp_point(c, o, lp_vert(slots[0])); return; }
    if (mode == PF_LINES) { lp_line(c, o, lp_vert(slots[0]), lp_vert(slots[1])); return; }
    uint32_t s[6];
    bool stored = false;
    for (int k = 0; k < nf; k++) {
        if (pm[k] == PF_POINT) {
            for (PFsizei i = 0; i < n; i++) lp_point(c, o, lp_vert(slots[i]));
        } else if (pm[k] == PF_LINE) {
            for (PFsizei i = 0; i < n; i++)
                if (!lp_line(c, o, lp_vert(slots[i]), lp_vert(slots[(i + 1) % n]))) break;
        } else {
            if (!stored) {
                for (PFsizei i = 0; i < n; i++) { s[i] = (uint32_t)rec.records.size(); rec.records.push_back(slots[i]); }
                stored = true;
            }
            emit_items(rec.explicitItems, mode, s, &faces[k], 1);
        }
    }
}

// pfVertex4fv path: a primitive completed in immediate mode.
void immediate_primitive(Ctx *c) { record_primitive(c, c->drawMode, c->slots); }

// ---------------------------------------------------------------------------
// device side
// ---------------------------------------------------------------------------
bool device_init(Renderer *r)
{
    if (r->devInit) return r->devOk;
    r->devInit = true;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        report_device_failure("cudaGetDeviceCount", e == cudaSuccess ? cudaErrorNoDevice : e);
        cudaGetLastError();
        r->devStatus |= PF_DEVICE_NO_GPU;
        return false;
    }
    e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&r->upStream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&r->pinStream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->upDone, cudaEventDisableTiming);
    if (e != cudaSuccess) { report_device_failure("cudaStreamCreate", e); r->devStatus |= PF_DEVICE_NO_GPU; return false; }
    if (!r->counters.ensure(sizeof(PFDevCounters))) { r->devStatus |= PF_DEVICE_ALLOC_FAIL; return false; }
    if (cudaMallocHost((void **)&r->hostCounters, sizeof(PFDevCounters)) != cudaSuccess) {
        cudaGetLastError(); r->devStatus |= PF_DEVICE_ALLOC_FAIL; return false;
    }
    r->devOk = true;
    return true;
}

void release_renderer(Renderer *r)
{
    if (r->graph) { cudaGraphExecDestroy(r->graph); r->graph = nullptr; }
    if (r->devOk) {
        r->arena.release(); r->vout.release(); r->prims.release(); r->primsPh.release(); r->pool.release();
        r->poolPh.release(); r->binCount.release(); r->bins.release(); r->counters.release();
        r->rowInfo.release(); r->rowGroup.release();
        if (r->hostCounters) cudaFreeHost(r->hostCounters);
        if (r->evStart) { cudaEventDestroy(r->evStart); cudaEventDestroy(r->evEnd); }
        for (auto &pr : r->rasterEv) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
        if (r->stream) cudaStreamDestroy(r->stream);
        if (r->upStream) cudaStreamDestroy(r->upStream);
        if (r->pinStream) cudaStreamDestroy(r->pinStream);
        if (r->upDone) cudaEventDestroy(r->upDone);
        if (r->dMax) cudaFree(r->dMax);
        if (r->hMax) cudaFreeHost(r->hMax);
        r->dMax = r->hMax = nullptr;
        for (auto &u : r->up) cudaFree(u.p);
        r->up.clear();
        for (auto &u : r->hostUp) cudaFreeHost(u.p);
        r->hostUp.clear();
        for (void *q : r->splitMem) cudaFree(q);
        r->splitMem.clear();
    }
    r->staging.release();
    r->devOk = r->devInit = false;
}

FBMirror *mirror_for(Renderer *r, PFframebuffer *fb)
{
    std::lock_guard<std::mutex> lk(gMirrorMutex);
    Tex *t = (Tex *)fb->texture;
    FBMirror &m = gMirrors[t];
    const size_t w = t->w, h = t->h;
    const uint32_t fmt = (uint32_t)fb_code(t->format, t->type);
    const size_t bpp = (size_t)pff_bytes(fmt);
    if (m.dColor && (m.w != w || m.h != h || m.fmt != fmt)) {
        cudaFree(m.dColor); cudaFree(m.dDepth); m.dColor = nullptr; m.dDepth = nullptr;
    }
    if (!m.dColor) {
        if (cudaMalloc(&m.dColor, w * h * bpp) != cudaSuccess ||
            cudaMalloc((void **)&m.dDepth, w * h * 4) != cudaSuccess) {
            cudaGetLastError(); r->devStatus |= PF_DEVICE_ALLOC_FAIL; return nullptr;
        }
        m.w = w; m.h = h; m.fmt = fmt; m.bpp = bpp; m.depthOnDevice = false;
    }
    m.tex = t;
    m.hostDepth = fb->zbuffer;
    m.depthUserVisible = !t->isMain;
    if (m.registered != t->pixels && !t->ownsPinned) {
        // (no copy may be in flight on the pages being pinned or released)
        if (cudaDeviceSynchronize() != cudaSuccess) cudaGetLastError();
        if (m.registered) cudaHostUnregister(m.registered);
        m.registered = nullptr;
        if (cudaHostRegister(t->pixels, w * h * bpp, cudaHostRegisterDefault) == cudaSuccess) m.registered = t->pixels;
        else cudaGetLastError();
    }
    return &m;
}

FBMirror *find_mirror(const void *tex)
{
    std::lock_guard<std::mutex> lk(gMirrorMutex);
    auto it = gMirrors.find(tex);
    return it == gMirrors.end() ? nullptr : &it->second;
}

void drop_mirror(const void *tex)
{
    std::lock_guard<std::mutex> lk(gMirrorMutex);
    auto it = gMirrors.find(tex);
    if (it == gMirrors.end()) return;
    if (cudaDeviceSynchronize() != cudaSuccess) cudaGetLastError();   // its write-back may be in flight
    if (it->second.registered) cudaHostUnregister(it->second.registered);
    if (it->second.dColor) cudaFree(it->second.dColor);
    if (it->second.dDepth) cudaFree(it->second.dDepth);
    gMirrors.erase(it);
}

void discard_recording(Renderer *r)
{
    r->states.clear(); r->segs.clear(); r->cmds.clear(); r->snaps.clear(); r->conversions.clear();
    r->staging.used = 0;
    settle_pinned(r);
    r->upSnaps.clear();
    if (r->upBytes) {
        cudaStreamSynchronize(r->upStream);            // (the host chunks' DMAs too)
        r->upChunk = r->upOff = r->upBytes = 0;
        r->hostChunk = r->hostOff = 0;
    }
}

// One unit of device work of a flush: a multi-target raster batch (a run of
// DRAW commands, each framebuffer's leading clear folded in), a standalone
// clear / fill, or a post-process hook.
struct FlushOp {
    int kind;                  // 0 batch, 1 clear/fill, 2 hook
    int cmd;                   // first command index (abort bookkeeping)
    int cmdEnd;                // one past the last command covered
    int segBegin, segEnd;
    std::vector<PFframebuffer *> targets;
    std::vector<int> clearCmd; // per target: fused clear command or -1
};

// Render everything recorded, then write colour (and user-visible depth) back
// to host memory.  Returns false if the device could not be used.
bool flush(Renderer *r)
{
    if (r->cmds.empty()) { discard_recording(r); return true; }
    if (!device_init(r)) { set_err(PF_INVALID_OPERATION); discard_recording(r); return false; }
    cudaStream_t st = r->stream;
    auto fail = [&](const char *what, cudaError_t e) {
        report_device_failure(what, e);
        r->devStatus |= PF_DEVICE_LAUNCH_FAIL;
        set_err(PF_INVALID_OPERATION);
        cudaGetLastError();
        cudaStreamSynchronize(st);
        discard_recording(r);
        r->graphValid = false;
        return false;
    };
    const std::vector<Cmd> &cmds = r->cmds;

    // --- group commands into device operations ---------------------------------
    std::vector<FlushOp> ops;
    {
        FlushOp cur; cur.kind = -1;
        auto close = [&]() { if (cur.kind == 0) ops.push_back(cur); cur = FlushOp(); cur.kind = -1; };
        auto targetIndex = [&](PFframebuffer *fb) {
            for (size_t i = 0; i < cur.targets.size(); i++) if (cur.targets[i] == fb) return (int)i;
            return -1;
        };
        for (size_t ci = 0; ci < cmds.size(); ci++) {
            const Cmd &cmd = cmds[ci];
            if (cmd.kind == CMD_DRAW) {
                if (cur.kind != 0) { close(); cur.kind = 0; cur.cmd = (int)ci; cur.segBegin = cmd.segBegin; }
                if (targetIndex(cmd.fb) < 0) { cur.targets.push_back(cmd.fb); cur.clearCmd.push_back(-1); }
                cur.segEnd = cmd.segEnd; cur.cmdEnd = (int)ci + 1;
                continue;
            }
            if (cmd.kind == CMD_CLEAR || cmd.kind == CMD_FILL) {
                // fold into the next DRAW of the same framebuffer when that
                // framebuffer has not been drawn yet in the current batch
                const bool nextDraw = ci + 1 < cmds.size() && cmds[ci + 1].kind == CMD_DRAW && cmds[ci + 1].fb == cmd.fb;
                const Tex *t = (const Tex *)cmd.fb->texture;
                const bool fusable = nextDraw && (cmd.kind == CMD_FILL || ((size_t)t->w * t->h) % 8 == 0);
                if (fusable && (cur.kind != 0 || targetIndex(cmd.fb) < 0)) {
                    if (cur.kind != 0) { close(); cur.kind = 0; cur.cmd = (int)ci; cur.segBegin = cmds[ci + 1].segBegin; cur.segEnd = cur.segBegin; }
                    cur.targets.push_back(cmd.fb); cur.clearCmd.push_back((int)ci);
                    cur.cmdEnd = (int)ci + 1;
                    continue;
                }
            }
            close();
            FlushOp o; o.kind = (cmd.kind == CMD_HOOK) ? 2 : 1; o.cmd = (int)ci; o.cmdEnd = (int)ci + 1;
            o.segBegin = o.segEnd = 0;
            o.targets.push_back(cmd.fb); o.clearCmd.push_back(-1);
            ops.push_back(o);
        }
        close();
    }

    // --- framebuffers used: device copies ------------------------------------------
    std::vector<PFframebuffer *> used;
    for (auto &cmd : cmds)
        if (std::find(used.begin(), used.end(), cmd.fb) == used.end()) used.push_back(cmd.fb);
    std::vector<FBMirror *> mirrors;
    for (PFframebuffer *fb : used) {
        FBMirror *m = mirror_for(r, fb);
        if (!m) return fail("cudaMalloc(framebuffer)", cudaErrorMemoryAllocation);
        mirrors.push_back(m);
    }
    auto mirrorOf = [&](PFframebuffer *fb) { return mirrors[std::find(used.begin(), used.end(), fb) - used.begin()]; };

    // --- staging: states, segments, explicit items, targets join the block --------
    const size_t nStates = r->states.size(), nSegs = r->segs.size();
    int64_t statesOff = r->staging.alloc(nStates * sizeof(PFDrawState));
    int64_t segsOff = r->staging.alloc(nSegs * sizeof(PFSegment));
    size_t nTargetsTotal = 0;
    for (auto &o : ops) if (o.kind == 0) nTargetsTotal += o.targets.size();
    int64_t targetsOff = r->staging.alloc(std::max<size_t>(nTargetsTotal, 1) * sizeof(PFTarget));
    for (auto &rec : r->segs) {
        if (!rec.records.empty()) {
            rec.recordsOff = r->staging.alloc(rec.records.size() * sizeof(PFVertexIn));
            std::memcpy(r->staging.base + rec.recordsOff, rec.records.data(), rec.records.size() * sizeof(PFVertexIn));
            rec.seg.nVerts = (uint32_t)rec.records.size();
        }
        if (rec.seg.itemKind == PF_ITEMS_EXPLICIT) {
            rec.itemsOff = r->staging.alloc(rec.explicitItems.size() * 4 + 16);
            if (!rec.explicitItems.empty())
                std::memcpy(r->staging.base + rec.itemsOff, rec.explicitItems.data(), rec.explicitItems.size() * 4);
            rec.seg.nItems = (uint32_t)(rec.explicitItems.size() / 4);
        }
        if (!rec.prebuilt.empty()) {
            rec.prebuiltOff = r->staging.alloc(rec.prebuilt.size() * sizeof(PFPrim));
            std::memcpy(r->staging.base + rec.prebuiltOff, rec.prebuilt.data(), rec.prebuilt.size() * sizeof(PFPrim));
        }
    }
    const size_t total = r->staging.used;
    if (!r->arena.ensure(total)) { r->devStatus |= PF_DEVICE_ALLOC_FAIL; return fail("cudaMalloc(arena)", cudaErrorMemoryAllocation); }
    uint8_t *dbase = (uint8_t *)r->arena.p;
    auto dptr = [&](int64_t off) -> const void * {
        if (off < -1) return (const void *)(uintptr_t)(-off);    // uploaded at record time
        return off < 0 ? nullptr : (const void *)(dbase + off);
    };
    PFDrawState *hs = (PFDrawState *)(r->staging.base + statesOff);
    for (size_t i = 0; i < nStates; i++) {
        hs[i] = r->states[i].st;
        hs[i].tex = (const uint32_t *)dptr(r->states[i].texOff);
    }
    PFSegment *hseg = (PFSegment *)(r->staging.base + segsOff);
    PFTarget *htg = (PFTarget *)(r->staging.base + targetsOff);
    for (size_t i = 0; i < nSegs; i++) {
        SegRec &rec = r->segs[i];
        PFSegment s = rec.seg;
        s.records = (const PFVertexIn *)dptr(rec.recordsOff);
        s.pos = (const float *)dptr(rec.posOff);
        s.nrm = (const float *)dptr(rec.nrmOff);
        s.uv = (const float *)dptr(rec.uvOff);
        s.col = (const uint8_t *)dptr(rec.colOff);
        s.idx = (const uint32_t *)dptr(rec.idxOff);
        s.explicitItems = (const int32_t *)dptr(rec.itemsOff);
        s.prebuilt = dptr(rec.prebuiltOff);
        if (!rec.blitSrc.empty()) {
            PFPrim *pp = (PFPrim *)(r->staging.base + rec.prebuiltOff);
            for (auto &bs : rec.blitSrc) pp[bs.first].src = (uint64_t)(uintptr_t)dptr(bs.second);
        }
        hseg[i] = s;
    }
    // per batch: vertex / item bases, targets, tile numbering
    uint32_t maxVerts = 0, maxItems = 0, maxTiles = 0;
    bool anyPhong = false, anyRows = false;
    std::vector<PFBatchLaunch> launches(ops.size());
    size_t tgCursor = 0;
    for (size_t oi = 0; oi < ops.size(); oi++) {
        FlushOp &o = ops[oi];
        if (o.kind != 0) continue;
        PFBatchLaunch &L = launches[oi];
        L = PFBatchLaunch{};
        if (o.targets.size() > 1) {
            // the raster's work queue hands out tiles in target order: put the
            // targets with the most triangles first, so that their (longest)
            // tiles do not start last
            std::vector<uint64_t> load(o.targets.size(), 0);
            for (int si = o.segBegin; si < o.segEnd; si++)
                load[std::find(o.targets.begin(), o.targets.end(), r->segs[si].fb) - o.targets.begin()] += hseg[si].nItems;
            std::vector<size_t> perm(o.targets.size());
            for (size_t k = 0; k < perm.size(); k++) perm[k] = k;
            std::stable_sort(perm.begin(), perm.end(), [&](size_t x, size_t y) { return load[x] > load[y]; });
            std::vector<PFframebuffer *> tg(perm.size());
            std::vector<int> cl(perm.size());
            for (size_t k = 0; k < perm.size(); k++) { tg[k] = o.targets[perm[k]]; cl[k] = o.clearCmd[perm[k]]; }
            o.targets.swap(tg);
            o.clearCmd.swap(cl);
        }
        uint32_t v = 0, it = 0, tiles = 0;
        for (int si = o.segBegin; si < o.segEnd; si++) {
            hseg[si].vtxBase = v; hseg[si].itemBase = it;
            v += hseg[si].nVerts; it += hseg[si].nItems;
            PFframebuffer *fb = r->segs[si].fb;
            hseg[si].target = (int32_t)(std::find(o.targets.begin(), o.targets.end(), fb) - o.targets.begin());
            if (hs[hseg[si].state].flags & PFS_PHONG) anyPhong = true;
        }
        for (size_t k = 0; k < o.targets.size(); k++) {
            FBMirror *m = mirrorOf(o.targets[k]);
            PFTarget &T = htg[tgCursor + k];
            std::memset(&T, 0, sizeof T);
            T.color = m->dColor; T.depth = m->dDepth; T.fmt = m->fmt;
            if (m->fmt != PFF_RGBA8) L.generic = 1;
            T.W = (uint32_t)m->w; T.H = (uint32_t)m->h;
            T.tilesX = (T.W + PF_TILE - 1) / PF_TILE; T.tilesY = (T.H + PF_TILE - 1) / PF_TILE;
            T.tileBase = tiles;
            tiles += T.tilesX * T.tilesY;
            if (m->fmt == PFF_BGRA8) {                                            // row by row (k_rows)
                L.rowCount += T.H; L.rowMaxW = std::max(L.rowMaxW, T.W); anyRows = true;
            }
            if (o.clearCmd[k] >= 0) {
                const Cmd &cl = cmds[o.clearCmd[k]];
                T.clearMode = (cl.kind == CMD_FILL) ? 2 : 1; T.clearDepth = cl.depth;
                clear_raw(m->fmt, cl, T.clearRaw);
            }
        }
        L.segs = (const PFSegment *)(dbase + segsOff) + o.segBegin;
        L.nSegs = o.segEnd - o.segBegin;
        L.states = (const PFDrawState *)(dbase + statesOff);
        L.targets = (const PFTarget *)(dbase + targetsOff) + tgCursor;
        L.nTargets = (int)o.targets.size();
        L.totalTiles = tiles;
        L.nVerts = v; L.nItems = it;
        L.command = (uint32_t)oi;
        tgCursor += o.targets.size();
        maxVerts = std::max(maxVerts, v); maxItems = std::max(maxItems, it); maxTiles = std::max(maxTiles, tiles);
    }
    cudaError_t e = cudaMemcpyAsync(dbase, r->staging.base, total, cudaMemcpyHostToDevice, st);
    settle_pinned(r);                               // (a flush inside a drawing call)
    if (e == cudaSuccess && r->upBytes) {            // the record-time uploads come first
        e = cudaEventRecord(r->upDone, r->upStream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, r->upDone, 0);
    }
    if (e != cudaSuccess) return fail("cudaMemcpyAsync(staging)", e);

    // --- framebuffers: bring host content to the device unless the first
    //     operation touching a framebuffer overwrites it --------------------------
    for (size_t u = 0; u < used.size(); u++) {
        PFframebuffer *fb = used[u];
        FBMirror *m = mirrors[u];
        const size_t n = m->w * m->h;
        const Cmd *first = nullptr;
        for (auto &cmd : cmds) if (cmd.fb == fb) { first = &cmd; break; }
        const bool uploadDepth = m->depthUserVisible || !m->depthOnDevice;
        if (first->kind == CMD_FILL) {
            // every pixel is overwritten first
        } else if (first->kind == CMD_CLEAR) {
            // the clear leaves pixels 0..7 (and reads pixel 0 for the tail;
            // the packed 16-bit formats keep their tail, see k_clear)
            const size_t k = std::min<size_t>(8, n);
            cudaMemcpyAsync(m->dColor, m->tex->pixels, k * m->bpp, cudaMemcpyHostToDevice, st);
            const size_t aligned = n - n % 8;
            if (m->bpp == 2 && aligned < n && aligned >= k)
                cudaMemcpyAsync((uint8_t *)m->dColor + aligned * 2, (const uint8_t *)m->tex->pixels + aligned * 2,
                                (n - aligned) * 2, cudaMemcpyHostToDevice, st);
            if (uploadDepth) cudaMemcpyAsync(m->dDepth, m->hostDepth, k * 4, cudaMemcpyHostToDevice, st);
        } else {
            cudaMemcpyAsync(m->dColor, m->tex->pixels, n * m->bpp, cudaMemcpyHostToDevice, st);
            if (uploadDepth) cudaMemcpyAsync(m->dDepth, m->hostDepth, n * 4, cudaMemcpyHostToDevice, st);
        }
        m->depthOnDevice = true;
    }

    PFDevCounters *dcnt = (PFDevCounters *)r->counters.p;
    uint32_t startOp = 0;
    r->lastOps.clear();
    for (void *q : r->splitMem) cudaFree(q);
    r->splitMem.clear();
    // Host copies of the segments and targets of each draw group, for
    // splitting a group whose tile bins exceed the largest capacity.
    std::vector<std::vector<PFSegment>> opSegs(ops.size());
    std::vector<std::vector<PFTarget>> opTargets(ops.size());
    {
        size_t tc = 0;
        for (size_t oi = 0; oi < ops.size(); oi++) {
            if (ops[oi].kind != 0) continue;
            opSegs[oi].assign(hseg + ops[oi].segBegin, hseg + ops[oi].segEnd);
            opTargets[oi].assign(htg + tc, htg + tc + ops[oi].targets.size());
            tc += ops[oi].targets.size();
        }
    }
    // Split draw group oi into two passes of half its items each; the second
    // pass starts from the first one's framebuffers (no fused clear).
    auto split_op = [&](size_t oi) -> bool {
        const std::vector<PFSegment> S = opSegs[oi];
        uint64_t N = 0;
        for (auto &sg : S) N += sg.nItems;
        if (ops[oi].kind != 0 || N < 2) return false;
        const uint64_t half = N / 2;
        std::vector<PFSegment> A, B;
        uint64_t acc = 0;
        for (const PFSegment &sg : S) {
            if (acc + sg.nItems <= half) A.push_back(sg);
            else if (acc >= half) B.push_back(sg);
            else {
                const uint32_t h = (uint32_t)(half - acc);
                PFSegment a = sg, b = sg;
                a.nItems = h;
                b.itemSkip = sg.itemSkip + h; b.nItems = sg.nItems - h;
                A.push_back(a); B.push_back(b);
            }
            acc += sg.nItems;
        }
        std::vector<PFTarget> TA = opTargets[oi], TB = opTargets[oi];
        for (auto &t : TB) t.clearMode = 0;
        PFBatchLaunch LA = launches[oi], LB = launches[oi];
        auto place = [&](std::vector<PFSegment> &segs, std::vector<PFTarget> &tg, PFBatchLaunch &L) -> bool {
            uint32_t v = 0, it = 0;
            for (auto &sg : segs) { sg.vtxBase = v; sg.itemBase = it; v += sg.nVerts; it += sg.nItems; }
            const size_t sb = segs.size() * sizeof(PFSegment), tb = tg.size() * sizeof(PFTarget);
            void *mem = nullptr;
            if (cudaMalloc(&mem, sb + tb) != cudaSuccess) { cudaGetLastError(); return false; }
            r->splitMem.push_back(mem);
            if (cudaMemcpyAsync(mem, segs.data(), sb, cudaMemcpyHostToDevice, st) != cudaSuccess ||
                cudaMemcpyAsync((uint8_t *)mem + sb, tg.data(), tb, cudaMemcpyHostToDevice, st) != cudaSuccess) {
                cudaGetLastError();
                return false;
            }
            L.segs = (const PFSegment *)mem; L.nSegs = (int)segs.size();
            L.targets = (const PFTarget *)((uint8_t *)mem + sb);
            L.nVerts = v; L.nItems = it;
            return true;
        };
        if (!place(A, TA, LA) || !place(B, TB, LB)) return false;
        ops.insert(ops.begin() + (long)oi + 1, ops[oi]);
        launches[oi] = LA;
        launches.insert(launches.begin() + (long)oi + 1, LB);
        opSegs[oi] = A; opSegs.insert(opSegs.begin() + (long)oi + 1, B);
        opTargets[oi] = TA; opTargets.insert(opTargets.begin() + (long)oi + 1, TB);
        for (size_t j = oi; j < launches.size(); j++) launches[j].command = (uint32_t)j;
        r->stats.draw_splits += 1;
        return true;
    };
    for (int attempt = 0;; attempt++) {
        if (!r->vout.ensure((size_t)maxVerts * sizeof(PFVertexOut) + 64) ||
            !r->prims.ensure((size_t)maxItems * sizeof(PFPrim) + 128) ||
            !r->primsPh.ensure(anyPhong ? (size_t)maxItems * sizeof(PFPrimPhong) + 128 : 128) ||
            !r->pool.ensure((size_t)r->poolCap * sizeof(PFPrim)) ||
            !r->poolPh.ensure(anyPhong ? (size_t)r->poolCap * sizeof(PFPrimPhong) : 128) ||
            !r->binCount.ensure((size_t)(((size_t)maxTiles + 31) & ~(size_t)31) * 4 * (2 + PF_HEAVY_LEVELS)) ||   // bin counters, tile lists
            !r->bins.ensure((size_t)maxTiles * r->cap * 4 + 64) ||
            !r->rowInfo.ensure(anyRows ? (size_t)maxItems * sizeof(uint64_t) + 64 : 64) ||
            !r->rowGroup.ensure(anyRows ? ((size_t)maxItems / 32 + 8) * sizeof(uint64_t) : 64)) {   // every k_items warp
            r->devStatus |= PF_DEVICE_ALLOC_FAIL;
            return fail("cudaMalloc(scratch)", cudaErrorMemoryAllocation);
        }
        PFDevCounters init{};
        init.abortCommand = 0xffffffffu;
        *r->hostCounters = init;
        e = cudaMemcpyAsync(dcnt, r->hostCounters, sizeof(PFDevCounters), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return fail("cudaMemcpyAsync(counters)", e);
        size_t nRaster = 0;
        if (r->timing) {
            if (!r->evStart) { cudaEventCreate(&r->evStart); cudaEventCreate(&r->evEnd); }
            cudaEventRecord(r->evStart, st);
        }
        std::vector<Renderer::Op> doneOps;
        for (size_t oi = startOp; oi < ops.size(); oi++) {
            const FlushOp &o = ops[oi];
            Renderer::Op rop{};
            rop.kind = o.kind; rop.cmd = (int)oi;
            if (o.kind == 1 || o.kind == 2) {
                const Cmd &cmd = cmds[o.cmd];
                FBMirror *m = mirrorOf(cmd.fb);
                rop.n = m->w * m->h; rop.color = m->dColor; rop.fmt = m->fmt; rop.depth = m->dDepth;
                clear_raw(m->fmt, cmd, rop.cc);
                rop.cd = cmd.depth; rop.all = cmd.kind == CMD_FILL; rop.hook = cmd.hook; rop.hp = cmd.hp;
                rop.hp.width = (uint32_t)m->w;
                r->stats.kernel_launches += 1;
                e = (o.kind == 1) ? pfd_launch_clear(rop.color, rop.fmt, rop.depth, rop.n, rop.cc, rop.cd, rop.all, dcnt, (uint32_t)oi, st)
                                  : pfd_launch_hook(rop.color, rop.fmt, rop.depth, rop.n, rop.hook, rop.hp, dcnt, (uint32_t)oi, st);
            } else {
                PFBatchLaunch L = launches[oi];
                L.vout = (PFVertexOut *)r->vout.p;
                L.prims = (PFPrim *)r->prims.p; L.primsPh = (PFPrimPhong *)r->primsPh.p;
                L.pool = (PFPrim *)r->pool.p; L.poolPh = (PFPrimPhong *)r->poolPh.p; L.poolCap = r->poolCap;
                L.binCount = (uint32_t *)r->binCount.p; L.bins = (uint32_t *)r->bins.p; L.cap = r->cap;
                L.listStride = (uint32_t)(((size_t)maxTiles + 31) & ~(size_t)31);
                L.tileList = (uint32_t *)r->binCount.p + L.listStride;
                L.rasterCtasPerSM = r->rasterCtasPerSM;
                L.rasterWarps = r->rasterWarps;
                L.anyPhong = anyPhong ? 1 : 0;
                L.rowInfo = L.rowCount ? (uint64_t *)r->rowInfo.p : nullptr;
                L.rowGroup = L.rowCount ? (uint64_t *)r->rowGroup.p : nullptr;
                L.cnt = dcnt;
                rop.L = L;
                r->stats.kernel_launches += L.rowCount ? 5 : 4;
                e = pfd_launch_vertex(L, st);
                if (e == cudaSuccess) e = pfd_launch_items(L, st);
                if (e == cudaSuccess) e = pfd_launch_binsort(L, st);
                if (r->timing) {
                    if (r->rasterEv.size() <= nRaster) {
                        cudaEvent_t ev0, ev1; cudaEventCreate(&ev0); cudaEventCreate(&ev1);
                        r->rasterEv.push_back({ ev0, ev1 });
                    }
                    cudaEventRecord(r->rasterEv[nRaster].first, st);
                }
                if (e == cudaSuccess) e = pfd_launch_raster(L, st);
                if (r->timing) cudaEventRecord(r->rasterEv[nRaster].second, st);
                nRaster++;
            }
            if (e != cudaSuccess) return fail("kernel launch", e);
            doneOps.push_back(rop);
        }
        if (r->timing) cudaEventRecord(r->evEnd, st);
        e = cudaMemcpyAsync(r->hostCounters, dcnt, sizeof(PFDevCounters), cudaMemcpyDeviceToHost, st);
        // write back colour (and user-visible depth); if a bin overflowed the
        // replay below writes back again
        for (FBMirror *m : mirrors) {
            if (e != cudaSuccess) break;
            const size_t n = m->w * m->h;
            e = cudaMemcpyAsync(m->tex->pixels, m->dColor, n * m->bpp, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess && m->depthUserVisible)
                e = cudaMemcpyAsync(m->hostDepth, m->dDepth, n * 4, cudaMemcpyDeviceToHost, st);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return fail("pipeline", e);
        if (r->timing) {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, r->evStart, r->evEnd);
            r->stats.device_ms += ms;
            for (size_t k = 0; k < nRaster; k++) {
                cudaEventElapsedTime(&ms, r->rasterEv[k].first, r->rasterEv[k].second);
                r->stats.raster_ms += ms;
            }
        }
        r->stats.raster_launches += nRaster;
        const PFDevCounters hc = *r->hostCounters;
        if (hc.status & PFD_BOUNDS) r->devStatus |= PF_DEVICE_INDEX_RANGE;
        r->stats.fragments += hc.fragments;
        r->stats.rasterized += hc.rasterized;
        if (hc.abortCommand == 0xffffffffu) {
            r->lastOps.insert(r->lastOps.end(), doneOps.begin(), doneOps.end());
            break;
        }
        // A bin or the clip pool overflowed in operation hc.abortCommand.  The
        // operations before it completed; it and every later one wrote nothing
        // to any framebuffer.  Grow the capacity and resume from it.
        for (auto &d : doneOps) if ((uint32_t)d.cmd < hc.abortCommand) r->lastOps.push_back(d);
        r->stats.bin_overflows += 1;
        if (hc.status & PFD_BIN_OVERFLOW) {
            uint32_t need = std::max(hc.maxBin, r->cap * 2);
            uint32_t nc = 1; while (nc < need) nc <<= 1;
            if (nc > kCapMax) {
                // more sub-triangles in one tile than a bin can sort: render
                // the draw group in two passes of half its items each
                if (!split_op(hc.abortCommand)) {
                    r->devStatus |= PF_DEVICE_BIN_LIMIT;
                    return fail("tile bin capacity", cudaErrorMemoryAllocation);
                }
                nc = kCapMax;
            }
            r->cap = nc;
        }
        if (hc.status & PFD_CLIP_OVERFLOW) r->poolCap = std::max(r->poolCap * 4, hc.clipCount * 2);
        if (attempt > 64) return fail("overflow retries", cudaErrorUnknown);
        startOp = hc.abortCommand;
    }
    r->stats.flushes += 1;
    r->graphValid = false;      // a new flush: a replay graph must be captured again
    discard_recording(r);
    return true;
}

bool flush(Ctx *c) { return flush(c->rend); }

// Bring a main framebuffer's internal depth back to the host (it stays on
// the device otherwise: the reference exposes it only to pfPostProcess).
void pull_main_depth(Ctx *c)
{
    FBMirror *m = find_mirror(c->mainFB.texture);
    if (!m || !m->depthOnDevice) return;
    cudaMemcpy(m->hostDepth, m->dDepth, m->w * m->h * 4, cudaMemcpyDeviceToHost);
    m->depthOnDevice = false;    // host copy authoritative again
}

void sync_host(Ctx *c) { flush(c); }

// Re-run the device work of the renderer's last flush (inputs already on the
// device) `n` times from a CUDA graph; returns the mean GPU ms per run.
float replay(Renderer *r, uint32_t n)
{
    if (!r->devOk || r->lastOps.empty() || n == 0) return -1.0f;
    cudaStream_t st = r->stream;
    PFDevCounters *dcnt = (PFDevCounters *)r->counters.p;
    if (!r->graphValid) {
        if (r->graph) { cudaGraphExecDestroy(r->graph); r->graph = nullptr; }
        PFDevCounters init{};
        init.abortCommand = 0xffffffffu;
        *r->hostCounters = init;
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { cudaGetLastError(); return -1.0f; }
        cudaMemcpyAsync(dcnt, r->hostCounters, sizeof(PFDevCounters), cudaMemcpyHostToDevice, st);
        for (const auto &op : r->lastOps) {
            if (op.kind == 1) pfd_launch_clear(op.color, op.fmt, op.depth, op.n, op.cc, op.cd, op.all, dcnt, (uint32_t)op.cmd, st);
            else if (op.kind == 2) pfd_launch_hook(op.color, op.fmt, op.depth, op.n, op.hook, op.hp, dcnt, (uint32_t)op.cmd, st);
            else {
                pfd_launch_vertex(op.L, st);
                pfd_launch_items(op.L, st);
                pfd_launch_binsort(op.L, st);
                pfd_launch_raster(op.L, st);
            }
        }
        cudaError_t e = cudaStreamEndCapture(st, &g);
        if (e != cudaSuccess || !g) { cudaGetLastError(); return -1.0f; }
        e = cudaGraphInstantiate(&r->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { cudaGetLastError(); r->graph = nullptr; return -1.0f; }
        r->graphValid = true;
        cudaGraphLaunch(r->graph, st);                     // warm
        cudaStreamSynchronize(st);
    }
    cudaEvent_t a, b;
    cudaEventCreate(&a); cudaEventCreate(&b);
    cudaEventRecord(a, st);
    for (uint32_t i = 0; i < n; i++) cudaGraphLaunch(r->graph, st);
    cudaEventRecord(b, st);
    cudaError_t e = cudaEventSynchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a); cudaEventDestroy(b);
    if (e != cudaSuccess) { cudaGetLastError(); return -1.0f; }
    return ms / (float)n;
}

}  // namespace

// ===========================================================================
// C API
// ===========================================================================
// Getters (getter.c:24-521): the same cases as the reference; any other
// name sets PF_INVALID_ENUM and leaves the output untouched.
static const double kInv255 = 1.0 / 255;

template <typename T>
static bool get_real(PFenum p, T *v, T inv255)                           // getter.c:235-491
{
    switch (p) {
    case PF_COLOR_CLEAR_VALUE:
        v[0] = G->clearColor.r * inv255; v[1] = G->clearColor.g * inv255;
        v[2] = G->clearColor.b * inv255; v[3] = G->clearColor.a * inv255; return true;
    case PF_DEPTH_CLEAR_VALUE: v[0] = G->clearDepth; return true;
    case PF_CURRENT_COLOR:
        v[0] = G->curColor.r * inv255; v[1] = G->curColor.g * inv255;
        v[2] = G->curColor.b * inv255; v[3] = G->curColor.a * inv255; return true;
    case PF_CURRENT_NORMAL: for (int i = 0; i < 3; i++) v[i] = G->curNormal[i]; return true;
    case PF_CURRENT_TEXTURE_COORDS: for (int i = 0; i < 2; i++) v[i] = G->curTex[i]; return true;
    case PF_CURRENT_RASTER_POSITION: v[0] = G->rasterPos[0]; v[1] = G->rasterPos[1]; return true;
    case PF_POINT_SIZE: v[0] = G->pointSize; return true;
    case PF_LINE_WIDTH: v[0] = G->lineWidth; return true;
    case PF_PROJECTION_MATRIX: for (int i = 0; i < 16; i++) v[i] = G->proj[i]; return true;
    case PF_MODELVIEW_MATRIX: {
        Mat mv; m_mul(mv, G->model, G->view);
        for (int i = 0; i < 16; i++) v[i] = mv[i];
        return true;
    }
    case PF_TEXTURE_MATRIX: for (int i = 0; i < 16; i++) v[i] = G->tex[i]; return true;
    case PF_ZOOM_X: v[0] = G->pixelZoom[0]; return true;
    case PF_ZOOM_Y: v[0] = G->pixelZoom[1]; return true;
    default: G->err = PF_INVALID_ENUM; return false;
    }
}

extern "C" {

PFcontext pfCreateContext(void *buf, PFsizei w, PFsizei h, PFpixelformat f, PFdatatype t)
{
    Ctx *c = new Ctx();
    Ctx *prev = G; G = c;
    c->mainFB.texture = tex_new(buf, w, h, f, t, false);
    G = prev;
    if (!c->mainFB.texture) { delete c; return nullptr; }
    ((Tex *)c->mainFB.texture)->isMain = true;
    c->mainFB.zbuffer = (float *)std::malloc((size_t)w * h * sizeof(float));
    if (!c->mainFB.zbuffer) { delete (Tex *)c->mainFB.texture; delete c; return nullptr; }
    if (gBatch) { c->rend = &gBatch->r; gBatch->members.push_back(c); }
    for (size_t i = 0; i < (size_t)w * h; i++) c->mainFB.zbuffer[i] = FLT_MAX;
    c->current = &c->mainFB;
    c->vpDim[0] = w - 1; c->vpMax[0] = (PFint)w - 1;
    c->vpDim[1] = h - 1; c->vpMax[1] = (PFint)h - 1;
    std::memset(c->proj, 0, 64);                                     // pfmMat4Ortho(-1,1,-1,1,-1,1)
    c->proj[0] = 2.0f / 2.0f; c->proj[5] = 2.0f / 2.0f; c->proj[10] = -2.0f / 2.0f;
    c->proj[12] = -(-1.0f + 1.0f) / 2.0f; c->proj[13] = -(1.0f + -1.0f) / 2.0f;
    c->proj[14] = -(1.0f + -1.0f) / 2.0f; c->proj[15] = 1.0f;
    m_identity(c->tex); m_identity(c->normal); m_identity(c->model); m_identity(c->view); m_identity(c->mvp);
    c->cur = c->view;
    std::memset(c->slots, 0, sizeof c->slots);
    return c;
}

void pfDeleteContext(PFcontext ctx)
{
    Ctx *c = (Ctx *)ctx;
    if (!c) return;
    Ctx *prev = G; G = c;
    flush(c);
    G = (prev == c) ? nullptr : prev;
    if (gBatch) {
        auto &mm = gBatch->members;
        mm.erase(std::remove(mm.begin(), mm.end(), c), mm.end());
    }
    drop_mirror(c->mainFB.texture);
    release_renderer(&c->own);
    std::free(c->mainFB.zbuffer);
    delete (Tex *)c->mainFB.texture;
    delete c;
}

void pfSetMainBuffer(void *buf, PFsizei w, PFsizei h, PFpixelformat f, PFdatatype t)
{
    if (!buf || !w || !h) { G->err = PF_INVALID_VALUE; return; }
    if (fb_code(f, t) < 0) { G->err = PF_INVALID_ENUM; return; }   // the main buffer stays as it was
    flush(G);
    pull_main_depth(G);
    Tex *old = (Tex *)G->mainFB.texture;
    if (old->w != w || old->h != h) {
        std::free(G->mainFB.zbuffer);
        G->mainFB.zbuffer = (float *)std::malloc((size_t)w * h * sizeof(float));
        for (size_t i = 0; i < (size_t)w * h; i++) G->mainFB.zbuffer[i] = G->clearDepth;
    }
    drop_mirror(old);
    delete old;
    G->mainFB.texture = tex_new(buf, w, h, f, t, false);
    if (G->mainFB.texture) ((Tex *)G->mainFB.texture)->isMain = true;
    G->aux = nullptr;
}

void pfSetAuxBuffer(void *aux) { G->aux = aux; }

void pfSwapBuffers(void)
{
    if (!G->aux) { G->err = PF_INVALID_OPERATION; return; }
    flush(G);
    Tex *t = (Tex *)G->current->texture;
    void *tmp = t->pixels; t->pixels = G->aux; G->aux = tmp;
}

PFcontext pfGetCurrentContext(void) { return G; }

void pfMakeCurrent(PFcontext ctx)
{
    Ctx *c = (Ctx *)ctx;
    // outside a batch, switching away is an observation point of the context
    if (G && G != c && !gBatch) flush(G);
    G = c;
    if (c && gBatch && c->rend != &gBatch->r) {
        flush(c);                                   // what it recorded alone renders first
        c->rend = &gBatch->r;
        c->openImmSeg = -1;
        gBatch->members.push_back(c);
    }
}

PFboolean pfIsEnabled(PFstate s) { return (G->state & s) != 0; }
void pfEnable(PFstate s)
{
    G->state |= s; G->stateDirty = true;
    if (s & PF_FRAMEBUFFER) G->current = G->bound ? G->bound : &G->mainFB;
}
void pfDisable(PFstate s)
{
    G->state &= ~(PFuint)s; G->stateDirty = true;
    if (s & PF_FRAMEBUFFER) G->current = &G->mainFB;
}

PFerrcode pfGetError(void) { PFerrcode e = G->err; G->err = PF_NO_ERROR; return e; }

void pfGetBooleanv(PFenum p, PFboolean *v)                            // getter.c:24-113
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
void pfGetIntegerv(PFenum p, PFint *v)                                // getter.c:115-233
{
    switch (p) {
    case PF_VIEWPORT: v[0] = G->vpPos[0]; v[1] = G->vpPos[1]; v[2] = (PFint)G->vpDim[0] + 1; v[3] = (PFint)G->vpDim[1] + 1; break;
    case PF_COLOR_CLEAR_VALUE: v[0] = G->clearColor.r; v[1] = G->clearColor.g; v[2] = G->clearColor.b; v[3] = G->clearColor.a; break;
    case PF_CULL_FACE_MODE: v[0] = G->cullFace; break;
    case PF_CURRENT_COLOR: v[0] = G->curColor.r; v[1] = G->curColor.g; v[2] = G->curColor.b; v[3] = G->curColor.a; break;
    case PF_CURRENT_RASTER_POSITION: v[0] = ftoi_x86(G->rasterPos[0]); v[1] = ftoi_x86(G->rasterPos[1]); break;
    case PF_POLYGON_MODE: v[0] = G->polygonMode[0]; v[1] = G->polygonMode[1]; break;
    case PF_MATRIX_MODE: v[0] = G->matMode; break;
    case PF_MAX_PROJECTION_STACK_DEPTH: v[0] = 2; break;
    case PF_MAX_MODELVIEW_STACK_DEPTH: v[0] = 8; break;
    case PF_MAX_TEXTURE_STACK_DEPTH: v[0] = 4; break;
    case PF_SHADE_MODEL: v[0] = G->shade; break;
    case PF_MAX_LIGHTS: v[0] = PF_MAX_LIGHTS; break;
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
void pfGetFloatv(PFenum p, PFfloat *v) { get_real<PFfloat>(p, v, (PFfloat)kInv255); }
void pfGetDoublev(PFenum p, PFdouble *v) { get_real<PFdouble>(p, v, kInv255); }
void pfGetPointerv(PFenum p, const void **v)                          // getter.c:493-521
{
    switch (p) {
    case PF_TEXTURE_2D: *v = G->texture; break;
    case PF_FRAMEBUFFER: *v = G->bound; break;
    // the reference returns the address of its internal function pointer
    case PF_BLEND_FUNC: *v = &G->blend; break;
    case PF_DEPTH_FUNC: *v = &G->depthFunc; break;
    default: G->err = PF_INVALID_ENUM; break;
    }
}

// --- matrices (context.c:392-548) -------------------------------------------
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
        std::memcpy(G->stackProj[G->nProj++], G->proj, 64); break;
    case PF_MODELVIEW:
        if (G->nMV >= 8) { G->err = PF_STACK_OVERFLOW; return; }
        if (G->modelUsed) std::memcpy(G->stackMV[G->nMV++], G->model, 64);
        else { G->cur = G->model; G->modelUsed = true; }
        break;
    case PF_TEXTURE:
        if (G->nTex >= 4) { G->err = PF_STACK_OVERFLOW; return; }
        std::memcpy(G->stackTex[G->nTex++], G->tex, 64); break;
    }
}
void pfPopMatrix(void)
{
    switch (G->matMode) {
    case PF_PROJECTION:
        if (G->nProj == 0) { G->err = PF_STACK_UNDERFLOW; return; }
        std::memcpy(G->proj, G->stackProj[--G->nProj], 64); break;
    case PF_MODELVIEW:
        if (G->nMV == 0) {
            if (!G->modelUsed) { G->err = PF_STACK_UNDERFLOW; return; }
            m_identity(G->model); G->modelUsed = false; G->cur = G->view;
        } else std::memcpy(G->model, G->stackMV[--G->nMV], 64);
        break;
    case PF_TEXTURE:
        if (G->nTex == 0) { G->err = PF_STACK_UNDERFLOW; return; }
        std::memcpy(G->tex, G->stackTex[--G->nTex], 64); break;
    }
}
void pfLoadIdentity(void) { m_identity(G->cur); G->stateDirty = true; }
void pfTranslatef(PFfloat x, PFfloat y, PFfloat z)
{
    float t[16]; m_identity(t); t[12] = x; t[13] = y; t[14] = z;
    m_mul(G->cur, t, G->cur); G->stateDirty = true;
}
void pfRotatef(PFfloat angle, PFfloat x, PFfloat y, PFfloat z)        // pfm.h:2227-2262
{
    float a = (float)(angle * kDeg2Rad);
    float r[16]; m_identity(r);
    float lsq = x*x + y*y + z*z;
    if (lsq != 1.0f && lsq != 0.0f) { float il = 1.0f / std::sqrt(lsq); x *= il; y *= il; z *= il; }
    float s = sinf(a), co = cosf(a), t = 1.0f - co;
    r[0] = x*x*t + co; r[1] = y*x*t + z*s; r[2] = z*x*t - y*s;
    r[4] = x*y*t - z*s; r[5] = y*y*t + co; r[6] = z*y*t + x*s;
    r[8] = x*z*t + y*s; r[9] = y*z*t - x*s; r[10] = z*z*t + co;
    m_mul(G->cur, r, G->cur); G->stateDirty = true;
}
void pfScalef(PFfloat x, PFfloat y, PFfloat z)
{
    float s[16]; std::memset(s, 0, 64); s[0] = x; s[5] = y; s[10] = z; s[15] = 1.0f;
    m_mul(G->cur, s, G->cur); G->stateDirty = true;
}
void pfMultMatrixf(const PFfloat *m) { m_mul(G->cur, G->cur, m); G->stateDirty = true; }
void pfFrustum(PFfloat l, PFfloat r, PFfloat b, PFfloat t, PFfloat n, PFfloat f)   // pfm.h:2375-2393
{
    float m[16]; std::memset(m, 0, 64);
    float rl = r - l, tb = t - b, fn = f - n;
    m[0] = (n*2.0f)/rl; m[5] = (n*2.0f)/tb; m[8] = (r + l)/rl; m[9] = (t + b)/tb;
    m[10] = -(f + n)/fn; m[11] = -1.0f; m[14] = -(f*n*2.0f)/fn;
    m_mul(G->cur, G->cur, m); G->stateDirty = true;
}
void pfOrtho(PFfloat l, PFfloat r, PFfloat b, PFfloat t, PFfloat n, PFfloat f)     // pfm.h:2422-2440
{
    float m[16]; std::memset(m, 0, 64);
    float rl = r - l, tb = t - b, fn = f - n;
    m[0] = 2.0f/rl; m[5] = 2.0f/tb; m[10] = -2.0f/fn;
    m[12] = -(l + r)/rl; m[13] = -(t + b)/tb; m[14] = -(f + n)/fn; m[15] = 1.0f;
    m_mul(G->cur, G->cur, m); G->stateDirty = true;
}

// --- render configuration (context.c:553-797) --------------------------------
void pfViewport(PFint x, PFint y, PFsizei w, PFsizei h)
{
    if (x <= -(PFint)w || y <= -(PFint)h) { G->err = PF_INVALID_OPERATION; return; }
    Tex *mt = (Tex *)G->mainFB.texture;
    G->vpPos[0] = x; G->vpPos[1] = y; G->vpDim[0] = w - 1; G->vpDim[1] = h - 1;
    G->vpMin[0] = std::max(x, 0); G->vpMin[1] = std::max(y, 0);
    G->vpMax[0] = (PFint)std::min((PFsizei)(x + (PFint)w), mt->w - 1);
    G->vpMax[1] = (PFint)std::min((PFsizei)(y + (PFint)h), mt->h - 1);
    G->stateDirty = true;
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
void pfShadeModel(PFshademode m) { G->shade = m; G->stateDirty = true; }
void pfLightModel(PFlightmode m) { G->lightMode = m; G->stateDirty = true; }
void pfLineWidth(PFfloat w) { if (w <= 0.0f) { G->err = PF_INVALID_VALUE; return; } G->lineWidth = w; }
void pfPointSize(PFfloat s) { if (s <= 0.0f) { G->err = PF_INVALID_VALUE; return; } G->pointSize = s; }
void pfCullFace(PFface f)
{
    if (f < PF_FRONT || f > PF_BACK) { G->err = PF_INVALID_ENUM; return; }
    G->cullFace = f;
}
void pfBlendFunc(PFblendmode m)
{
    if (m < PF_BLEND_AVERAGE || m > PF_BLEND_DARKEN) { G->err = PF_INVALID_ENUM; return; }
    G->blend = m; G->stateDirty = true;
}
void pfDepthFunc(PFdepthmode m)
{
    if (m < PF_EQUAL || m > PF_GEQUAL) { G->err = PF_INVALID_ENUM; return; }
    G->depthFunc = m; G->stateDirty = true;
}
void pfDepthMask(PFboolean f) { G->depthMask = f; G->stateDirty = true; }
void pfBindFramebuffer(PFframebuffer *fb)
{
    G->bound = fb;
    if (G->state & PF_FRAMEBUFFER) G->current = fb ? fb : &G->mainFB;
    G->stateDirty = true;
}
void pfBindTexture(PFtexture t) { G->texture = (Tex *)t; G->stateDirty = true; }

void pfClear(PFclearflag flag)
{
    if (!flag) return;
    Cmd cmd{};
    cmd.kind = CMD_CLEAR; cmd.fb = G->current; cmd.color = pack(G->clearColor); cmd.depth = G->clearDepth;
    push_cmd(G, cmd);
}
void pfClearDepth(PFfloat d) { G->clearDepth = d; }
void pfClearColor(PFubyte r, PFubyte g, PFubyte b, PFubyte a) { G->clearColor = PFcolor{ r, g, b, a }; }

// --- lights and materials (context.c:802-1156) --------------------------------
void pfEnableLight(PFsizei l)
{
    if (l >= PF_MAX_LIGHTS) { G->err = PF_INVALID_VALUE; return; }
    for (int a : G->activeLights) if (a == (int)l) { G->err = PF_INVALID_OPERATION; return; }
    G->activeLights.push_back((int)l); G->stateDirty = true;
}
void pfDisableLight(PFsizei l)
{
    if (l >= PF_MAX_LIGHTS) { G->err = PF_INVALID_VALUE; return; }
    auto it = std::find(G->activeLights.begin(), G->activeLights.end(), (int)l);
    if (it == G->activeLights.end()) { G->err = PF_INVALID_OPERATION; return; }
    G->activeLights.erase(it); G->stateDirty = true;
}
PFboolean pfIsEnabledLight(PFsizei l)
{
    if (l >= PF_MAX_LIGHTS) { G->err = PF_INVALID_VALUE; return PF_FALSE; }
    return std::find(G->activeLights.begin(), G->activeLights.end(), (int)l) != G->activeLights.end();
}
static PFcolor f3_color(const float *v) { return PFcolor{ ftoub(v[0]*255.0f), ftoub(v[1]*255.0f), ftoub(v[2]*255.0f), 255 }; }
static bool cutoff_ok(float v) { return (v >= 0 && v <= 90) || v == 180; }
void pfLightf(PFsizei li, PFenum p, PFfloat v)
{
    if (li >= PF_MAX_LIGHTS) { G->err = PF_STACK_OVERFLOW; return; }
    Light &l = G->lights[li];
    switch (p) {
    case PF_SPOT_INNER_CUTOFF: if (cutoff_ok(v)) l.inner = cosf((float)(v * kDeg2Rad)); else G->err = PF_INVALID_VALUE; break;
    case PF_SPOT_OUTER_CUTOFF: if (cutoff_ok(v)) l.outer = cosf((float)(v * kDeg2Rad)); else G->err = PF_INVALID_VALUE; break;
    case PF_CONSTANT_ATTENUATION: l.attC = v; break;
    case PF_LINEAR_ATTENUATION: l.attL = v; break;
    case PF_QUADRATIC_ATTENUATION: l.attQ = v; break;
    default: G->err = PF_INVALID_ENUM; break;
    }
    G->stateDirty = true;
}
void pfLightfv(PFsizei li, PFenum p, const void *value)
{
    if (li >= PF_MAX_LIGHTS) { G->err = PF_STACK_OVERFLOW; return; }
    Light &l = G->lights[li];
    const float *v = (const float *)value;
    switch (p) {
    case PF_POSITION: std::memcpy(l.position, v, 12); break;
    case PF_SPOT_DIRECTION: std::memcpy(l.direction, v, 12); break;
    case PF_SPOT_INNER_CUTOFF: case PF_SPOT_OUTER_CUTOFF: case PF_CONSTANT_ATTENUATION:
    case PF_LINEAR_ATTENUATION: case PF_QUADRATIC_ATTENUATION: pfLightf(li, p, v[0]); break;
    case PF_AMBIENT: l.ambient = f3_color(v); break;
    case PF_DIFFUSE: l.diffuse = f3_color(v); break;
    case PF_SPECULAR: l.specular = f3_color(v); break;
    default: G->err = PF_INVALID_ENUM; break;
    }
    G->stateDirty = true;
}
static void mat_set(PFface f, PFenum p, const float *v)
{
    Material *a, *b;
    switch (f) {
    case PF_FRONT: a = b = &G->mat[0]; break;
    case PF_BACK: a = b = &G->mat[1]; break;
    case PF_FRONT_AND_BACK: a = &G->mat[0]; b = &G->mat[1]; break;
    default: G->err = PF_INVALID_ENUM; return;
    }
    PFcolor c = f3_color(v);
    switch (p) {
    case PF_AMBIENT: a->ambient = b->ambient = c; break;
    case PF_DIFFUSE: a->diffuse = b->diffuse = c; break;
    case PF_SPECULAR: a->specular = b->specular = c; break;
    case PF_EMISSION: a->emission = b->emission = c; break;
    case PF_SHININESS: a->shininess = b->shininess = v[0]; break;
    case PF_AMBIENT_AND_DIFFUSE: a->ambient = b->ambient = c; a->diffuse = b->diffuse = c; break;
    default: G->err = PF_INVALID_ENUM; return;
    }
    G->stateDirty = true;
}
void pfMaterialf(PFface f, PFenum p, PFfloat v) { float vv[3] = { v, v, v }; mat_set(f, p, vv); }
void pfMaterialfv(PFface f, PFenum p, const void *v) { mat_set(f, p, (const float *)v); }
void pfColorMaterial(PFface f, PFenum m)
{
    if (f < PF_FRONT || f > PF_FRONT_AND_BACK) { G->err = PF_INVALID_ENUM; return; }
    if (m < PF_AMBIENT_AND_DIFFUSE || m > PF_EMISSION) { G->err = PF_INVALID_ENUM; return; }
    G->colMatFace = f; G->colMatMode = m;
}

// --- vertex arrays and draws (context.c:1161-1575) ----------------------------
void pfVertexPointer(PFint size, PFenum type, PFsizei stride, const void *p)
{
    if (size < 2 || size > 4) { G->err = PF_INVALID_VALUE; return; }
    if (!(type == PF_SHORT || type == PF_INT || type == PF_FLOAT || type == PF_DOUBLE)) { G->err = PF_INVALID_ENUM; return; }
    G->positions = Attrib{ p, stride, size, type };
}
void pfNormalPointer(PFenum type, PFsizei stride, const void *p)
{
    if (!(type == PF_FLOAT || type == PF_DOUBLE)) { G->err = PF_INVALID_ENUM; return; }
    G->normals = Attrib{ p, stride, 3, type };
}
void pfTexCoordPointer(PFenum type, PFsizei stride, const void *p)
{
    if (!(type == PF_FLOAT || type == PF_DOUBLE)) { G->err = PF_INVALID_ENUM; return; }
    G->texcoords = Attrib{ p, stride, 2, type };
}
void pfColorPointer(PFint size, PFenum type, PFsizei stride, const void *p)
{
    if (size < 3 || size > 4) { G->err = PF_INVALID_VALUE; return; }
    if (!(type == PF_UNSIGNED_BYTE || type == PF_UNSIGNED_SHORT || type == PF_UNSIGNED_INT ||
          type == PF_FLOAT || type == PF_DOUBLE)) { G->err = PF_INVALID_ENUM; return; }
    G->colors = Attrib{ p, stride, size, type };
}

static float attr_f(const Attrib &a, size_t i)
{
    switch (a.type) {
    case PF_SHORT: return (float)((const PFshort *)a.buf)[i];
    case PF_INT: return (float)((const PFint *)a.buf)[i];
    case PF_FLOAT: return ((const PFfloat *)a.buf)[i];
    case PF_DOUBLE: return (float)((const PFdouble *)a.buf)[i];
    }
    return 0.0f;
}

// Snapshot `count` elements of one attribute array as floats (positions,
// normals, texcoords) starting at element `first`.
static int64_t stage_float_attr(Ctx *c, const Attrib &a, int comps, size_t first, size_t count)
{
    if (a.dev) return -(int64_t)(uintptr_t)((const float *)a.buf + first * comps);   // read in place at the flush
    if (a.type == PF_FLOAT) return snapshot(c, (const float *)a.buf + first * comps, count * comps * 4);
    int64_t off = c->rend->staging.alloc(count * comps * 4);
    float *dst = (float *)(c->rend->staging.base + off);
    for (size_t i = 0; i < count * comps; i++) dst[i] = attr_f(a, first * comps + i);
    return off;
}

static int64_t stage_color_attr(Ctx *c, const Attrib &a, size_t first, size_t count)
{
    const size_t k = (size_t)a.size;
    if (a.dev) return -(int64_t)(uintptr_t)((const uint8_t *)a.buf + first * k);
    if (a.type == PF_UNSIGNED_BYTE) return snapshot(c, (const uint8_t *)a.buf + first * k, count * k);
    int64_t off = c->rend->staging.alloc(count * k);
    uint8_t *dst = c->rend->staging.base + off;
    for (size_t i = 0; i < count * k; i++) {
        const size_t o = first * k + i;
        switch (a.type) {
        case PF_UNSIGNED_SHORT: dst[i] = (uint8_t)(((const PFushort *)a.buf)[o] >> 8); break;
        case PF_UNSIGNED_INT: dst[i] = (uint8_t)(((const PFuint *)a.buf)[o] >> 24); break;
        case PF_FLOAT: dst[i] = ftoub(((const PFfloat *)a.buf)[o] * 255); break;
        case PF_DOUBLE: dst[i] = dtoub(((const PFdouble *)a.buf)[o] * 255); break;
        }
    }
    return off;
}

// Colour component o of the colour array as the reference converts it.
static uint8_t color_comp(const Attrib &a, size_t o)
{
    switch (a.type) {
    case PF_UNSIGNED_BYTE: return ((const PFubyte *)a.buf)[o];
    case PF_UNSIGNED_SHORT: return (uint8_t)(((const PFushort *)a.buf)[o] >> 8);
    case PF_UNSIGNED_INT: return (uint8_t)(((const PFuint *)a.buf)[o] >> 24);
    case PF_FLOAT: return ftoub(((const PFfloat *)a.buf)[o] * 255);
    case PF_DOUBLE: return dtoub(((const PFdouble *)a.buf)[o] * 255);
    }
    return 0;
}

// A draw with points or lines (the modes, or a PF_POINT / PF_LINE polygon
// mode): the reference's slot assembly (context.c:1231-1300, 1415-1460) on
// the host, each element read into a vertex record; slots start zeroed with
// the current colour, and attributes whose array is off keep what the slot
// held.
static void assemble_arrays(Ctx *c, PFdrawmode mode, PFsizei count, const void *indices, PFdatatype itype, PFint first)
{
    const bool useT = (c->state & PF_TEXTURE_COORD_ARRAY) && c->texcoords.buf;
    const bool useN = (c->state & PF_NORMAL_ARRAY) && c->normals.buf;
    const bool useC = (c->state & PF_COLOR_ARRAY) && c->colors.buf;
    const PFsizei nv = mode_count(mode);
    PFVertexIn slots[6];
    std::memset(slots, 0, sizeof slots);
    for (PFVertexIn &v : slots) v.color = pack(c->curColor);
    PFsizei vc = 0;
    for (PFsizei i = 0; i < count; i++) {
        size_t j = (size_t)first + (size_t)i;
        if (indices) {
            if (itype == PF_UNSIGNED_BYTE) j = ((const uint8_t *)indices)[i];
            else if (itype == PF_UNSIGNED_SHORT) j = ((const uint16_t *)indices)[i];
            else j = ((const uint32_t *)indices)[i];
        }
        PFVertexIn &v = slots[vc++];
        v.pos[0] = v.pos[1] = v.pos[2] = 0.0f; v.pos[3] = 1.0f;
        const size_t ps = (size_t)c->positions.size;
        for (size_t k = 0; k < ps; k++) v.pos[k] = attr_f(c->positions, j * ps + k);
        if (useN) for (size_t k = 0; k < 3; k++) v.normal[k] = attr_f(c->normals, j * 3 + k);
        if (useT) for (size_t k = 0; k < 2; k++) v.uv[k] = attr_f(c->texcoords, j * 2 + k);
        if (useC) {
            uint8_t cb[4] = { 255, 255, 255, 255 };
            const size_t cs = (size_t)c->colors.size;
            for (size_t k = 0; k < cs; k++) cb[k] = color_comp(c->colors, j * cs + k);
            std::memcpy(&v.color, cb, 4);
        }
        if (vc == nv) { record_primitive(c, mode, slots); vc = reset_for_next(mode, slots); }
    }
}

// pfDrawElements / pfDrawArrays: one segment whose vertices are the arrays'
// elements [first, first + nverts) and whose primitives follow `indices`
// (or the sequence 0..count-1).
static void draw_arrays(PFdrawmode mode, PFsizei count, const void *indices, PFdatatype itype, PFint first,
                        size_t devVerts = 0)
{
    Ctx *c = G;
    CopyScope scope(c->rend);
    update_matrices(c, !(mode == PF_POINTS || mode == PF_LINES));     // pfBegin inside the draw
    c->drawMode = mode; c->vcount = 0;
    c->stateDirty = true;
    c->openImmSeg = -1;
    if (mode > PF_QUAD_STRIP) { c->err = PF_INVALID_ENUM; return; }
    const PFsizei nv = mode_count(mode);
    const PFsizei nprim = count / nv;
    int faces[2];
    bool allFill = false;
    const int nf = fill_faces(c, mode, faces, allFill);
    if (nprim == 0) return;
    // device arrays (and device indices, devVerts > 0) are read by the
    // kernels only: the host assembles points and lines itself
    const bool anyDev = devVerts > 0 || c->positions.dev ||
                        ((c->state & PF_NORMAL_ARRAY) && c->normals.buf && c->normals.dev) ||
                        ((c->state & PF_TEXTURE_COORD_ARRAY) && c->texcoords.buf && c->texcoords.dev) ||
                        ((c->state & PF_COLOR_ARRAY) && c->colors.buf && c->colors.dev);
    if (anyDev && !allFill) { c->err = PF_INVALID_OPERATION; return; }
    if (!allFill) {
        assemble_arrays(c, mode, count, indices, itype, first);
        c->stateDirty = true;
        c->openImmSeg = -1;
        return;
    }

    // the segment and its draw state first: the texture's copy is then
    // under way while the indices are copied and their range is found
    const int si = new_segment(c, PF_SRC_ARRAYS, mode == PF_TRIANGLES ? PF_ITEMS_TRIS : PF_ITEMS_EXPLICIT);

    // indices: stage as u32 and find the vertex range
    int64_t idxOff = -1;
    size_t nverts;
    if (devVerts) {
        idxOff = -(int64_t)(uintptr_t)indices;           // the caller's device indices, read in place
        nverts = devVerts;
        first = 0;
    } else if (indices) {
        uint32_t mx = 0;
        if (itype == PF_UNSIGNED_INT) {
            idxOff = snapshot_u32(c->rend, (const uint32_t *)indices, (size_t)count, mx);
        } else {
            idxOff = c->rend->staging.alloc((size_t)count * 4);
            uint32_t *dst = (uint32_t *)(c->rend->staging.base + idxOff);
            if (itype == PF_UNSIGNED_SHORT) {
                const uint16_t *s = (const uint16_t *)indices;
                for (PFsizei i = 0; i < count; i++) { dst[i] = s[i]; mx = std::max(mx, dst[i]); }
            } else {
                const uint8_t *s = (const uint8_t *)indices;
                for (PFsizei i = 0; i < count; i++) { dst[i] = s[i]; mx = std::max(mx, dst[i]); }
            }
        }
        nverts = (size_t)mx + 1;
        first = 0;
    } else {
        nverts = count;
    }
    const bool useT = (c->state & PF_TEXTURE_COORD_ARRAY) && c->texcoords.buf;
    const bool useN = (c->state & PF_NORMAL_ARRAY) && c->normals.buf;
    const bool useC = (c->state & PF_COLOR_ARRAY) && c->colors.buf;

    SegRec &r = c->rend->segs[si];
    r.posOff = stage_float_attr(c, c->positions, c->positions.size, (size_t)first, nverts);
    // the normals are often the positions' own array (unit spheres): one copy
    // taken in the same call serves both
    if (useN) r.nrmOff = (c->normals.buf == c->positions.buf && c->normals.dev == c->positions.dev &&
                          c->normals.type == PF_FLOAT && c->positions.type == PF_FLOAT && c->positions.size == 3)
                             ? r.posOff : stage_float_attr(c, c->normals, 3, (size_t)first, nverts);
    if (useT) r.uvOff = stage_float_attr(c, c->texcoords, 2, (size_t)first, nverts);
    if (useC) r.colOff = stage_color_attr(c, c->colors, (size_t)first, nverts);
    r.idxOff = idxOff;
    PFSegment &s = r.seg;
    s.nVerts = (uint32_t)nverts;
    s.posSize = c->positions.size;
    s.colSize = c->colors.size;
    s.constColor = pack(c->curColor);
    if (mode == PF_TRIANGLES) {
        s.nFaces = nf; s.face0 = faces[0];
        s.nItems = nprim * (uint32_t)nf;
    } else {
        // simulate the reference's vertex-buffer slots over sequence positions
        uint32_t slot[6];
        PFsizei vc = 0;
        for (PFsizei i = 0; i < count; i++) {
            slot[vc++] = i;
            if (vc == nv) { emit_items(r.explicitItems, mode, slot, faces, nf); vc = reset_for_next(mode, slot); }
        }
    }
    c->stateDirty = true;
}

void pfDrawElements(PFdrawmode mode, PFsizei count, PFdatatype type, const void *indices)
{
    if (!(type == PF_UNSIGNED_BYTE || type == PF_UNSIGNED_SHORT || type == PF_UNSIGNED_INT)) { G->err = PF_INVALID_ENUM; return; }
    if (!(G->state & PF_VERTEX_ARRAY)) { G->err = PF_INVALID_OPERATION; return; }
    draw_arrays(mode, count, indices, type, 0);
}
void pfDrawArrays(PFdrawmode mode, PFint first, PFsizei count)
{
    if (!(G->state & PF_VERTEX_ARRAY)) { G->err = PF_INVALID_OPERATION; return; }
    draw_arrays(mode, count, nullptr, PF_UNSIGNED_INT, first);
}

// --- zero-copy device arrays and textures (extension) --------------------------
// The pointers are device memory of the current GPU (cudaMalloc or managed),
// read by the kernels when the frame is rendered, at the next observation
// point: nothing is copied at the call, and the caller keeps the memory
// allocated and unchanged until then.
static bool device_memory(Ctx *c, const void *p, size_t align)
{
    if (!p || ((uintptr_t)p % align) != 0 || !device_init(c->rend)) return false;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}
void pfVertexPointerDevice(PFint size, PFenum type, PFsizei stride, const void *p)
{
    if (size < 2 || size > 4) { G->err = PF_INVALID_VALUE; return; }
    if (type != PF_FLOAT) { G->err = PF_INVALID_ENUM; return; }
    if (!device_memory(G, p, 4)) { G->err = PF_INVALID_VALUE; return; }
    G->positions = Attrib{ p, stride, size, type, true };
}
void pfNormalPointerDevice(PFenum type, PFsizei stride, const void *p)
{
    if (type != PF_FLOAT) { G->err = PF_INVALID_ENUM; return; }
    if (!device_memory(G, p, 4)) { G->err = PF_INVALID_VALUE; return; }
    G->normals = Attrib{ p, stride, 3, type, true };
}
void pfTexCoordPointerDevice(PFenum type, PFsizei stride, const void *p)
{
    if (type != PF_FLOAT) { G->err = PF_INVALID_ENUM; return; }
    if (!device_memory(G, p, 4)) { G->err = PF_INVALID_VALUE; return; }
    G->texcoords = Attrib{ p, stride, 2, type, true };
}
void pfColorPointerDevice(PFint size, PFenum type, PFsizei stride, const void *p)
{
    if (size < 3 || size > 4) { G->err = PF_INVALID_VALUE; return; }
    if (type != PF_UNSIGNED_BYTE) { G->err = PF_INVALID_ENUM; return; }
    if (!device_memory(G, p, 1)) { G->err = PF_INVALID_VALUE; return; }
    G->colors = Attrib{ p, stride, size, type, true };
}
void pfDrawElementsDevice(PFdrawmode mode, PFsizei count, PFsizei vertexCount, const PFuint *indices)
{
    if (!(G->state & PF_VERTEX_ARRAY)) { G->err = PF_INVALID_OPERATION; return; }
    if (vertexCount == 0) { G->err = PF_INVALID_VALUE; return; }
    if (!device_memory(G, indices, 4)) { G->err = PF_INVALID_VALUE; return; }
    draw_arrays(mode, count, indices, PF_UNSIGNED_INT, 0, (size_t)vertexCount);
}
PFtexture pfGenTextureDevice(const void *pixels, PFsizei w, PFsizei h)
{
    if (w == 0 || h == 0 || !G || !device_memory(G, pixels, 4)) { set_err(PF_INVALID_VALUE); return nullptr; }
    Tex *t = tex_new(const_cast<void *>(pixels), w, h, PF_RGBA, PF_UNSIGNED_BYTE, true);
    if (t) t->device = true;
    return t;
}

static void list_begin(Ctx *c, PFdrawmode mode);
static void list_vertex(Ctx *c, const PFfloat *v);

void pfBegin(PFdrawmode mode)                                        // context.c:1580-1603
{
    if (G->curList) { list_begin(G, mode); return; }
    if (mode > PF_QUAD_STRIP) { G->err = PF_INVALID_ENUM; return; }
    update_matrices(G, !(mode == PF_POINTS || mode == PF_LINES));
    G->drawMode = mode; G->vcount = 0;
    G->stateDirty = true;
}
void pfEnd(void) { G->vcount = 0; }

void pfVertex4fv(const PFfloat *v)                                   // context.c:1655-1685
{
    Ctx *c = G;
    if (c->curList) { list_vertex(c, v); return; }
    PFVertexIn &x = c->slots[c->vcount++];
    std::memcpy(x.pos, v, 16);
    std::memcpy(x.normal, c->curNormal, 12);
    std::memcpy(x.uv, c->curTex, 8);
    x.color = pack(c->curColor);
    x.pad[0] = x.pad[1] = 0;
    if (c->vcount == mode_count(c->drawMode)) {
        immediate_primitive(c);
        c->vcount = reset_for_next(c->drawMode, c->slots);
    }
}
void pfVertex2i(PFint x, PFint y) { float v[4] = { (float)x, (float)y, 0.0f, 1.0f }; pfVertex4fv(v); }
void pfVertex2f(PFfloat x, PFfloat y) { float v[4] = { x, y, 0.0f, 1.0f }; pfVertex4fv(v); }
void pfVertex2fv(const PFfloat *p) { float v[4] = { p[0], p[1], 0.0f, 1.0f }; pfVertex4fv(v); }
void pfVertex3i(PFint x, PFint y, PFint z) { float v[4] = { (float)x, (float)y, (float)z, 1.0f }; pfVertex4fv(v); }
void pfVertex3f(PFfloat x, PFfloat y, PFfloat z) { float v[4] = { x, y, z, 1.0f }; pfVertex4fv(v); }
void pfVertex3fv(const PFfloat *p) { float v[4] = { p[0], p[1], p[2], 1.0f }; pfVertex4fv(v); }
void pfVertex4i(PFint x, PFint y, PFint z, PFint w) { float v[4] = { (float)x, (float)y, (float)z, (float)w }; pfVertex4fv(v); }
void pfVertex4f(PFfloat x, PFfloat y, PFfloat z, PFfloat w) { float v[4] = { x, y, z, w }; pfVertex4fv(v); }

void pfColor(PFcolor col)                                           // context.c:1687-1717
{
    if (G->state & PF_COLOR_MATERIAL) {
        Material *m1 = &G->mat[0], *m2 = &G->mat[1];
        if (G->colMatFace == PF_FRONT) m2 = m1; else if (G->colMatFace == PF_BACK) m1 = m2;
        switch (G->colMatMode) {
        case PF_AMBIENT_AND_DIFFUSE: m1->ambient = m2->ambient = col; m1->diffuse = m2->diffuse = col; break;
        case PF_AMBIENT: m1->ambient = m2->ambient = col; break;
        case PF_DIFFUSE: m1->diffuse = m2->diffuse = col; break;
        case PF_SPECULAR: m1->specular = m2->specular = col; break;
        case PF_EMISSION: m1->emission = m2->emission = col; break;
        }
        G->stateDirty = true;
    } else G->curColor = col;
}
void pfColor1ui(PFuint u) { pfColor(unpack(u)); }
void pfColor3ub(PFubyte r, PFubyte g, PFubyte b) { pfColor(PFcolor{ r, g, b, 255 }); }
void pfColor3ubv(const PFubyte *v) { pfColor3ub(v[0], v[1], v[2]); }
void pfColor3us(PFushort r, PFushort g, PFushort b) { pfColor3ub((PFubyte)(r >> 8), (PFubyte)(g >> 8), (PFubyte)(b >> 8)); }
void pfColor3usv(const PFushort *v) { pfColor3us(v[0], v[1], v[2]); }
void pfColor3ui(PFuint r, PFuint g, PFuint b) { pfColor3ub((PFubyte)(r >> 24), (PFubyte)(g >> 24), (PFubyte)(b >> 24)); }
void pfColor3uiv(const PFuint *v) { pfColor3ui(v[0], v[1], v[2]); }
void pfColor3f(PFfloat r, PFfloat g, PFfloat b) { pfColor3ub(ftoub(r*255), ftoub(g*255), ftoub(b*255)); }
void pfColor3fv(const PFfloat *v) { pfColor3f(v[0], v[1], v[2]); }
void pfColor4ub(PFubyte r, PFubyte g, PFubyte b, PFubyte a) { pfColor(PFcolor{ r, g, b, a }); }
void pfColor4ubv(const PFubyte *v) { pfColor4ub(v[0], v[1], v[2], v[3]); }
void pfColor4us(PFushort r, PFushort g, PFushort b, PFushort a) { pfColor4ub((PFubyte)(r >> 8), (PFubyte)(g >> 8), (PFubyte)(b >> 8), (PFubyte)(a >> 8)); }
void pfColor4usv(const PFushort *v) { pfColor4us(v[0], v[1], v[2], v[3]); }
void pfColor4ui(PFuint r, PFuint g, PFuint b, PFuint a) { pfColor4ub((PFubyte)(r >> 24), (PFubyte)(g >> 24), (PFubyte)(b >> 24), (PFubyte)(a >> 24)); }
void pfColor4uiv(const PFuint *v) { pfColor4ui(v[0], v[1], v[2], v[3]); }
void pfColor4f(PFfloat r, PFfloat g, PFfloat b, PFfloat a) { pfColor4ub(ftoub(r*255), ftoub(g*255), ftoub(b*255), ftoub(a*255)); }
void pfColor4fv(const PFfloat *v) { pfColor4f(v[0], v[1], v[2], v[3]); }
void pfTexCoord2f(PFfloat u, PFfloat v)                              // context.c:1874-1893
{
    const float *m = G->tex;
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

// --- outside the triangle pipeline -------------------------------------------
// --- rectangles and images (context.c:1936-2159) ----------------------------
// Both become PFP_BLIT records of the recording, in submission order with
// the primitives: the tile rasterizer fills their pixels (image pixels with
// the scalar depth test and blending of the state).  Pixels outside the
// framebuffer are not drawn (the reference writes them at y*w + x).

// (PFsizei)(float) as the reference's x86-64 build converts it: a 64-bit
// truncating conversion, low 32 bits kept; 0 for NaN and out of range.
static inline uint32_t ftou32_x86(float x)
{
    if (!(x > -9.2e18f && x < 9.2e18f)) return 0u;
    return (uint32_t)(int64_t)x;
}

static int32_t screen_x(const Ctx *c, float hx) { return ftoi_x86((float)c->vpPos[0] + (hx + 1.0f) * 0.5f * (float)c->vpDim[0]); }
static int32_t screen_y(const Ctx *c, float hy) { return ftoi_x86((float)c->vpPos[1] + (1.0f - hy) * 0.5f * (float)c->vpDim[1]); }
static int32_t iclamp(int32_t v, int32_t lo, int32_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

void pfRectf(PFfloat x1, PFfloat y1, PFfloat x2, PFfloat y2)          // context.c:1936-1981
{
    Ctx *c = G;
    update_matrices(c, false);
    float v1[4] = { x1, y1, 0.0f, 1.0f }, v2[4] = { x2, y2, 0.0f, 1.0f };
    v4_transform(v1, v1, c->mvp);
    v4_transform(v2, v2, c->mvp);
    int32_t iX1 = screen_x(c, v1[0]), iY1 = screen_y(c, v1[1]), iX2 = screen_x(c, v2[0]), iY2 = screen_y(c, v2[1]);
    if (iX2 < iX1) std::swap(iX1, iX2);
    if (iY2 < iY1) std::swap(iY1, iY2);
    iX1 = iclamp(iX1, c->vpMin[0], c->vpMax[0]); iY1 = iclamp(iY1, c->vpMin[1], c->vpMax[1]);
    iX2 = iclamp(iX2, c->vpMin[0], c->vpMax[0]); iY2 = iclamp(iY2, c->vpMin[1], c->vpMax[1]);
    PFPrim P;
    std::memset(&P, 0, sizeof P);
    P.flags = PFP_BLIT;                                    // no depth test, blending or depth write
    P.c1 = pack(c->curColor);
    SegRec &rec = open_segment(c);
    const Tex *fbt = (const Tex *)c->current->texture;
    LPOut o{ rec.prebuilt, rec.explicitItems, (int32_t)fbt->w, (int32_t)fbt->h };
    lp_emit(o, P, iX1, iX2, iY1, iY2);
}
void pfRects(PFshort x1, PFshort y1, PFshort x2, PFshort y2) { pfRectf((PFfloat)x1, (PFfloat)y1, (PFfloat)x2, (PFfloat)y2); }
void pfRectsv(const PFshort *a, const PFshort *b) { pfRectf((PFfloat)a[0], (PFfloat)a[1], (PFfloat)b[0], (PFfloat)b[1]); }
void pfRectfv(const PFfloat *a, const PFfloat *b) { pfRectf(a[0], a[1], b[0], b[1]); }

// RGBA8 value of the reference's scalar pixel getter for element o
// (src/internal/pixel.h:410-760): plain reads, (PFubyte)(255 x) for half
// and float channels, (PFubyte)(field * 255/31 ...) for packed shorts.
static uint32_t pixel_sisd(PFpixelformat f, PFdatatype t, const void *p, size_t o)
{
    const uint8_t *b = (const uint8_t *)p;
    const uint16_t *h = (const uint16_t *)p;
    const float *fl = (const float *)p;
    uint32_t r = 0, g = 0, bl = 0, a = 255;
    if (t == PF_UNSIGNED_BYTE || t == PF_HALF_FLOAT || t == PF_FLOAT) {
        const int n = f == PF_LUMINANCE_ALPHA ? 2 : (f == PF_RGB || f == PF_BGR) ? 3 : (f == PF_RGBA || f == PF_BGRA) ? 4 : 1;
        uint32_t v[4] = { 0, 0, 0, 0 };
        for (int k = 0; k < n; k++) {
            const size_t i = o * (size_t)n + (size_t)k;
            if (t == PF_UNSIGNED_BYTE) v[k] = b[i];
            else if (t == PF_HALF_FLOAT) v[k] = ftoub(255.0f * half_to_float(h[i]));
            else v[k] = ftoub(255.0f * fl[i]);
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
        default: r = v[2]; g = v[1]; bl = v[0]; a = v[3]; break;              // BGRA
        }
    } else {
        const uint32_t px = h[o];
        const uint32_t hi5 = ftoub((float)((px & 0xF800u) >> 11) * (255.0f / 31));
        if (t == PF_UNSIGNED_SHORT_5_6_5) {
            const uint32_t mid = ftoub((float)((px & 0x7E0u) >> 5) * (255.0f / 63));
            const uint32_t lo = ftoub((float)(px & 0x1Fu) * (255.0f / 31));
            r = f == PF_RGB ? hi5 : lo; g = mid; bl = f == PF_RGB ? lo : hi5;
        } else if (t == PF_UNSIGNED_SHORT_5_5_5_1) {
            const uint32_t mid = ftoub((float)((px & 0x7C0u) >> 6) * (255.0f / 31));
            const uint32_t lo = ftoub((float)((px & 0x3Eu) >> 1) * (255.0f / 31));
            r = f == PF_RGBA ? hi5 : lo; g = mid; bl = f == PF_RGBA ? lo : hi5;
            a = (px & 1u) * 255u;
        } else {                                                              // 4-4-4-4
            const uint32_t c3 = ftoub((float)((px & 0xF000u) >> 12) * (255.0f / 15));
            const uint32_t c2 = ftoub((float)((px & 0xF00u) >> 8) * (255.0f / 15));
            const uint32_t c1 = ftoub((float)((px & 0xF0u) >> 4) * (255.0f / 15));
            a = ftoub((float)(px & 0xFu) * (255.0f / 15));
            r = f == PF_RGBA ? c3 : c1; g = c2; bl = f == PF_RGBA ? c1 : c3;
        }
    }
    return (r & 255u) | (g & 255u) << 8 | (bl & 255u) << 16 | (a & 255u) << 24;
}

void pfDrawPixels(PFsizei width, PFsizei height, PFpixelformat format, PFdatatype type, const void *pixels)
{                                                                          // context.c:1990-2087
    Ctx *c = G;
    if (width == 0 || height == 0) { c->err = PF_INVALID_VALUE; return; }
    if (!(format >= PF_RED && format <= PF_BGRA && type >= PF_UNSIGNED_BYTE && type <= PF_DOUBLE)) { c->err = PF_INVALID_ENUM; return; }
    if (!texel_bytes(format, type)) { c->err = PF_INVALID_ENUM; return; }
    const size_t n = (size_t)width * height;
    if (n > 0xffffffffu) { c->err = PF_INVALID_VALUE; return; }
    update_matrices(c, false);
    float rp[4];
    v4_transform(rp, c->rasterPos, c->mvp);
    const int32_t xScreen = screen_x(c, rp[0]), yScreen = screen_y(c, rp[1]);
    const int32_t xMin = iclamp(xScreen, c->vpMin[0], c->vpMax[0]), yMin = iclamp(yScreen, c->vpMin[1], c->vpMax[1]);
    // PF_CLAMP of a float against int bounds evaluates to a float
    auto fclamp = [](float v, int32_t lo, int32_t hi) { return v < (float)lo ? (float)lo : (v > (float)hi ? (float)hi : v); };
    const int32_t xMax = ftoi_x86(fclamp((float)xScreen + (float)width * c->pixelZoom[0], c->vpMin[0], c->vpMax[0]));
    const int32_t yMax = ftoi_x86(fclamp((float)yScreen + (float)height * c->pixelZoom[1], c->vpMin[1], c->vpMax[1]));
    PFPrim P;
    std::memset(&P, 0, sizeof P);
    P.flags = PFP_BLIT | ((c->state & PF_DEPTH_TEST) ? (uint32_t)PFP_DEPTH_TEST : 0u) |
              ((c->state & PF_BLEND) ? (uint32_t)PFP_BLEND : 0u) | (c->depthMask ? (uint32_t)PFP_DEPTH_WRITE : 0u);
    P.x1 = xScreen; P.y1 = yScreen;
    P.x2 = (int32_t)width; P.y2 = (int32_t)(width - 1); P.x3 = (int32_t)(height - 1);
    P.wInvSum = 1.0f / ((float)width * c->pixelZoom[0]);
    P.z2 = 1.0f / ((float)height * c->pixelZoom[1]);
    P.z1 = rp[2];
    P.nSrc = (uint32_t)n;
    SegRec &rec = open_segment(c);
    const Tex *fbt = (const Tex *)c->current->texture;
    LPOut o{ rec.prebuilt, rec.explicitItems, (int32_t)fbt->w, (int32_t)fbt->h };
    const int64_t ri = lp_emit(o, P, xMin, xMax, yMin, yMax);
    if (ri < 0) return;
    // the image, converted once with the scalar getter
    const int64_t off = c->rend->staging.alloc(n * 4);
    uint32_t *dst = (uint32_t *)(c->rend->staging.base + off);
    for (size_t i = 0; i < n; i++) dst[i] = pixel_sisd(format, type, pixels, i);
    rec.blitSrc.push_back({ (uint32_t)ri, off });
}

void pfPixelZoom(PFfloat x, PFfloat y) { G->pixelZoom[0] = x; G->pixelZoom[1] = y; }   // context.c:2089-2093
static void raster_pos(float x, float y, float z, float w)
{
    G->rasterPos[0] = x; G->rasterPos[1] = y; G->rasterPos[2] = z; G->rasterPos[3] = w;
}
void pfRasterPos2i(PFint x, PFint y) { raster_pos((PFfloat)x, (PFfloat)y, 0.0f, 1.0f); }
void pfRasterPos2f(PFfloat x, PFfloat y) { raster_pos(x, y, 0.0f, 1.0f); }
void pfRasterPos2fv(const PFfloat *v) { raster_pos(v[0], v[1], 0.0f, 1.0f); }
void pfRasterPos3i(PFint x, PFint y, PFint z) { raster_pos((PFfloat)x, (PFfloat)y, (PFfloat)z, 1.0f); }
void pfRasterPos3f(PFfloat x, PFfloat y, PFfloat z) { raster_pos(x, y, z, 1.0f); }
void pfRasterPos3fv(const PFfloat *v) { raster_pos(v[0], v[1], v[2], 1.0f); }
void pfRasterPos4i(PFint x, PFint y, PFint z, PFint w) { raster_pos((PFfloat)x, (PFfloat)y, (PFfloat)z, (PFfloat)w); }
void pfRasterPos4f(PFfloat x, PFfloat y, PFfloat z, PFfloat w) { raster_pos(x, y, z, w); }
void pfRasterPos4fv(const PFfloat *v) { raster_pos(v[0], v[1], v[2], v[3]); }

// --- fog (context.c:2161-2351) -------------------------------------------------
// The parameter setters keep the reference's behaviour: a density sets the
// mode (truncated), and the vector forms accept any mode or density (their
// range tests are always true).
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
    case PF_FOG_DENSITY: if (v >= 0 && v <= 1) G->fog.mode = ftou32_x86(v); else G->err = PF_INVALID_VALUE; break;
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
    case PF_FOG_COLOR: G->fog.color = PFcolor{ (PFubyte)v[0], (PFubyte)v[1], (PFubyte)v[2], (PFubyte)v[3] }; break;
    default: G->err = PF_INVALID_ENUM; break;
    }
}
void pfFogfv(PFfogparam p, PFfloat *v)
{
    switch (p) {
    case PF_FOG_DENSITY: if (*v >= 0 || *v <= 1) G->fog.mode = ftou32_x86(*v); else G->err = PF_INVALID_VALUE; break;
    case PF_FOG_START: G->fog.start = *v; break;
    case PF_FOG_END: G->fog.end = *v; break;
    case PF_FOG_COLOR: G->fog.color = PFcolor{ ftoub(255 * v[0]), ftoub(255 * v[1]), ftoub(255 * v[2]), ftoub(255 * v[3]) }; break;
    default: G->err = PF_INVALID_ENUM; break;
    }
}
// A framebuffer-wide device pass over the current framebuffer, in order
// with the recorded draws.
void pfFogProcess(void)
{
    Cmd cmd{};
    cmd.kind = CMD_HOOK; cmd.fb = G->current; cmd.hook = 3;
    cmd.hp.start = G->fog.start; cmd.hp.end = G->fog.end; cmd.hp.density = G->fog.density;
    cmd.hp.mode = G->fog.mode; cmd.hp.color = pack(G->fog.color);
    push_cmd(G, cmd);
}

// --- render lists (src/renderlist.c:6-97, context.c:1580-1685) ---------------
// Recorded on the host as the reference records them (RenderList) and
// replayed through the immediate-mode calls, which record into the deferred
// renderer like any other draw.

static void ctx_backup(Ctx *c)                       // pfiMakeContextBackup (internal/context/context.c:26-36)
{
    c->backup.mat[0] = c->mat[0]; c->backup.mat[1] = c->mat[1];
    std::memcpy(c->backup.tex, c->curTex, 8); std::memcpy(c->backup.nrm, c->curNormal, 12);
    c->backup.col = c->curColor; c->backup.texture = c->texture; c->backup.state = c->state;
}
static void ctx_restore(Ctx *c)                      // pfiRestoreContext (:38-48)
{
    c->mat[0] = c->backup.mat[0]; c->mat[1] = c->backup.mat[1];
    std::memcpy(c->curTex, c->backup.tex, 8); std::memcpy(c->curNormal, c->backup.nrm, 12);
    c->curColor = c->backup.col; c->texture = c->backup.texture; c->state = c->backup.state;
    c->stateDirty = true;
}
static void list_begin(Ctx *c, PFdrawmode mode)
{
    RenderCall k;
    k.mode = mode; k.mat[0] = c->mat[0]; k.mat[1] = c->mat[1]; k.texture = c->texture;
    c->curList->calls.push_back(std::move(k));
}
static void list_vertex(Ctx *c, const PFfloat *v)
{
    if (c->curList->calls.empty()) return;           // the reference indexes call -1
    RenderCall &k = c->curList->calls.back();
    k.pos.insert(k.pos.end(), v, v + 4);
    k.uv.insert(k.uv.end(), c->curTex, c->curTex + 2);
    k.nrm.insert(k.nrm.end(), c->curNormal, c->curNormal + 3);
    k.col.push_back(c->curColor);
}

PFrenderlist pfGenList(void) { return new RenderList(); }
void pfDeleteList(PFrenderlist *pl)
{
    if (!pl) return;
    RenderList *l = (RenderList *)*pl;
    if (G && G->curList == l) G->curList = nullptr;
    delete l;
    *pl = nullptr;
}
void pfNewList(PFrenderlist pl)
{
    if (!pl) { G->err = PF_INVALID_VALUE; return; }
    RenderList *l = (RenderList *)pl;
    l->calls.clear();
    G->curList = l;
    ctx_backup(G);
}
void pfEndList(void)
{
    if (!G->curList) G->err = PF_INVALID_OPERATION;
    G->curList = nullptr;
    ctx_restore(G);
}
void pfCallList(const PFrenderlist pl)
{
    const RenderList *l = (const RenderList *)pl;
    if (!l) { G->err = PF_INVALID_VALUE; return; }
    Ctx *c = G;
    ctx_backup(c);
    for (const RenderCall &k : l->calls) {
        c->mat[0] = k.mat[0]; c->mat[1] = k.mat[1];
        c->stateDirty = true;
        pfBindTexture(k.texture);
        pfBegin(k.mode);
        for (size_t j = 0; j < k.col.size(); j++) {
            pfColor4ubv((const PFubyte *)&k.col[j]);
            pfTexCoordfv(&k.uv[2 * j]);
            pfNormal3fv(&k.nrm[3 * j]);
            pfVertex4fv(&k.pos[4 * j]);
        }
        pfEnd();
    }
    ctx_restore(c);
}

// --- readback, post-process -----------------------------------------------------
void pfFinish(void) { if (G) flush(G); }

// pfmFloatToHalfI (src/pfm.h:108-126): round half up on the dropped bits,
// flush below 2^-14, infinity from 2^16, all NaNs quiet.
static uint16_t float_to_half(float x)
{
    uint32_t ui; std::memcpy(&ui, &x, 4);
    const int s = (int)((ui >> 16) & 0x8000u);
    const int em = (int)(ui & 0x7fffffffu);
    int h = (em - (112 << 23) + (1 << 12)) >> 13;
    h = (em < (113 << 23)) ? 0 : h;
    h = (em >= (143 << 23)) ? 0x7c00 : h;
    h = (em > (255 << 23)) ? 0x7e00 : h;
    return (uint16_t)(s | h);
}

// The reference's scalar pixel setter (src/internal/pixel.h:52-405) writing
// RGBA8 colour col as element o of a buffer of format f / type t.
#define FTOUB ftoub
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
        const uint32_t c0 = (uint8_t)std::round(n[0] * 31.0f), c1 = (uint8_t)std::round(n[1] * 63.0f), c2 = (uint8_t)std::round(n[2] * 31.0f);
        p16[o] = (uint16_t)(c0 << 11 | c1 << 5 | c2);
        return;
    }
    if (t == PF_UNSIGNED_SHORT_5_5_5_1) {
        const uint32_t c0 = (uint8_t)std::round(n[0] * 31.0f), c1 = (uint8_t)std::round(n[1] * 31.0f), c2 = (uint8_t)std::round(n[2] * 31.0f);
        const uint32_t al = ((double)n[3] > (double)(float)50 * (1.0 / 255)) ? 1u : 0u;
        p16[o] = (uint16_t)(c0 << 11 | c1 << 6 | c2 << 1 | al);
        return;
    }
    if (t == PF_UNSIGNED_SHORT_4_4_4_4) {
        const uint32_t c0 = (uint8_t)std::round(n[0] * 15.0f), c1 = (uint8_t)std::round(n[1] * 15.0f);
        const uint32_t c2 = (uint8_t)std::round(n[2] * 15.0f), c3 = (uint8_t)std::round(n[3] * 15.0f);
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

// A framebuffer's scalar getter and setter for pixel o (host side: the
// framebuffer functions, pfReadPixels, host post-processing).
static uint32_t fb_get(const Tex *t, size_t o)
{
    uint32_t raw[4];
    const uint32_t f = (uint32_t)fb_code(t->format, t->type);
    pff_load(f, t->pixels, o, raw);
    return pff_get_sisd(f, raw);
}
static void fb_set(Tex *t, size_t o, uint32_t col)
{
    uint32_t raw[4];
    const uint32_t f = (uint32_t)fb_code(t->format, t->type);
    pff_set_sisd(f, col, raw);
    pff_store(f, t->pixels, o, raw);
}

void pfReadPixels(PFint x, PFint y, PFsizei w, PFsizei h, PFpixelformat f, PFdatatype t, void *pixels)
{                                                                    // context.c:2353-2395
    if (!(f >= PF_RED && f <= PF_BGRA && t >= PF_UNSIGNED_BYTE && t <= PF_DOUBLE)) { G->err = PF_INVALID_ENUM; return; }
    if (!texel_bytes(f, t)) { G->err = PF_INVALID_ENUM; return; }
    sync_host(G);
    const Tex *s = (const Tex *)G->current->texture;
    auto cl = [](PFint v, PFint lo, PFint hi) { return v < lo ? lo : (v > hi ? hi : v); };
    PFint xMin = cl(x, 0, (PFint)s->w - 1), yMin = cl(y, 0, (PFint)s->h - 1);
    PFint xMax = cl(x + (PFint)w, 0, (PFint)s->w), yMax = cl(y + (PFint)h, 0, (PFint)s->h);
    if (f == PF_RGBA && t == PF_UNSIGNED_BYTE) {
        uint32_t *dst = (uint32_t *)pixels;
        for (PFint yy = yMin; yy < yMax; yy++)
            for (PFint xx = xMin; xx < xMax; xx++)
                dst[(size_t)(yy - yMin) * w + (size_t)(xx - xMin)] = fb_get(s, (size_t)yy * s->w + (size_t)xx);
        return;
    }
    for (PFint yy = yMin; yy < yMax; yy++)
        for (PFint xx = xMin; xx < xMax; xx++)
            pixel_set_sisd(f, t, pixels, (size_t)(yy - yMin) * w + (size_t)(xx - xMin), fb_get(s, (size_t)yy * s->w + (size_t)xx));
}

void pfPostProcess(PFpostprocessfunc fn)                             // context.c:2397-2441
{
    sync_host(G);
    if (G->current == &G->mainFB) pull_main_depth(G);
    Tex *t = (Tex *)G->current->texture;
    const float *zb = G->current->zbuffer;
    for (PFint y = 0; y < (PFint)t->h; y++)
        for (PFint x = 0; x < (PFint)t->w; x++) {
            size_t o = (size_t)y * t->w + (size_t)x;
            fb_set(t, o, pack(fn(x, y, zb[o], unpack(fb_get(t, o)))));
        }
}

void pfPostProcessDevice(PFuint hookId, const void *params, PFsizei size)
{
    Cmd cmd{};
    cmd.kind = CMD_HOOK; cmd.fb = G->current; cmd.hook = (int)hookId;
    switch (hookId) {
    case PF_HOOK_IDENTITY: case PF_HOOK_GRAYSCALE: break;
    case PF_HOOK_DITHER: cmd.hook = 4; break;        // device hook 3 is pfFogProcess
    case PF_HOOK_FOG_LINEAR: {
        if (!params || size < sizeof(PFhookfog)) { G->err = PF_INVALID_VALUE; return; }
        PFhookfog f; std::memcpy(&f, params, sizeof f);
        cmd.hp.znear = f.znear; cmd.hp.zfar = f.zfar; cmd.hp.start = f.start; cmd.hp.end = f.end;
        cmd.hp.color = pack(f.color);
    } break;
    default: G->err = PF_INVALID_ENUM; return;
    }
    push_cmd(G, cmd);
}

// --- batches: many contexts, one launch of each pipeline kernel --------------
PFgbbatch pfgbBatchCreate(void) { return new Batch(); }

void pfgbBatchDelete(PFgbbatch batch)
{
    Batch *b = (Batch *)batch;
    if (!b) return;
    if (gBatch == b) pfgbBatchEnd(batch);
    release_renderer(&b->r);
    delete b;
}

void pfgbBatchBegin(PFgbbatch batch)
{
    Batch *b = (Batch *)batch;
    if (!b || gBatch) { set_err(PF_INVALID_OPERATION); return; }
    gBatch = b;
    b->open = true;
    if (G) {
        flush(G);                         // the current context's own work renders first
        G->rend = &b->r;
        G->openImmSeg = -1;
        b->members.push_back(G);
    }
}

void pfgbBatchEnd(PFgbbatch batch)
{
    Batch *b = (Batch *)batch;
    if (!b || gBatch != b) { set_err(PF_INVALID_OPERATION); return; }
    flush(&b->r);
    for (Ctx *c : b->members) { c->rend = &c->own; c->openImmSeg = -1; }
    b->members.clear();
    b->open = false;
    gBatch = nullptr;
}

PFfloat pfgbBatchReplay(PFgbbatch batch, PFuint n)
{
    Batch *b = (Batch *)batch;
    if (!b || b->open) return -1.0f;
    return replay(&b->r, n);
}

void pfgbBatchGetStats(PFgbbatch batch, PFstats *s) { *s = ((Batch *)batch)->r.stats; }
void pfgbBatchEnableTiming(PFgbbatch batch, PFboolean enable) { ((Batch *)batch)->r.timing = enable; }

void pfgbBatchTune(PFgbbatch batch, PFuint binCapacity, PFuint rasterCtasPerSM)
{
    Renderer *r = batch ? &((Batch *)batch)->r : (G ? &G->own : nullptr);
    if (!r) return;
    if (binCapacity >= 32 && binCapacity <= kCapMax && (binCapacity & (binCapacity - 1)) == 0) r->cap = binCapacity;
    if (rasterCtasPerSM <= 32) r->rasterCtasPerSM = (int)rasterCtasPerSM;
}

void pfgbBatchTuneShape(PFgbbatch batch, PFuint rasterWarpsPerCta)
{
    Renderer *r = batch ? &((Batch *)batch)->r : (G ? &G->own : nullptr);
    if (!r) return;
    if (rasterWarpsPerCta == 2 || rasterWarpsPerCta == 4 || rasterWarpsPerCta == 8) r->rasterWarps = (int)rasterWarpsPerCta;
}

PFfloat pfgbReplay(PFuint n) { return G ? replay(&G->own, n) : -1.0f; }

void pfGetStats(PFstats *s) { *s = G->own.stats; }
void pfResetStats(void) { G->own.stats = PFstats{}; }
void pfEnableTiming(PFboolean enable) { G->own.timing = enable; }
PFuint pfGetDeviceStatus(void) { return G ? G->own.devStatus : 0; }

// --- framebuffers (framebuffer.c) ----------------------------------------------
PFframebuffer pfGenFramebuffer(PFsizei w, PFsizei h, PFpixelformat f, PFdatatype t)
{
    PFframebuffer fb{ nullptr, nullptr };
    const int code = fb_code(f, t);
    if (code < 0) { set_err(PF_INVALID_ENUM); return fb; }
    const size_t n = (size_t)w * h, bytes = n * (size_t)pff_bytes((uint32_t)code);
    void *px = nullptr;
    bool pinned = cudaMallocHost(&px, bytes) == cudaSuccess;
    if (!pinned) { cudaGetLastError(); px = std::malloc(bytes); }
    if (!px) { set_err(PF_ERROR_OUT_OF_MEMORY); return fb; }
    std::memset(px, 0, bytes);
    Tex *tx = tex_new(px, w, h, f, t, false);
    tx->ownsPinned = pinned;
    float *z = nullptr;
    bool zp = cudaMallocHost((void **)&z, n * 4) == cudaSuccess;
    if (!zp) { cudaGetLastError(); z = (float *)std::malloc(n * 4); }
    for (size_t i = 0; i < n; i++) z[i] = FLT_MAX;
    tx->depthPinned = zp;
    fb.texture = tx; fb.zbuffer = z;
    return fb;
}

void pfDeleteFramebuffer(PFframebuffer *fb)
{
    if (!fb) return;
    if (G) flush(G);
    Tex *t = (Tex *)fb->texture;
    if (t) {
        drop_mirror(t);
        if (t->ownsPinned) cudaFreeHost(t->pixels); else std::free(t->pixels);
        if (fb->zbuffer) {
            if (t->depthPinned) { if (cudaFreeHost(fb->zbuffer) != cudaSuccess) cudaGetLastError(); }
            else std::free(fb->zbuffer);
        }
        delete t;
    }
    fb->texture = nullptr; fb->zbuffer = nullptr;
}

PFboolean pfIsValidFramebuffer(PFframebuffer *fb)
{
    const Tex *t = (const Tex *)fb->texture;
    return t && fb->zbuffer && t->w > 0 && t->h > 0 && t->pixels;
}

void pfClearFramebuffer(PFframebuffer *fb, PFcolor color, PFfloat depth)
{
    Cmd cmd{};
    cmd.kind = CMD_FILL; cmd.fb = fb; cmd.color = pack(color); cmd.depth = depth;
    if (G) push_cmd(G, cmd);
}

PFcolor pfGetFramebufferPixel(const PFframebuffer *fb, PFsizei x, PFsizei y)
{
    if (G) sync_host(G);
    const Tex *t = (const Tex *)fb->texture;
    return unpack(fb_get(t, (size_t)y * t->w + x));
}
PFfloat pfGetFramebufferDepth(const PFframebuffer *fb, PFsizei x, PFsizei y)
{
    if (G) { sync_host(G); if (fb == &G->mainFB) pull_main_depth(G); }
    const Tex *t = (const Tex *)fb->texture;
    return fb->zbuffer[(size_t)y * t->w + x];
}
void pfSetFramebufferPixelDepthTest(PFframebuffer *fb, PFsizei x, PFsizei y, PFfloat z, PFcolor col, PFdepthmode m)
{
    if (m > PF_GEQUAL) { set_err(PF_INVALID_ENUM); return; }
    if (G) { sync_host(G); if (fb == &G->mainFB) pull_main_depth(G); }
    Tex *t = (Tex *)fb->texture;
    size_t o = (size_t)y * t->w + x;
    bool pass;
    switch (m) {                                                    // depth.h:30-70
    case PF_EQUAL: pass = z == fb->zbuffer[o]; break;
    case PF_NOTEQUAL: pass = z != fb->zbuffer[o]; break;
    case PF_LESS: pass = z < fb->zbuffer[o]; break;
    case PF_LEQUAL: pass = z <= fb->zbuffer[o]; break;
    case PF_GREATER: pass = z > fb->zbuffer[o]; break;
    default: pass = z >= fb->zbuffer[o]; break;
    }
    if (pass) { fb_set(t, o, pack(col)); fb->zbuffer[o] = z; }
}
void pfSetFramebufferPixelDepth(PFframebuffer *fb, PFsizei x, PFsizei y, PFfloat z, PFcolor col)
{
    if (G) { sync_host(G); if (fb == &G->mainFB) pull_main_depth(G); }
    Tex *t = (Tex *)fb->texture;
    size_t o = (size_t)y * t->w + x;
    fb_set(t, o, pack(col)); fb->zbuffer[o] = z;
}
void pfSetFramebufferPixel(PFframebuffer *fb, PFsizei x, PFsizei y, PFcolor col)
{
    if (G) sync_host(G);
    Tex *t = (Tex *)fb->texture;
    fb_set(t, (size_t)y * t->w + x, pack(col));
}

// --- textures (texture.c) --------------------------------------------------------
PFtexture pfGenTexture(void *pixels, PFsizei w, PFsizei h, PFpixelformat f, PFdatatype t) { return tex_new(pixels, w, h, f, t, true); }
void pfDeleteTexture(PFtexture *tex, PFboolean freeBuffer)
{
    Tex *t = (Tex *)*tex;
    if (!t) return;
    if (G && G->texture == t) G->texture = nullptr;   // snapshots already hold the texels
    if (t->hostRegistered) {
        if (cudaDeviceSynchronize() != cudaSuccess) cudaGetLastError();   // no upload from it in flight
        cudaHostUnregister(t->pixels);
    }
    if (freeBuffer && !t->device) std::free(t->pixels);      // device texels stay the caller's
    delete t;
    *tex = nullptr;
}
PFboolean pfIsValidTexture(const PFtexture tex)
{
    const Tex *t = (const Tex *)tex;
    return t && t->pixels && t->w > 0 && t->h > 0;
}
void pfTextureParameter(PFtexture tex, PFtexturewrap wrap, PFtexturefilter filter)
{
    if (!(wrap <= PF_CLAMP_TO_EDGE && filter <= PF_BILINEAR)) { set_err(PF_INVALID_ENUM); return; }
    Tex *t = (Tex *)tex; t->wrap = wrap; t->filter = filter;
    if (G) G->stateDirty = true;
}
void *pfGetTexturePixels(const PFtexture tex, PFsizei *w, PFsizei *h, PFpixelformat *f, PFdatatype *t)
{
    const Tex *x = (const Tex *)tex;
    if (!x) return nullptr;
    if (G) sync_host(G);
    if (w) *w = x->w;
    if (h) *h = x->h;
    if (f) *f = x->format;
    if (t) *t = x->type;
    return x->pixels;
}

}  // extern "C"
