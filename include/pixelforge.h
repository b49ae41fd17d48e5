/*
 * pixelforge.h -- C99 interface of pixelforge-gb300.
 *
 * Drop-in replacement of PixelForge's public header (src/pixelforge.h) for
 * the triangle pipeline, rendered on a GB300 (sm_103a) by hand-written CUDA
 * kernels.  Every type, enumerator value and prototype below has the same
 * name, value, argument meaning and C linkage as the reference, so a program
 * written against PixelForge recompiles (or relinks against
 * libpixelforge_gb300.so) unchanged.  Each prototype cites the reference
 * declaration it replaces as `pixelforge.h:LINE`.
 *
 * Execution model.  The reference rasterises synchronously inside every
 * pfVertex / pfDrawElements call.  This library records the calls and renders
 * them on the GPU when an observation point is reached: pfFinish (extension),
 * pfReadPixels, pfGetFramebufferPixel / pfGetFramebufferDepth, pfPostProcess,
 * pfSwapBuffers, pfMakeCurrent (switching away), pfSetMainBuffer,
 * pfDeleteContext, pfDeleteTexture of a bound texture, and any getter that
 * returns pixel memory.  At those points the colour is written back to the
 * caller's buffer and the depth to the framebuffer's host z-buffer.  Textures
 * are read from the caller's pixel memory at flush time, as the reference
 * reads them at draw time.
 *
 * Entry points outside the triangle pipeline (lines, points, render lists,
 * pixel rectangles, fog) are exported so that programs link; they set
 * PF_INVALID_OPERATION and draw nothing.
 */
#ifndef PIXELFORGE_GB300_H
#define PIXELFORGE_GB300_H

#include <stdint.h>

#ifndef PF_API
#   if defined(__GNUC__)
#       define PF_API __attribute__((visibility("default")))
#   else
#       define PF_API
#   endif
#endif

#if !defined(__cplusplus)
#   include <stdbool.h>
#endif

/* ---- scalar types (pixelforge.h:129-149) ---------------------------------- */

typedef bool        PFboolean;
#define PF_FALSE 0
#define PF_TRUE  1

typedef int8_t      PFbyte;
typedef uint8_t     PFubyte;
typedef int16_t     PFshort;
typedef uint16_t    PFushort;
typedef int32_t     PFint;
typedef uint32_t    PFuint;
typedef int64_t     PFint64;
typedef uint64_t    PFuint64;
typedef uint32_t    PFsizei;
typedef uint32_t    PFenum;
typedef intptr_t    PFintptr;
typedef uintptr_t   PFsizeiptr;
typedef float       PFfloat;
typedef double      PFdouble;

/* ---- enumerations (pixelforge.h:151-392); values identical ----------------- */

typedef enum {
    PF_UNSIGNED_BYTE, PF_UNSIGNED_SHORT, PF_UNSIGNED_SHORT_5_6_5,
    PF_UNSIGNED_SHORT_5_5_5_1, PF_UNSIGNED_SHORT_4_4_4_4, PF_UNSIGNED_INT,
    PF_BYTE, PF_SHORT, PF_INT, PF_HALF_FLOAT, PF_FLOAT, PF_DOUBLE
} PFdatatype;

typedef void* PFcontext;

typedef enum {
    PF_TEXTURE_2D          = 0x0001,
    PF_FRAMEBUFFER         = 0x0002,
    PF_BLEND               = 0x0004,
    PF_DEPTH_TEST          = 0x0008,
    PF_CULL_FACE           = 0x0010,
    PF_NORMALIZE           = 0x0020,
    PF_LIGHTING            = 0x0040,
    PF_COLOR_MATERIAL      = 0x0080,
    PF_VERTEX_ARRAY        = 0x0100,
    PF_NORMAL_ARRAY        = 0x0200,
    PF_COLOR_ARRAY         = 0x0400,
    PF_TEXTURE_COORD_ARRAY = 0x0800
} PFstate;

typedef enum {
    PF_VIEWPORT = 10000, PF_COLOR_CLEAR_VALUE, PF_DEPTH_CLEAR_VALUE,
    PF_CULL_FACE_MODE, PF_CURRENT_COLOR, PF_CURRENT_NORMAL,
    PF_CURRENT_TEXTURE_COORDS, PF_CURRENT_RASTER_POSITION, PF_BLEND_FUNC,
    PF_DEPTH_FUNC, PF_POLYGON_MODE, PF_POINT_SIZE, PF_LINE_WIDTH,
    PF_MATRIX_MODE, PF_PROJECTION_MATRIX, PF_MODELVIEW_MATRIX,
    PF_TEXTURE_MATRIX, PF_MAX_PROJECTION_STACK_DEPTH,
    PF_MAX_MODELVIEW_STACK_DEPTH, PF_MAX_TEXTURE_STACK_DEPTH, PF_SHADE_MODEL,
    PF_MAX_LIGHTS, PF_VERTEX_ARRAY_SIZE, PF_VERTEX_ARRAY_STRIDE,
    PF_VERTEX_ARRAY_TYPE, PF_NORMAL_ARRAY_STRIDE, PF_NORMAL_ARRAY_TYPE,
    PF_TEXTURE_COORD_ARRAY_STRIDE, PF_TEXTURE_COORD_ARRAY_TYPE,
    PF_COLOR_ARRAY_SIZE, PF_COLOR_ARRAY_STRIDE, PF_COLOR_ARRAY_TYPE,
    PF_ZOOM_X, PF_ZOOM_Y
} PFgettable;

/* Release-build error codes (the reference adds PF_DEBUG_* codes only when
 * compiled without NDEBUG). */
typedef enum {
    PF_NO_ERROR, PF_INVALID_ENUM, PF_INVALID_VALUE, PF_STACK_OVERFLOW,
    PF_STACK_UNDERFLOW, PF_INVALID_OPERATION, PF_ERROR_OUT_OF_MEMORY
} PFerrcode;

typedef enum { PF_COLOR_BUFFER_BIT = 0x01, PF_DEPTH_BUFFER_BIT = 0x02 } PFclearflag;
typedef enum { PF_MODELVIEW, PF_PROJECTION, PF_TEXTURE } PFmatrixmode;
typedef enum {
    PF_POINTS, PF_LINES, PF_TRIANGLES, PF_TRIANGLE_FAN, PF_TRIANGLE_STRIP,
    PF_QUADS, PF_QUAD_FAN, PF_QUAD_STRIP
} PFdrawmode;
typedef enum {
    PF_BLEND_AVERAGE, PF_BLEND_ALPHA, PF_BLEND_ADD, PF_BLEND_SUB,
    PF_BLEND_MUL, PF_BLEND_SCREEN, PF_BLEND_LIGHTEN, PF_BLEND_DARKEN
} PFblendmode;
typedef enum {
    PF_EQUAL, PF_NOTEQUAL, PF_LESS, PF_LEQUAL, PF_GREATER, PF_GEQUAL
} PFdepthmode;
typedef enum { PF_POINT, PF_LINE, PF_FILL } PFpolygonmode;
typedef enum { PF_FLAT, PF_SMOOTH } PFshademode;
typedef enum { PF_GOURAUD, PF_PHONG } PFlightmode;
typedef enum { PF_FRONT = 0, PF_BACK = 1, PF_FRONT_AND_BACK } PFface;
typedef enum { PF_REPEAT, PF_MIRRORED_REPEAT, PF_CLAMP_TO_EDGE } PFtexturewrap;
typedef enum { PF_NEAREST, PF_BILINEAR } PFtexturefilter;
typedef enum {
    PF_LIGHT0 = 0, PF_LIGHT1, PF_LIGHT2, PF_LIGHT3, PF_LIGHT4, PF_LIGHT5,
    PF_LIGHT6, PF_LIGHT7, PF_LIGHT8
} PFlights;
typedef enum {
    PF_AMBIENT_AND_DIFFUSE = 1, PF_AMBIENT = 2, PF_DIFFUSE = 3, PF_SPECULAR = 4
} PFrendercolor;
typedef enum { PF_EMISSION = 5, PF_SHININESS = 6 } PFmaterialparam;
typedef enum {
    PF_POSITION = 7, PF_SPOT_DIRECTION = 8, PF_SPOT_INNER_CUTOFF = 10,
    PF_SPOT_OUTER_CUTOFF = 11, PF_CONSTANT_ATTENUATION = 12,
    PF_LINEAR_ATTENUATION = 13, PF_QUADRATIC_ATTENUATION = 14
} PFlightparam;
typedef enum { PF_FOG_MODE, PF_FOG_DENSITY, PF_FOG_START, PF_FOG_END, PF_FOG_COLOR } PFfogparam;
typedef enum { PF_LINEAR, PF_EXP, PF_EXP2 } PFfogmode;

typedef struct { PFubyte r, g, b, a; } PFcolor;                       /* pixelforge.h:399-401 */
typedef PFcolor (*PFpostprocessfunc)(PFint, PFint, PFfloat, PFcolor); /* pixelforge.h:403 */

typedef enum {
    PF_RED, PF_GREEN, PF_BLUE, PF_ALPHA, PF_LUMINANCE, PF_LUMINANCE_ALPHA,
    PF_RGB, PF_RGBA, PF_BGR, PF_BGRA
} PFpixelformat;

typedef void* PFtexture;
typedef void* PFrenderlist;

/* By-value framebuffer with a public host z-buffer (pixelforge.h:428-431). */
typedef struct {
    PFtexture texture;
    PFfloat  *zbuffer;
} PFframebuffer;

#if defined(__cplusplus)
extern "C" {
#endif

/* ---- contexts (pixelforge.h:453-560) --------------------------------------- */
PF_API PFcontext pfCreateContext(void* targetBuffer, PFsizei width, PFsizei height,
                                 PFpixelformat format, PFdatatype type);       /* pixelforge.h:453 */
PF_API void      pfDeleteContext(PFcontext ctx);                               /* pixelforge.h:466 */
PF_API void      pfSetMainBuffer(void* targetBuffer, PFsizei width, PFsizei height,
                                 PFpixelformat format, PFdatatype type);       /* pixelforge.h:487 */
PF_API void      pfSetAuxBuffer(void* auxFramebuffer);                         /* pixelforge.h:500 */
PF_API void      pfSwapBuffers(void);                                          /* pixelforge.h:508 */
PF_API PFcontext pfGetCurrentContext(void);                                    /* pixelforge.h:518 */
PF_API void      pfMakeCurrent(PFcontext ctx);                                 /* pixelforge.h:528 */
PF_API PFboolean pfIsEnabled(PFstate state);                                   /* pixelforge.h:540 */
PF_API void      pfEnable(PFstate state);                                      /* pixelforge.h:550 */
PF_API void      pfDisable(PFstate state);                                     /* pixelforge.h:560 */

/* ---- getters (pixelforge.h:574-628) ----------------------------------------- */
PF_API void      pfGetBooleanv(PFenum pname, PFboolean* params);               /* pixelforge.h:574 */
PF_API void      pfGetIntegerv(PFenum pname, PFint* params);                   /* pixelforge.h:585 */
PF_API void      pfGetFloatv(PFenum pname, PFfloat* params);                   /* pixelforge.h:596 */
PF_API void      pfGetDoublev(PFenum pname, PFdouble* params);                 /* pixelforge.h:607 */
PF_API void      pfGetPointerv(PFenum pname, const void** params);             /* pixelforge.h:618 */
PF_API PFerrcode pfGetError(void);                                             /* pixelforge.h:628 */

/* ---- matrices (pixelforge.h:641-744) ----------------------------------------- */
PF_API void pfMatrixMode(PFmatrixmode mode);                                   /* pixelforge.h:641 */
PF_API void pfPushMatrix(void);                                                /* pixelforge.h:649 */
PF_API void pfPopMatrix(void);                                                 /* pixelforge.h:657 */
PF_API void pfLoadIdentity(void);                                              /* pixelforge.h:665 */
PF_API void pfTranslatef(PFfloat x, PFfloat y, PFfloat z);                     /* pixelforge.h:677 */
PF_API void pfRotatef(PFfloat angle, PFfloat x, PFfloat y, PFfloat z);         /* pixelforge.h:690 */
PF_API void pfScalef(PFfloat x, PFfloat y, PFfloat z);                         /* pixelforge.h:702 */
PF_API void pfMultMatrixf(const PFfloat* mat);                                 /* pixelforge.h:712 */
PF_API void pfFrustum(PFfloat left, PFfloat right, PFfloat bottom, PFfloat top,
                      PFfloat znear, PFfloat zfar);                            /* pixelforge.h:727 */
PF_API void pfOrtho(PFfloat left, PFfloat right, PFfloat bottom, PFfloat top,
                    PFfloat znear, PFfloat zfar);                              /* pixelforge.h:744 */

/* ---- render configuration (pixelforge.h:762-922) ----------------------------- */
PF_API void pfViewport(PFint x, PFint y, PFsizei width, PFsizei height);       /* pixelforge.h:762 */
PF_API void pfPolygonMode(PFface face, PFpolygonmode mode);                    /* pixelforge.h:777 */
PF_API void pfShadeModel(PFshademode mode);                                    /* pixelforge.h:791 */
PF_API void pfLightModel(PFlightmode mode);                                    /* pixelforge.h:813 */
PF_API void pfLineWidth(PFfloat width);                                        /* pixelforge.h:823 */
PF_API void pfPointSize(PFfloat size);                                         /* pixelforge.h:833 */
PF_API void pfCullFace(PFface face);                                           /* pixelforge.h:843 */
PF_API void pfBlendFunc(PFblendmode mode);                                     /* pixelforge.h:853 */
PF_API void pfDepthFunc(PFdepthmode mode);                                     /* pixelforge.h:863 */
PF_API void pfBindFramebuffer(PFframebuffer* framebuffer);                     /* pixelforge.h:876 */
PF_API void pfBindTexture(PFtexture texture);                                  /* pixelforge.h:889 */
PF_API void pfClear(PFclearflag flag);                                         /* pixelforge.h:899 */
PF_API void pfClearDepth(PFfloat depth);                                       /* pixelforge.h:909 */
PF_API void pfClearColor(PFubyte r, PFubyte g, PFubyte b, PFubyte a);          /* pixelforge.h:922 */

/* ---- lights and materials (pixelforge.h:935-1015) ----------------------------- */
PF_API void      pfEnableLight(PFsizei light);                                 /* pixelforge.h:935 */
PF_API void      pfDisableLight(PFsizei light);                                /* pixelforge.h:945 */
PF_API PFboolean pfIsEnabledLight(PFsizei light);                              /* pixelforge.h:956 */
PF_API void      pfLightf(PFsizei light, PFenum param, PFfloat value);         /* pixelforge.h:968 */
PF_API void      pfLightfv(PFsizei light, PFenum param, const void* value);    /* pixelforge.h:980 */
PF_API void      pfMaterialf(PFface face, PFenum param, PFfloat value);        /* pixelforge.h:992 */
PF_API void      pfMaterialfv(PFface face, PFenum param, const void* value);   /* pixelforge.h:1004 */
PF_API void      pfColorMaterial(PFface face, PFenum mode);                    /* pixelforge.h:1015 */

/* ---- vertex arrays and draws (pixelforge.h:1031-1116) ------------------------ */
PF_API void pfVertexPointer(PFint size, PFenum type, PFsizei stride, const void* pointer);   /* pixelforge.h:1031 */
PF_API void pfNormalPointer(PFenum type, PFsizei stride, const void* pointer);               /* pixelforge.h:1044 */
PF_API void pfTexCoordPointer(PFenum type, PFsizei stride, const void* pointer);             /* pixelforge.h:1056 */
PF_API void pfColorPointer(PFint size, PFenum type, PFsizei stride, const void* pointer);    /* pixelforge.h:1069 */
PF_API void pfDrawElements(PFdrawmode mode, PFsizei count, PFdatatype type, const void* indices); /* pixelforge.h:1082 */
PF_API void pfDrawArrays(PFdrawmode mode, PFint first, PFsizei count);                       /* pixelforge.h:1095 */
PF_API void pfBegin(PFdrawmode mode);                                                         /* pixelforge.h:1108 */
PF_API void pfEnd(void);                                                                      /* pixelforge.h:1116 */

/* ---- immediate-mode attributes (pixelforge.h:1127-1461) ---------------------- */
PF_API void pfVertex2i(PFint x, PFint y);                                      /* pixelforge.h:1127 */
PF_API void pfVertex2f(PFfloat x, PFfloat y);                                  /* pixelforge.h:1138 */
PF_API void pfVertex2fv(const PFfloat* v);                                     /* pixelforge.h:1148 */
PF_API void pfVertex3i(PFint x, PFint y, PFint z);                             /* pixelforge.h:1160 */
PF_API void pfVertex3f(PFfloat x, PFfloat y, PFfloat z);                       /* pixelforge.h:1172 */
PF_API void pfVertex3fv(const PFfloat* v);                                     /* pixelforge.h:1182 */
PF_API void pfVertex4i(PFint x, PFint y, PFint z, PFint w);                    /* pixelforge.h:1195 */
PF_API void pfVertex4f(PFfloat x, PFfloat y, PFfloat z, PFfloat w);            /* pixelforge.h:1208 */
PF_API void pfVertex4fv(const PFfloat* v);                                     /* pixelforge.h:1218 */
PF_API void pfColor(PFcolor color);                                            /* pixelforge.h:1228 */
PF_API void pfColor1ui(PFuint color);                                          /* pixelforge.h:1238 */
PF_API void pfColor3ub(PFubyte r, PFubyte g, PFubyte b);                       /* pixelforge.h:1250 */
PF_API void pfColor3ubv(const PFubyte* v);                                     /* pixelforge.h:1260 */
PF_API void pfColor3us(PFushort r, PFushort g, PFushort b);                    /* pixelforge.h:1272 */
PF_API void pfColor3usv(const PFushort* v);                                    /* pixelforge.h:1282 */
PF_API void pfColor3ui(PFuint r, PFuint g, PFuint b);                          /* pixelforge.h:1294 */
PF_API void pfColor3uiv(const PFuint* v);                                      /* pixelforge.h:1304 */
PF_API void pfColor3f(PFfloat r, PFfloat g, PFfloat b);                        /* pixelforge.h:1316 */
PF_API void pfColor3fv(const PFfloat* v);                                      /* pixelforge.h:1326 */
PF_API void pfColor4ub(PFubyte r, PFubyte g, PFubyte b, PFubyte a);            /* pixelforge.h:1339 */
PF_API void pfColor4ubv(const PFubyte* v);                                     /* pixelforge.h:1349 */
PF_API void pfColor4us(PFushort r, PFushort g, PFushort b, PFushort a);        /* pixelforge.h:1362 */
PF_API void pfColor4usv(const PFushort* v);                                    /* pixelforge.h:1372 */
PF_API void pfColor4ui(PFuint r, PFuint g, PFuint b, PFuint a);                /* pixelforge.h:1385 */
PF_API void pfColor4uiv(const PFuint* v);                                      /* pixelforge.h:1395 */
PF_API void pfColor4f(PFfloat r, PFfloat g, PFfloat b, PFfloat a);             /* pixelforge.h:1408 */
PF_API void pfColor4fv(const PFfloat* v);                                      /* pixelforge.h:1418 */
PF_API void pfTexCoord2f(PFfloat u, PFfloat v);                                /* pixelforge.h:1429 */
PF_API void pfTexCoordfv(const PFfloat* v);                                    /* pixelforge.h:1439 */
PF_API void pfNormal3f(PFfloat x, PFfloat y, PFfloat z);                       /* pixelforge.h:1451 */
PF_API void pfNormal3fv(const PFfloat* v);                                     /* pixelforge.h:1461 */

/* ---- outside the triangle pipeline: exported, set PF_INVALID_OPERATION ------- */
PF_API void pfRects(PFshort x1, PFshort y1, PFshort x2, PFshort y2);           /* pixelforge.h:1477 */
PF_API void pfRectsv(const PFshort* v1, const PFshort* v2);                    /* pixelforge.h:1488 */
PF_API void pfRectf(PFfloat x1, PFfloat y1, PFfloat x2, PFfloat y2);           /* pixelforge.h:1501 */
PF_API void pfRectfv(const PFfloat* v1, const PFfloat* v2);                    /* pixelforge.h:1501 */
PF_API void pfDrawPixels(PFsizei width, PFsizei height, PFpixelformat format,
                         PFdatatype type, const void* pixels);                 /* pixelforge.h:1527 */
PF_API void pfPixelZoom(PFfloat xfactor, PFfloat yfactor);                     /* pixelforge.h:1540 */
PF_API void pfRasterPos2i(PFint x, PFint y);                                   /* pixelforge.h:1551 */
PF_API void pfRasterPos2f(PFfloat x, PFfloat y);                               /* pixelforge.h:1562 */
PF_API void pfRasterPos2fv(const PFfloat* v);                                  /* pixelforge.h:1572 */
PF_API void pfRasterPos3i(PFint x, PFint y, PFint z);                          /* pixelforge.h:1584 */
PF_API void pfRasterPos3f(PFfloat x, PFfloat y, PFfloat z);                    /* pixelforge.h:1596 */
PF_API void pfRasterPos3fv(const PFfloat* v);                                  /* pixelforge.h:1606 */
PF_API void pfRasterPos4i(PFint x, PFint y, PFint z, PFint w);                 /* pixelforge.h:1619 */
PF_API void pfRasterPos4f(PFfloat x, PFfloat y, PFfloat z, PFfloat w);         /* pixelforge.h:1632 */
PF_API void pfRasterPos4fv(const PFfloat* v);                                  /* pixelforge.h:1642 */
PF_API void pfFogi(PFfogparam pname, PFint param);                             /* pixelforge.h:1656 */
PF_API void pfFogf(PFfogparam pname, PFfloat param);                           /* pixelforge.h:1667 */
PF_API void pfFogiv(PFfogparam pname, PFint* param);                           /* pixelforge.h:1678 */
PF_API void pfFogfv(PFfogparam pname, PFfloat* param);                         /* pixelforge.h:1689 */
PF_API void pfFogProcess(void);                                                /* pixelforge.h:1697 */
PF_API PFrenderlist pfGenList(void);                                           /* pixelforge.h:1768 */
PF_API void pfDeleteList(PFrenderlist* renderList);                            /* pixelforge.h:1793 */
PF_API void pfNewList(PFrenderlist renderList);                                /* pixelforge.h:1817 */
PF_API void pfEndList(void);                                                   /* pixelforge.h:1838 */
PF_API void pfCallList(const PFrenderlist renderList);                         /* pixelforge.h:1867 */

/* ---- readback and post-process (pixelforge.h:1718-1735) ---------------------- */
PF_API void pfReadPixels(PFint x, PFint y, PFsizei width, PFsizei height,
                         PFpixelformat format, PFdatatype type, void* pixels); /* pixelforge.h:1718 */
PF_API void pfPostProcess(PFpostprocessfunc postProcessFunction);              /* pixelforge.h:1735 */

/* ---- framebuffers (pixelforge.h:1887-2003) -----------------------------------
 * A framebuffer -- a context's main buffer or a pfGenFramebuffer object -- may
 * be RGBA, RGB, BGR or BGRA unsigned byte, RGB / BGR 5-6-5, RGBA / BGRA
 * 5-5-5-1 or 4-4-4-4, or luminance-alpha, RGB, BGR, RGBA or BGRA half or
 * float.  In BGRA unsigned byte a triangle writes each 4-pixel half of the
 * reference's 8-pixel vector with the value of the half's first pixel, as
 * the reference's SIMD setter does.  The other pairs (single-channel and
 * luminance formats, luminance-alpha unsigned byte) set PF_INVALID_ENUM in
 * pfCreateContext, pfSetMainBuffer and pfGenFramebuffer: in the reference
 * a pixel of those depends on its neighbours' values. */
PF_API PFframebuffer pfGenFramebuffer(PFsizei width, PFsizei height,
                                      PFpixelformat format, PFdatatype type);  /* pixelforge.h:1887 */
PF_API void      pfDeleteFramebuffer(PFframebuffer* framebuffer);              /* pixelforge.h:1899 */
PF_API PFboolean pfIsValidFramebuffer(PFframebuffer* framebuffer);             /* pixelforge.h:1911 */
PF_API void      pfClearFramebuffer(PFframebuffer* framebuffer, PFcolor color, PFfloat depth); /* pixelforge.h:1924 */
PF_API PFcolor   pfGetFramebufferPixel(const PFframebuffer* framebuffer, PFsizei x, PFsizei y); /* pixelforge.h:1938 */
PF_API PFfloat   pfGetFramebufferDepth(const PFframebuffer* framebuffer, PFsizei x, PFsizei y); /* pixelforge.h:1952 */
PF_API void      pfSetFramebufferPixelDepthTest(PFframebuffer* framebuffer, PFsizei x, PFsizei y,
                                                PFfloat z, PFcolor color, PFdepthmode depthMode); /* pixelforge.h:1969 */
PF_API void      pfSetFramebufferPixelDepth(PFframebuffer* framebuffer, PFsizei x, PFsizei y,
                                            PFfloat z, PFcolor color);         /* pixelforge.h:1986 */
PF_API void      pfSetFramebufferPixel(PFframebuffer* framebuffer, PFsizei x, PFsizei y,
                                       PFcolor color);                         /* pixelforge.h:2003 */

/* ---- textures (pixelforge.h:2025-2086) --------------------------------------- */
PF_API PFtexture pfGenTexture(void* pixels, PFsizei width, PFsizei height,
                              PFpixelformat format, PFdatatype type);          /* pixelforge.h:2025 */
PF_API void      pfDeleteTexture(PFtexture* texture, PFboolean freeBuffer);    /* pixelforge.h:2040 */
PF_API PFboolean pfIsValidTexture(const PFtexture texture);                    /* pixelforge.h:2053 */
PF_API void      pfTextureParameter(PFtexture texture, PFtexturewrap wrapMode,
                                    PFtexturefilter filterMode);               /* pixelforge.h:2067 */
PF_API void*     pfGetTexturePixels(const PFtexture texture, PFsizei* width, PFsizei* height,
                                    PFpixelformat* format, PFdatatype* type);  /* pixelforge.h:2086 */

/* ============================================================================
 * Extensions (no counterpart in the reference).
 * ========================================================================== */

/* Render everything recorded so far and write the colour back to the caller's
 * buffer (and depth to the host z-buffer).  The reference needs no such call
 * because it draws synchronously. */
PF_API void pfFinish(void);

/* Enable or disable depth writes (default PF_TRUE, which is the reference's
 * only behaviour, src/internal/primitives/triangles.c:529). */
PF_API void pfDepthMask(PFboolean flag);

/* Zero-copy vertex arrays, indices and textures in device memory.
 *
 * Counterparts of pfVertexPointer, pfNormalPointer, pfTexCoordPointer,
 * pfColorPointer (pixelforge.h:1031-1069), pfDrawElements (:1082) and
 * pfGenTexture (:2025) whose pointers are device memory of the current GPU
 * (cudaMalloc or managed; a host pointer sets PF_INVALID_VALUE and binds
 * nothing).  Nothing is copied when a draw is recorded: the kernels read the
 * arrays and texels when the frame is rendered, at the next observation
 * point, so the caller keeps that memory allocated and unchanged until then
 * (the host-pointer calls copy at the draw call instead).  Stride is ignored,
 * as in the reference.  Types: positions float with 2 to 4 components,
 * normals and texture coordinates float, colours unsigned byte with 3 or 4
 * components (other types: PF_INVALID_ENUM), every pointer but colours
 * 4-byte aligned.  Device arrays draw triangles in every triangle draw mode
 * with PF_FILL polygon modes; points, lines and the PF_POINT / PF_LINE
 * polygon modes are assembled on the host and set PF_INVALID_OPERATION.
 *
 * pfDrawElementsDevice draws `count` unsigned-int indices read from device
 * memory; vertexCount is the number of array elements they may reference
 * (the largest index + 1), which the library cannot find without reading
 * them: the vertex kernel transforms that many.  An index at or past
 * vertexCount is clamped to vertexCount - 1 and sets PF_DEVICE_INDEX_RANGE
 * in pfGetDeviceStatus.  vertexCount 0 sets PF_INVALID_VALUE.
 *
 * pfGenTextureDevice wraps width x height RGBA / unsigned-byte texels in
 * device memory; pfDeleteTexture never frees them. */
PF_API void pfVertexPointerDevice(PFint size, PFenum type, PFsizei stride, const void* devicePointer);
PF_API void pfNormalPointerDevice(PFenum type, PFsizei stride, const void* devicePointer);
PF_API void pfTexCoordPointerDevice(PFenum type, PFsizei stride, const void* devicePointer);
PF_API void pfColorPointerDevice(PFint size, PFenum type, PFsizei stride, const void* devicePointer);
PF_API void pfDrawElementsDevice(PFdrawmode mode, PFsizei count, PFsizei vertexCount, const PFuint* deviceIndices);
PF_API PFtexture pfGenTextureDevice(const void* devicePixels, PFsizei width, PFsizei height);

/* Built-in device post-process hooks, the GPU form of pfPostProcess.  A hook
 * is a __device__ function compiled into the library and applied to every
 * pixel of the current framebuffer, in order with the recorded draws. */
typedef enum {
    PF_HOOK_IDENTITY   = 0,  /* params: none */
    PF_HOOK_FOG_LINEAR = 1,  /* params: PFhookfog */
    PF_HOOK_GRAYSCALE  = 2,  /* params: none */
    PF_HOOK_DITHER     = 3   /* params: none.  The ordered 3x3 dither of the reference's post-process
                                example (examples/raylib/raylib_PostProcess.c:7-19): the pixel at
                                column x, row y becomes white (all four channels 255) when
                                (r + g + b) / 3 >= M[x % 3][y % 3], else 0, with
                                M = {{230, 51, 128}, {25, 102, 179}, {154, 205, 77}} */
} PFhookid;

/* Linear fog on the stored depth.  d = (depth + znear) / (zfar + znear)
 * normalises a frustum's clip-space z (which spans [-znear, zfar]) to [0, 1];
 * f = clamp((end - d) / (end - start), 0, 1); every colour channel c (alpha
 * included) becomes (c*k + fog*(255-k)) / 255 with k = (int)(f*255). */
typedef struct {
    PFfloat znear, zfar, start, end;
    PFcolor color;
} PFhookfog;

PF_API void pfPostProcessDevice(PFuint hookId, const void* params, PFsizei size);

/* Counters accumulated by the current context since its creation or the last
 * pfResetStats.  A fragment is a (pixel, sub-triangle) pair that passes the
 * coverage test inside the viewport, counted before the depth test. */
typedef struct {
    PFuint64 fragments;        /* covered fragments (before depth test) */
    PFuint64 primitives;       /* triangle-face items submitted */
    PFuint64 rasterized;       /* sub-triangles that survived clip and cull */
    PFuint64 flushes;          /* GPU flushes executed */
    PFuint64 bin_overflows;    /* flushes re-binned because a tile bin overflowed */
    PFdouble device_ms;        /* with pfEnableTiming: GPU time of the pipeline kernels */
    PFdouble raster_ms;        /* with pfEnableTiming: GPU time of the tile-raster kernel */
    PFuint64 raster_launches;  /* tile-raster kernel launches */
    PFuint64 kernel_launches;  /* all kernels launched by this library */
    PFuint64 draw_splits;      /* draw groups rendered in two passes because a tile held more
                                  sub-triangles than one bin can sort */
    PFuint64 copy_launches;    /* of kernel_launches: kernels run while draws are recorded
                                  (the index range of an uploaded index array) */
} PFstats;

PF_API void pfGetStats(PFstats* stats);
/* Time the pipeline with CUDA events on the context's stream (adds a few
 * event records per flush; off by default). */
PF_API void pfEnableTiming(PFboolean enable);
PF_API void pfResetStats(void);

/* Device status of the last flush: 0 = no error, otherwise a bit set of
 * PF_DEVICE_* conditions (the context also records PF_INVALID_OPERATION). */
enum {
    PF_DEVICE_OK          = 0,
    PF_DEVICE_NO_GPU      = 1,   /* no CUDA device, or the CUDA runtime failed */
    PF_DEVICE_ALLOC_FAIL  = 2,   /* device memory allocation failed */
    PF_DEVICE_LAUNCH_FAIL = 4,   /* a kernel launch or copy reported an error */
    PF_DEVICE_BIN_LIMIT   = 8,   /* a tile bin exceeded its hard capacity */
    PF_DEVICE_INDEX_RANGE = 16   /* a pfDrawElementsDevice index reached its vertexCount (clamped) */
};
PF_API PFuint pfGetDeviceStatus(void);

/* ---- batches (no counterpart in the reference) -----------------------------
 *
 * Between pfgbBatchBegin and pfgbBatchEnd every context made current on the
 * calling thread records into the batch instead of rendering at its own
 * observation points; pfgbBatchEnd renders all of it -- hundreds of contexts
 * of uneven sizes -- with one launch of each pipeline kernel (the tile
 * rasterizer is a persistent kernel over a work list of (framebuffer, tile)
 * items) and writes every colour buffer back.  Observation points inside the
 * batch (pfFinish, pfReadPixels, ...) render the whole batch so far. */
typedef void* PFgbbatch;
PF_API PFgbbatch pfgbBatchCreate(void);
PF_API void      pfgbBatchDelete(PFgbbatch batch);
PF_API void      pfgbBatchBegin(PFgbbatch batch);
PF_API void      pfgbBatchEnd(PFgbbatch batch);
/* Re-run the device work of the batch's last render `n` times from a CUDA
 * graph (inputs already on the device; framebuffers are rewritten, so a
 * batch that starts each framebuffer with a clear gives the same pixels
 * every time).  Returns the mean GPU milliseconds per run, or < 0. */
PF_API PFfloat   pfgbBatchReplay(PFgbbatch batch, PFuint n);
PF_API void      pfgbBatchGetStats(PFgbbatch batch, PFstats* stats);
PF_API void      pfgbBatchEnableTiming(PFgbbatch batch, PFboolean enable);
/* Tuning knobs (set by the project's autotuner): tile-bin capacity (a power
 * of two, 32..16384; bins still grow on overflow; other values leave the
 * setting) and persistent raster CTAs per SM (1..32, at most as many as fit;
 * 0: as many as fit, the default; larger values leave the setting).
 * batch == NULL tunes the current context. */
PF_API void      pfgbBatchTune(PFgbbatch batch, PFuint binCapacity, PFuint rasterCtasPerSM);
/* The raster's block shape: warps per CTA, 2, 4 (the default) or 8; each
 * warp rasterizes one 8x8 tile at a time.  Other values leave the setting. */
PF_API void      pfgbBatchTuneShape(PFgbbatch batch, PFuint rasterWarpsPerCta);
/* The same graph replay for the current context's last render. */
PF_API PFfloat   pfgbReplay(PFuint n);

/* ---- allocation-free entry point (no counterpart in the reference) --------
 *
 * pfgbDrawTrianglesStatic renders `ntris` triangles straight into device
 * colour (RGBA8, width*height words) and depth (float) buffers that the
 * caller owns, and allocates nothing.  It is for callers that cannot call
 * cudaMalloc: a real-time frame path, where an allocation may block and
 * synchronise the whole device, or an engine or plugin host that owns all
 * device memory through its own pool and only lends out pre-allocated
 * buffers.  It runs the same kernels as the pf* API and gives the same
 * pixels as
 *     pfMatrixMode(PF_PROJECTION); pfLoadIdentity(); pfMultMatrixf(mvp);
 *     pfMatrixMode(PF_MODELVIEW);  pfLoadIdentity();
 *     depthFunc < 0 ? pfDisable(PF_DEPTH_TEST) : pfEnable + pfDepthFunc(depthFunc);
 *     cullMode 0: pfDisable(PF_CULL_FACE); 1: cull PF_BACK; 2: cull PF_FRONT;
 *     pfBegin(PF_TRIANGLES); per vertex pfColor(colors[i]); pfVertex3fv(&positions[3*i]); pfEnd();
 * on a framebuffer already holding `color` and `depth` (no clear), smooth
 * shading, no lighting, texture or blending.
 *
 * positions: device, 9 floats per triangle (object-space x, y, z of its 3
 * vertices); colors: device, one packed RGBA8 word per vertex; mvp: host,
 * 16 floats in the reference's layout; stream: a cudaStream_t or NULL.  The
 * call reads its overflow counters back and waits for `stream` before it
 * returns.
 *
 * Its intermediates live in one file-scope __device__ array of
 * PFGB_STATIC_SCRATCH_BYTES that every GPU loading the library holds until
 * the process exits.  The first call on a device looks up that array's
 * device address (cudaGetSymbolAddress) with the device current; make that
 * first call before any stream capture.  All calls share the array: calls
 * that overlap on the GPU (other streams, other threads) race and corrupt
 * each other, so issue them one after another.  Returns 0, or a negative
 * PFGB_STATIC_E_* code; sizes beyond the limits below are rejected. */
#define PFGB_STATIC_MAX_TRIANGLES   8192      /* culling off: 16,384 face items */
#define PFGB_STATIC_MAX_WIDTH       512
#define PFGB_STATIC_MAX_HEIGHT      512
#define PFGB_STATIC_BIN_CAPACITY    512       /* sub-triangles per 8x8 tile */
#define PFGB_STATIC_CLIP_CAPACITY   32768     /* extra sub-triangles of clipped triangles */
#define PFGB_STATIC_SCRATCH_BYTES   16353024  /* 15.6 MiB */
#define PFGB_STATIC_E_TOO_LARGE     (-1)      /* more triangles or pixels than the limits */
#define PFGB_STATIC_E_INVALID       (-2)      /* null pointer or invalid mode */
#define PFGB_STATIC_E_CUDA          (-3)      /* a CUDA call failed */
#define PFGB_STATIC_E_CAPACITY      (-4)      /* a tile needed more than PFGB_STATIC_BIN_CAPACITY entries,
                                                 or clipping more than PFGB_STATIC_CLIP_CAPACITY
                                                 sub-triangles; the buffers were not modified */
PF_API int pfgbDrawTrianglesStatic(const float* positions, const uint32_t* colors, uint32_t ntris,
                                   const float* mvp, uint32_t* color, float* depth,
                                   uint32_t width, uint32_t height, int depthFunc, int cullMode,
                                   void* stream);

#if defined(__cplusplus)
}
#endif

#endif /* PIXELFORGE_GB300_H */
