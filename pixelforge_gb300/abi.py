"""ctypes binding of the PixelForge C ABI (include/pixelforge.h).

The same binding drives any shared library that exports the ``pf*`` API:
libpixelforge_gb300.so (this package's GPU library), and -- in tests and the
CPU-baseline leg of bench.py only -- the reference build and the CPU oracle.
Argument types follow the reference prototypes (src/pixelforge.h:452-2090).
"""
from __future__ import annotations

import ctypes as C

PFsizei = C.c_uint32
PFenum = C.c_uint32
PFint = C.c_int32
PFuint = C.c_uint32
PFfloat = C.c_float
PFbool = C.c_bool
PFubyte = C.c_uint8
PFushort = C.c_uint16
PFshort = C.c_int16
PFptr = C.c_void_p
PFenum_i = C.c_int   # C enums are int-sized


class PFcolor(C.Structure):
    _fields_ = [("r", C.c_uint8), ("g", C.c_uint8), ("b", C.c_uint8), ("a", C.c_uint8)]


class PFframebuffer(C.Structure):
    _fields_ = [("texture", C.c_void_p), ("zbuffer", C.POINTER(C.c_float))]


class PFstats(C.Structure):
    _fields_ = [("fragments", C.c_uint64), ("primitives", C.c_uint64),
                ("rasterized", C.c_uint64), ("flushes", C.c_uint64),
                ("bin_overflows", C.c_uint64), ("device_ms", C.c_double),
                ("raster_ms", C.c_double), ("raster_launches", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("draw_splits", C.c_uint64),
                ("copy_launches", C.c_uint64)]


class PFhookfog(C.Structure):
    _fields_ = [("znear", C.c_float), ("zfar", C.c_float), ("start", C.c_float),
                ("end", C.c_float), ("color", PFcolor)]


POSTPROCESS = C.CFUNCTYPE(PFcolor, PFint, PFint, PFfloat, PFcolor)

# enum values (src/pixelforge.h:151-392)
PF_UNSIGNED_BYTE, PF_UNSIGNED_SHORT = 0, 1
PF_UNSIGNED_INT, PF_BYTE, PF_SHORT, PF_INT, PF_HALF_FLOAT, PF_FLOAT, PF_DOUBLE = 5, 6, 7, 8, 9, 10, 11
PF_TEXTURE_2D, PF_FRAMEBUFFER, PF_BLEND, PF_DEPTH_TEST = 0x1, 0x2, 0x4, 0x8
PF_CULL_FACE, PF_NORMALIZE, PF_LIGHTING, PF_COLOR_MATERIAL = 0x10, 0x20, 0x40, 0x80
PF_VERTEX_ARRAY, PF_NORMAL_ARRAY, PF_COLOR_ARRAY, PF_TEXTURE_COORD_ARRAY = 0x100, 0x200, 0x400, 0x800
PF_NO_ERROR, PF_INVALID_ENUM, PF_INVALID_VALUE, PF_STACK_OVERFLOW = 0, 1, 2, 3
PF_STACK_UNDERFLOW, PF_INVALID_OPERATION, PF_ERROR_OUT_OF_MEMORY = 4, 5, 6
PF_COLOR_BUFFER_BIT, PF_DEPTH_BUFFER_BIT = 1, 2
PF_MODELVIEW, PF_PROJECTION, PF_TEXTURE = 0, 1, 2
(PF_POINTS, PF_LINES, PF_TRIANGLES, PF_TRIANGLE_FAN, PF_TRIANGLE_STRIP,
 PF_QUADS, PF_QUAD_FAN, PF_QUAD_STRIP) = range(8)
(PF_BLEND_AVERAGE, PF_BLEND_ALPHA, PF_BLEND_ADD, PF_BLEND_SUB, PF_BLEND_MUL,
 PF_BLEND_SCREEN, PF_BLEND_LIGHTEN, PF_BLEND_DARKEN) = range(8)
PF_EQUAL, PF_NOTEQUAL, PF_LESS, PF_LEQUAL, PF_GREATER, PF_GEQUAL = range(6)
PF_POINT, PF_LINE, PF_FILL = range(3)
PF_FLAT, PF_SMOOTH = 0, 1
PF_GOURAUD, PF_PHONG = 0, 1
PF_FRONT, PF_BACK, PF_FRONT_AND_BACK = 0, 1, 2
PF_REPEAT, PF_MIRRORED_REPEAT, PF_CLAMP_TO_EDGE = 0, 1, 2
PF_NEAREST, PF_BILINEAR = 0, 1
PF_AMBIENT_AND_DIFFUSE, PF_AMBIENT, PF_DIFFUSE, PF_SPECULAR = 1, 2, 3, 4
PF_EMISSION, PF_SHININESS = 5, 6
PF_POSITION, PF_SPOT_DIRECTION = 7, 8
PF_SPOT_INNER_CUTOFF, PF_SPOT_OUTER_CUTOFF = 10, 11
PF_CONSTANT_ATTENUATION, PF_LINEAR_ATTENUATION, PF_QUADRATIC_ATTENUATION = 12, 13, 14
(PF_RED, PF_GREEN, PF_BLUE, PF_ALPHA, PF_LUMINANCE, PF_LUMINANCE_ALPHA, PF_RGB, PF_RGBA,
 PF_BGR, PF_BGRA) = range(10)
PF_UNSIGNED_SHORT_5_6_5, PF_UNSIGNED_SHORT_5_5_5_1, PF_UNSIGNED_SHORT_4_4_4_4 = 2, 3, 4


def pixel_bytes(fmt: int, typ: int) -> int:
    """Bytes of one pixel of a format / type pair (0: no such pixel)."""
    comps = [1, 1, 1, 1, 1, 2, 3, 4, 3, 4][fmt] if 0 <= fmt < 10 else 0
    if typ in (PF_UNSIGNED_SHORT_5_6_5, PF_UNSIGNED_SHORT_5_5_5_1, PF_UNSIGNED_SHORT_4_4_4_4):
        return 2
    return comps * {PF_UNSIGNED_BYTE: 1, PF_HALF_FLOAT: 2, PF_FLOAT: 4}.get(typ, 0)
(PF_VIEWPORT, PF_COLOR_CLEAR_VALUE, PF_DEPTH_CLEAR_VALUE, PF_CULL_FACE_MODE, PF_CURRENT_COLOR,
 PF_CURRENT_NORMAL, PF_CURRENT_TEXTURE_COORDS, PF_CURRENT_RASTER_POSITION, PF_BLEND_FUNC, PF_DEPTH_FUNC,
 PF_POLYGON_MODE, PF_POINT_SIZE, PF_LINE_WIDTH, PF_MATRIX_MODE, PF_PROJECTION_MATRIX, PF_MODELVIEW_MATRIX,
 PF_TEXTURE_MATRIX, PF_MAX_PROJECTION_STACK_DEPTH, PF_MAX_MODELVIEW_STACK_DEPTH, PF_MAX_TEXTURE_STACK_DEPTH,
 PF_SHADE_MODEL) = range(10000, 10021)
PF_HOOK_IDENTITY, PF_HOOK_FOG_LINEAR, PF_HOOK_GRAYSCALE, PF_HOOK_DITHER = 0, 1, 2, 3
PF_DEVICE_INDEX_RANGE = 16

_V = None
_FP = C.POINTER(C.c_float)

# name -> (restype, argtypes); the reference's prototypes.
PROTOTYPES = {
    "pfCreateContext": (PFptr, [PFptr, PFsizei, PFsizei, PFenum_i, PFenum_i]),
    "pfDeleteContext": (_V, [PFptr]),
    "pfSetMainBuffer": (_V, [PFptr, PFsizei, PFsizei, PFenum_i, PFenum_i]),
    "pfSetAuxBuffer": (_V, [PFptr]),
    "pfSwapBuffers": (_V, []),
    "pfGetCurrentContext": (PFptr, []),
    "pfMakeCurrent": (_V, [PFptr]),
    "pfIsEnabled": (PFbool, [PFenum_i]),
    "pfEnable": (_V, [PFenum_i]),
    "pfDisable": (_V, [PFenum_i]),
    "pfGetIntegerv": (_V, [PFenum, C.POINTER(PFint)]),
    "pfGetFloatv": (_V, [PFenum, _FP]),
    "pfGetError": (PFenum_i, []),
    "pfMatrixMode": (_V, [PFenum_i]),
    "pfPushMatrix": (_V, []),
    "pfPopMatrix": (_V, []),
    "pfLoadIdentity": (_V, []),
    "pfTranslatef": (_V, [PFfloat] * 3),
    "pfRotatef": (_V, [PFfloat] * 4),
    "pfScalef": (_V, [PFfloat] * 3),
    "pfMultMatrixf": (_V, [_FP]),
    "pfFrustum": (_V, [PFfloat] * 6),
    "pfOrtho": (_V, [PFfloat] * 6),
    "pfViewport": (_V, [PFint, PFint, PFsizei, PFsizei]),
    "pfPolygonMode": (_V, [PFenum_i, PFenum_i]),
    "pfShadeModel": (_V, [PFenum_i]),
    "pfLightModel": (_V, [PFenum_i]),
    "pfCullFace": (_V, [PFenum_i]),
    "pfBlendFunc": (_V, [PFenum_i]),
    "pfDepthFunc": (_V, [PFenum_i]),
    "pfBindFramebuffer": (_V, [C.POINTER(PFframebuffer)]),
    "pfBindTexture": (_V, [PFptr]),
    "pfClear": (_V, [PFenum_i]),
    "pfClearDepth": (_V, [PFfloat]),
    "pfClearColor": (_V, [PFubyte] * 4),
    "pfEnableLight": (_V, [PFsizei]),
    "pfDisableLight": (_V, [PFsizei]),
    "pfIsEnabledLight": (PFbool, [PFsizei]),
    "pfLightf": (_V, [PFsizei, PFenum, PFfloat]),
    "pfLightfv": (_V, [PFsizei, PFenum, PFptr]),
    "pfMaterialf": (_V, [PFenum_i, PFenum, PFfloat]),
    "pfMaterialfv": (_V, [PFenum_i, PFenum, PFptr]),
    "pfColorMaterial": (_V, [PFenum_i, PFenum]),
    "pfVertexPointer": (_V, [PFint, PFenum, PFsizei, PFptr]),
    "pfNormalPointer": (_V, [PFenum, PFsizei, PFptr]),
    "pfTexCoordPointer": (_V, [PFenum, PFsizei, PFptr]),
    "pfColorPointer": (_V, [PFint, PFenum, PFsizei, PFptr]),
    "pfDrawElements": (_V, [PFenum_i, PFsizei, PFenum_i, PFptr]),
    "pfDrawArrays": (_V, [PFenum_i, PFint, PFsizei]),
    "pfBegin": (_V, [PFenum_i]),
    "pfEnd": (_V, []),
    "pfVertex2f": (_V, [PFfloat] * 2),
    "pfVertex3f": (_V, [PFfloat] * 3),
    "pfVertex4f": (_V, [PFfloat] * 4),
    "pfVertex3fv": (_V, [_FP]),
    "pfColor3ub": (_V, [PFubyte] * 3),
    "pfColor4ub": (_V, [PFubyte] * 4),
    "pfColor4f": (_V, [PFfloat] * 4),
    "pfColor3f": (_V, [PFfloat] * 3),
    "pfTexCoord2f": (_V, [PFfloat] * 2),
    "pfNormal3f": (_V, [PFfloat] * 3),
    "pfReadPixels": (_V, [PFint, PFint, PFsizei, PFsizei, PFenum_i, PFenum_i, PFptr]),
    "pfPostProcess": (_V, [POSTPROCESS]),
    "pfGenFramebuffer": (PFframebuffer, [PFsizei, PFsizei, PFenum_i, PFenum_i]),
    "pfDeleteFramebuffer": (_V, [C.POINTER(PFframebuffer)]),
    "pfClearFramebuffer": (_V, [C.POINTER(PFframebuffer), PFcolor, PFfloat]),
    "pfGetFramebufferPixel": (PFcolor, [C.POINTER(PFframebuffer), PFsizei, PFsizei]),
    "pfGetFramebufferDepth": (PFfloat, [C.POINTER(PFframebuffer), PFsizei, PFsizei]),
    "pfGenTexture": (PFptr, [PFptr, PFsizei, PFsizei, PFenum_i, PFenum_i]),
    "pfDeleteTexture": (_V, [C.POINTER(C.c_void_p), PFbool]),
    "pfTextureParameter": (_V, [PFptr, PFenum_i, PFenum_i]),
    "pfGetBooleanv": (_V, [PFenum, C.POINTER(PFbool)]),
    "pfGetDoublev": (_V, [PFenum, C.POINTER(C.c_double)]),
    "pfGetPointerv": (_V, [PFenum, C.POINTER(C.c_void_p)]),
    "pfLineWidth": (_V, [PFfloat]),
    "pfPointSize": (_V, [PFfloat]),
    "pfVertex2i": (_V, [PFint] * 2),
    "pfVertex2fv": (_V, [_FP]),
    "pfVertex3i": (_V, [PFint] * 3),
    "pfVertex4i": (_V, [PFint] * 4),
    "pfVertex4fv": (_V, [_FP]),
    "pfColor": (_V, [PFcolor]),
    "pfColor1ui": (_V, [PFuint]),
    "pfColor3ubv": (_V, [C.POINTER(PFubyte)]),
    "pfColor3us": (_V, [PFushort] * 3),
    "pfColor3usv": (_V, [C.POINTER(PFushort)]),
    "pfColor3ui": (_V, [PFuint] * 3),
    "pfColor3uiv": (_V, [C.POINTER(PFuint)]),
    "pfColor3fv": (_V, [_FP]),
    "pfColor4ubv": (_V, [C.POINTER(PFubyte)]),
    "pfColor4us": (_V, [PFushort] * 4),
    "pfColor4usv": (_V, [C.POINTER(PFushort)]),
    "pfColor4ui": (_V, [PFuint] * 4),
    "pfColor4uiv": (_V, [C.POINTER(PFuint)]),
    "pfColor4fv": (_V, [_FP]),
    "pfTexCoordfv": (_V, [_FP]),
    "pfNormal3fv": (_V, [_FP]),
    "pfRects": (_V, [PFshort] * 4),
    "pfRectsv": (_V, [C.POINTER(PFshort)] * 2),
    "pfRectf": (_V, [PFfloat] * 4),
    "pfRectfv": (_V, [_FP] * 2),
    "pfDrawPixels": (_V, [PFsizei, PFsizei, PFenum_i, PFenum_i, PFptr]),
    "pfPixelZoom": (_V, [PFfloat] * 2),
    "pfRasterPos2i": (_V, [PFint] * 2),
    "pfRasterPos2f": (_V, [PFfloat] * 2),
    "pfRasterPos2fv": (_V, [_FP]),
    "pfRasterPos3i": (_V, [PFint] * 3),
    "pfRasterPos3f": (_V, [PFfloat] * 3),
    "pfRasterPos3fv": (_V, [_FP]),
    "pfRasterPos4i": (_V, [PFint] * 4),
    "pfRasterPos4f": (_V, [PFfloat] * 4),
    "pfRasterPos4fv": (_V, [_FP]),
    "pfFogi": (_V, [PFenum_i, PFint]),
    "pfFogf": (_V, [PFenum_i, PFfloat]),
    "pfFogiv": (_V, [PFenum_i, C.POINTER(PFint)]),
    "pfFogfv": (_V, [PFenum_i, _FP]),
    "pfFogProcess": (_V, []),
    "pfGenList": (PFptr, []),
    "pfDeleteList": (_V, [C.POINTER(C.c_void_p)]),
    "pfNewList": (_V, [PFptr]),
    "pfEndList": (_V, []),
    "pfCallList": (_V, [PFptr]),
    "pfIsValidFramebuffer": (PFbool, [C.POINTER(PFframebuffer)]),
    "pfSetFramebufferPixelDepthTest": (_V, [C.POINTER(PFframebuffer), PFsizei, PFsizei, PFfloat, PFcolor,
                                            PFenum_i]),
    "pfSetFramebufferPixelDepth": (_V, [C.POINTER(PFframebuffer), PFsizei, PFsizei, PFfloat, PFcolor]),
    "pfSetFramebufferPixel": (_V, [C.POINTER(PFframebuffer), PFsizei, PFsizei, PFcolor]),
    "pfIsValidTexture": (PFbool, [PFptr]),
    "pfgbDrawTrianglesStatic": (C.c_int, [PFptr, PFptr, C.c_uint32, PFptr, PFptr, PFptr, C.c_uint32, C.c_uint32,
                                          C.c_int, C.c_int, PFptr]),
    # extensions (absent from the reference build)
    "pfFinish": (_V, []),
    "pfDepthMask": (_V, [PFbool]),
    "pfPostProcessDevice": (_V, [PFuint, PFptr, PFsizei]),
    "pfGetStats": (_V, [C.POINTER(PFstats)]),
    "pfResetStats": (_V, []),
    "pfGetDeviceStatus": (PFuint, []),
    "pfEnableTiming": (_V, [PFbool]),
    "pfGetTexturePixels": (PFptr, [PFptr, PFptr, PFptr, PFptr, PFptr]),
    "pfVertexPointerDevice": (_V, [PFint, PFenum, PFsizei, PFptr]),
    "pfNormalPointerDevice": (_V, [PFenum, PFsizei, PFptr]),
    "pfTexCoordPointerDevice": (_V, [PFenum, PFsizei, PFptr]),
    "pfColorPointerDevice": (_V, [PFint, PFenum, PFsizei, PFptr]),
    "pfDrawElementsDevice": (_V, [PFenum_i, PFsizei, PFsizei, PFptr]),
    "pfGenTextureDevice": (PFptr, [PFptr, PFsizei, PFsizei]),
    "pfgbBatchCreate": (PFptr, []),
    "pfgbBatchDelete": (_V, [PFptr]),
    "pfgbBatchBegin": (_V, [PFptr]),
    "pfgbBatchEnd": (_V, [PFptr]),
    "pfgbBatchReplay": (PFfloat, [PFptr, PFuint]),
    "pfgbBatchGetStats": (_V, [PFptr, C.POINTER(PFstats)]),
    "pfgbBatchEnableTiming": (_V, [PFptr, PFbool]),
    "pfgbBatchTune": (_V, [PFptr, PFuint, PFuint]),
    "pfgbBatchTuneShape": (_V, [PFptr, PFuint]),
    "pfgbReplay": (PFfloat, [PFuint]),
}


class PixelForgeLib:
    """Thin attribute access to one ``pf*`` shared library.

    ``lib.pfVertex3f(...)`` calls the C function with the reference's argument
    types.  Functions that the loaded library does not export (the extensions,
    when it is the reference build) are ``None``.
    """

    def __init__(self, path: str, mode: int = C.RTLD_LOCAL):
        self.path = path
        self._dll = C.CDLL(path, mode=mode)
        for name, (res, args) in PROTOTYPES.items():
            try:
                fn = getattr(self._dll, name)
            except AttributeError:
                setattr(self, name, None)
                continue
            fn.restype = res
            fn.argtypes = args
            setattr(self, name, fn)

    def has(self, name: str) -> bool:
        return getattr(self, name, None) is not None

    def raw(self, name: str):
        return getattr(self._dll, name)
