"""The drop-in boundary, without a GPU.

libpixelforge_gb300.so must load on a host without a GPU, export every
function that include/pixelforge.h and include/pixelforge_grad.h declare,
and keep the reference's host-side state semantics (errors, matrix stacks,
getters) -- those run on the host and are compared here with the CPU oracle
and, where it can be built, the reference.  Rendering calls on a host
without a device must fail loudly (a device status bit and
PF_INVALID_OPERATION), never fall back to the CPU.
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from pixelforge_gb300 import LIB_PATH, abi as A, load_library

ROOT = Path(__file__).resolve().parent.parent


def declared(header: str, macro: str):
    text = (ROOT / "include" / header).read_text()
    return sorted(set(re.findall(macro + r"\s+[\w\s\*]+?\b(pf\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    return load_library()


def test_exports_every_declared_function(lib):
    names = declared("pixelforge.h", "PF_API") + declared("pixelforge_grad.h", "PFGRAD_API")
    assert len(names) > 140
    dll = C.CDLL(str(LIB_PATH))
    missing = [n for n in names if not hasattr(dll, n)]
    assert not missing, f"not exported: {missing}"


def test_reference_api_is_complete():
    """Every pf* function of the reference header (as re-declared, with its
    line citation, in include/pixelforge.h) is bound by the ctypes layer."""
    text = (ROOT / "include" / "pixelforge.h").read_text()
    cited = re.findall(r"PF_API[^;]*?\b(pf\w+)\s*\([^;]*;\s*/\* pixelforge\.h:\d+", text, re.S)
    assert len(cited) >= 120
    assert not [n for n in cited if n not in A.PROTOTYPES]


def _ctx(lib, w=16, h=16):
    buf = np.zeros((h, w, 4), np.uint8)
    c = lib.pfCreateContext(buf.ctypes.data_as(C.c_void_p), w, h, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
    assert c
    lib.pfMakeCurrent(c)
    return c, buf


def state_script(lib):
    """A sequence of host-side state calls; returns every observable result."""
    out = []
    c, buf = _ctx(lib)
    try:
        out.append(("err0", lib.pfGetError()))
        lib.pfMatrixMode(A.PF_PROJECTION)
        for _ in range(3):
            lib.pfPushMatrix()
            out.append(("push", lib.pfGetError()))
        for _ in range(4):
            lib.pfPopMatrix()
            out.append(("pop", lib.pfGetError()))
        lib.pfMatrixMode(A.PF_MODELVIEW)
        for _ in range(9):
            lib.pfPushMatrix()
        out.append(("mv overflow", lib.pfGetError()))
        for _ in range(9):
            lib.pfPopMatrix()
        out.append(("mv pops", lib.pfGetError()))
        lib.pfLoadIdentity()
        lib.pfTranslatef(0.25, -1.5, 3.0)
        lib.pfRotatef(33.0, 0.3, 0.9, -0.2)
        lib.pfScalef(1.5, 0.75, 2.0)
        m = (C.c_float * 16)()
        lib.pfGetFloatv(A.PF_MODELVIEW_MATRIX, m)
        out.append(("modelview", [np.float32(x).view(np.uint32).item() for x in m]))
        lib.pfMatrixMode(A.PF_PROJECTION)
        lib.pfLoadIdentity()
        lib.pfFrustum(-0.1, 0.1, -0.075, 0.075, 0.1, 100.0)
        lib.pfGetFloatv(A.PF_PROJECTION_MATRIX, m)
        out.append(("frustum", [np.float32(x).view(np.uint32).item() for x in m]))
        lib.pfLoadIdentity()
        lib.pfOrtho(-2.0, 3.0, -1.0, 1.5, 0.5, 20.0)
        lib.pfGetFloatv(A.PF_PROJECTION_MATRIX, m)
        out.append(("ortho", [np.float32(x).view(np.uint32).item() for x in m]))
        lib.pfViewport(2, 3, 10, 9)
        v = (C.c_int32 * 4)()
        lib.pfGetIntegerv(A.PF_VIEWPORT, v)
        out.append(("viewport", list(v)))
        lib.pfEnable(A.PF_BLEND | A.PF_DEPTH_TEST)
        lib.pfDisable(A.PF_CULL_FACE)
        out.append(("enabled", [bool(lib.pfIsEnabled(s)) for s in
                                (A.PF_BLEND, A.PF_DEPTH_TEST, A.PF_CULL_FACE, A.PF_TEXTURE_2D, A.PF_LIGHTING)]))
        lib.pfBlendFunc(A.PF_BLEND_ADD)
        lib.pfDepthFunc(A.PF_GREATER)
        lib.pfClearDepth(0.5)
        f = (C.c_float * 4)()
        lib.pfGetFloatv(A.PF_DEPTH_CLEAR_VALUE, f)
        out.append(("clear depth", f[0]))
        lib.pfGetIntegerv(A.PF_DEPTH_FUNC, v)
        out.append(("depth func", v[0]))
        lib.pfGetIntegerv(A.PF_BLEND_FUNC, v)
        out.append(("blend func", v[0]))
        out.append(("err end", lib.pfGetError()))
        # raster position, pixel zoom, fog and render-list parameter errors
        lib.pfRasterPos3f(2.75, -1.5, 0.25)
        lib.pfGetFloatv(A.PF_CURRENT_RASTER_POSITION, f)
        out.append(("raster pos f", [f[0], f[1]]))
        lib.pfGetIntegerv(A.PF_CURRENT_RASTER_POSITION, v)
        out.append(("raster pos i", [v[0], v[1]]))
        lib.pfPixelZoom(2.5, 0.5)
        for name, e in (("zoom x", 10032), ("zoom y", 10033)):
            lib.pfGetFloatv(e, f)
            out.append((name, f[0]))
        for call in (lambda: lib.pfFogi(0, 3), lambda: lib.pfFogi(1, 2), lambda: lib.pfFogf(0, 1.0),
                     lambda: lib.pfFogf(1, 1.5), lambda: lib.pfFogi(4, 1), lambda: lib.pfFogi(9, 1)):
            call()
            out.append(("fog param", lib.pfGetError()))
        lib.pfNewList(None)
        out.append(("new null list", lib.pfGetError()))
        lib.pfEndList()
        out.append(("end without list", lib.pfGetError()))
        px = (C.c_uint8 * 16)()
        lib.pfDrawPixels(0, 2, A.PF_RGBA, A.PF_UNSIGNED_BYTE, px)
        out.append(("draw pixels empty", lib.pfGetError()))
        lib.pfDrawPixels(2, 2, 11, A.PF_UNSIGNED_BYTE, px)
        out.append(("draw pixels format", lib.pfGetError()))
        lib.pfDrawPixels(2, 2, A.PF_RGBA, 2, px)
        out.append(("draw pixels no getter", lib.pfGetError()))
        lib.pfMatrixMode(12345)
        out.append(("bad matrix mode", lib.pfGetError()))
        out.append(("error reset", lib.pfGetError()))
    finally:
        lib.pfDeleteContext(c)
    return out


def test_host_state_matches_oracle(lib, oracle):
    got, ref = state_script(lib), state_script(oracle)
    for g, r in zip(got, ref):
        assert g == r, f"{g[0]}: {g[1]} vs oracle {r[1]}"


def test_host_state_matches_reference(lib, ref_shim):
    got, ref = state_script(lib), state_script(ref_shim)
    for g, r in zip(got, ref):
        assert g == r, f"{g[0]}: {g[1]} vs reference {r[1]}"


def test_no_device_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    c, buf = _ctx(lib)
    try:
        lib.pfBegin(A.PF_TRIANGLES)
        lib.pfVertex2f(0.0, 0.0)
        lib.pfVertex2f(1.0, 0.0)
        lib.pfVertex2f(0.0, 1.0)
        lib.pfEnd()
        lib.pfFinish()
        assert lib.pfGetDeviceStatus() != 0
        assert lib.pfGetError() == A.PF_INVALID_OPERATION
    finally:
        lib.pfDeleteContext(c)


def test_static_entry_rejects_oversize_without_device(lib):
    f = lib.raw("pfgbDrawTrianglesStatic")
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                  C.c_uint32, C.c_int, C.c_int, C.c_void_p]
    dummy = C.c_void_p(16)
    assert f(dummy, dummy, 8193, dummy, dummy, dummy, 64, 64, 0, 0, None) == -1    # too many triangles
    assert f(dummy, dummy, 1, dummy, dummy, dummy, 513, 64, 0, 0, None) == -1      # too wide
    assert f(None, dummy, 1, dummy, dummy, dummy, 64, 64, 0, 0, None) == -2        # no positions
    assert f(dummy, dummy, 1, dummy, dummy, dummy, 64, 64, 6, 0, None) == -2       # depth function
    assert f(dummy, dummy, 1, dummy, dummy, dummy, 64, 64, 2, 3, None) == -2       # cull mode


def test_device_pointer_calls_refuse_host_memory(lib):
    """The zero-copy calls take device memory only: a host pointer (or no
    GPU at all) sets PF_INVALID_VALUE and binds nothing, other types
    PF_INVALID_ENUM; pfGenTextureDevice returns no texture."""
    buf = np.zeros((8, 8, 4), np.uint8)
    arr = np.zeros(64, np.float32)
    p = arr.ctypes.data_as(C.c_void_p)
    ctx = lib.pfCreateContext(buf.ctypes.data_as(C.c_void_p), 8, 8, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
    lib.pfMakeCurrent(ctx)
    try:
        for call in (lambda: lib.pfVertexPointerDevice(3, A.PF_FLOAT, 0, p),
                     lambda: lib.pfNormalPointerDevice(A.PF_FLOAT, 0, p),
                     lambda: lib.pfTexCoordPointerDevice(A.PF_FLOAT, 0, p),
                     lambda: lib.pfColorPointerDevice(4, A.PF_UNSIGNED_BYTE, 0, p)):
            call()
            assert lib.pfGetError() == A.PF_INVALID_VALUE
        lib.pfVertexPointerDevice(3, A.PF_DOUBLE, 0, p)
        assert lib.pfGetError() == A.PF_INVALID_ENUM
        lib.pfColorPointerDevice(4, A.PF_FLOAT, 0, p)
        assert lib.pfGetError() == A.PF_INVALID_ENUM
        lib.pfEnable(A.PF_VERTEX_ARRAY)
        lib.pfDrawElementsDevice(A.PF_TRIANGLES, 3, 3, p)
        assert lib.pfGetError() == A.PF_INVALID_VALUE
        assert not lib.pfGenTextureDevice(p, 4, 4)
        assert lib.pfGetError() == A.PF_INVALID_VALUE
    finally:
        lib.pfDeleteContext(ctx)


def test_framebuffer_formats_refused(lib, oracle):
    """Framebuffer formats whose reference results depend on other pixels or
    on the SIMD lane are refused with PF_INVALID_ENUM, by the library and
    the oracle alike; every accepted pair is a valid pixel format."""
    from fbscenes import FB_ACCEPTED, FB_REFUSED, refused_formats
    for lb in (lib, oracle):
        res = refused_formats(lb)
        assert len(res) == len(FB_REFUSED)
        for pair, null, err in res:
            assert null and err == A.PF_INVALID_ENUM, pair
    assert len(FB_ACCEPTED) == 20 and all(A.pixel_bytes(*p) for p in FB_ACCEPTED)


def test_framebuffer_pixel_functions_every_format(lib, oracle):
    """pfSetFramebufferPixel / pfGetFramebufferPixel and the stored bytes of
    a framebuffer object of every accepted format, library against oracle
    (host-side: the scalar setter and getter of pf_pixfmt.h, no device)."""
    from fbscenes import FB_ACCEPTED
    rng = np.random.default_rng(77)
    cols = rng.integers(0, 256, (64, 4)).astype(np.uint8)
    for fmt in FB_ACCEPTED:
        res = []
        for lb in (lib, oracle):
            buf = np.zeros((4, 4, 4), np.uint8)
            ctx = lb.pfCreateContext(buf.ctypes.data_as(C.c_void_p), 4, 4, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
            lb.pfMakeCurrent(ctx)
            fb = lb.pfGenFramebuffer(8, 8, *fmt)
            ref = C.pointer(fb)
            got = []
            for i, c in enumerate(cols):
                lb.pfSetFramebufferPixel(ref, i % 8, i // 8, A.PFcolor(*map(int, c)))
                g = lb.pfGetFramebufferPixel(ref, i % 8, i // 8)
                got.append((g.r, g.g, g.b, g.a))
            px = lb.raw("pfGetTexturePixels")
            px.restype = C.c_void_p
            px.argtypes = [C.c_void_p] * 5
            base = px(fb.texture, None, None, None, None)
            raw = np.ctypeslib.as_array(C.cast(base, C.POINTER(C.c_uint8)), shape=(64 * A.pixel_bytes(*fmt),)).copy()
            res.append((np.array(got), raw, lb.pfGetError()))
            lb.pfDeleteFramebuffer(ref)
            lb.pfDeleteContext(ctx)
        (g1, r1, e1), (g2, r2, e2) = res
        assert e1 == e2 == A.PF_NO_ERROR, fmt
        assert np.array_equal(r1, r2), f"{fmt}: stored bytes differ"
        assert np.array_equal(g1, g2), f"{fmt}: read-back colours differ"
