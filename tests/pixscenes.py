"""Seeded scenes of the API outside the triangle path (render lists,
pfRect*, pfDrawPixels with every source format, pfFog* / pfFogProcess),
interleaved with triangles and replayable on any pf* library."""
from __future__ import annotations

import ctypes as C

import numpy as np

from pixelforge_gb300 import abi as A
from pixelforge_gb300.scenes import Frame, Target, _ptr

# every (format, type) pair the reference has a scalar getter for
# (src/internal/pixel.h:765-809): format ids and type ids of src/pixelforge.h
PIXEL_FORMATS = [(f, 0) for f in range(10)] + [(f, 9) for f in range(10)] + [(f, 10) for f in range(10)] + \
    [(6, 2), (8, 2), (7, 3), (9, 3), (7, 4), (9, 4)]
_COMPS = [1, 1, 1, 1, 1, 2, 3, 4, 3, 4]
PF_FOG_MODE, PF_FOG_DENSITY, PF_FOG_START, PF_FOG_END, PF_FOG_COLOR = range(5)


def pixel_source(fmt: int, typ: int, w: int, h: int, rng) -> np.ndarray:
    """Source pixels of a format: bytes, halves / floats in [-0.05, 1.05],
    or packed shorts."""
    n = w * h
    if typ == 0:
        return rng.integers(0, 256, n * _COMPS[fmt]).astype(np.uint8)
    if typ in (2, 3, 4):
        return rng.integers(0, 65536, n).astype(np.uint16)
    v = rng.uniform(-0.05, 1.05, n * _COMPS[fmt])
    return v.astype(np.float16).view(np.uint16) if typ == 9 else v.astype(np.float32)


def px_case(seed: int) -> dict:
    r = np.random.default_rng(seed)
    kind = ["rects", "pixels", "fog", "list"][seed % 4]
    proj = ["default", "frustum"][int(r.integers(2))]
    return dict(seed=seed, kind=kind, depth=int(r.integers(-1, 6)), blend=int(r.integers(-1, 8)),
                # pfDrawPixels does not divide by w: a raster position under a
                # perspective projection lands outside the viewport, where the
                # reference reads before its source buffer
                proj="default" if kind == "pixels" else proj, n=int(r.integers(4, 9)))


def _soup(lib, r, n, proj):
    lib.pfBegin(A.PF_TRIANGLES)
    for _ in range(n):
        c = r.integers(0, 256, 4)
        lib.pfColor4ub(int(c[0]), int(c[1]), int(c[2]), int(r.integers(120, 256)))
        zr = (-0.9, 0.9) if proj == "default" else (-1.5, 1.5)
        for _k in range(3):
            p = r.uniform(-1.1, 1.1, 2)
            lib.pfVertex3f(float(p[0]), float(p[1]), float(r.uniform(*zr)))
    lib.pfEnd()


def _setup(lib, case):
    if case["proj"] == "frustum":
        lib.pfMatrixMode(A.PF_PROJECTION)
        lib.pfLoadIdentity()
        lib.pfFrustum(-0.08, 0.08, -0.06, 0.06, 0.1, 10.0)
        lib.pfMatrixMode(A.PF_MODELVIEW)
        lib.pfLoadIdentity()
        lib.pfTranslatef(0.0, 0.0, -2.2)
    lib.pfDisable(A.PF_CULL_FACE)
    if case["depth"] >= 0:
        lib.pfEnable(A.PF_DEPTH_TEST)
        lib.pfDepthFunc(case["depth"])
    if case["blend"] >= 0:
        lib.pfEnable(A.PF_BLEND)
        lib.pfBlendFunc(case["blend"])


def _rects(lib, case, r):
    for i in range(case["n"]):
        _soup(lib, r, 6, case["proj"])
        c = r.integers(0, 256, 4)
        lib.pfColor4ub(int(c[0]), int(c[1]), int(c[2]), int(c[3]))
        a, b = r.uniform(-1.3, 1.3, 2), r.uniform(-1.3, 1.3, 2)
        form = i % 3
        if form == 0:
            lib.pfRectf(float(a[0]), float(a[1]), float(b[0]), float(b[1]))
        elif form == 1:
            v1, v2 = a.astype(np.float32), b.astype(np.float32)
            lib.pfRectfv(C.cast(_ptr(v1), C.POINTER(C.c_float)), C.cast(_ptr(v2), C.POINTER(C.c_float)))
        else:
            s = r.integers(-1, 2, 4)
            lib.pfRects(int(s[0]), int(s[1]), int(s[2]), int(s[3]))


def _pixels(lib, case, r):
    # the raster position stays inside the viewport (else the reference
    # reads before its source buffer); the default projection keeps w = 1
    keep = []
    for i in range(case["n"]):
        _soup(lib, r, 5, "default")
        fmt, typ = PIXEL_FORMATS[int(r.integers(len(PIXEL_FORMATS)))]
        w, h = int(r.integers(3, 40)), int(r.integers(3, 30))
        src = pixel_source(fmt, typ, w, h, r)
        keep.append(src)
        zoom = [(1.0, 1.0), (2.0, 1.5), (0.5, 0.75), (3.0, 3.0), (1.25, 0.5)][int(r.integers(5))]
        lib.pfPixelZoom(*zoom)
        p = r.uniform(-0.95, 0.9, 2)
        z = float(r.uniform(-0.9, 0.9))
        if i % 3 == 0:
            lib.pfRasterPos3f(float(p[0]), float(p[1]), z)
        elif i % 3 == 1:
            v = np.array([p[0], p[1], z, 1.0], np.float32)
            lib.pfRasterPos4fv(C.cast(_ptr(v), C.POINTER(C.c_float)))
        else:
            lib.pfRasterPos2f(float(p[0]), float(p[1]))
        lib.pfDrawPixels(w, h, fmt, typ, _ptr(src))
    return keep


def _fog(lib, case, r):
    for rep in range(2):
        _soup(lib, r, 12, case["proj"])
        if case["proj"] == "default":
            start = float(r.choice([-1.0, -0.5, 0.0, 0.4]))
        else:
            start = float(r.choice([0.5, 1.5, 2.0, 2.5]))
        end = start + float(r.choice([0.3, 1.0, 2.5]))
        mode = int(r.integers(3))
        form = int(r.integers(3))
        if form == 0:
            lib.pfFogi(PF_FOG_MODE, mode)
            lib.pfFogf(PF_FOG_START, start)
            lib.pfFogf(PF_FOG_END, end)
        elif form == 1:
            iv = (C.c_int * 4)(mode, 0, 0, 0)
            lib.pfFogiv(PF_FOG_MODE, iv)
            fv = (C.c_float * 4)(start, 0, 0, 0)
            lib.pfFogfv(PF_FOG_START, fv)
            fv = (C.c_float * 4)(end, 0, 0, 0)
            lib.pfFogfv(PF_FOG_END, fv)
        else:
            lib.pfFogi(PF_FOG_DENSITY, mode & 1)          # sets the mode
            lib.pfFogi(PF_FOG_START, int(np.floor(start)))
            lib.pfFogi(PF_FOG_END, int(np.floor(start)) + 2)
        c = r.integers(0, 256, 4)
        alpha = 255 if r.random() < 0.3 else int(c[3])
        if r.random() < 0.5:
            lib.pfFogiv(PF_FOG_COLOR, (C.c_int * 4)(int(c[0]), int(c[1]), int(c[2]), alpha))
        else:
            lib.pfFogfv(PF_FOG_COLOR, (C.c_float * 4)(c[0] / 255.0, c[1] / 255.0, c[2] / 255.0, alpha / 255.0))
        lib.pfFogProcess()


def _list(lib, case, r, tex):
    lst = lib.pfGenList()
    lib.pfNewList(lst)
    lib.pfColor4ub(200, 30, 30, 255)
    lib.pfBindTexture(tex)
    for blk in range(3):
        mode = [A.PF_TRIANGLES, A.PF_QUADS, A.PF_TRIANGLE_FAN][blk]
        per = [3, 4, 5][blk]
        lib.pfBegin(mode)
        for _ in range(per * (2 if blk == 0 else 1)):
            c = r.integers(0, 256, 4)
            lib.pfColor4ub(int(c[0]), int(c[1]), int(c[2]), int(c[3]))
            t = r.uniform(0, 1, 2)
            lib.pfTexCoord2f(float(t[0]), float(t[1]))
            nv = r.normal(size=3)
            lib.pfNormal3f(float(nv[0]), float(nv[1]), float(nv[2]))
            p = r.uniform(-0.6, 0.6, 3)
            lib.pfVertex3f(float(p[0]), float(p[1]), float(p[2]) * 0.5)
        lib.pfEnd()
    lib.pfEndList()
    # state restored by pfEndList: this triangle takes the colour set before
    lib.pfBegin(A.PF_TRIANGLES)
    lib.pfVertex2f(-1.0, -1.0)
    lib.pfVertex2f(-0.6, -1.0)
    lib.pfVertex2f(-1.0, -0.6)
    lib.pfEnd()
    lib.pfMatrixMode(A.PF_MODELVIEW)
    for k in range(case["n"]):
        lib.pfPushMatrix()
        lib.pfTranslatef(float(r.uniform(-0.4, 0.4)), float(r.uniform(-0.4, 0.4)), 0.0)
        lib.pfRotatef(float(r.uniform(0, 360)), 0.0, 0.0, 1.0)
        if k % 3 == 1:
            lib.pfEnable(A.PF_TEXTURE_2D)
        if k % 4 == 2:
            lib.pfEnable(A.PF_LIGHTING)
            lib.pfEnableLight(0)
        if k % 4 == 3:
            lib.pfEnable(A.PF_COLOR_MATERIAL)
        lib.pfCallList(lst)
        lib.pfDisable(A.PF_TEXTURE_2D)
        lib.pfDisable(A.PF_LIGHTING)
        lib.pfDisable(A.PF_COLOR_MATERIAL)
        lib.pfPopMatrix()
    ref = C.c_void_p(lst)
    lib.pfDeleteList(C.byref(ref))


def run_px(lib: A.PixelForgeLib, case: dict, target: str = "fbo") -> Frame:
    r = np.random.default_rng(case["seed"] + 303)
    W, H = 96, 80
    tg = Target(lib, W, H, target)
    tex_px = r.integers(0, 256, (16, 16, 4)).astype(np.uint8)
    tex = None
    try:
        far = 1e30 if case["proj"] == "frustum" else 1.0
        lib.pfClearDepth(-far if case["depth"] in (A.PF_GREATER, A.PF_GEQUAL) else far)
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        _setup(lib, case)
        keep = None
        if case["kind"] == "rects":
            _rects(lib, case, r)
        elif case["kind"] == "pixels":
            keep = _pixels(lib, case, r)
        elif case["kind"] == "fog":
            _fog(lib, case, r)
        else:
            tex = lib.pfGenTexture(_ptr(tex_px), 16, 16, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
            _list(lib, case, r, tex)
        fr = tg.finish()
        del keep
        return fr
    finally:
        if tex:
            th = C.c_void_p(tex)
            lib.pfDeleteTexture(C.byref(th), False)
        tg.close()


_TYPE_BYTES = {0: 1, 2: 2, 3: 2, 4: 2, 9: 2, 10: 4}


def run_readback(lib: A.PixelForgeLib, seed: int, target: str = "fbo") -> dict:
    """A small scene read back with pfReadPixels into every format the
    reference has a setter for, over regions partly outside the
    framebuffer; returns the bytes of each read."""
    r = np.random.default_rng(seed + 404)
    W, H = 40, 30
    tg = Target(lib, W, H, target)
    out = {}
    try:
        lib.pfClearColor(10, 20, 30, 200)
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        lib.pfDisable(A.PF_CULL_FACE)
        _soup(lib, r, 20, "default")
        for fmt, typ in PIXEL_FORMATS:
            x, y = int(r.integers(-5, 30)), int(r.integers(-5, 24))
            w, h = int(r.integers(1, 30)), int(r.integers(1, 20))
            n = w * h * (1 if typ in (2, 3, 4) else _COMPS[fmt]) * _TYPE_BYTES[typ]
            buf = np.full(n + 16, 0xA5, np.uint8)
            lib.pfReadPixels(x, y, w, h, fmt, typ, _ptr(buf))
            out[(fmt, typ)] = (buf, lib.pfGetError())
        return out
    finally:
        tg.close()
