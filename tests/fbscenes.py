"""Seeded scenes rendered into framebuffers of every format a framebuffer
may have: fills and clears, triangles with blending and depth, points,
lines, rectangles, pixel images, fog, device post-processing and the
per-pixel framebuffer functions, replayable on any pf* library."""
from __future__ import annotations

import ctypes as C

import numpy as np

from pixelforge_gb300 import abi as A
from pixelforge_gb300.scenes import Frame, Target, _ptr

from pixscenes import PIXEL_FORMATS, pixel_source

# (format, type) pairs a framebuffer may have, RGBA / unsigned byte first:
# the formats of the seeded cases (case `seed` draws into format
# seed % 19) ...
FB_FORMATS = [(A.PF_RGBA, 0), (A.PF_RGB, 0), (A.PF_BGR, 0),
              (A.PF_RGB, 2), (A.PF_BGR, 2), (A.PF_RGBA, 3), (A.PF_BGRA, 3), (A.PF_RGBA, 4), (A.PF_BGRA, 4)] + \
    [(f, t) for t in (A.PF_HALF_FLOAT, A.PF_FLOAT)
     for f in (A.PF_LUMINANCE_ALPHA, A.PF_RGB, A.PF_BGR, A.PF_RGBA, A.PF_BGRA)]
# ... and BGRA / unsigned byte, whose SIMD getter and setter shuffle each
# 4-pixel half vector with the bytes of its first pixel (its cases name it)
FB_BGRA8 = (A.PF_BGRA, A.PF_UNSIGNED_BYTE)
FB_ACCEPTED = FB_FORMATS + [FB_BGRA8]
# the seeded cases of the parity tests: five per format of FB_FORMATS, then
# twelve BGRA / unsigned byte
FB_SEEDS = [(s, None) for s in range(5 * len(FB_FORMATS))] + [(s, FB_BGRA8) for s in range(200, 212)]
# pairs that are valid pixel formats but not framebuffer formats
FB_REFUSED = [(f, 0) for f in (A.PF_RED, A.PF_GREEN, A.PF_BLUE, A.PF_ALPHA, A.PF_LUMINANCE,
                               A.PF_LUMINANCE_ALPHA)] + \
    [(f, t) for t in (A.PF_HALF_FLOAT, A.PF_FLOAT)
     for f in (A.PF_RED, A.PF_GREEN, A.PF_BLUE, A.PF_ALPHA, A.PF_LUMINANCE)]


def fb_case(seed: int, fmt: tuple | None = None) -> dict:
    r = np.random.default_rng(seed)
    fmt = fmt or FB_FORMATS[seed % len(FB_FORMATS)]
    # odd sizes leave a tail of W*H % 8 pixels for pfClear to copy pixel 0 into
    W, H = [(61, 37), (64, 40), (45, 29), (80, 48)][int(r.integers(4))]
    return dict(seed=seed, fmt=fmt, W=W, H=H, target=["main", "fbo"][int(r.integers(2))],
                depth=int(r.integers(-1, 6)), blend=int(r.integers(-1, 8)))


def _init_pixels(fmt, W, H, r) -> np.ndarray:
    """Initial content of a main buffer: raw pixels of the format, half and
    float channels in [0, 1]."""
    f, t = fmt
    if t in (A.PF_HALF_FLOAT, A.PF_FLOAT):
        n = W * H * (A.pixel_bytes(f, t) // (2 if t == A.PF_HALF_FLOAT else 4))
        v = r.uniform(0.0, 1.0, n)
        raw = v.astype(np.float16 if t == A.PF_HALF_FLOAT else np.float32).view(np.uint8)
    else:
        raw = r.integers(0, 256, W * H * A.pixel_bytes(f, t)).astype(np.uint8)
    return raw.reshape(H, W, -1)


def _color(r, alpha_lo=0):
    c = r.integers(0, 256, 4)
    return int(c[0]), int(c[1]), int(c[2]), int(r.integers(alpha_lo, 256))


def _soup(lib, r, n):
    lib.pfBegin(A.PF_TRIANGLES)
    for _ in range(n):
        lib.pfColor4ub(*_color(r, 60))
        for _k in range(3):
            p = r.uniform(-1.1, 1.1, 2)
            lib.pfVertex3f(float(p[0]), float(p[1]), float(r.uniform(-0.9, 0.9)))
    lib.pfEnd()


def run_fb(lib: A.PixelForgeLib, case: dict, device_hook: bool = True) -> dict:
    """Render the case; returns the framebuffer's raw pixels and depth and
    what the per-pixel functions and pfReadPixels returned.  device_hook:
    run the grayscale device post-process on every third seed and the
    dither one on the next (libraries that have pfPostProcessDevice)."""
    r = np.random.default_rng(case["seed"] + 505)
    W, H, fmt = case["W"], case["H"], case["fmt"]
    init = _init_pixels(fmt, W, H, r) if case["target"] == "main" else None
    tg = Target(lib, W, H, case["target"], init=init, fmt=fmt)
    out = {}
    keep = []
    try:
        if tg.fb is not None:
            lib.pfClearFramebuffer(tg._fbref, A.PFcolor(*_color(r)), 0.5)
        lib.pfClearColor(*_color(r))
        lib.pfClearDepth(-1.0 if case["depth"] in (A.PF_GREATER, A.PF_GEQUAL) else 1.0)
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        lib.pfDisable(A.PF_CULL_FACE)
        if case["depth"] >= 0:
            lib.pfEnable(A.PF_DEPTH_TEST)
            lib.pfDepthFunc(case["depth"])
        if case["blend"] >= 0:
            lib.pfEnable(A.PF_BLEND)
            lib.pfBlendFunc(case["blend"])
        _soup(lib, r, 14)
        # points and lines (scalar getter and setter)
        lib.pfPointSize(float(r.choice([1.0, 3.0])))
        lib.pfBegin(A.PF_POINTS)
        for _ in range(12):
            lib.pfColor4ub(*_color(r, 60))
            p = r.uniform(-1.0, 1.0, 3)
            lib.pfVertex3f(float(p[0]), float(p[1]), float(p[2]) * 0.9)
        lib.pfEnd()
        lib.pfBegin(A.PF_LINES)
        for _ in range(8):
            lib.pfColor4ub(*_color(r, 60))
            p = r.uniform(-1.0, 1.0, 3)
            lib.pfVertex3f(float(p[0]), float(p[1]), float(p[2]) * 0.9)
        lib.pfEnd()
        _soup(lib, r, 6)
        # a rectangle and a pixel image
        lib.pfColor4ub(*_color(r))
        a, b = r.uniform(-1.2, 1.2, 2), r.uniform(-1.2, 1.2, 2)
        lib.pfRectf(float(a[0]), float(a[1]), float(b[0]), float(b[1]))
        sf, st = PIXEL_FORMATS[int(r.integers(len(PIXEL_FORMATS)))]
        w, h = int(r.integers(3, 20)), int(r.integers(3, 16))
        src = pixel_source(sf, st, w, h, r)
        keep.append(src)
        lib.pfPixelZoom(float(r.choice([1.0, 1.5])), float(r.choice([1.0, 0.75])))
        p = r.uniform(-0.9, 0.6, 2)
        lib.pfRasterPos3f(float(p[0]), float(p[1]), float(r.uniform(-0.5, 0.5)))
        lib.pfDrawPixels(w, h, sf, st, _ptr(src))
        _soup(lib, r, 6)
        # linear fog over the depth buffer (the exponential modes go through
        # the host's libm; they are covered on RGBA8 framebuffers)
        lib.pfFogi(0, 0)
        lib.pfFogf(2, float(r.uniform(-1.0, 0.0)))
        lib.pfFogf(3, float(r.uniform(0.2, 1.0)))
        lib.pfFogiv(4, (C.c_int * 4)(*_color(r)))
        lib.pfFogProcess()
        if device_hook and case["seed"] % 3 == 0:
            lib.pfPostProcessDevice(A.PF_HOOK_GRAYSCALE, None, 0)
        elif device_hook and case["seed"] % 3 == 1:
            lib.pfPostProcessDevice(A.PF_HOOK_DITHER, None, 0)
        _soup(lib, r, 4)
        # per-pixel framebuffer functions (framebuffer objects only)
        if tg.fb is not None:
            for k in range(6):
                x, y = int(r.integers(W)), int(r.integers(H))
                col = A.PFcolor(*_color(r))
                if k % 3 == 0:
                    lib.pfSetFramebufferPixel(tg._fbref, x, y, col)
                elif k % 3 == 1:
                    lib.pfSetFramebufferPixelDepth(tg._fbref, x, y, float(r.uniform(-1, 1)), col)
                else:
                    lib.pfSetFramebufferPixelDepthTest(tg._fbref, x, y, float(r.uniform(-1, 1)), col, A.PF_LESS)
            got = []
            for _ in range(8):
                x, y = int(r.integers(W)), int(r.integers(H))
                c = lib.pfGetFramebufferPixel(tg._fbref, x, y)
                got.append((c.r, c.g, c.b, c.a))
            out["get"] = np.array(got, np.uint8)
        rb = np.zeros((H, W, 4), np.uint8)
        lib.pfReadPixels(0, 0, W, H, A.PF_RGBA, A.PF_UNSIGNED_BYTE, _ptr(rb))
        out["read"] = rb
        fr: Frame = tg.finish()
        out["color"] = fr.color
        if fr.depth is not None:
            out["depth"] = fr.depth
        out["err"] = lib.pfGetError()
        return out
    finally:
        del keep
        tg.close()


def refused_formats(lib: A.PixelForgeLib) -> list:
    """pfGenFramebuffer of each refused pair: (pair, texture pointer null,
    error code)."""
    buf = np.zeros((8, 8, 4), np.uint8)
    ctx = lib.pfCreateContext(_ptr(buf), 8, 8, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
    lib.pfMakeCurrent(ctx)
    res = []
    try:
        for f, t in FB_REFUSED:
            fb = lib.pfGenFramebuffer(8, 8, f, t)
            res.append(((f, t), not fb.texture, lib.pfGetError()))
            if fb.texture:
                ref = C.pointer(fb)
                lib.pfDeleteFramebuffer(ref)
        return res
    finally:
        lib.pfDeleteContext(ctx)


def fb_frame(seed: int, fmt: tuple | None = None):
    """A golden-vector runner: the case's framebuffer as a Frame."""
    def run(lib):
        out = run_fb(lib, fb_case(seed, fmt), device_hook=False)
        return Frame(out["color"], out.get("depth"))
    return run


# ragged framebuffers: fewer than 8 pixels (pfClear's vector loop does not
# run and its tail copies pixel 0 over every pixel), a single row or column,
# sides that are no multiple of the 16-pixel tile
TINY_SIZES = [(1, 1), (2, 3), (7, 1), (1, 9), (17, 5), (33, 2), (5, 31)]
TINY_FORMATS = [(A.PF_RGBA, 0), (A.PF_RGB, 0), (A.PF_RGBA, A.PF_HALF_FLOAT), (A.PF_BGRA, A.PF_FLOAT),
                (A.PF_RGB, 2), (A.PF_RGBA, 4), (A.PF_BGRA, 0)]


def tiny_case(k: int) -> dict:
    """Case k of the ragged-size set: every size with every format of
    TINY_FORMATS, except the packed 16-bit formats below 10 pixels (there the
    reference's pfClear tail, stepped by components x 2 bytes, writes pixels
    inside the buffer at 3-4x their index; not reproduced)."""
    cases = []
    for (W, H) in TINY_SIZES:
        for fmt in TINY_FORMATS:
            if fmt[1] in (2, 3, 4) and W * H < 10:
                continue
            cases.append((W, H, fmt))
    W, H, fmt = cases[k]
    r = np.random.default_rng(2000 + k)
    return dict(seed=2000 + k, fmt=fmt, W=W, H=H, target=["main", "fbo"][k % 2],
                depth=int(r.integers(-1, 6)), blend=int(r.integers(-1, 8)))


TINY_CASES = sum(1 for (W, H) in TINY_SIZES for f in TINY_FORMATS if not (f[1] in (2, 3, 4) and W * H < 10))
