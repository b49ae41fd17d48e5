"""Golden cases: scenes driven through the pf* API of any library.

Each case renders into a small framebuffer and returns a Frame (colour and
depth).  ``make_golden.py`` runs them on the reference compiled from its own
sources (the exact-reciprocal flavour, oracle/_ref/libpf_shim.so) and stores
the images in ``golden.npz``; ``tests/test_oracle_golden.py`` checks the CPU
oracle against them on any host, including the aarch64 GPU host where the
reference cannot be built.

Known-answer cases (``kat_*``) isolate one rule each, with the reference
lines they exercise:
  kat_edge_*      coverage (w1|w2|w3) > 0, x < xMax, y <= yMax (triangles.c:404-424)
  kat_cull_*      FRONT iff integer area < 0, culling default BACK (triangles.c:299-306, context.c:243-246)
  kat_blend_*     each blend function on known colour pairs (blend.h:140-277)
  kat_tex_*       each wrap mode with the nearest filter on a 4x4 texture (sampler.h:203-258)
  kat_clip_*      a triangle crossing each clip plane (triangles.c:157-244)
  kat_depth_*     each depth function, including NOTEQUAL behaving as EQUAL (depth.h:80-124)
  kat_clear       pfClear leaving pixels 0..7 (context.c:680-745)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from pixelforge_gb300 import abi as A
from pixelforge_gb300.scenes import PhongScene, SoupScene, SphereScene, Target, _ptr


def _tri(lib, pts, cols, uvs=None):
    lib.pfBegin(A.PF_TRIANGLES)
    for k, p in enumerate(pts):
        c = cols[k % len(cols)]
        lib.pfColor4ub(*c)
        if uvs is not None:
            lib.pfTexCoord2f(*uvs[k])
        lib.pfVertex3f(*p)
    lib.pfEnd()


def _frame(lib, w, h, body, init=None):
    # with initial contents: the context's own buffer (a framebuffer object
    # starts cleared); its depth buffer is not public, so only colour is kept
    tg = Target(lib, w, h, "main" if init is not None else "fbo", init=init)
    try:
        body(lib)
        return tg.finish()
    finally:
        tg.close()


def kat_edge(variant):
    # 2D path (default projection, w = 1): screen x = (x+1)/2*(W-1)+0.5;
    # the stored depth is 1/h.z (h.z = -z under the default orthographic
    # projection), so z = 0 would store infinity
    tris = {
        "a": [(-1.0, -1.0, 0.5), (1.0, -1.0, 0.5), (-1.0, 1.0, 0.5)],
        "b": [(-0.6, 0.7, 0.2), (0.9, 0.1, 0.2), (-0.2, -0.8, 0.2)],
        "c": [(-0.95, -0.95, 0.5), (0.95, 0.95, 0.5), (-0.95, 0.95, 0.5), (0.95, -0.95, 0.5), (0.95, 0.95, 0.5),
              (-0.95, -0.95, 0.5)],
    }[variant]

    def body(lib):
        lib.pfClearDepth(1.0)
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        lib.pfDisable(A.PF_CULL_FACE)
        lib.pfEnable(A.PF_DEPTH_TEST)
        lib.pfDepthFunc(A.PF_LEQUAL)
        _tri(lib, tris, [(255, 0, 0, 255), (0, 255, 0, 255), (0, 0, 255, 255)])
    return lambda lib: _frame(lib, 9, 8, body)


def kat_cull(mode):
    def body(lib):
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        if mode == "none":
            lib.pfDisable(A.PF_CULL_FACE)
        elif mode == "front":
            lib.pfCullFace(A.PF_FRONT)
        # one triangle of each winding
        _tri(lib, [(-0.9, -0.9, 0.0), (-0.1, -0.9, 0.0), (-0.9, 0.9, 0.0)], [(255, 255, 255, 255)])
        _tri(lib, [(0.1, -0.9, 0.0), (0.1, 0.9, 0.0), (0.9, -0.9, 0.0)], [(90, 160, 30, 255)])
    return lambda lib: _frame(lib, 12, 8, body)


def kat_blend(mode):
    init = np.zeros((4, 8, 4), np.uint8)
    init[..., 0] = np.arange(8) * 32
    init[..., 1] = 255 - np.arange(8)[None, :] * 30
    init[..., 2] = 77
    init[..., 3] = np.arange(4)[:, None] * 80

    def body(lib):
        lib.pfDisable(A.PF_CULL_FACE)
        lib.pfEnable(A.PF_BLEND)
        lib.pfBlendFunc(mode)
        quad = [(-1.0, -1.0, 0.0), (1.0, -1.0, 0.0), (1.0, 1.0, 0.0),
                (-1.0, -1.0, 0.0), (1.0, 1.0, 0.0), (-1.0, 1.0, 0.0)]
        lib.pfBegin(A.PF_TRIANGLES)
        for p in quad:
            lib.pfColor4ub(200, 60, 140, 128)
            lib.pfVertex3f(*p)
        lib.pfEnd()
    return lambda lib: _frame(lib, 8, 4, body, init=init)


def kat_tex(wrap):
    tex = np.arange(4 * 4 * 4, dtype=np.uint8).reshape(4, 4, 4) * 3
    tex[..., 3] = 255
    handle = {}

    def body(lib):
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        lib.pfDisable(A.PF_CULL_FACE)
        t = lib.pfGenTexture(_ptr(tex), 4, 4, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
        handle["t"] = t
        lib.pfTextureParameter(t, wrap, A.PF_NEAREST)
        lib.pfBindTexture(t)
        lib.pfEnable(A.PF_TEXTURE_2D)
        lo, hi = (-0.7, 1.6) if wrap != A.PF_CLAMP_TO_EDGE else (-0.7, 0.95)
        quad = [(-1.0, -1.0, 0.0), (1.0, -1.0, 0.0), (1.0, 1.0, 0.0),
                (-1.0, -1.0, 0.0), (1.0, 1.0, 0.0), (-1.0, 1.0, 0.0)]
        uvs = [(lo, lo), (hi, lo), (hi, hi), (lo, lo), (hi, hi), (lo, hi)]
        _tri(lib, quad, [(255, 255, 255, 255)], uvs)

    def run(lib):
        fr = _frame(lib, 12, 12, body)
        if "t" in handle:
            th = C.c_void_p(handle["t"])
            lib.pfDeleteTexture(C.byref(th), False)
        return fr
    return run


def kat_clip(plane):
    # a triangle through the frustum with one vertex beyond the named plane
    base = {"near": [(-0.5, -0.4, -1.0), (0.6, -0.3, -1.2), (0.0, 0.5, 0.3)],
            "far": [(-0.5, -0.4, -1.0), (0.6, -0.3, -1.2), (0.0, 0.5, -40.0)],
            "left": [(-3.0, 0.0, -1.5), (0.5, -0.5, -1.5), (0.3, 0.6, -1.5)],
            "right": [(3.0, 0.1, -1.5), (-0.5, -0.5, -1.5), (-0.3, 0.6, -1.5)],
            "bottom": [(0.0, -3.0, -1.5), (0.5, 0.4, -1.5), (-0.6, 0.5, -1.5)],
            "top": [(0.1, 3.0, -1.5), (0.5, -0.4, -1.5), (-0.6, -0.5, -1.5)]}[plane]

    def body(lib):
        lib.pfClearDepth(1e30)
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        lib.pfDisable(A.PF_CULL_FACE)
        lib.pfEnable(A.PF_DEPTH_TEST)
        lib.pfMatrixMode(A.PF_PROJECTION)
        lib.pfLoadIdentity()
        lib.pfFrustum(-0.1, 0.1, -0.1, 0.1, 0.1, 20.0)
        lib.pfMatrixMode(A.PF_MODELVIEW)
        lib.pfLoadIdentity()
        _tri(lib, base, [(250, 10, 10, 255), (10, 250, 10, 255), (10, 10, 250, 255)])
    return lambda lib: _frame(lib, 24, 24, body)


def kat_depth(func):
    def body(lib):
        lib.pfClearDepth(0.5)
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        lib.pfDisable(A.PF_CULL_FACE)
        lib.pfEnable(A.PF_DEPTH_TEST)
        lib.pfDepthFunc(func)
        # 2D path: stored depth = z; a slanted triangle crosses the clear depth
        lib.pfBegin(A.PF_TRIANGLES)
        for p, c in (((-1.0, -1.0, 0.0), (255, 0, 0, 255)), ((1.0, -1.0, 1.0), (0, 255, 0, 255)),
                     ((0.0, 1.0, 0.5), (0, 0, 255, 255))):
            lib.pfColor4ub(*c)
            lib.pfVertex3f(*p)
        lib.pfEnd()
    return lambda lib: _frame(lib, 10, 10, body)


def kat_clear():
    init = (np.arange(6 * 5 * 4) % 251).astype(np.uint8).reshape(5, 6, 4)

    def body(lib):
        lib.pfClearColor(10, 20, 30, 40)
        lib.pfClearDepth(0.25)
        lib.pfClear(A.PF_COLOR_BUFFER_BIT)
    return lambda lib: _frame(lib, 6, 5, body, init=init)


TEX_FORMATS = [(f, t) for f in ("RED", "GREEN", "BLUE", "ALPHA", "LUMINANCE", "LUMINANCE_ALPHA", "RGB", "RGBA",
                                 "BGR", "BGRA") for t in ("UBYTE", "HALF", "FLOAT")] + \
              [("RGB", "S565"), ("BGR", "S565"), ("RGBA", "S5551"), ("BGRA", "S5551"), ("RGBA", "S4444"),
               ("BGRA", "S4444")]
_FMT = dict(RED=0, GREEN=1, BLUE=2, ALPHA=3, LUMINANCE=4, LUMINANCE_ALPHA=5, RGB=6, RGBA=7, BGR=8, BGRA=9)
_TYP = dict(UBYTE=0, S565=2, S5551=3, S4444=4, HALF=9, FLOAT=10)
_COMPS = dict(RED=1, GREEN=1, BLUE=1, ALPHA=1, LUMINANCE=1, LUMINANCE_ALPHA=2, RGB=3, RGBA=4, BGR=3, BGRA=4)


def tex_format_data(f, t, w=8, h=8, seed=3):
    """Texels of format f / type t (values slightly outside [0, 1] for the
    floating types), padded so that the getters' wide loads stay inside."""
    rng = np.random.default_rng(seed + 17 * _FMT[f] + _TYP[t])
    n = w * h
    if t == "UBYTE":
        d = rng.integers(0, 256, n * _COMPS[f] + 8).astype(np.uint8)
    elif t == "HALF":
        d = rng.uniform(-0.2, 1.2, n * _COMPS[f] + 8).astype(np.float16)
    elif t == "FLOAT":
        d = rng.uniform(-0.2, 1.2, n * _COMPS[f] + 8).astype(np.float32)
    else:
        d = rng.integers(0, 65536, n + 8).astype(np.uint16)
    d[-8:] = 0
    return d


def kat_texfmt(f, t, filt=A.PF_NEAREST):
    """A textured quad sampling an 8x8 texture of format f / type t
    (src/texture.c:30-70, src/internal/pixel.h:2253-3097)."""
    data = tex_format_data(f, t)
    handle = {}

    def body(lib):
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        lib.pfDisable(A.PF_CULL_FACE)
        tx = lib.pfGenTexture(_ptr(data), 8, 8, _FMT[f], _TYP[t])
        handle["t"] = tx
        lib.pfTextureParameter(tx, A.PF_REPEAT, filt)
        lib.pfBindTexture(tx)
        lib.pfEnable(A.PF_TEXTURE_2D)
        quad = [(-1.0, -1.0, 0.0), (1.0, -1.0, 0.0), (1.0, 1.0, 0.0),
                (-1.0, -1.0, 0.0), (1.0, 1.0, 0.0), (-1.0, 1.0, 0.0)]
        uvs = [(0.0, 0.0), (0.97, 0.0), (0.97, 0.97), (0.0, 0.0), (0.97, 0.97), (0.0, 0.97)]
        _tri(lib, quad, [(255, 255, 255, 255)], uvs)

    def run(lib):
        fr = _frame(lib, 16, 16, body)
        if handle.get("t"):
            th = C.c_void_p(handle["t"])
            lib.pfDeleteTexture(C.byref(th), False)
        return fr
    return run


def mix(seed):
    from mixscenes import mix_case, run_mix
    return lambda lib: run_mix(lib, mix_case(seed))


def lp(seed):
    from lpscenes import lp_case, run_lp
    return lambda lib: run_lp(lib, lp_case(seed))


def px(seed):
    from pixscenes import px_case, run_px
    return lambda lib: run_px(lib, px_case(seed))


def _scene(sc, **kw):
    return lambda lib: sc.render(lib, "fbo", **kw)


def cases() -> dict:
    c = {}
    for v in ("a", "b", "c"):
        c[f"kat_edge_{v}"] = kat_edge(v)
    for m in ("back", "front", "none"):
        c[f"kat_cull_{m}"] = kat_cull(m)
    for name, m in (("average", A.PF_BLEND_AVERAGE), ("alpha", A.PF_BLEND_ALPHA), ("add", A.PF_BLEND_ADD),
                    ("sub", A.PF_BLEND_SUB), ("mul", A.PF_BLEND_MUL), ("screen", A.PF_BLEND_SCREEN),
                    ("lighten", A.PF_BLEND_LIGHTEN), ("darken", A.PF_BLEND_DARKEN)):
        c[f"kat_blend_{name}"] = kat_blend(m)
    for name, w in (("repeat", A.PF_REPEAT), ("mirrored", A.PF_MIRRORED_REPEAT), ("clamp", A.PF_CLAMP_TO_EDGE)):
        c[f"kat_tex_{name}"] = kat_tex(w)
    for p in ("near", "far", "left", "right", "bottom", "top"):
        c[f"kat_clip_{p}"] = kat_clip(p)
    for name, f in (("equal", A.PF_EQUAL), ("notequal", A.PF_NOTEQUAL), ("less", A.PF_LESS),
                    ("lequal", A.PF_LEQUAL), ("greater", A.PF_GREATER), ("gequal", A.PF_GEQUAL)):
        c[f"kat_depth_{name}"] = kat_depth(f)
    c["kat_clear"] = kat_clear()
    for f, t in TEX_FORMATS:
        if (f, t) == ("BGRA", "UBYTE"):
            continue   # the reference repeats one texel per half vector here (simd.h:564-583); pinned to the per-texel swizzle
        c[f"kat_texfmt_{f}_{t}"] = kat_texfmt(f, t)
    c["soup256"] = _scene(SoupScene())
    c["soup128_nocull_flat_lequal"] = _scene(SoupScene(width=128, height=128, ntris=600, seed=11, cull=False,
                                                       shade=A.PF_FLAT, depth_func=A.PF_LEQUAL))
    c["soup128_alpha"] = _scene(SoupScene(width=128, height=96, ntris=500, seed=12, blend=A.PF_BLEND_ALPHA))
    c["sphere_nearest_320"] = _scene(SphereScene(width=320, height=180, segments=64, rings=32, tex_size=128,
                                                 filt=A.PF_NEAREST, depth_mask_off=False))
    c["phong_320"] = _scene(PhongScene(width=320, height=180, subdiv=4, tex_size=128, fog=False))
    for s in range(40):
        c[f"mix_{s}"] = mix(5000 + s)
    for s in range(24):
        c[f"lp_{s}"] = lp(7000 + s)
    for s in range(16):
        c[f"px_{s}"] = px(9000 + s)
    from fbscenes import FB_BGRA8, FB_FORMATS, fb_frame
    for s in range(len(FB_FORMATS)):
        c[f"fb_{s}"] = fb_frame(11000 + s)
    for s in range(4):
        c[f"fb_bgra8_{s}"] = fb_frame(11100 + s, FB_BGRA8)
    return c


# cases whose colour goes through the host libm (the Gouraud specular powf,
# the fog's expf / exp2f)
def uses_host_powf(name: str) -> bool:
    if name.startswith("sphere"):
        return True
    if name.startswith("px_"):
        from pixscenes import px_case
        return px_case(9000 + int(name.split("_")[1]))["kind"] in ("fog", "list")
    if name.startswith("mix_"):
        from mixscenes import mix_case
        return mix_case(5000 + int(name.split("_")[1]))["lighting"] == "gouraud"
    return False
