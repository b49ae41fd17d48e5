"""Randomised feature-mix scenes for parity tests.

``mix_case(seed)`` draws one combination of pipeline state (projection path,
culling, shading, depth function, blend mode, texture wrap/filter, Gouraud or
Phong lighting with spot and attenuation terms, draw mode and vertex source)
and ``run_mix(lib, case)`` replays it through the pf* API of any library.
The same case therefore runs on the reference build, the CPU oracle and the
GPU library.  Sizes are small so the scalar oracle finishes in milliseconds.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from pixelforge_gb300 import abi as A
from pixelforge_gb300.scenes import Frame, Target, _ptr

DRAW_MODES = [A.PF_TRIANGLES, A.PF_TRIANGLE_FAN, A.PF_TRIANGLE_STRIP, A.PF_QUADS,
              A.PF_QUAD_FAN, A.PF_QUAD_STRIP]


def mix_case(seed: int, bilinear: bool = False, edge_wraps: bool = True) -> dict:
    r = np.random.default_rng(seed)
    proj = ["default", "frustum", "ortho"][int(r.integers(3))]
    lighting = ["none", "gouraud", "phong"][int(r.integers(3))]
    tex = bool(r.random() < 0.6)
    wraps = [A.PF_REPEAT, A.PF_MIRRORED_REPEAT, A.PF_CLAMP_TO_EDGE] if edge_wraps else [A.PF_REPEAT]
    return dict(
        seed=seed,
        width=int(r.choice([64, 96, 100, 128])), height=int(r.choice([48, 64, 80, 81])),
        proj=proj,
        cull=int(r.integers(3)),              # 0 off, 1 back (default), 2 front
        shade=A.PF_SMOOTH if r.random() < 0.75 else A.PF_FLAT,
        depth=int(r.integers(-1, 6)),         # -1 = depth test off
        blend=int(r.integers(-1, 8)),         # -1 = blending off
        tex=tex, wrap=int(r.choice(wraps)),
        filt=A.PF_BILINEAR if (bilinear and r.random() < 0.5) else A.PF_NEAREST,
        lighting=lighting, nlights=int(r.integers(1, 4)),
        spot=bool(r.random() < 0.3), atten=bool(r.random() < 0.3),
        mode=int(r.choice(DRAW_MODES)),
        source=["immediate", "elements", "arrays"][int(r.integers(3))],
        ntris=int(r.integers(20, 120)),
        model=bool(r.random() < 0.5),
        viewport=bool(r.random() < 0.2),
        colmat=bool(r.random() < 0.2),
        alpha=bool(r.random() < 0.5),
    )


def _geometry(case: dict, r: np.random.Generator):
    n = case["ntris"] * 3 + 6
    if case["proj"] == "default":
        xy = r.uniform(-1.2, 1.2, (n, 2))
        z = r.uniform(-0.9, 0.9, (n, 1))
    else:
        xy = r.uniform(-1.6, 1.6, (n, 2))
        z = r.uniform(-1.6, 1.6, (n, 1))
    pos = np.concatenate([xy, z], 1).astype(np.float32)
    nrm = r.normal(size=(n, 3)).astype(np.float32)
    if case["wrap"] == A.PF_CLAMP_TO_EDGE:
        # Clamped coordinates >= 1 round to texel w (row h for v): the
        # reference then reads past its texture buffer, so keep them below 1.
        uv = r.uniform(-0.5, 0.97, (n, 2)).astype(np.float32)
    else:
        uv = r.uniform(0.01, 1.95, (n, 2)).astype(np.float32)
    col = r.integers(0, 256, (n, 4)).astype(np.uint8)
    if not case["alpha"]:
        col[:, 3] = 255
    return pos, nrm, uv, col


def run_mix(lib: A.PixelForgeLib, case: dict, target: str = "fbo",
            fmt: tuple = (A.PF_RGBA, A.PF_UNSIGNED_BYTE)) -> Frame:
    """fmt: the framebuffer's format, RGBA or BGRA unsigned byte."""
    r = np.random.default_rng(case["seed"] + 7919)
    W, H = case["width"], case["height"]
    init = r.integers(0, 256, (H, W, 4)).astype(np.uint8)
    tg = Target(lib, W, H, target, init=init, fmt=fmt)
    texh = None
    try:
        pos, nrm, uv, col = _geometry(case, r)
        texture = r.integers(0, 256, (16, 32, 4)).astype(np.uint8)
        lib.pfClearColor(*[int(v) for v in r.integers(0, 256, 4)])
        if case["proj"] == "frustum":
            lib.pfClearDepth(1e30)
        else:
            lib.pfClearDepth(float(r.choice([1.0, -1.0, 5.0])))
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        if case["proj"] == "frustum":
            lib.pfMatrixMode(A.PF_PROJECTION)
            lib.pfLoadIdentity()
            lib.pfFrustum(-0.08, 0.08, -0.06, 0.06, 0.1, 10.0)
            lib.pfMatrixMode(A.PF_MODELVIEW)
            lib.pfLoadIdentity()
            lib.pfTranslatef(0.0, 0.0, -2.2)
        elif case["proj"] == "ortho":
            lib.pfMatrixMode(A.PF_PROJECTION)
            lib.pfLoadIdentity()
            lib.pfOrtho(-1.5, 1.3, -1.2, 1.4, -3.0, 3.0)
            lib.pfMatrixMode(A.PF_MODELVIEW)
            lib.pfLoadIdentity()
        if case["model"]:
            lib.pfPushMatrix()
            lib.pfRotatef(float(r.uniform(-40, 40)), 0.3, 1.0, 0.2)
            lib.pfScalef(1.1, 0.9, 1.0)
        if case["viewport"]:
            # Inside the framebuffer: a larger viewport makes the reference write
            # outside its buffers on the 3D path (its bbox is not clamped there).
            vx, vy = int(r.integers(0, 6)), int(r.integers(0, 5))
            lib.pfViewport(vx, vy, W - vx - int(r.integers(0, 6)), H - vy - int(r.integers(0, 6)))
        if case["cull"] == 0:
            lib.pfDisable(A.PF_CULL_FACE)
        elif case["cull"] == 2:
            lib.pfCullFace(A.PF_FRONT)
        lib.pfShadeModel(case["shade"])
        if case["depth"] >= 0:
            lib.pfEnable(A.PF_DEPTH_TEST)
            lib.pfDepthFunc(case["depth"])
        if case["blend"] >= 0:
            lib.pfEnable(A.PF_BLEND)
            lib.pfBlendFunc(case["blend"])
        if case["tex"]:
            texh = lib.pfGenTexture(_ptr(texture), 32, 16, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
            lib.pfTextureParameter(texh, case["wrap"], case["filt"])
            lib.pfBindTexture(texh)
            lib.pfEnable(A.PF_TEXTURE_2D)
        if case["lighting"] != "none":
            lib.pfEnable(A.PF_LIGHTING)
            lib.pfLightModel(A.PF_GOURAUD if case["lighting"] == "gouraud" else A.PF_PHONG)
            for i in range(case["nlights"]):
                lib.pfEnableLight(i)
                p = r.uniform(-3, 3, 3).astype(np.float32)
                lib.pfLightfv(i, A.PF_POSITION, _ptr(p))
                for prm in (A.PF_AMBIENT, A.PF_DIFFUSE, A.PF_SPECULAR):
                    lib.pfLightfv(i, prm, _ptr(r.uniform(0, 1, 3).astype(np.float32)))
                if case["spot"]:
                    d = r.normal(size=3).astype(np.float32)
                    lib.pfLightfv(i, A.PF_SPOT_DIRECTION, _ptr(d))
                    lib.pfLightf(i, A.PF_SPOT_INNER_CUTOFF, float(r.uniform(20, 40)))
                    lib.pfLightf(i, A.PF_SPOT_OUTER_CUTOFF, float(r.uniform(45, 80)))
                if case["atten"]:
                    lib.pfLightf(i, A.PF_LINEAR_ATTENUATION, float(r.uniform(0.0, 0.3)))
                    lib.pfLightf(i, A.PF_QUADRATIC_ATTENUATION, float(r.uniform(0.0, 0.2)))
            for face in (A.PF_FRONT, A.PF_BACK):
                lib.pfMaterialfv(face, A.PF_DIFFUSE, _ptr(r.uniform(0.2, 1, 3).astype(np.float32)))
                lib.pfMaterialfv(face, A.PF_AMBIENT, _ptr(r.uniform(0, 1, 3).astype(np.float32)))
                lib.pfMaterialfv(face, A.PF_SPECULAR, _ptr(r.uniform(0, 1, 3).astype(np.float32)))
                lib.pfMaterialf(face, A.PF_SHININESS, float(r.uniform(4, 64)))
            lib.pfMaterialfv(A.PF_FRONT_AND_BACK, A.PF_EMISSION, _ptr(r.uniform(0, 0.2, 3).astype(np.float32)))
        if case["colmat"]:
            lib.pfEnable(A.PF_COLOR_MATERIAL)
            lib.pfColorMaterial(A.PF_FRONT_AND_BACK, A.PF_DIFFUSE)
            lib.pfColor4ub(200, 120, 90, 255)
            lib.pfDisable(A.PF_COLOR_MATERIAL)
        mode, n = case["mode"], len(pos)
        if case["source"] == "immediate":
            lib.pfBegin(mode)
            for i in range(n):
                c = col[i]
                lib.pfColor4ub(int(c[0]), int(c[1]), int(c[2]), int(c[3]))
                lib.pfTexCoord2f(float(uv[i, 0]), float(uv[i, 1]))
                lib.pfNormal3f(float(nrm[i, 0]), float(nrm[i, 1]), float(nrm[i, 2]))
                lib.pfVertex3f(float(pos[i, 0]), float(pos[i, 1]), float(pos[i, 2]))
            lib.pfEnd()
        else:
            lib.pfEnable(A.PF_VERTEX_ARRAY | A.PF_NORMAL_ARRAY | A.PF_TEXTURE_COORD_ARRAY | A.PF_COLOR_ARRAY)
            lib.pfVertexPointer(3, A.PF_FLOAT, 0, _ptr(pos))
            lib.pfNormalPointer(A.PF_FLOAT, 0, _ptr(nrm))
            lib.pfTexCoordPointer(A.PF_FLOAT, 0, _ptr(uv))
            lib.pfColorPointer(4, A.PF_UNSIGNED_BYTE, 0, _ptr(col))
            if case["source"] == "elements":
                idx = r.integers(0, n, n).astype(np.uint32)
                lib.pfDrawElements(mode, n, A.PF_UNSIGNED_INT, _ptr(idx))
            else:
                lib.pfDrawArrays(mode, 2, n - 2)
        if case["model"]:
            lib.pfMatrixMode(A.PF_MODELVIEW)
            lib.pfPopMatrix()
        fr = tg.finish()
        if texh is not None:
            th = C.c_void_p(texh)
            lib.pfDeleteTexture(C.byref(th), False)
        return fr
    finally:
        tg.close()


TYPE_CASES = [
    # (position type, normal/uv type, colour type, index type)
    (A.PF_SHORT, A.PF_FLOAT, A.PF_UNSIGNED_SHORT, A.PF_UNSIGNED_BYTE),
    (A.PF_INT, A.PF_DOUBLE, A.PF_UNSIGNED_INT, A.PF_UNSIGNED_SHORT),
    (A.PF_DOUBLE, A.PF_DOUBLE, A.PF_FLOAT, A.PF_UNSIGNED_INT),
    (A.PF_FLOAT, A.PF_FLOAT, A.PF_DOUBLE, A.PF_UNSIGNED_BYTE),
]

_NP = {A.PF_SHORT: np.int16, A.PF_INT: np.int32, A.PF_FLOAT: np.float32, A.PF_DOUBLE: np.float64,
       A.PF_UNSIGNED_BYTE: np.uint8, A.PF_UNSIGNED_SHORT: np.uint16, A.PF_UNSIGNED_INT: np.uint32}


def run_types(lib: A.PixelForgeLib, seed: int, types, target: str = "fbo") -> Frame:
    """Vertex arrays of every accepted element type (context.c:1231-1575):
    integer or floating positions, float or double normals and texture
    coordinates, 8/16/32-bit or floating colours, 8/16/32-bit indices."""
    ptype, ntype, ctype, itype = types
    r = np.random.default_rng(seed)
    W, H = 96, 72
    tg = Target(lib, W, H, target)
    texh = None
    try:
        n = 60
        pos = r.integers(-100, 101, (n, 3)).astype(np.float64)
        pos[:, 2] = r.integers(-90, 91, n)
        nrm = r.normal(size=(n, 3))
        uv = r.uniform(0.0, 0.95, (n, 2))
        colf = r.uniform(0, 1, (n, 4))
        colf[:, 3] = 1.0
        if ctype in (A.PF_FLOAT, A.PF_DOUBLE):
            col = colf.astype(_NP[ctype])
        else:
            scale = {A.PF_UNSIGNED_BYTE: 255, A.PF_UNSIGNED_SHORT: 65535, A.PF_UNSIGNED_INT: 4294967295}[ctype]
            col = np.floor(colf * scale).astype(_NP[ctype])
        idx = r.integers(0, n, 90).astype(_NP[itype])
        pos_t = pos.astype(_NP[ptype])
        nrm_t, uv_t = nrm.astype(_NP[ntype]), uv.astype(_NP[ntype])
        texture = r.integers(0, 256, (8, 8, 4)).astype(np.uint8)
        lib.pfClearDepth(1e30)
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        lib.pfMatrixMode(A.PF_PROJECTION)
        lib.pfLoadIdentity()
        lib.pfOrtho(-110.0, 110.0, -110.0, 110.0, -120.0, 120.0)
        lib.pfMatrixMode(A.PF_MODELVIEW)
        lib.pfLoadIdentity()
        lib.pfDisable(A.PF_CULL_FACE)
        lib.pfEnable(A.PF_DEPTH_TEST)
        texh = lib.pfGenTexture(_ptr(texture), 8, 8, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
        lib.pfBindTexture(texh)
        lib.pfEnable(A.PF_TEXTURE_2D)
        lib.pfEnable(A.PF_LIGHTING)
        lib.pfEnableLight(0)
        lp = np.array([50.0, 80.0, 150.0], np.float32)
        lib.pfLightfv(0, A.PF_POSITION, _ptr(lp))
        lib.pfEnable(A.PF_VERTEX_ARRAY | A.PF_NORMAL_ARRAY | A.PF_TEXTURE_COORD_ARRAY | A.PF_COLOR_ARRAY)
        lib.pfVertexPointer(3, ptype, 0, _ptr(pos_t))
        lib.pfNormalPointer(ntype, 0, _ptr(nrm_t))
        lib.pfTexCoordPointer(ntype, 0, _ptr(uv_t))
        lib.pfColorPointer(4, ctype, 0, _ptr(col))
        lib.pfDrawElements(A.PF_TRIANGLES, len(idx), itype, _ptr(idx))
        fr = tg.finish()
        if texh is not None:
            th = C.c_void_p(texh)
            lib.pfDeleteTexture(C.byref(th), False)
        return fr
    finally:
        tg.close()
