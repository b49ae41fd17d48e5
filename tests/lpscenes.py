"""Seeded point and line scenes (immediate mode, vertex arrays and the
PF_POINT / PF_LINE polygon modes), replayable on any pf* library."""
from __future__ import annotations

import numpy as np

from pixelforge_gb300 import abi as A
from pixelforge_gb300.scenes import Frame, Target, _ptr


def lp_case(seed: int) -> dict:
    r = np.random.default_rng(seed)
    return dict(
        seed=seed,
        kind=["points", "lines", "poly"][int(r.integers(3))],
        proj=["default", "frustum"][int(r.integers(2))],
        size=float(r.choice([1.0, 2.0, 3.5, 6.0])),
        width=float(r.choice([1.0, 1.2, 3.0, 5.5])),
        depth=int(r.integers(-1, 6)),
        blend=int(r.integers(-1, 8)),
        cull=int(r.integers(3)),
        front=int(r.choice([A.PF_POINT, A.PF_LINE, A.PF_FILL])),
        back=int(r.choice([A.PF_POINT, A.PF_LINE, A.PF_FILL])),
        quads=bool(r.random() < 0.4),
        source=["immediate", "arrays"][int(r.integers(2))],
        n=int(r.integers(10, 60)),
    )


def run_lp(lib: A.PixelForgeLib, case: dict, target: str = "fbo") -> Frame:
    r = np.random.default_rng(case["seed"] + 101)
    W, H = 96, 80
    tg = Target(lib, W, H, target)
    try:
        lib.pfClearDepth(1e30 if case["proj"] == "frustum" else 1.0)
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        if case["proj"] == "frustum":
            lib.pfMatrixMode(A.PF_PROJECTION)
            lib.pfLoadIdentity()
            lib.pfFrustum(-0.08, 0.08, -0.06, 0.06, 0.1, 10.0)
            lib.pfMatrixMode(A.PF_MODELVIEW)
            lib.pfLoadIdentity()
            lib.pfTranslatef(0.0, 0.0, -2.2)
        if case["depth"] >= 0:
            lib.pfEnable(A.PF_DEPTH_TEST)
            lib.pfDepthFunc(case["depth"])
        if case["blend"] >= 0:
            lib.pfEnable(A.PF_BLEND)
            lib.pfBlendFunc(case["blend"])
        if case["cull"] == 0:
            lib.pfDisable(A.PF_CULL_FACE)
        elif case["cull"] == 2:
            lib.pfCullFace(A.PF_FRONT)
        lib.pfPointSize(case["size"])
        lib.pfLineWidth(case["width"])
        lib.pfPolygonMode(A.PF_FRONT, case["front"])
        lib.pfPolygonMode(A.PF_BACK, case["back"])
        if case["kind"] == "points":
            mode, per = A.PF_POINTS, 1
        elif case["kind"] == "lines":
            mode, per = A.PF_LINES, 2
        else:
            mode, per = (A.PF_QUADS, 4) if case["quads"] else (A.PF_TRIANGLES, 3)
        n = case["n"] * per
        # Thick lines stay inside the framebuffer with a margin wider than
        # their offsets (past the edges the reference writes outside its
        # buffers); thin ones may be clipped by the viewport or the frustum.
        thick = case["width"] > 1.5 and case["kind"] != "points"
        if case["proj"] == "default":
            lim = 0.72 if thick else 1.3
            pos = np.concatenate([r.uniform(-lim, lim, (n, 2)), r.uniform(-0.9, 0.9, (n, 1))], 1)
        else:
            lim, zr = (0.3, 1.2) if thick else (1.4, 2.6)
            pos = np.concatenate([r.uniform(-lim, lim, (n, 2)), r.uniform(-zr, zr, (n, 1))], 1)
        pos = pos.astype(np.float32)
        col = r.integers(0, 256, (n, 4)).astype(np.uint8)
        if case["source"] == "immediate":
            lib.pfBegin(mode)
            for i in range(n):
                c = col[i]
                lib.pfColor4ub(int(c[0]), int(c[1]), int(c[2]), int(c[3]))
                lib.pfVertex3f(float(pos[i, 0]), float(pos[i, 1]), float(pos[i, 2]))
            lib.pfEnd()
        else:
            lib.pfEnable(A.PF_VERTEX_ARRAY | A.PF_COLOR_ARRAY)
            lib.pfVertexPointer(3, A.PF_FLOAT, 0, _ptr(pos))
            lib.pfColorPointer(4, A.PF_UNSIGNED_BYTE, 0, _ptr(col))
            idx = r.integers(0, n, n).astype(np.uint32)
            lib.pfDrawElements(mode, n, A.PF_UNSIGNED_INT, _ptr(idx))
        return tg.finish()
    finally:
        tg.close()


def run_wire(lib: A.PixelForgeLib, W: int = 1920, H: int = 1080, target: str = "fbo", seed: int = 5) -> Frame:
    """A full-HD wireframe: a warped grid drawn as triangles with front faces
    in PF_LINE mode and back faces filled, a thick polyline and a cloud of
    large points over it, depth-tested, through vertex arrays."""
    r = np.random.default_rng(seed)
    tg = Target(lib, W, H, target)
    try:
        lib.pfClearDepth(1.0)
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        lib.pfEnable(A.PF_DEPTH_TEST)
        lib.pfDepthFunc(A.PF_LEQUAL)
        lib.pfDisable(A.PF_CULL_FACE)
        g = 60
        u, v = np.meshgrid(np.linspace(-0.92, 0.92, g + 1), np.linspace(-0.9, 0.9, g + 1))
        z = 0.5 * np.sin(3.0 * u) * np.cos(2.0 * v)
        pos = np.stack([u + 0.02 * np.sin(9 * v), v, z], -1).reshape(-1, 3).astype(np.float32)
        col = r.integers(0, 256, (pos.shape[0], 4)).astype(np.uint8)
        q = np.arange(g * g)
        a = (q // g) * (g + 1) + q % g
        tri = np.stack([a, a + 1, a + g + 2, a, a + g + 2, a + g + 1], -1).reshape(-1).astype(np.uint32)
        lib.pfPolygonMode(A.PF_FRONT, A.PF_LINE)
        lib.pfPolygonMode(A.PF_BACK, A.PF_FILL)
        lib.pfEnable(A.PF_VERTEX_ARRAY | A.PF_COLOR_ARRAY)
        lib.pfVertexPointer(3, A.PF_FLOAT, 0, _ptr(pos))
        lib.pfColorPointer(4, A.PF_UNSIGNED_BYTE, 0, _ptr(col))
        lib.pfDrawElements(A.PF_TRIANGLES, tri.size, A.PF_UNSIGNED_INT, _ptr(tri))
        lib.pfDisable(A.PF_VERTEX_ARRAY | A.PF_COLOR_ARRAY)
        lib.pfLineWidth(4.0)
        lib.pfBegin(A.PF_LINES)
        t = np.linspace(0, 2 * np.pi, 201)
        for i in range(200):
            lib.pfColor4ub(255, (i * 7) % 256, 40, 255)
            for k in (i, i + 1):
                lib.pfVertex3f(float(0.7 * np.cos(t[k])), float(0.7 * np.sin(2 * t[k])), -0.2)
        lib.pfEnd()
        lib.pfEnable(A.PF_BLEND)
        lib.pfBlendFunc(A.PF_BLEND_ALPHA)
        lib.pfPointSize(7.0)
        lib.pfBegin(A.PF_POINTS)
        for p in r.uniform(-0.95, 0.95, (500, 3)):
            lib.pfColor4ub(40, 200, 255, 160)
            lib.pfVertex3f(float(p[0]), float(p[1]), float(p[2]))
        lib.pfEnd()
        return tg.finish()
    finally:
        tg.close()
