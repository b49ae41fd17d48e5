"""Seeded synthetic workloads of the PixelForge triangle pipeline.

Every scene is built with numpy's PCG64 generator from a fixed seed and is
replayed through the ``pf*`` C API of whichever library it is given (the GPU
library, or in tests the CPU oracle / reference build), so that all of them
see exactly the same call sequence and inputs.  Sizes follow the five
workloads the project measures:

  0  soup256   256x256, 2,000-triangle immediate-mode soup, default projection
  1  sphere1080  1920x1080 textured lit UV sphere (256x128 segments) drawn
                twice: opaque, then scaled 1.05 with alpha 0.5 blending
  2  phong1080  1920x1080 displaced icosphere (subdivision 8, 1.31M triangles),
                per-fragment Phong with 8 point lights, nearest mirrored
                texture, 30% of triangles additively blended, device fog
  3  batched    512 independent contexts of uneven sizes (see batch.py)
  4  fit        inverse texture/material fit (see fit.py)

The reference has no published benchmark suite; these stand in for it.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi as A

FLT_MAX = float(np.finfo(np.float32).max)


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


@dataclass
class Frame:
    """Result of one rendered scene: colour (H, W, 4) uint8, depth (H, W) f32."""
    color: np.ndarray
    depth: np.ndarray | None
    stats: dict = field(default_factory=dict)


class Target:
    """Where a scene renders.

    ``main``: the context's own buffer (the caller's numpy array), as
    pfCreateContext wraps it.  ``fbo``: a framebuffer object made by
    pfGenFramebuffer and bound with PF_FRAMEBUFFER, which also exposes the
    depth buffer through its public ``zbuffer`` pointer.
    """

    def __init__(self, lib: A.PixelForgeLib, width: int, height: int, kind: str = "fbo",
                 init: np.ndarray | None = None, fmt: tuple = (A.PF_RGBA, A.PF_UNSIGNED_BYTE)):
        self.lib, self.w, self.h, self.kind = lib, width, height, kind
        self.fmt, self.bpp = fmt, A.pixel_bytes(*fmt)
        # packed 16-bit formats: the reference's pfClear copies its tail at
        # components x 2 bytes per pixel (src/internal/pixel.h:3156-3210),
        # past the pixels; the buffer gets room for those writes
        n = height * width * self.bpp
        self._backing = np.zeros(n * (4 if self.bpp == 2 else 1), np.uint8)
        self.main = self._backing[:n].reshape(height, width, self.bpp)
        if init is not None:
            self.main[...] = init
        self.ctx = lib.pfCreateContext(_ptr(self.main), width, height, *fmt)
        if not self.ctx:
            raise RuntimeError("pfCreateContext failed")
        lib.pfMakeCurrent(self.ctx)
        self.fb = None
        if kind == "fbo":
            self.fb = lib.pfGenFramebuffer(width, height, *fmt)
            self._fbref = C.pointer(self.fb)
            lib.pfBindFramebuffer(self._fbref)
            lib.pfEnable(A.PF_FRAMEBUFFER)

    def finish(self) -> Frame:
        lib = self.lib
        if lib.has("pfFinish"):
            lib.pfFinish()
        stats = {}
        if lib.has("pfGetStats"):
            s = A.PFstats()
            lib.pfGetStats(C.byref(s))
            stats = {k: int(getattr(s, k)) for k, _ in A.PFstats._fields_}
        if self.kind == "fbo":
            px = lib.raw("pfGetTexturePixels")
            px.restype = C.c_void_p
            px.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
            base = px(self.fb.texture, None, None, None, None)
            color = np.ctypeslib.as_array(C.cast(base, C.POINTER(C.c_uint8)),
                                          shape=(self.h, self.w, self.bpp)).copy()
            depth = np.ctypeslib.as_array(self.fb.zbuffer, shape=(self.h, self.w)).copy()
            return Frame(color, depth, stats)
        return Frame(self.main.copy(), None, stats)

    def close(self):
        lib = self.lib
        if self.fb is not None:
            lib.pfDisable(A.PF_FRAMEBUFFER)
            lib.pfBindFramebuffer(None)
            lib.pfDeleteFramebuffer(self._fbref)
            self.fb = None
        lib.pfDeleteContext(self.ctx)
        self.ctx = None


# ---------------------------------------------------------------------------
# geometry
# ---------------------------------------------------------------------------

def uv_sphere(segments: int = 256, rings: int = 128):
    """UV sphere: (rings+1)*(segments+1) vertices, 2*segments*rings triangles.

    Returns float32 positions (N,3) (unit radius, also the normals), float32
    texcoords (N,2) and uint32 indices (T*3,), wound so that the outside faces
    the camera as PF_FRONT under the reference's cull rule.
    """
    r = np.arange(rings + 1, dtype=np.float64)[:, None]
    s = np.arange(segments + 1, dtype=np.float64)[None, :]
    theta = np.pi * r / rings
    phi = 2.0 * np.pi * s / segments
    x = np.sin(theta) * np.cos(phi)
    y = np.cos(theta) * np.ones_like(phi)
    z = np.sin(theta) * np.sin(phi)
    pos = np.stack([x, y, z], -1).reshape(-1, 3).astype(np.float32)
    uv = np.stack([np.broadcast_to(s / segments, x.shape), np.broadcast_to(r / rings, x.shape)],
                  -1).reshape(-1, 2).astype(np.float32)
    rr, ss = np.meshgrid(np.arange(rings), np.arange(segments), indexing="ij")
    a = (rr * (segments + 1) + ss).ravel()
    b = a + segments + 1
    tri = np.stack([np.stack([a, a + 1, b], -1), np.stack([a + 1, b + 1, b], -1)], 1).reshape(-1, 3)
    return pos, uv, tri.astype(np.uint32).ravel()


def icosphere(subdiv: int):
    """Icosphere: 10*4^s+2 vertices, 20*4^s triangles (float32 unit positions)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
         (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = np.array(v, np.float64)
    verts /= np.linalg.norm(verts, axis=1, keepdims=True)
    faces = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9),
                      (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2),
                      (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
                      (8, 6, 7), (9, 8, 1)], np.int64)
    for _ in range(subdiv):
        nv = len(verts)
        e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * (nv + 1) + e[:, 1]
        uk, inv = np.unique(key, return_inverse=True)
        a, b = uk // (nv + 1), uk % (nv + 1)
        mid = verts[a] + verts[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        verts = np.concatenate([verts, mid])
        nf = len(faces)
        m01, m12, m20 = (inv[:nf] + nv, inv[nf:2 * nf] + nv, inv[2 * nf:] + nv)
        f0, f1, f2 = faces[:, 0], faces[:, 1], faces[:, 2]
        faces = np.concatenate([np.stack([f0, m01, m20], 1), np.stack([f1, m12, m01], 1),
                                np.stack([f2, m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return verts, faces


def noise_texture(size: int, seed: int) -> np.ndarray:
    """Uniform RGBA8 noise, alpha 255."""
    rng = np.random.default_rng(seed)
    tex = rng.integers(0, 256, (size, size, 4), dtype=np.uint8)
    tex[..., 3] = 255
    return np.ascontiguousarray(tex)


def value_noise_texture(size: int, seed: int, cells: int = 32) -> np.ndarray:
    """Smooth value noise (bilinear interpolation of a random lattice), RGBA8."""
    rng = np.random.default_rng(seed)
    lat = rng.random((cells + 1, cells + 1, 3))
    g = np.arange(size, dtype=np.float64) * cells / size
    i0 = np.floor(g).astype(np.int64)
    f = g - i0
    f = f * f * (3 - 2 * f)
    a = lat[i0][:, i0]
    b = lat[i0][:, i0 + 1]
    c = lat[i0 + 1][:, i0]
    d = lat[i0 + 1][:, i0 + 1]
    fy, fx = f[:, None, None], f[None, :, None]
    val = (a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy
    tex = np.empty((size, size, 4), np.uint8)
    tex[..., :3] = np.clip(val * 255.0, 0, 255).astype(np.uint8)
    tex[..., 3] = 255
    return tex


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

@dataclass
class SoupScene:
    """Config 0 and its variants: an immediate-mode triangle soup."""
    width: int = 256
    height: int = 256
    ntris: int = 2000
    seed: int = 1000
    cull: bool = True
    depth_func: int = A.PF_LESS
    shade: int = A.PF_SMOOTH
    blend: int | None = None
    clear_depth: float = 1.0
    z_range: tuple = (0.1, 0.9)
    xy_range: tuple = (-1.0, 1.0)

    def data(self):
        rng = np.random.default_rng(self.seed)
        xy = rng.uniform(self.xy_range[0], self.xy_range[1], (self.ntris, 3, 2)).astype(np.float32)
        z = rng.uniform(self.z_range[0], self.z_range[1], (self.ntris, 3)).astype(np.float32)
        rgb = rng.integers(0, 256, (self.ntris, 3, 3), dtype=np.int64)
        a = np.full((self.ntris, 3, 1), 255, np.int64)
        if self.blend is not None:
            a = rng.integers(0, 256, (self.ntris, 3, 1), dtype=np.int64)
        return xy, z, np.concatenate([rgb, a], -1).astype(np.uint8)

    def record(self, lib: A.PixelForgeLib):
        xy, z, col = self.data()
        lib.pfClearDepth(self.clear_depth)
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        lib.pfEnable(A.PF_DEPTH_TEST)
        lib.pfDepthFunc(self.depth_func)
        lib.pfShadeModel(self.shade)
        if not self.cull:
            lib.pfDisable(A.PF_CULL_FACE)
        if self.blend is not None:
            lib.pfEnable(A.PF_BLEND)
            lib.pfBlendFunc(self.blend)
        color4ub, vertex3f = lib.pfColor4ub, lib.pfVertex3f
        xl, zl, cl = xy.tolist(), z.tolist(), col.tolist()
        lib.pfBegin(A.PF_TRIANGLES)
        for t in range(self.ntris):
            for k in range(3):
                c = cl[t][k]
                color4ub(c[0], c[1], c[2], c[3])
                vertex3f(xl[t][k][0], xl[t][k][1], zl[t][k])
        lib.pfEnd()

    def render(self, lib, target: str = "fbo") -> Frame:
        tg = Target(lib, self.width, self.height, target)
        try:
            self.record(lib)
            return tg.finish()
        finally:
            tg.close()


@dataclass
class SphereScene:
    """Config 1: textured, Gouraud-lit UV sphere at 1920x1080, drawn twice."""
    width: int = 1920
    height: int = 1080
    segments: int = 256
    rings: int = 128
    tex_size: int = 1024
    tex_seed: int = 1001
    filt: int = A.PF_BILINEAR
    wrap: int = A.PF_REPEAT
    second_draw: bool = True
    lighting: int | None = A.PF_GOURAUD
    distance: float = 3.0
    fov_deg: float = 60.0
    znear: float = 0.1
    zfar: float = 100.0
    depth_mask_off: bool = True   # second draw without depth writes (extension)
    device_arrays: bool = False   # arrays, indices and texture in device memory (zero-copy extension)

    def __post_init__(self):
        self.pos, self.uv, self.idx = uv_sphere(self.segments, self.rings)
        self.tex = noise_texture(self.tex_size, self.tex_seed)
        self._dev = None

    @property
    def ntris(self) -> int:
        return len(self.idx) // 3

    def setup(self, lib):
        """State that persists across frames (camera, light, material, texture)."""
        aspect = self.width / self.height
        top = self.znear * float(np.tan(np.radians(self.fov_deg) / 2))
        right = top * aspect
        lib.pfMatrixMode(A.PF_PROJECTION)
        lib.pfLoadIdentity()
        lib.pfFrustum(-right, right, -top, top, self.znear, self.zfar)
        lib.pfMatrixMode(A.PF_MODELVIEW)
        lib.pfLoadIdentity()
        lib.pfTranslatef(0.0, 0.0, -self.distance)
        lib.pfEnable(A.PF_DEPTH_TEST)
        lib.pfDepthFunc(A.PF_LESS)
        if self.lighting is not None:
            lib.pfEnable(A.PF_LIGHTING)
            lib.pfLightModel(self.lighting)
            lib.pfEnableLight(0)
            d = np.array([-1.0, 1.0, 1.0]) / np.sqrt(3.0) * 1000.0
            lib.pfLightfv(0, A.PF_POSITION, _ptr(np.ascontiguousarray(d, np.float32)))
            lib.pfMaterialf(A.PF_FRONT_AND_BACK, A.PF_DIFFUSE, 0.8)
            lib.pfMaterialf(A.PF_FRONT_AND_BACK, A.PF_SPECULAR, 0.5)
            lib.pfMaterialf(A.PF_FRONT_AND_BACK, A.PF_SHININESS, 32.0)
        lib.pfEnable(A.PF_TEXTURE_2D)
        lib.pfEnable(A.PF_VERTEX_ARRAY | A.PF_NORMAL_ARRAY | A.PF_TEXTURE_COORD_ARRAY)
        if self.device_arrays:
            import torch
            dev = torch.device("cuda:0")
            self._dev = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
                         for k, v in (("pos", self.pos), ("uv", self.uv), ("idx", self.idx), ("tex", self.tex))}
            torch.cuda.synchronize()
            dp = lambda k: C.c_void_p(self._dev[k].data_ptr())
            self.texh = lib.pfGenTextureDevice(dp("tex"), self.tex_size, self.tex_size)
            lib.pfVertexPointerDevice(3, A.PF_FLOAT, 0, dp("pos"))
            lib.pfNormalPointerDevice(A.PF_FLOAT, 0, dp("pos"))
            lib.pfTexCoordPointerDevice(A.PF_FLOAT, 0, dp("uv"))
        else:
            self.texh = lib.pfGenTexture(_ptr(self.tex), self.tex_size, self.tex_size, A.PF_RGBA,
                                         A.PF_UNSIGNED_BYTE)
            lib.pfVertexPointer(3, A.PF_FLOAT, 0, _ptr(self.pos))
            lib.pfNormalPointer(A.PF_FLOAT, 0, _ptr(self.pos))
            lib.pfTexCoordPointer(A.PF_FLOAT, 0, _ptr(self.uv))
        lib.pfTextureParameter(self.texh, self.wrap, self.filt)
        lib.pfBindTexture(self.texh)

    def _draw(self, lib):
        if self._dev is not None:
            lib.pfDrawElementsDevice(A.PF_TRIANGLES, len(self.idx), len(self.pos), C.c_void_p(self._dev["idx"].data_ptr()))
        else:
            lib.pfDrawElements(A.PF_TRIANGLES, len(self.idx), A.PF_UNSIGNED_INT, _ptr(self.idx))

    def frame(self, lib):
        """One frame: clear, opaque draw, scaled alpha-blended draw."""
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        lib.pfColor4ub(255, 255, 255, 255)
        self._draw(lib)
        if self.second_draw:
            lib.pfPushMatrix()
            lib.pfScalef(1.05, 1.05, 1.05)
            lib.pfColor4f(1.0, 1.0, 1.0, 0.5)
            lib.pfEnable(A.PF_BLEND)
            lib.pfBlendFunc(A.PF_BLEND_ALPHA)
            mask = self.depth_mask_off and lib.has("pfDepthMask")
            if mask:
                lib.pfDepthMask(False)
            self._draw(lib)
            if mask:
                lib.pfDepthMask(True)
            lib.pfDisable(A.PF_BLEND)
            lib.pfPopMatrix()

    def teardown(self, lib):
        th = C.c_void_p(self.texh)
        lib.pfDeleteTexture(C.byref(th), False)
        self._dev = None

    def render(self, lib, target: str = "fbo", fmt: tuple = (A.PF_RGBA, A.PF_UNSIGNED_BYTE)) -> Frame:
        tg = Target(lib, self.width, self.height, target, fmt=fmt)
        try:
            self.setup(lib)
            self.frame(lib)
            fr = tg.finish()
            self.teardown(lib)
            return fr
        finally:
            tg.close()


@dataclass
class PhongScene:
    """Config 2: fragment-heavy Phong on a displaced icosphere."""
    width: int = 1920
    height: int = 1080
    subdiv: int = 8
    seed: int = 1002
    tex_size: int = 2048
    nlights: int = 8
    add_frac: float = 0.3
    distance: float = 3.0
    fov_deg: float = 60.0
    znear: float = 0.1
    zfar: float = 6.0
    fog: bool = True
    filt: int = A.PF_NEAREST
    wrap: int = A.PF_MIRRORED_REPEAT
    light_model: int = A.PF_PHONG

    def __post_init__(self):
        rng = np.random.default_rng(self.seed)
        v, f = icosphere(self.subdiv)
        disp = 1.0 + 0.04 * rng.standard_normal(len(v))
        p = v * disp[:, None]
        self.pos = p.astype(np.float32)
        self.nrm = v.astype(np.float32)
        u = 0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2 * np.pi)
        w = np.arccos(np.clip(v[:, 1], -1, 1)) / np.pi
        # scaled by 1.9 rather than 2 so that no vertex sits exactly on the
        # mirrored edge (coordinate 1.0), where the reference's nearest map
        # rounds to texel w and reads past its texture
        self.uv = (np.stack([u, w], 1) * 1.9).astype(np.float32)
        add = rng.random(len(f)) < self.add_frac
        self.idx_opaque = f[~add].astype(np.uint32).ravel()
        self.idx_add = f[add].astype(np.uint32).ravel()
        self.tex = value_noise_texture(self.tex_size, self.seed + 1)
        d = rng.standard_normal((self.nlights, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        self.lights = (d * 4.0).astype(np.float32)
        self.light_col = rng.uniform(0.3, 1.0, (self.nlights, 3)).astype(np.float32)

    @property
    def ntris(self) -> int:
        return (len(self.idx_opaque) + len(self.idx_add)) // 3

    def setup(self, lib):
        aspect = self.width / self.height
        top = self.znear * float(np.tan(np.radians(self.fov_deg) / 2))
        right = top * aspect
        lib.pfMatrixMode(A.PF_PROJECTION)
        lib.pfLoadIdentity()
        lib.pfFrustum(-right, right, -top, top, self.znear, self.zfar)
        lib.pfMatrixMode(A.PF_MODELVIEW)
        lib.pfLoadIdentity()
        lib.pfTranslatef(0.0, 0.0, -self.distance)
        lib.pfEnable(A.PF_DEPTH_TEST)
        lib.pfDepthFunc(A.PF_LESS)
        lib.pfEnable(A.PF_LIGHTING)
        lib.pfLightModel(self.light_model)
        for i in range(self.nlights):
            lib.pfEnableLight(i)
            lib.pfLightfv(i, A.PF_POSITION, _ptr(np.ascontiguousarray(self.lights[i])))
            lib.pfLightfv(i, A.PF_DIFFUSE, _ptr(np.ascontiguousarray(self.light_col[i])))
        lib.pfMaterialf(A.PF_FRONT_AND_BACK, A.PF_DIFFUSE, 0.9)
        lib.pfMaterialf(A.PF_FRONT_AND_BACK, A.PF_SPECULAR, 0.3)
        lib.pfMaterialf(A.PF_FRONT_AND_BACK, A.PF_SHININESS, 24.0)
        self.texh = lib.pfGenTexture(_ptr(self.tex), self.tex_size, self.tex_size, A.PF_RGBA,
                                     A.PF_UNSIGNED_BYTE)
        lib.pfTextureParameter(self.texh, self.wrap, self.filt)
        lib.pfBindTexture(self.texh)
        lib.pfEnable(A.PF_TEXTURE_2D)
        lib.pfEnable(A.PF_VERTEX_ARRAY | A.PF_NORMAL_ARRAY | A.PF_TEXTURE_COORD_ARRAY)
        lib.pfVertexPointer(3, A.PF_FLOAT, 0, _ptr(self.pos))
        lib.pfNormalPointer(A.PF_FLOAT, 0, _ptr(self.nrm))
        lib.pfTexCoordPointer(A.PF_FLOAT, 0, _ptr(self.uv))

    def fog_params(self) -> A.PFhookfog:
        return A.PFhookfog(self.znear, self.zfar, 0.3, 0.9, A.PFcolor(160, 170, 190, 255))

    def frame(self, lib, host_fog=None):
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        lib.pfDrawElements(A.PF_TRIANGLES, len(self.idx_opaque), A.PF_UNSIGNED_INT, _ptr(self.idx_opaque))
        lib.pfEnable(A.PF_BLEND)
        lib.pfBlendFunc(A.PF_BLEND_ADD)
        lib.pfDrawElements(A.PF_TRIANGLES, len(self.idx_add), A.PF_UNSIGNED_INT, _ptr(self.idx_add))
        lib.pfDisable(A.PF_BLEND)
        if self.fog:
            fp = self.fog_params()
            if lib.has("pfPostProcessDevice"):
                lib.pfPostProcessDevice(A.PF_HOOK_FOG_LINEAR, C.c_void_p(C.addressof(fp)), C.sizeof(fp))
            elif host_fog is not None:
                host_fog(fp)

    def teardown(self, lib):
        th = C.c_void_p(self.texh)
        lib.pfDeleteTexture(C.byref(th), False)

    def render(self, lib, target: str = "fbo", host_fog=None) -> Frame:
        tg = Target(lib, self.width, self.height, target)
        try:
            self.setup(lib)
            self.frame(lib, host_fog)
            fr = tg.finish()
            self.teardown(lib)
            return fr
        finally:
            tg.close()


@dataclass
class BatchScene:
    """Config 3: many independent contexts of uneven size and load.

    Context i: square framebuffer of side ~ U{64, 128, ..., max_side}; a
    triangle soup as in the 256x256 workload (xy in [-1, 1], z in [0.1, 0.9],
    RGB uniform, alpha 255) plus UVs in [0, 2], triangle count lognormal
    (median ``tri_median``, sigma ``tri_sigma``) clipped to ``tri_clip``; one
    256x256 noise texture with a uniformly chosen filter and wrap; blending
    uniformly one of alpha / additive / multiply / none; depth test LESS
    against a depth cleared to 1.0.  Triangles are submitted with
    pfDrawArrays(PF_TRIANGLES), which processes them exactly as
    pfBegin/pfVertex does.
    """
    n: int = 512
    seed: int = 1003
    max_side: int = 512
    tri_median: float = 2000.0
    tri_sigma: float = 1.0
    tri_clip: tuple = (100, 50000)
    tex_size: int = 256
    fmts: tuple = ()                 # framebuffer (format, type) of context i: fmts[i % len]; RGBA8 if empty

    def __post_init__(self):
        rng = np.random.default_rng(self.seed)
        steps = self.max_side // 64
        self.sides = (rng.integers(1, steps + 1, self.n) * 64).astype(int)
        nt = np.exp(np.log(self.tri_median) + self.tri_sigma * rng.standard_normal(self.n))
        self.ntris = np.clip(nt.astype(int), self.tri_clip[0], self.tri_clip[1])
        self.filters = rng.integers(0, 2, self.n)
        self.wraps = rng.integers(0, 3, self.n)
        self.blends = rng.choice([A.PF_BLEND_ALPHA, A.PF_BLEND_ADD, A.PF_BLEND_MUL, -1], self.n)
        self.pos, self.col, self.uv, self.tex = [], [], [], []
        for i in range(self.n):
            m = int(self.ntris[i]) * 3
            p = np.empty((m, 3), np.float32)
            p[:, :2] = rng.uniform(-1, 1, (m, 2))
            p[:, 2] = rng.uniform(0.1, 0.9, m)
            c = rng.integers(0, 256, (m, 4), dtype=np.uint8)
            c[:, 3] = 255
            self.pos.append(p)
            self.col.append(c)
            self.uv.append(rng.uniform(0, 2, (m, 2)).astype(np.float32))
            self.tex.append(noise_texture(self.tex_size, self.seed * 1000 + i))
        self.ctx = []
        self.buf = []
        self.texh = []

    @property
    def total_tris(self) -> int:
        return int(self.ntris.sum())

    def create(self, lib):
        for i in range(self.n):
            s = int(self.sides[i])
            fmt = self.fmts[i % len(self.fmts)] if self.fmts else (A.PF_RGBA, A.PF_UNSIGNED_BYTE)
            b = np.zeros((s, s, A.pixel_bytes(*fmt)), np.uint8)
            c = lib.pfCreateContext(_ptr(b), s, s, *fmt)
            lib.pfMakeCurrent(c)
            t = lib.pfGenTexture(_ptr(self.tex[i]), self.tex_size, self.tex_size, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
            lib.pfTextureParameter(t, int(self.wraps[i]), int(self.filters[i]))
            self.ctx.append(c)
            self.buf.append(b)
            self.texh.append(t)

    def record(self, lib, i):
        lib.pfMakeCurrent(self.ctx[i])
        lib.pfClearDepth(1.0)
        lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
        lib.pfEnable(A.PF_DEPTH_TEST)
        lib.pfDepthFunc(A.PF_LESS)
        lib.pfBindTexture(self.texh[i])
        lib.pfEnable(A.PF_TEXTURE_2D)
        if self.blends[i] >= 0:
            lib.pfEnable(A.PF_BLEND)
            lib.pfBlendFunc(int(self.blends[i]))
        else:
            lib.pfDisable(A.PF_BLEND)
        lib.pfEnable(A.PF_VERTEX_ARRAY | A.PF_COLOR_ARRAY | A.PF_TEXTURE_COORD_ARRAY)
        lib.pfVertexPointer(3, A.PF_FLOAT, 0, _ptr(self.pos[i]))
        lib.pfColorPointer(4, A.PF_UNSIGNED_BYTE, 0, _ptr(self.col[i]))
        lib.pfTexCoordPointer(A.PF_FLOAT, 0, _ptr(self.uv[i]))
        lib.pfDrawArrays(A.PF_TRIANGLES, 0, int(self.ntris[i]) * 3)

    def render_loop(self, lib, finish=True):
        """Each context on its own: record, then its own observation point."""
        for i in range(self.n):
            self.record(lib, i)
            if finish and lib.has("pfFinish"):
                lib.pfFinish()
        return [b.copy() for b in self.buf]

    def render_batch(self, lib, batch):
        """All contexts recorded into one batch and rendered together."""
        lib.pfgbBatchBegin(batch)
        for i in range(self.n):
            self.record(lib, i)
        lib.pfgbBatchEnd(batch)
        return [b.copy() for b in self.buf]

    def destroy(self, lib):
        for i, c in enumerate(self.ctx):
            lib.pfMakeCurrent(c)
            th = C.c_void_p(self.texh[i])
            lib.pfDeleteTexture(C.byref(th), False)
            lib.pfDeleteContext(c)
        self.ctx, self.buf, self.texh = [], [], []
