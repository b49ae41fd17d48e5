"""Differentiable rendering over the C ABI (include/pixelforge_grad.h).

``GradScene`` wraps a pfgrad scene: a fixed mesh seen from a set of views,
set up and binned once on the device.  ``GradScene.render`` is a
``torch.autograd.Function``: its forward calls ``pfgradForward`` and its
backward calls ``pfgradBackward`` (which recomputes the fragments tile by
tile) on torch's current CUDA stream, passing ``tensor.data_ptr()`` device
pointers.  Visibility (coverage and depth-test outcome) is held fixed; the
parameters are the RGBA texture, per-vertex colours and alphas, the material
(diffuse, specular, shininess) and the light direction.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

PFGRAD_ERRORS = {-2: "invalid argument", -3: "CUDA error", -4: "a tile holds too many triangles",
                 -5: "a triangle crosses the view volume (clipping is not differentiated)"}


class PFgradSceneDesc(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("texcoords", C.c_void_p),
                ("indices", C.c_void_p), ("nVertices", C.c_uint32), ("nTriangles", C.c_uint32),
                ("mvp", C.c_void_p), ("eye", C.c_void_p), ("nViews", C.c_uint32), ("width", C.c_uint32),
                ("height", C.c_uint32), ("cullFace", C.c_int32), ("texWidth", C.c_uint32),
                ("texHeight", C.c_uint32), ("texFilter", C.c_int32), ("texWrap", C.c_int32),
                ("ambient", C.c_float), ("background", C.c_float * 3), ("clearDepth", C.c_float)]


class PFgradParams(C.Structure):
    _fields_ = [("texture", C.c_void_p), ("colors", C.c_void_p), ("alphas", C.c_void_p),
                ("material", C.c_void_p), ("light", C.c_void_p)]


class PFgradGrads(C.Structure):
    _fields_ = [("texture", C.c_void_p), ("colors", C.c_void_p), ("alphas", C.c_void_p),
                ("material", C.c_void_p), ("light", C.c_void_p)]


class PFgradInfo(C.Structure):
    _fields_ = [("primitives", C.c_uint64), ("tileEntries", C.c_uint64), ("maxTilePrims", C.c_uint32),
                ("tiles", C.c_uint32)]


PROTOTYPES = {
    "pfgradSceneCreate": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(PFgradSceneDesc), C.c_void_p]),
    "pfgradSceneDestroy": (C.c_int, [C.c_void_p]),
    "pfgradSceneInfo": (C.c_int, [C.c_void_p, C.POINTER(PFgradInfo)]),
    "pfgradForward": (C.c_int, [C.c_void_p, C.POINTER(PFgradParams), C.c_void_p, C.c_void_p]),
    "pfgradBackward": (C.c_int, [C.c_void_p, C.POINTER(PFgradParams), C.c_void_p, C.POINTER(PFgradGrads),
                                 C.c_void_p]),
}


def bind(cdll: C.CDLL) -> C.CDLL:
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(cdll, name)
        fn.restype, fn.argtypes = res, args
    return cdll


def _check(rc: int, what: str):
    if rc != 0:
        raise RuntimeError(f"{what} failed: {PFGRAD_ERRORS.get(rc, rc)}")


@dataclass
class Mesh:
    positions: np.ndarray        # (nv, 3) float32
    normals: np.ndarray          # (nv, 3) float32
    texcoords: np.ndarray        # (nv, 2) float32
    indices: np.ndarray          # (nt, 3) uint32


PARAM_NAMES = ("texture", "colors", "alphas", "material", "light")


class GradScene:
    """A mesh, its views and the sampling state, set up on cuda:0."""

    def __init__(self, mesh: Mesh, mvp: np.ndarray, eye: np.ndarray, width: int, height: int,
                 tex_size: tuple, filter: int = 1, wrap: int = 0, cull: int = 1, ambient: float = 0.2,
                 background=(0.0, 0.0, 0.0), clear_depth: float = np.finfo(np.float32).max):
        import torch
        from . import LIB_PATH, load_library
        load_library()                       # builds the library if needed; no CPU fallback
        self.lib = bind(C.CDLL(str(LIB_PATH)))
        dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        self.mesh = mesh
        self.nv, self.nt = len(mesh.positions), len(mesh.indices)
        self.width, self.height = int(width), int(height)
        self.tex_h, self.tex_w = int(tex_size[0]), int(tex_size[1])
        self.mvp = np.ascontiguousarray(mvp, np.float32).reshape(-1, 16)
        self.eye = np.ascontiguousarray(eye, np.float32).reshape(-1, 3)
        self.n_views = len(self.mvp)
        self._pos = torch.from_numpy(np.ascontiguousarray(mesh.positions, np.float32)).to(dev)
        self._nrm = torch.from_numpy(np.ascontiguousarray(mesh.normals, np.float32)).to(dev)
        self._uv = torch.from_numpy(np.ascontiguousarray(mesh.texcoords, np.float32)).to(dev)
        self._idx = torch.from_numpy(np.ascontiguousarray(mesh.indices, np.int32)).to(dev)
        d = PFgradSceneDesc()
        d.positions, d.normals = self._pos.data_ptr(), self._nrm.data_ptr()
        d.texcoords, d.indices = self._uv.data_ptr(), self._idx.data_ptr()
        d.nVertices, d.nTriangles = self.nv, self.nt
        d.mvp, d.eye = self.mvp.ctypes.data, self.eye.ctypes.data
        d.nViews, d.width, d.height = self.n_views, self.width, self.height
        d.cullFace = cull
        d.texWidth, d.texHeight = self.tex_w, self.tex_h
        d.texFilter, d.texWrap = filter, wrap
        d.ambient = ambient
        d.background = (C.c_float * 3)(*background)
        d.clearDepth = clear_depth
        self.desc = d
        self.filter, self.wrap, self.cull, self.ambient = filter, wrap, cull, ambient
        self.background, self.clear_depth = tuple(background), clear_depth
        h = C.c_void_p()
        _check(self.lib.pfgradSceneCreate(C.byref(h), C.byref(d), self._stream()), "pfgradSceneCreate")
        self.handle = h

    @staticmethod
    def _stream():
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def info(self) -> dict:
        i = PFgradInfo()
        _check(self.lib.pfgradSceneInfo(self.handle, C.byref(i)), "pfgradSceneInfo")
        return {k: getattr(i, k) for k, _ in PFgradInfo._fields_}

    def close(self):
        if getattr(self, "handle", None):
            self.lib.pfgradSceneDestroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def image_shape(self):
        return (self.n_views, self.height, self.width, 3)

    def _params(self, tensors) -> PFgradParams:
        p = PFgradParams()
        for name, t in zip(PARAM_NAMES, tensors):
            if t.dtype != _torch().float32 or not t.is_cuda or not t.is_contiguous():
                raise ValueError(f"{name}: expected a contiguous float32 CUDA tensor")
            setattr(p, name, t.data_ptr())
        return p

    def forward_raw(self, tensors, image):
        p = self._params(tensors)
        _check(self.lib.pfgradForward(self.handle, C.byref(p), C.c_void_p(image.data_ptr()), self._stream()),
               "pfgradForward")

    def backward_raw(self, tensors, d_image, grads):
        p = self._params(tensors)
        g = PFgradGrads()
        for name, t in zip(PARAM_NAMES, grads):
            setattr(g, name, t.data_ptr())
        _check(self.lib.pfgradBackward(self.handle, C.byref(p), C.c_void_p(d_image.data_ptr()), C.byref(g),
                                       self._stream()), "pfgradBackward")

    def render(self, texture, colors, alphas, material, light):
        """Images of all views, (nViews, H, W, 3) float32, differentiable in
        every argument."""
        return _Render.apply(self, texture, colors, alphas, material, light)


def _torch():
    import torch
    return torch


def _make_fn():
    torch = _torch()

    class Render(torch.autograd.Function):
        @staticmethod
        def forward(ctx, scene, texture, colors, alphas, material, light):
            ts = tuple(t.detach().contiguous() for t in (texture, colors, alphas, material, light))
            img = torch.empty(scene.image_shape(), dtype=torch.float32, device=texture.device)
            scene.forward_raw(ts, img)
            ctx.scene = scene
            ctx.save_for_backward(*ts)
            return img

        @staticmethod
        def backward(ctx, d_image):
            ts = ctx.saved_tensors
            grads = [torch.empty_like(t) for t in ts]
            ctx.scene.backward_raw(ts, d_image.contiguous(), grads)
            return (None, *grads)

    return Render


class _Lazy:
    fn = None

    def apply(self, *args):
        if _Lazy.fn is None:
            _Lazy.fn = _make_fn()
        return _Lazy.fn.apply(*args)


_Render = _Lazy()
