"""ctypes wrapper of the FP64 differentiable-path oracle (oracle/pfgrad_ref.c).

TEST INFRASTRUCTURE ONLY: used by tests/ to check the GPU forward images and
gradients against an FP64 restatement and against FP64 central finite
differences.  Builds oracle/_build/libpfgrad.so with make on first use.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libpfgrad.so"

_dll = None


def _lib():
    global _dll
    if _dll is None:
        subprocess.run(["make", "-s", "-C", str(HERE), "pfgrad"], check=True)
        d = C.CDLL(str(LIB))
        fp, ip = C.POINTER(C.c_float), C.POINTER(C.c_int)
        d.pgref_create.restype = C.c_void_p
        d.pgref_create.argtypes = [fp, fp, fp, C.POINTER(C.c_uint32), C.c_int, C.c_int, fp, fp, C.c_int, C.c_int,
                                   C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, fp, C.c_float, ip]
        d.pgref_destroy.argtypes = [C.c_void_p]
        d.pgref_fragments.restype = C.c_int64
        d.pgref_fragments.argtypes = [C.c_void_p]
        d.pgref_fragment_counts.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        d.pgref_depth.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
        dp = C.POINTER(C.c_double)
        d.pgref_forward.restype = C.c_double
        d.pgref_forward.argtypes = [C.c_void_p, dp, fp, C.c_double, dp]
        d.pgref_loss_local.restype = C.c_double
        d.pgref_loss_local.argtypes = [C.c_void_p, dp, fp, C.c_double, C.c_int64]
        d.pgref_backward.restype = C.c_int
        d.pgref_backward.argtypes = [C.c_void_p, dp, fp, C.c_double, dp]
        _dll = d
    return _dll


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


PARAM_NAMES = ("texture", "colors", "alphas", "material", "light")


class RefScene:
    """FP64 oracle of one pfgrad scene (same arguments as GradScene)."""

    def __init__(self, mesh, mvp, eye, width, height, tex_size, filter=1, wrap=0, cull=1, ambient=0.2,
                 background=(0.0, 0.0, 0.0), clear_depth=float(np.finfo(np.float32).max)):
        d = _lib()
        self.pos = np.ascontiguousarray(mesh.positions, np.float32)
        self.nrm = np.ascontiguousarray(mesh.normals, np.float32)
        self.uv = np.ascontiguousarray(mesh.texcoords, np.float32)
        self.idx = np.ascontiguousarray(mesh.indices, np.uint32)
        self.mvp = np.ascontiguousarray(mvp, np.float32).reshape(-1, 16)
        self.eye = np.ascontiguousarray(eye, np.float32).reshape(-1, 3)
        self.nv, self.n_views = len(self.pos), len(self.mvp)
        self.width, self.height = int(width), int(height)
        self.tex_h, self.tex_w = int(tex_size[0]), int(tex_size[1])
        bg = np.asarray(background, np.float32)
        st = C.c_int(0)
        self.h = d.pgref_create(_fp(self.pos), _fp(self.nrm), _fp(self.uv),
                                self.idx.ctypes.data_as(C.POINTER(C.c_uint32)), self.nv, len(self.idx),
                                _fp(self.mvp), _fp(self.eye), self.n_views, self.width, self.height, cull,
                                self.tex_w, self.tex_h, filter, wrap, ambient, _fp(bg), clear_depth, C.byref(st))
        if not self.h:
            raise RuntimeError(f"pgref_create failed ({st.value})")

    def close(self):
        if self.h:
            _lib().pgref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_params(self) -> int:
        return self.tex_h * self.tex_w * 4 + 4 * self.nv + 6

    def pack(self, params: dict) -> np.ndarray:
        return np.concatenate([np.asarray(params[k], np.float64).ravel() for k in PARAM_NAMES])

    def unpack(self, vec: np.ndarray) -> dict:
        sizes = [self.tex_h * self.tex_w * 4, 3 * self.nv, self.nv, 3, 3]
        shapes = [(self.tex_h, self.tex_w, 4), (self.nv, 3), (self.nv,), (3,), (3,)]
        out, o = {}, 0
        for k, n, s in zip(PARAM_NAMES, sizes, shapes):
            out[k] = vec[o:o + n].reshape(s)
            o += n
        return out

    def fragments(self) -> int:
        return int(_lib().pgref_fragments(self.h))

    def fragment_counts(self) -> np.ndarray:
        out = np.zeros((self.n_views, self.height, self.width), np.int32)
        _lib().pgref_fragment_counts(self.h, out.ctypes.data_as(C.POINTER(C.c_int32)))
        return out

    def depth(self) -> np.ndarray:
        """Final depth buffer of every view (nViews, H, W)."""
        out = np.zeros((self.n_views, self.height, self.width), np.float32)
        _lib().pgref_depth(self.h, _fp(out))
        return out

    def forward(self, vec: np.ndarray, target: np.ndarray = None, scale: float = 1.0):
        """(loss, image) -- image (nViews, H, W, 3) float64."""
        img = np.zeros((self.n_views, self.height, self.width, 3), np.float64)
        tgt = np.zeros_like(img, dtype=np.float32) if target is None else np.ascontiguousarray(target, np.float32)
        vec = np.ascontiguousarray(vec, np.float64)
        loss = _lib().pgref_forward(self.h, _dp(vec), _fp(tgt), scale, _dp(img))
        return loss, img

    def gradient(self, vec: np.ndarray, target: np.ndarray, scale: float) -> np.ndarray:
        vec = np.ascontiguousarray(vec, np.float64)
        tgt = np.ascontiguousarray(target, np.float32)
        g = np.zeros(self.n_params, np.float64)
        rc = _lib().pgref_backward(self.h, _dp(vec), _fp(tgt), scale, _dp(g))
        if rc != 0:
            raise RuntimeError("pgref_backward failed")
        return g

    def central_difference(self, vec: np.ndarray, target: np.ndarray, scale: float, q: int,
                           h: float = 1e-4) -> float:
        """FP64 central difference of the loss in parameter q, over the
        pixels that depend on q."""
        tgt = np.ascontiguousarray(target, np.float32)
        v = np.array(vec, np.float64)
        v[q] += h
        lp = _lib().pgref_loss_local(self.h, _dp(v), _fp(tgt), scale, q)
        v[q] -= 2 * h
        lm = _lib().pgref_loss_local(self.h, _dp(v), _fp(tgt), scale, q)
        return (lp - lm) / (2 * h)
