"""pfgbDrawTrianglesStatic: the allocation-free entry point.

It is meant for callers that cannot allocate device memory (inside another
component's stream capture, on a real-time frame path, or in a host that
lends out pre-allocated buffers).  This test calls it through the C ABI on
device buffers the test owns and checks, for two calls in a row on the same
scratch, that its pixels equal what the pf* API renders for the same
triangles, state and starting framebuffer: depth bit-exact, colour within
the 1 LSB the other parity tests allow.  The file is named so that pytest
collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from pixelforge_gb300 import abi as A
from pixelforge_gb300.scenes import Target, _ptr

pytestmark = pytest.mark.gpu

COLOR_TOL = 1


def _frustum(l, r, b, t, n, f):
    m = np.zeros(16, np.float32)
    m[0] = (n * 2) / (r - l); m[5] = (n * 2) / (t - b)
    m[8] = (r + l) / (r - l); m[9] = (t + b) / (t - b)
    m[10] = -(f + n) / (f - n); m[11] = -1.0; m[14] = -(f * n * 2) / (f - n)
    return m


def _translate_z(m, dz):
    # pfTranslatef then pfFrustum on PROJECTION: translation @ frustum, row-vector layout
    t = np.eye(4, dtype=np.float32)
    t[3, 2] = dz
    return (t @ m.reshape(4, 4)).astype(np.float32).ravel()


def _soup(seed, ntris):
    # small triangles (about 0.15 across in normalised units) scattered over
    # and past the viewport, so that no 16x16 tile needs more bin entries
    # than PFGB_STATIC_BIN_CAPACITY
    r = np.random.default_rng(seed)
    centre = r.uniform(-1.2, 1.2, (ntris, 1, 3))
    pos = (centre + r.uniform(-0.08, 0.08, (ntris, 3, 3))).reshape(-1, 3).astype(np.float32)
    pos[:, 2] = r.uniform(-0.9, 0.9, ntris * 3)
    col = r.integers(0, 256, (ntris * 3, 4), dtype=np.uint8)
    return pos, col


CASES = [
    # seed, ntris, W, H, mvp kind, depthFunc, cullMode, clear colour, clear depth
    (11, 1500, 256, 192, "ortho", A.PF_LESS, 1, (9, 8, 7, 255), 1.0),
    (12, 4000, 320, 200, "frustum", A.PF_GEQUAL, 0, (0, 40, 80, 255), -1e30),
]


def _mvp(kind):
    if kind == "ortho":   # the context's default projection, ortho(-1, 1, -1, 1, -1, 1)
        m = np.zeros(16, np.float32)
        m[0] = m[5] = 1.0; m[10] = -1.0; m[15] = 1.0
        return m
    return _translate_z(_frustum(-0.06, 0.06, -0.045, 0.045, 0.1, 10.0), -2.0)


def _render_api(lib, pos, col, mvp, W, H, depth_func, cull, cc, cd):
    tg = Target(lib, W, H, "fbo")
    try:
        lib.pfClearFramebuffer(tg._fbref, A.PFcolor(*cc), cd)
        lib.pfMatrixMode(A.PF_PROJECTION)
        lib.pfLoadIdentity()
        lib.pfMultMatrixf(mvp.ctypes.data_as(C.POINTER(C.c_float)))
        lib.pfMatrixMode(A.PF_MODELVIEW)
        lib.pfLoadIdentity()
        if depth_func < 0:
            lib.pfDisable(A.PF_DEPTH_TEST)
        else:
            lib.pfEnable(A.PF_DEPTH_TEST)
            lib.pfDepthFunc(depth_func)
        if cull == 0:
            lib.pfDisable(A.PF_CULL_FACE)
        else:
            lib.pfEnable(A.PF_CULL_FACE)
            lib.pfCullFace(A.PF_BACK if cull == 1 else A.PF_FRONT)
        lib.pfBegin(A.PF_TRIANGLES)
        for i in range(len(pos)):
            c = col[i]
            lib.pfColor4ub(int(c[0]), int(c[1]), int(c[2]), int(c[3]))
            lib.pfVertex3f(float(pos[i, 0]), float(pos[i, 1]), float(pos[i, 2]))
        lib.pfEnd()
        return tg.finish()
    finally:
        tg.close()


def test_static_entry_matches_api_twice():
    torch = pytest.importorskip("torch")
    from pixelforge_gb300 import load_library
    lib = load_library()
    fn = lib.raw("pfgbDrawTrianglesStatic")
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_void_p]
    dev = torch.device("cuda:0")
    for seed, ntris, W, H, kind, depth_func, cull, cc, cd in CASES:
        pos, col = _soup(seed, ntris)
        mvp = _mvp(kind)
        ref = _render_api(lib, pos, col, mvp, W, H, depth_func, cull, cc, cd)
        assert lib.pfGetDeviceStatus() == 0

        d_pos = torch.from_numpy(pos.ravel().copy()).to(dev)
        d_col = torch.from_numpy(col.view(np.int32).ravel().copy()).to(dev)
        packed = int(np.array(cc, np.uint8).view(np.int32)[0])
        d_color = torch.full((H * W,), packed, dtype=torch.int32, device=dev)
        d_depth = torch.full((H * W,), cd, dtype=torch.float32, device=dev)
        stream = torch.cuda.current_stream(dev)
        rc = fn(d_pos.data_ptr(), d_col.data_ptr(), ntris, _ptr(mvp), d_color.data_ptr(), d_depth.data_ptr(),
                W, H, depth_func, cull, stream.cuda_stream)
        assert rc == 0, f"pfgbDrawTrianglesStatic returned {rc}"
        torch.cuda.synchronize()
        got_color = d_color.cpu().numpy().view(np.uint8).reshape(H, W, 4)
        got_depth = d_depth.cpu().numpy().reshape(H, W)
        assert np.array_equal(got_depth.view(np.uint32), ref.depth.view(np.uint32)), f"depth differs (seed {seed})"
        diff = np.abs(got_color.astype(np.int32) - ref.color.astype(np.int32))
        assert int(diff.max()) <= COLOR_TOL, f"colour differs by {int(diff.max())} (seed {seed})"
        assert ref.stats["fragments"] > 0


def test_static_entry_rejects_oversize():
    from pixelforge_gb300 import load_library
    lib = load_library()
    fn = lib.raw("pfgbDrawTrianglesStatic")
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_void_p]
    assert fn(None, None, 8193, None, None, None, 64, 64, 2, 1, None) == -1
    assert fn(None, None, 10, None, None, None, 513, 64, 2, 1, None) == -1
