"""pfgbDrawTrianglesStatic: the allocation-free entry point.

Some callers cannot allocate device memory: a real-time frame path, where a
cudaMalloc may block and synchronise the whole device, or an engine that only
lends out buffers from its own pool.  This entry point renders into device
colour and depth buffers the caller owns and keeps its intermediates in one
fixed-size static device array.

The tests call it through the C ABI on device buffers the test owns, several
calls in a row on the same shared scratch, and check each call's pixels
against what the library's pf* API renders for the same triangles, state and
starting framebuffer, and against the CPU oracle: depth bit-exact, colour
within the 1 LSB the other parity tests allow.  The cases cover every cull
mode (culling off sets up each triangle twice, 16,384 face items at the
8,192-triangle limit), no depth test, triangles that cross the near and side
clip planes, the capacity error (the buffers stay untouched) and the invalid
arguments.  The file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from pixelforge_gb300 import abi as A
from pixelforge_gb300.scenes import Target, _ptr

pytestmark = pytest.mark.gpu

COLOR_TOL = 1
MAX_TRIS = 8192
E_INVALID, E_CAPACITY = -2, -4


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


def _mvp(kind):
    if kind == "ortho":   # the context's default projection, ortho(-1, 1, -1, 1, -1, 1)
        m = np.zeros(16, np.float32)
        m[0] = m[5] = 1.0; m[10] = -1.0; m[15] = 1.0
        return m
    return _translate_z(_frustum(-0.06, 0.06, -0.045, 0.045, 0.1, 10.0), -2.0)


def _soup(seed, ntris, near_share=0.0):
    """Small triangles (about 0.15 across) scattered over and past the
    viewport; a share of them gets one vertex behind the camera of the
    frustum view (object z > 2 is eye z > 0), so they cross the w and near
    planes as well as the side planes."""
    r = np.random.default_rng(seed)
    centre = r.uniform(-1.2, 1.2, (ntris, 1, 3))
    pos = (centre + r.uniform(-0.08, 0.08, (ntris, 3, 3))).astype(np.float32)
    pos[:, :, 2] = r.uniform(-0.9, 0.9, (ntris, 3))
    cross = r.random(ntris) < near_share
    pos[cross, 0, 2] = r.uniform(2.05, 2.6, int(cross.sum()))
    col = r.integers(0, 256, (ntris * 3, 4), dtype=np.uint8)
    return pos.reshape(-1, 3), col


def _one_tile_pile(seed, ntris):
    """Triangles inside the first 16x16 pixels of the ortho view (more of
    them in each 8x8 tile than a tile bin holds)."""
    r = np.random.default_rng(seed)
    # in a 64x48 ortho view these land on pixels 0..14 of x and 0..14 of y
    x = r.uniform(-1.0, -0.55, (ntris, 3))
    y = r.uniform(0.4, 1.0, (ntris, 3))
    z = r.uniform(-0.5, 0.5, (ntris, 3))
    pos = np.stack([x, y, z], -1).astype(np.float32).reshape(-1, 3)
    col = r.integers(0, 256, (ntris * 3, 4), dtype=np.uint8)
    return pos, col


CASES = [
    # seed, ntris, W, H, mvp kind, depthFunc, cullMode, clear colour, clear depth, near share
    (11, 1500, 256, 192, "ortho", A.PF_LESS, 1, (9, 8, 7, 255), 1.0, 0.0),
    (12, 4000, 320, 200, "frustum", A.PF_GEQUAL, 0, (0, 40, 80, 255), -1e30, 0.0),
    (13, MAX_TRIS, 320, 200, "frustum", A.PF_LESS, 0, (20, 30, 40, 255), 1e30, 0.03),
    (14, 3000, 512, 512, "frustum", A.PF_LEQUAL, 2, (1, 2, 3, 4), 1e30, 0.02),
    (15, 2500, 200, 130, "ortho", -1, 1, (200, 100, 50, 255), 1.0, 0.0),
]


def _static_fn(lib):
    fn = lib.raw("pfgbDrawTrianglesStatic")
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_void_p]
    return fn


def _render_api(lib, pos, col, mvp, W, H, depth_func, cull, cc, cd):
    """The same draw through the pf* API (library or oracle)."""
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


class _Device:
    def __init__(self, torch, lib):
        self.torch, self.fn = torch, _static_fn(lib)
        self.dev = torch.device("cuda:0")

    def buffers(self, W, H, cc, cd):
        packed = int(np.array(cc, np.uint8).view(np.int32)[0])
        color = self.torch.full((H * W,), packed, dtype=self.torch.int32, device=self.dev)
        depth = self.torch.full((H * W,), cd, dtype=self.torch.float32, device=self.dev)
        return color, depth

    def draw(self, pos, col, mvp, color, depth, W, H, depth_func, cull):
        t = self.torch
        d_pos = t.from_numpy(pos.ravel().copy()).to(self.dev)
        d_col = t.from_numpy(col.view(np.int32).ravel().copy()).to(self.dev)
        stream = t.cuda.current_stream(self.dev)
        rc = self.fn(d_pos.data_ptr(), d_col.data_ptr(), len(pos) // 3, _ptr(mvp), color.data_ptr(),
                     depth.data_ptr(), W, H, depth_func, cull, stream.cuda_stream)
        t.cuda.synchronize()
        return rc

    @staticmethod
    def read(color, depth, W, H):
        return (color.cpu().numpy().view(np.uint8).reshape(H, W, 4).copy(),
                depth.cpu().numpy().reshape(H, W).copy())


def _compare(got_color, got_depth, ref, label):
    assert np.array_equal(got_depth.view(np.uint32), ref.depth.view(np.uint32)), f"{label}: depth differs"
    diff = np.abs(got_color.astype(np.int32) - ref.color.astype(np.int32))
    assert int(diff.max()) <= COLOR_TOL, f"{label}: colour differs by {int(diff.max())}"


def test_static_entry_matches_api_and_oracle(gpu, oracle):
    torch = pytest.importorskip("torch")
    d = _Device(torch, gpu)
    for seed, ntris, W, H, kind, depth_func, cull, cc, cd, near in CASES:
        pos, col = _soup(seed, ntris, near)
        mvp = _mvp(kind)
        api = _render_api(gpu, pos, col, mvp, W, H, depth_func, cull, cc, cd)
        assert gpu.pfGetDeviceStatus() == 0
        orc = _render_api(oracle, pos, col, mvp, W, H, depth_func, cull, cc, cd)
        assert api.stats["fragments"] > 0
        # consecutive calls on the shared scratch: each one must start from
        # a clean state (bin counters, device counters)
        for call in range(2):
            color, depth = d.buffers(W, H, cc, cd)
            rc = d.draw(pos, col, mvp, color, depth, W, H, depth_func, cull)
            assert rc == 0, f"seed {seed} call {call}: pfgbDrawTrianglesStatic returned {rc}"
            got_color, got_depth = d.read(color, depth, W, H)
            _compare(got_color, got_depth, api, f"seed {seed} call {call} vs pf* API")
            _compare(got_color, got_depth, orc, f"seed {seed} call {call} vs oracle")


def test_static_entry_capacity_leaves_buffers(gpu):
    """More sub-triangles in one tile than a bin holds: -4, and neither
    buffer is written; the next call works again."""
    torch = pytest.importorskip("torch")
    d = _Device(torch, gpu)
    W, H, cc, cd = 64, 48, (5, 6, 7, 255), 1.0
    pos, col = _one_tile_pile(21, 2600)
    color, depth = d.buffers(W, H, cc, cd)
    before = d.read(color, depth, W, H)
    rc = d.draw(pos, col, _mvp("ortho"), color, depth, W, H, A.PF_LESS, 0)
    assert rc == E_CAPACITY
    after = d.read(color, depth, W, H)
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1].view(np.uint32), after[1].view(np.uint32))
    # the same scratch right after the failed call
    pos, col = _soup(22, 800)
    mvp = _mvp("ortho")
    ref = _render_api(gpu, pos, col, mvp, W, H, A.PF_LESS, 1, cc, cd)
    color, depth = d.buffers(W, H, cc, cd)
    assert d.draw(pos, col, mvp, color, depth, W, H, A.PF_LESS, 1) == 0
    _compare(*d.read(color, depth, W, H), ref, "after the capacity error")


def test_static_entry_rejects_bad_arguments(gpu):
    fn = _static_fn(gpu)
    dummy = C.c_void_p(16)
    assert fn(None, None, MAX_TRIS + 1, None, None, None, 64, 64, 2, 1, None) == -1
    assert fn(None, None, 10, None, None, None, 513, 64, 2, 1, None) == -1
    assert fn(None, None, 10, None, None, None, 64, 0, 2, 1, None) == -1
    assert fn(dummy, dummy, 10, None, dummy, dummy, 64, 64, 2, 1, None) == E_INVALID     # no MVP
    assert fn(dummy, dummy, 10, dummy, dummy, None, 64, 64, 2, 1, None) == E_INVALID     # no depth
    assert fn(dummy, dummy, 10, dummy, dummy, dummy, 64, 64, 6, 1, None) == E_INVALID    # depth function
    assert fn(dummy, dummy, 10, dummy, dummy, dummy, 64, 64, -2, 1, None) == E_INVALID
    assert fn(dummy, dummy, 10, dummy, dummy, dummy, 64, 64, 2, 3, None) == E_INVALID    # cull mode
