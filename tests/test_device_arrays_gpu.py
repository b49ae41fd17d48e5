"""Zero-copy device arrays, indices and textures (pfVertexPointerDevice,
pfNormalPointerDevice, pfTexCoordPointerDevice, pfColorPointerDevice,
pfDrawElementsDevice, pfGenTextureDevice): the same draws with the data in
device memory render what the oracle renders from host arrays, bit-exact."""
import ctypes as C

import numpy as np
import pytest

from pixelforge_gb300 import abi as A
from pixelforge_gb300.scenes import Target, _ptr

pytestmark = pytest.mark.gpu

W, H = 320, 200


def _scene(seed=5, ntri=6000):
    r = np.random.default_rng(seed)
    nv = ntri * 3 // 2
    pos = (r.uniform(-1.4, 1.4, (nv, 3)) * np.float32([1, 1, 1.5])).astype(np.float32)
    nrm = r.normal(size=(nv, 3)).astype(np.float32)
    uv = r.uniform(-0.5, 1.5, (nv, 2)).astype(np.float32)
    col = r.integers(0, 256, (nv, 4)).astype(np.uint8)
    idx = r.integers(0, nv, ntri * 3).astype(np.uint32)
    tex = r.integers(0, 256, (64, 128, 4)).astype(np.uint8)
    return dict(pos=pos, nrm=nrm, uv=uv, col=col, idx=idx, tex=tex, nv=nv)


def _state(lib):
    lib.pfMatrixMode(A.PF_PROJECTION)
    lib.pfLoadIdentity()
    lib.pfFrustum(-0.1, 0.1, -0.0625, 0.0625, 0.1, 10.0)
    lib.pfMatrixMode(A.PF_MODELVIEW)
    lib.pfLoadIdentity()
    lib.pfTranslatef(0.0, 0.0, -2.5)
    lib.pfClearDepth(1e30)
    lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
    lib.pfDisable(A.PF_CULL_FACE)
    lib.pfEnable(A.PF_DEPTH_TEST)
    lib.pfEnable(A.PF_LIGHTING)
    lib.pfLightModel(A.PF_PHONG)
    lib.pfEnableLight(0)
    lib.pfLightfv(0, A.PF_POSITION, (C.c_float * 3)(2.0, 3.0, 4.0))
    lib.pfEnable(A.PF_VERTEX_ARRAY | A.PF_NORMAL_ARRAY | A.PF_TEXTURE_COORD_ARRAY | A.PF_COLOR_ARRAY)
    lib.pfEnable(A.PF_TEXTURE_2D)


def _run(lib, s, device=None):
    """Two draws (indexed triangles, then a blended strip of the first
    vertices); device: None (host arrays) or a dict of torch device tensors,
    optionally only some of them."""
    tg = Target(lib, W, H, "fbo")
    th = None
    try:
        _state(lib)
        d = device or {}
        if "tex" in d:
            th = lib.pfGenTextureDevice(C.c_void_p(d["tex"].data_ptr()), 128, 64)
        else:
            th = lib.pfGenTexture(_ptr(s["tex"]), 128, 64, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
        lib.pfBindTexture(th)
        dp = lambda k: C.c_void_p(d[k].data_ptr())
        if "pos" in d:
            lib.pfVertexPointerDevice(3, A.PF_FLOAT, 0, dp("pos"))
        else:
            lib.pfVertexPointer(3, A.PF_FLOAT, 0, _ptr(s["pos"]))
        if "nrm" in d:
            lib.pfNormalPointerDevice(A.PF_FLOAT, 0, dp("nrm"))
        else:
            lib.pfNormalPointer(A.PF_FLOAT, 0, _ptr(s["nrm"]))
        if "uv" in d:
            lib.pfTexCoordPointerDevice(A.PF_FLOAT, 0, dp("uv"))
        else:
            lib.pfTexCoordPointer(A.PF_FLOAT, 0, _ptr(s["uv"]))
        if "col" in d:
            lib.pfColorPointerDevice(4, A.PF_UNSIGNED_BYTE, 0, dp("col"))
        else:
            lib.pfColorPointer(4, A.PF_UNSIGNED_BYTE, 0, _ptr(s["col"]))
        n = len(s["idx"])
        if "idx" in d:
            lib.pfDrawElementsDevice(A.PF_TRIANGLES, n, s["nv"], dp("idx"))
        else:
            lib.pfDrawElements(A.PF_TRIANGLES, n, A.PF_UNSIGNED_INT, _ptr(s["idx"]))
        lib.pfEnable(A.PF_BLEND)
        lib.pfBlendFunc(A.PF_BLEND_ALPHA)
        lib.pfDrawArrays(A.PF_TRIANGLE_STRIP, 7, 900)
        err = lib.pfGetError()
        fr = tg.finish()
        if lib.has("pfGetDeviceStatus"):
            assert lib.pfGetDeviceStatus() == 0
        return fr, err
    finally:
        if th:
            h = C.c_void_p(th)
            lib.pfDeleteTexture(C.byref(h), False)
        tg.close()


def _device(s, keys):
    import torch
    dev = torch.device("cuda:0")
    return {k: torch.from_numpy(np.ascontiguousarray(s[k])).to(dev) for k in keys}


@pytest.mark.parametrize("keys", [("pos", "nrm", "uv", "col", "idx", "tex"), ("pos", "idx"), ("uv", "tex"),
                                  ("col", "nrm")])
def test_device_arrays_match_host_arrays(gpu, oracle, keys):
    """Every combination of device and host arrays draws the oracle's image
    (Phong-lit, textured, depth-tested, then an alpha-blended strip)."""
    s = _scene()
    d = _device(s, keys)
    got, e1 = _run(gpu, s, d)
    ref, e2 = _run(oracle, s)
    assert e1 == e2 == A.PF_NO_ERROR
    assert (ref.depth < 1e30).sum() > 20000
    assert np.array_equal(got.depth.view(np.uint32), ref.depth.view(np.uint32)), "depth differs"
    nd = int((got.color != ref.color).any(-1).sum())
    assert nd == 0, f"{keys}: {nd} pixels differ"
    assert got.stats["fragments"] == ref.stats["fragments"]


def test_device_arrays_read_at_the_flush(gpu, oracle):
    """Device memory is read when the frame renders: positions changed on
    the device after the draw call and before pfFinish are the ones drawn
    (the host arrays of the same draw were copied at the call)."""
    import torch
    s = _scene(seed=6)
    d = _device(s, ("pos",))
    t = s.copy()
    t["pos"] = (s["pos"] * np.float32([0.7, 0.7, 1.0])).astype(np.float32)
    tg = Target(gpu, W, H, "fbo")
    th = None
    try:
        _state(gpu)
        th = gpu.pfGenTexture(_ptr(s["tex"]), 128, 64, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
        gpu.pfBindTexture(th)
        gpu.pfVertexPointerDevice(3, A.PF_FLOAT, 0, C.c_void_p(d["pos"].data_ptr()))
        gpu.pfNormalPointer(A.PF_FLOAT, 0, _ptr(s["nrm"]))
        gpu.pfTexCoordPointer(A.PF_FLOAT, 0, _ptr(s["uv"]))
        gpu.pfColorPointer(4, A.PF_UNSIGNED_BYTE, 0, _ptr(s["col"]))
        gpu.pfDrawElements(A.PF_TRIANGLES, len(s["idx"]), A.PF_UNSIGNED_INT, _ptr(s["idx"]))
        gpu.pfEnable(A.PF_BLEND)
        gpu.pfBlendFunc(A.PF_BLEND_ALPHA)
        gpu.pfDrawArrays(A.PF_TRIANGLE_STRIP, 7, 900)
        d["pos"].copy_(torch.from_numpy(t["pos"]).to(d["pos"].device))     # before the frame renders
        torch.cuda.synchronize()
        got = tg.finish()
    finally:
        if th:
            h = C.c_void_p(th)
            gpu.pfDeleteTexture(C.byref(h), False)
        tg.close()
    ref, _ = _run(oracle, t)
    assert np.array_equal(got.depth.view(np.uint32), ref.depth.view(np.uint32))
    assert np.array_equal(got.color, ref.color)


def test_device_indices_past_vertex_count(gpu, oracle):
    """Indices at or past pfDrawElementsDevice's vertexCount are clamped to
    vertexCount - 1 and flagged in the device status; the image is the one
    host indices clamped the same way draw."""
    s = _scene(seed=7)
    nv = s["nv"]
    lim = nv - 200
    d = _device(s, ("idx",))
    tg = Target(gpu, W, H, "fbo")
    try:
        _state(gpu)
        gpu.pfDisable(A.PF_TEXTURE_2D)
        gpu.pfVertexPointer(3, A.PF_FLOAT, 0, _ptr(s["pos"]))
        gpu.pfNormalPointer(A.PF_FLOAT, 0, _ptr(s["nrm"]))
        gpu.pfTexCoordPointer(A.PF_FLOAT, 0, _ptr(s["uv"]))
        gpu.pfColorPointer(4, A.PF_UNSIGNED_BYTE, 0, _ptr(s["col"]))
        gpu.pfDrawElementsDevice(A.PF_TRIANGLES, len(s["idx"]), lim, C.c_void_p(d["idx"].data_ptr()))
        got = tg.finish()
        assert gpu.pfGetDeviceStatus() & A.PF_DEVICE_INDEX_RANGE
    finally:
        tg.close()
    clamped = np.minimum(s["idx"], np.uint32(lim - 1))
    tg = Target(oracle, W, H, "fbo")
    try:
        _state(oracle)
        oracle.pfDisable(A.PF_TEXTURE_2D)
        oracle.pfVertexPointer(3, A.PF_FLOAT, 0, _ptr(s["pos"]))
        oracle.pfNormalPointer(A.PF_FLOAT, 0, _ptr(s["nrm"]))
        oracle.pfTexCoordPointer(A.PF_FLOAT, 0, _ptr(s["uv"]))
        oracle.pfColorPointer(4, A.PF_UNSIGNED_BYTE, 0, _ptr(s["col"]))
        oracle.pfDrawElements(A.PF_TRIANGLES, len(clamped), A.PF_UNSIGNED_INT, _ptr(clamped))
        ref = tg.finish()
    finally:
        tg.close()
    assert np.array_equal(got.depth.view(np.uint32), ref.depth.view(np.uint32))
    assert np.array_equal(got.color, ref.color)


def test_device_arrays_refusals(gpu):
    """Host pointers, other types and host-assembled modes are refused."""
    import torch
    s = _scene(seed=8, ntri=30)
    d = _device(s, ("pos", "idx"))
    tg = Target(gpu, 16, 16, "fbo")
    try:
        gpu.pfVertexPointerDevice(3, A.PF_FLOAT, 0, _ptr(s["pos"]))              # host memory
        assert gpu.pfGetError() == A.PF_INVALID_VALUE
        gpu.pfVertexPointerDevice(3, A.PF_DOUBLE, 0, C.c_void_p(d["pos"].data_ptr()))
        assert gpu.pfGetError() == A.PF_INVALID_ENUM
        gpu.pfEnable(A.PF_VERTEX_ARRAY)
        gpu.pfVertexPointerDevice(3, A.PF_FLOAT, 0, C.c_void_p(d["pos"].data_ptr()))
        assert gpu.pfGetError() == A.PF_NO_ERROR
        gpu.pfDrawArrays(A.PF_LINES, 0, 10)                                       # assembled on the host
        assert gpu.pfGetError() == A.PF_INVALID_OPERATION
        gpu.pfDrawElementsDevice(A.PF_TRIANGLES, 30, 0, C.c_void_p(d["idx"].data_ptr()))
        assert gpu.pfGetError() == A.PF_INVALID_VALUE
        assert not gpu.pfGenTextureDevice(_ptr(s["tex"]), 128, 64)
        assert gpu.pfGetError() == A.PF_INVALID_VALUE
        tg.finish()
        torch.cuda.synchronize()
    finally:
        tg.close()


def test_sphere_device_arrays_equal_host_arrays(gpu):
    """The 1080p sphere frame from device memory (zero-copy) and from host
    arrays: the same image and depth, bit for bit."""
    from pixelforge_gb300.scenes import SphereScene
    a = SphereScene(device_arrays=True).render(gpu)
    b = SphereScene().render(gpu)
    assert np.array_equal(a.color, b.color)
    assert np.array_equal(a.depth.view(np.uint32), b.depth.view(np.uint32))
    assert a.stats["fragments"] == b.stats["fragments"] > 500000
