"""The FP64 oracle of the differentiable path, on the CPU.

1. Its adjoint equals FP64 central finite differences of its own forward,
   for every kind of parameter, nearest and bilinear sampling, with and
   without face culling.  The step is 1e-5: the loss is a polynomial of
   degree up to six in a texel shared by two fragments of a pixel, and the
   O(h^2) truncation of h = 1e-4 reaches 2e-5 relative there.
2. Its visibility -- the depth buffer left by the visible fragments -- is
   bit-exact against the pipeline oracle (pfref, itself pinned to the
   reference build) and, where it can be built, the reference itself, each
   rendering the same mesh and views through the pf* API.
"""
import ctypes as C

import numpy as np
import pytest

from pixelforge_gb300 import abi as A
from pixelforge_gb300.fit import FitScene
from pixelforge_gb300.scenes import Target

pgref = pytest.importorskip("pgref")


def small_scene(subdiv=2, views=4, size=64, tex=32):
    return FitScene(subdiv=subdiv, n_views=views, size=size, tex_size=tex)


def random_params(rs, seed):
    rng = np.random.default_rng(seed)
    return {"texture": rng.uniform(0.2, 0.9, (rs.tex_h, rs.tex_w, 4)),
            "colors": rng.uniform(0.2, 0.9, (rs.nv, 3)),
            "alphas": rng.uniform(0.6, 1.0, rs.nv),
            "material": np.array([0.7, 0.4, 20.0]),
            "light": np.array([0.3, 0.8, 0.5])}


@pytest.mark.parametrize("filt,cull", [(0, 1), (1, 1), (1, -1), (0, -1)])
def test_oracle_adjoint_matches_finite_differences(filt, cull):
    fs = small_scene()
    mvp, eyes = fs.cameras()
    rs = pgref.RefScene(fs.mesh(), mvp, eyes, fs.size, fs.size, (fs.tex_size,) * 2, filter=filt, cull=cull)
    _, tgt = rs.forward(rs.pack(random_params(rs, 1)))
    vec = rs.pack(random_params(rs, 2))
    scale = 1.0 / tgt.size
    g = rs.gradient(vec, tgt.astype(np.float32), scale)
    rng = np.random.default_rng(3)
    nz = np.nonzero(g)[0]
    n_tex = rs.tex_h * rs.tex_w * 4
    tex_q = rng.choice(nz[nz < n_tex], 24, replace=False)
    vtx_q = rng.choice(nz[(nz >= n_tex) & (nz < rs.n_params - 6)], 24, replace=False)
    glob_q = np.arange(rs.n_params - 6, rs.n_params)
    for q in np.concatenate([tex_q, vtx_q, glob_q]):
        fd = rs.central_difference(vec, tgt.astype(np.float32), scale, int(q), h=1e-5)
        assert abs(fd - g[q]) <= 1e-5 * max(abs(fd), 1e-9), f"param {q}: adjoint {g[q]} vs FD {fd}"


def render_depth(lib, mesh, mvp, size, cull):
    tg = Target(lib, size, size, "fbo")
    try:
        lib.pfEnable(A.PF_DEPTH_TEST)
        if cull < 0:
            lib.pfDisable(A.PF_CULL_FACE)
        lib.pfMatrixMode(A.PF_PROJECTION)
        lib.pfLoadIdentity()
        lib.pfMultMatrixf(np.ascontiguousarray(mvp, np.float32).ctypes.data_as(C.POINTER(C.c_float)))
        lib.pfMatrixMode(A.PF_MODELVIEW)
        lib.pfLoadIdentity()
        lib.pfEnable(A.PF_VERTEX_ARRAY)
        pos = np.ascontiguousarray(mesh.positions, np.float32)
        idx = np.ascontiguousarray(mesh.indices, np.uint32)
        lib.pfVertexPointer(3, A.PF_FLOAT, 0, pos.ctypes.data_as(C.c_void_p))
        lib.pfDrawElements(A.PF_TRIANGLES, idx.size, A.PF_UNSIGNED_INT, idx.ctypes.data_as(C.c_void_p))
        return tg.finish().depth
    finally:
        tg.close()


@pytest.mark.parametrize("cull", [1, -1])
def test_oracle_visibility_pinned(oracle, cull):
    fs = small_scene(subdiv=3, views=5, size=96)
    mvp, eyes = fs.cameras()
    mesh = fs.mesh()
    rs = pgref.RefScene(mesh, mvp, eyes, fs.size, fs.size, (32, 32), cull=cull)
    dref = rs.depth()
    assert (dref < 1e30).sum() > 5 * 2000
    for v in range(len(mvp)):
        d = render_depth(oracle, mesh, mvp[v], fs.size, cull)
        assert np.array_equal(d.view(np.uint32), dref[v].view(np.uint32)), f"view {v}"


def test_oracle_visibility_vs_reference(ref_shim):
    fs = small_scene(subdiv=3, views=3, size=96)
    mvp, eyes = fs.cameras()
    mesh = fs.mesh()
    rs = pgref.RefScene(mesh, mvp, eyes, fs.size, fs.size, (32, 32), cull=1)
    dref = rs.depth()
    for v in range(len(mvp)):
        d = render_depth(ref_shim, mesh, mvp[v], fs.size, 1)
        assert np.array_equal(d.view(np.uint32), dref[v].view(np.uint32)), f"view {v}"


def test_oracle_rejects_clipping():
    fs = small_scene()
    mvp, eyes = fs.cameras()
    fs.radius = 0.5                  # cameras inside the sphere: triangles cross the near plane
    mvp2, eyes2 = fs.cameras()
    with pytest.raises(RuntimeError, match=r"\(5\)"):
        pgref.RefScene(fs.mesh(), mvp2, eyes2, 64, 64, (32, 32))
