"""Differentiable path on the GPU (pfgrad* through the C ABI) against the FP64
oracle (oracle/pfgrad_ref.c) and FP64 central finite differences.

Bars: forward images within 2e-5 absolute of the FP64 image (values in
[0, 1]; coverage and depth outcomes are the reference's, so any visibility
difference would show as an error of order 0.1); gradients within 1e-3
relative of FP64 central differences (h = 1e-4) on 256 seeded parameters of
the full 64-view fitting workload, and within 1e-4 (norm-wise per parameter
group) of the FP64 adjoint.
"""
import numpy as np
import pytest

from pixelforge_gb300.fit import FitScene, to_device
from pixelforge_gb300.grad import PARAM_NAMES

pgref = pytest.importorskip("pgref")
torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

GROUPS = ("texture", "colors", "alphas", "material", "light")


def scenes(fs, filt=None, cull=1):
    mvp, eyes = fs.cameras()
    f = fs.filter if filt is None else filt
    from pixelforge_gb300.grad import GradScene
    gs = GradScene(fs.mesh(), mvp, eyes, fs.size, fs.size, (fs.tex_size,) * 2, filter=f, wrap=fs.wrap,
                   cull=cull, ambient=fs.ambient)
    rs = pgref.RefScene(fs.mesh(), mvp, eyes, fs.size, fs.size, (fs.tex_size,) * 2, filter=f, wrap=fs.wrap,
                        cull=cull, ambient=fs.ambient)
    return gs, rs


def gpu_grad(gs, params: dict, target):
    ts = to_device(params)
    img = gs.render(*ts)
    loss = ((img - target) ** 2).mean()
    loss.backward()
    torch.cuda.synchronize()
    return img.detach(), {k: t.grad.detach().cpu().numpy().astype(np.float64) for k, t in zip(PARAM_NAMES, ts)}


def small_params(fs, seed):
    t = fs.truth()
    rng = np.random.default_rng(seed)
    t["texture"] = rng.uniform(0.2, 0.9, t["texture"].shape).astype(np.float32)
    t["colors"] = rng.uniform(0.2, 0.9, t["colors"].shape).astype(np.float32)
    return t


@pytest.mark.parametrize("filt,cull", [(1, 1), (0, 1), (1, -1)])
def test_forward_and_adjoint_vs_fp64(filt, cull):
    fs = FitScene(subdiv=3, n_views=6, size=128, tex_size=64)
    gs, rs = scenes(fs, filt, cull)
    try:
        truth, init = fs.truth(), small_params(fs, 7)
        with torch.no_grad():
            target = gs.render(*to_device(truth, requires_grad=False))
        _, ref_img = rs.forward(rs.pack(truth))
        assert np.abs(target.cpu().numpy() - ref_img).max() <= 2e-5
        img, g = gpu_grad(gs, init, target)
        scale = 1.0 / target.numel()
        gref = rs.unpack(rs.gradient(rs.pack(init), target.cpu().numpy(), scale))
        for k in GROUPS:
            err = np.linalg.norm(g[k] - gref[k]) / max(np.linalg.norm(gref[k]), 1e-30)
            assert err <= 1e-4, f"{k}: relative error {err:.2e} against the FP64 adjoint"
    finally:
        gs.close()


def test_fit_workload_gradients_vs_finite_differences():
    """The full 64-view, 512x512 workload: GPU gradients against FP64 central
    differences (h = 1e-4) on 256 seeded parameters."""
    fs = FitScene()
    gs, rs = scenes(fs)
    try:
        info = gs.info()
        assert info["primitives"] > 0
        with torch.no_grad():
            target = gs.render(*to_device(fs.truth(), requires_grad=False))
        init = fs.initial()
        _, g = gpu_grad(gs, init, target)
        vec = rs.pack(init)
        tgt = target.cpu().numpy()
        scale = 1.0 / tgt.size
        gvec = np.concatenate([g[k].ravel() for k in PARAM_NAMES])
        gref = rs.gradient(vec, tgt, scale)
        for k, gr in rs.unpack(gref).items():
            err = np.linalg.norm(g[k] - gr) / max(np.linalg.norm(gr), 1e-30)
            assert err <= 1e-4, f"{k}: relative error {err:.2e} against the FP64 adjoint"
        rng = np.random.default_rng(1004)
        n_tex = rs.tex_h * rs.tex_w * 4
        nz = np.nonzero(gref)[0]
        sel = np.concatenate([rng.choice(nz[nz < n_tex], 160, replace=False),
                              rng.choice(nz[(nz >= n_tex) & (nz < rs.n_params - 6)], 90, replace=False),
                              np.arange(rs.n_params - 6, rs.n_params)])
        assert len(sel) == 256
        rel = []
        for q in sel:
            fd = rs.central_difference(vec, tgt, scale, int(q), h=1e-4)
            rel.append(abs(gvec[q] - fd) / max(abs(fd), 1e-30))
        rel = np.array(rel)
        print(f"\nfit64 gradient vs FP64 central differences: max rel {rel.max():.2e}, "
              f"median {np.median(rel):.2e} over {len(rel)} parameters")
        assert rel.max() <= 1e-3
    finally:
        gs.close()


def test_fit_decreases_loss():
    from pixelforge_gb300.fit import fit
    fs = FitScene(subdiv=4, n_views=8, size=256, tex_size=256)
    r = fit(fs, iters=30, lr=0.02, log_every=29)
    try:
        (i0, l0), (i1, l1) = r["loss"][0], r["loss"][-1]
        assert l1 < 0.5 * l0, f"loss {l0} -> {l1}"
    finally:
        r["scene"].close()


def test_clipping_is_refused():
    fs = FitScene(subdiv=2, n_views=2, size=64, tex_size=32, radius=0.5)
    mvp, eyes = fs.cameras()
    from pixelforge_gb300.grad import GradScene
    with pytest.raises(RuntimeError, match="crosses the view volume"):
        GradScene(fs.mesh(), mvp, eyes, 64, 64, (32, 32))
