"""Inverse texture / material fitting over the differentiable path.

Workload ``fit64``: an icosphere of subdivision 5 (10,242 vertices, 20,480
triangles) with per-vertex normals and spherical texture coordinates, seen
by 64 cameras on a radius-3 Fibonacci sphere (60 degree perspective, 512x512
views, culling of back faces as the reference's default).  Learnable: a
512x512 RGBA float texture (initialised to 0.5), per-vertex RGB colours and
alphas, the material (diffuse, specular, shininess) and the light direction.
Targets are rendered from seeded ground-truth parameters (the texture is
seeded smooth value noise, per-vertex alpha uniform in [0.6, 1]).  Sampling
is bilinear with REPEAT wrap, lighting Gouraud Blinn-Phong, blending
alpha-over, loss the mean squared error over all views.

    python -m pixelforge_gb300.fit --iters 100
"""
from __future__ import annotations

import argparse
import math
import time
from dataclasses import dataclass

import numpy as np

from .grad import GradScene, Mesh, PARAM_NAMES
from .scenes import icosphere, value_noise_texture


def look_at(eye, center=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """View matrix in the row-vector layout of pfMultMatrixf (p' = p * V)."""
    e = np.asarray(eye, np.float64)
    f = np.asarray(center, np.float64) - e
    f /= np.linalg.norm(f)
    u = np.asarray(up, np.float64)
    if abs(np.dot(f, u)) > 0.99:
        u = np.array([0.0, 0.0, 1.0])
    r = np.cross(f, u)
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    V = np.eye(4)
    V[:3, 0], V[:3, 1], V[:3, 2] = r, u, -f
    V[3, :3] = [-np.dot(r, e), -np.dot(u, e), np.dot(f, e)]
    return V


def perspective(fov_deg: float, aspect: float, near: float, far: float) -> np.ndarray:
    """Projection matrix (row-vector layout); clip w = -z_eye."""
    f = 1.0 / math.tan(math.radians(fov_deg) / 2.0)
    P = np.zeros((4, 4))
    P[0, 0], P[1, 1] = f / aspect, f
    P[2, 2] = (far + near) / (near - far)
    P[2, 3] = -1.0
    P[3, 2] = 2.0 * far * near / (near - far)
    return P


def fibonacci_sphere(n: int, radius: float) -> np.ndarray:
    i = np.arange(n, dtype=np.float64) + 0.5
    y = 1.0 - 2.0 * i / n
    r = np.sqrt(1.0 - y * y)
    th = np.pi * (3.0 - math.sqrt(5.0)) * np.arange(n)
    return radius * np.stack([np.cos(th) * r, y, np.sin(th) * r], 1)


@dataclass
class FitScene:
    subdiv: int = 5
    n_views: int = 64
    size: int = 512
    tex_size: int = 512
    radius: float = 3.0
    fov: float = 60.0
    seed: int = 1004
    filter: int = 1          # PF_BILINEAR
    wrap: int = 0            # PF_REPEAT
    ambient: float = 0.2

    def mesh(self) -> Mesh:
        v, f = icosphere(self.subdiv)
        pos = v.astype(np.float32)
        u = 0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2 * np.pi)
        t = 0.5 - np.arcsin(np.clip(v[:, 1], -1, 1)) / np.pi
        uv = np.stack([u, t], 1).astype(np.float32)
        return Mesh(pos, pos.copy(), uv, f.astype(np.uint32))

    def cameras(self):
        eyes = fibonacci_sphere(self.n_views, self.radius)
        P = perspective(self.fov, 1.0, 0.1, 100.0)
        mvp = np.stack([(look_at(e) @ P).reshape(16) for e in eyes]).astype(np.float32)
        return mvp, eyes.astype(np.float32)

    def truth(self) -> dict:
        rng = np.random.default_rng(self.seed)
        nv = 10 * 4 ** self.subdiv + 2
        tex = value_noise_texture(self.tex_size, self.seed).astype(np.float32) / 255.0
        light = rng.normal(size=3)
        light[1] = abs(light[1]) + 0.5
        return {"texture": tex,
                "colors": rng.uniform(0.3, 1.0, (nv, 3)).astype(np.float32),
                "alphas": rng.uniform(0.6, 1.0, nv).astype(np.float32),
                "material": np.array([0.8, 0.5, 32.0], np.float32),
                "light": (light / np.linalg.norm(light)).astype(np.float32)}

    def initial(self) -> dict:
        t = self.truth()
        rng = np.random.default_rng(self.seed + 1)
        nv = len(t["colors"])
        light = t["light"] + rng.normal(scale=0.3, size=3).astype(np.float32)
        return {"texture": np.full((self.tex_size, self.tex_size, 4), 0.5, np.float32),
                "colors": np.full((nv, 3), 0.5, np.float32),
                "alphas": np.full(nv, 0.8, np.float32),
                "material": np.array([0.5, 0.3, 16.0], np.float32),
                "light": light.astype(np.float32)}

    def build(self) -> GradScene:
        mvp, eyes = self.cameras()
        return GradScene(self.mesh(), mvp, eyes, self.size, self.size, (self.tex_size, self.tex_size),
                         filter=self.filter, wrap=self.wrap, cull=1, ambient=self.ambient)


def to_device(params: dict, requires_grad: bool = True):
    import torch
    return [torch.tensor(params[k], device="cuda", requires_grad=requires_grad) for k in PARAM_NAMES]


def clamp_(tensors):
    """Keep the parameters in their valid ranges after an optimiser step."""
    import torch
    with torch.no_grad():
        tex, col, alpha, mat, _ = tensors
        tex.clamp_(0.0, 1.0)
        col.clamp_(0.0, 1.0)
        alpha.clamp_(0.0, 1.0)
        mat[:2].clamp_(0.0, 2.0)
        mat[2].clamp_(1.0, 256.0)


def fit(fs: FitScene, iters: int = 100, lr: float = 0.02, log_every: int = 10, scene: GradScene = None):
    import torch
    sc = scene or fs.build()
    with torch.no_grad():
        target = sc.render(*to_device(fs.truth(), requires_grad=False))
    params = to_device(fs.initial())
    groups = [{"params": params[:4], "lr": lr}, {"params": [params[4]], "lr": lr * 0.5}]
    opt = torch.optim.Adam(groups)
    hist = []
    t0 = time.perf_counter()
    for it in range(iters):
        opt.zero_grad(set_to_none=True)
        img = sc.render(*params)
        loss = ((img - target) ** 2).mean()
        loss.backward()
        opt.step()
        clamp_(params)
        if it % log_every == 0 or it == iters - 1:
            hist.append((it, float(loss.detach())))
    torch.cuda.synchronize()
    return {"loss": hist, "seconds": time.perf_counter() - t0, "params": params, "scene": sc}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--iters", type=int, default=100)
    ap.add_argument("--lr", type=float, default=0.02)
    args = ap.parse_args()
    r = fit(FitScene(), args.iters, args.lr)
    for it, l in r["loss"]:
        print(f"iter {it:5d}  loss {l:.6f}")
    print(f"{args.iters} iterations in {r['seconds']:.2f} s")


if __name__ == "__main__":
    main()
