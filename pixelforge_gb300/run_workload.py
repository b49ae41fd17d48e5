"""Render one of the seeded workloads a given number of times (for
profilers and quick checks).

    python -m pixelforge_gb300.run_workload sphere --frames 4
    python -m pixelforge_gb300.run_workload sphere --frames 4 --format RGBA16F
    python -m pixelforge_gb300.run_workload phong --frames 2 --width 960 --height 540
    python -m pixelforge_gb300.run_workload batch --contexts 64 --repeat 2
    python -m pixelforge_gb300.run_workload soup --frames 4
    python -m pixelforge_gb300.run_workload fit --views 8 --iters 2

Exits non-zero if the device reports an error.
"""
from __future__ import annotations

import argparse
import sys


FORMATS = {"RGBA8": (7, 0), "RGB8": (6, 0), "RGB565": (6, 2), "RGBA5551": (7, 3), "RGBA4444": (7, 4),
           "RGBA16F": (7, 9), "RGBA32F": (7, 10), "LA16F": (5, 9), "BGRA8": (9, 0)}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["sphere", "phong", "batch", "fit", "soup"])
    ap.add_argument("--frames", type=int, default=4)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--contexts", type=int, default=64)
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--views", type=int, default=8)
    ap.add_argument("--iters", type=int, default=2)
    ap.add_argument("--format", default="RGBA8", choices=sorted(FORMATS),
                    help="format of the main buffer (sphere and phong)")
    a = ap.parse_args(argv)

    from . import load_library
    if a.workload == "fit":
        import torch
        from .fit import FitScene, to_device
        fs = FitScene(n_views=a.views)
        sc = fs.build()
        with torch.no_grad():
            target = sc.render(*to_device(fs.truth(), requires_grad=False))
        params = to_device(fs.initial())
        for _ in range(a.iters):
            for p in params:
                p.grad = None
            loss = ((sc.render(*params) - target) ** 2).mean()
            loss.backward()
        torch.cuda.synchronize()
        print(f"fit: {a.iters} iterations, loss {float(loss.detach()):.6f}")
        sc.close()
        return 0

    lib = load_library()
    if a.workload == "batch":
        from .scenes import BatchScene
        sc = BatchScene(n=a.contexts)
        sc.create(lib)
        b = lib.pfgbBatchCreate()
        for _ in range(a.repeat):
            sc.render_batch(lib, b)
        status = 0
        for c in sc.ctx:
            lib.pfMakeCurrent(c)
            status |= lib.pfGetDeviceStatus()
        lib.pfgbBatchDelete(b)
        sc.destroy(lib)
        print(f"batch: {a.contexts} contexts x {a.repeat}, status {status}")
        return 1 if status else 0

    from .scenes import PhongScene, SoupScene, SphereScene, Target
    if a.workload == "soup":
        sc = SoupScene()
        tg = Target(lib, sc.width, sc.height, "main")
        for _ in range(a.frames):
            sc.record(lib)
            lib.pfFinish()
        status = lib.pfGetDeviceStatus()
        tg.close()
        print(f"soup: {a.frames} frames at {sc.width}x{sc.height}, status {status}")
        return 1 if status else 0
    sc = SphereScene(width=a.width, height=a.height) if a.workload == "sphere" else \
        PhongScene(width=a.width, height=a.height)
    tg = Target(lib, sc.width, sc.height, "main", fmt=FORMATS[a.format])
    sc.setup(lib)
    for _ in range(a.frames):
        sc.frame(lib)
        lib.pfFinish()
    status = lib.pfGetDeviceStatus()
    sc.teardown(lib)
    tg.close()
    print(f"{a.workload}: {a.frames} frames at {a.width}x{a.height} ({a.format}), status {status}")
    return 1 if status else 0


if __name__ == "__main__":
    sys.exit(main())
