"""Autotuner for the batched tile rasterizer.

Tunes, per GPU model and workload name, the two launch parameters the
library exposes through pfgbBatchTune: the initial tile-bin capacity (a
power of two; bins still grow on overflow) and the number of persistent
raster CTAs per SM.  The tile size itself is a compile-time constant
(16x16 pixels, one 256-thread CTA per tile at a time).  Each candidate is
measured by replaying the batch's CUDA graph (device time only); results are
cached in pixelforge_gb300/_build/autotune.json keyed by GPU name and
workload.
"""
from __future__ import annotations

import json
from pathlib import Path

from . import abi as A

CACHE = Path(__file__).resolve().parent / "_build" / "autotune.json"
BIN_CAPS = (256, 1024, 4096)
CTAS_PER_SM = (2, 3, 4)


def _gpu_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown"


def _load() -> dict:
    try:
        return json.loads(CACHE.read_text())
    except Exception:
        return {}


def tune_batch(lib: A.PixelForgeLib, batch, render, workload: str, replays: int = 5,
               use_cache: bool = True) -> dict:
    """Pick (bin capacity, CTAs per SM) for `render(batch)` (which records and
    renders the workload into `batch`).  Returns the chosen setting and the
    timings of every candidate."""
    key = f"{_gpu_name()}|{workload}"
    cache = _load()
    if use_cache and key in cache:
        best = cache[key]
        lib.pfgbBatchTune(batch, best["bin_capacity"], best["ctas_per_sm"])
        return {**best, "cached": True}
    trials = []
    for cap in BIN_CAPS:
        for per in CTAS_PER_SM:
            lib.pfgbBatchTune(batch, cap, per)
            render(batch)
            ms = lib.pfgbBatchReplay(batch, replays)
            trials.append({"bin_capacity": cap, "ctas_per_sm": per, "replay_ms": float(ms)})
    ok = [t for t in trials if t["replay_ms"] > 0]
    best = min(ok, key=lambda t: t["replay_ms"]) if ok else {"bin_capacity": 1024, "ctas_per_sm": 4,
                                                            "replay_ms": -1.0}
    lib.pfgbBatchTune(batch, best["bin_capacity"], best["ctas_per_sm"])
    cache[key] = {"bin_capacity": best["bin_capacity"], "ctas_per_sm": best["ctas_per_sm"],
                  "replay_ms": best["replay_ms"], "tile": 16}
    CACHE.parent.mkdir(exist_ok=True)
    CACHE.write_text(json.dumps(cache, indent=1))
    return {**cache[key], "cached": False, "trials": trials}
