"""Autotuner for the batched tile rasterizer.

Tunes, per GPU model and workload name, the launch parameters the library
exposes: the initial tile-bin capacity (a power of two; bins still grow on
overflow) and the persistent raster CTAs per SM (pfgbBatchTune), and the
raster's block shape, 2, 4 or 8 warps per CTA (pfgbBatchTuneShape).  The
tile size is fixed at 8x8 pixels: the rasterizer maps one warp to one tile,
two pixels per lane.  Each candidate is measured by replaying the batch's
CUDA graph (device time only); results are cached in
pixelforge_gb300/_build/autotune.json keyed by GPU name and workload.
"""
from __future__ import annotations

import json
from pathlib import Path

from . import abi as A

CACHE = Path(__file__).resolve().parent / "_build" / "autotune.json"
BIN_CAPS = (256, 1024, 4096)
WARPS_PER_CTA = (2, 4, 8)
# CTAs per SM: 0 = as many as fit (shared memory and registers decide);
# one lower setting for the default shape shows whether occupancy pays
EXTRA = ((1024, 4, 3),)
TILE = 8


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


def _apply(lib, batch, s: dict):
    lib.pfgbBatchTune(batch, s["bin_capacity"], s["ctas_per_sm"])
    lib.pfgbBatchTuneShape(batch, s["warps_per_cta"])


def tune_batch(lib: A.PixelForgeLib, batch, render, workload: str, replays: int = 5,
               use_cache: bool = True) -> dict:
    """Pick (bin capacity, warps per CTA, CTAs per SM) for `render(batch)`
    (which records and renders the workload into `batch`).  Returns the
    chosen setting and the timings of every candidate."""
    key = f"{_gpu_name()}|{workload}"
    cache = _load()
    if use_cache and key in cache and "warps_per_cta" in cache[key]:
        best = cache[key]
        _apply(lib, batch, best)
        return {**best, "cached": True}
    cands = [(c, w, 0) for c in BIN_CAPS for w in WARPS_PER_CTA] + list(EXTRA)
    trials = []
    for cap, warps, per in cands:
        s = {"bin_capacity": cap, "warps_per_cta": warps, "ctas_per_sm": per}
        _apply(lib, batch, s)
        render(batch)
        ms = lib.pfgbBatchReplay(batch, replays)
        trials.append({**s, "replay_ms": float(ms)})
    ok = [t for t in trials if t["replay_ms"] > 0]
    best = min(ok, key=lambda t: t["replay_ms"]) if ok else {"bin_capacity": 1024, "warps_per_cta": 4,
                                                            "ctas_per_sm": 0, "replay_ms": -1.0}
    _apply(lib, batch, best)
    cache[key] = {k: best[k] for k in ("bin_capacity", "warps_per_cta", "ctas_per_sm", "replay_ms")}
    cache[key]["tile"] = TILE
    CACHE.parent.mkdir(exist_ok=True)
    CACHE.write_text(json.dumps(cache, indent=1))
    return {**cache[key], "cached": False, "trials": trials}
