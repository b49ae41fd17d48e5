#!/usr/bin/env python3
"""Benchmark of the PixelForge triangle pipeline on GB300.

Workload (one step = one frame): the 1920x1080 textured, Gouraud-lit UV
sphere (256x128 segments, 65,536 triangles) drawn twice -- opaque, then
scaled 1.05 with alpha 0.5 and alpha blending -- after a clear; 1024x1024
RGBA8 noise texture, bilinear, repeat.  Metric: fragments/s (a fragment is a
covered (pixel, sub-triangle) pair before the depth test) and ms/frame.

  value  device throughput: fragments / GPU time of the pipeline kernels,
         timed with CUDA events on the library's own stream (inputs already
         uploaded when each kernel region starts)
  e2e    the same frames through the C ABI with host buffers: every pf*
         call, the snapshot and host-to-device copy of vertex arrays, indices
         and texture, the kernels and the device-to-host write-back of the
         colour into the caller's buffer
  --impl reference  times the reference's CPU implementation of the path on
         this host's cores: the reference build (x86-64 only) when present,
         else the portable restatement in oracle/

L2 is flushed (a 512 MiB device write) between timed frames.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
TRAFFIC_FILE = ROOT / "profiles" / "roofline_traffic.json"
FALLBACK_HBM_GBS = 6800.0


def _traffic(kernel: str):
    """DRAM bytes per launch of a kernel from the committed ncu summary (one
    capture of the same workload), or None."""
    try:
        return float(json.loads(TRAFFIC_FILE.read_text())[kernel]["bytes_per_launch"])
    except Exception:
        return None


def _peaks():
    try:
        d = json.loads(PEAKS_FILE.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = Path(os.environ.get("PF_CLOCKS_CSV", "/tmp/pf_bench_clocks.csv"))

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-i", "0", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                rows.append(parts)
        if not rows:
            return None
        sm = sorted(float(r[0]) for r in rows if r[0].replace(".", "").isdigit())
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, n in enumerate(names):
                if r[3 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": sm[len(sm) // 2] if sm else None,
                "sm_max_mhz": float(rows[0][1]) if rows[0][1].replace(".", "").isdigit() else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def frame_bytes(scene) -> dict:
    """Compulsory bytes of one frame (algorithmic): colour + depth written
    once, vertex attributes and indices of both draws read once, the texture
    read once."""
    W, H = scene.width, scene.height
    nv = len(scene.pos)
    fb = 8 * W * H
    vtx = nv * (12 + 12 + 8)
    idx = len(scene.idx) * 4
    tex = scene.tex.nbytes
    draws = 2 if scene.second_draw else 1
    return {"framebuffer": fb, "vertices": draws * vtx, "indices": draws * idx, "texture": tex,
            "total": fb + draws * (vtx + idx) + tex, "raster": fb + tex}


def run_gpu(args):
    import numpy as np
    import torch
    from pixelforge_gb300 import load_library, abi as A
    from pixelforge_gb300.scenes import SphereScene, Target

    lib = load_library()
    scene = SphereScene()
    tg = Target(lib, scene.width, scene.height, "main")
    scene.setup(lib)
    lib.pfEnableTiming(True)
    dev = torch.device("cuda:0")
    l2_flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def stats():
        s = A.PFstats()
        lib.pfGetStats(s)
        return {k: getattr(s, k) for k, _ in A.PFstats._fields_}

    for _ in range(args.warmup):
        scene.frame(lib)
        lib.pfFinish()
    if lib.pfGetDeviceStatus() != 0:
        raise RuntimeError(f"device status {lib.pfGetDeviceStatus():#x}")
    lib.pfResetStats()
    torch.cuda.synchronize()
    clocks = ClockSampler()
    clocks.start()
    wall = rec = 0.0
    for _ in range(args.steps):
        l2_flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        scene.frame(lib)
        t1 = time.perf_counter()
        lib.pfFinish()
        t2 = time.perf_counter()
        wall += t2 - t0
        rec += t1 - t0
    torch.cuda.synchronize()
    ck = clocks.stop()
    st = stats()
    # fragments of the opaque draw alone (one frame outside the timed region),
    # for the immediate-mode byte count: the blended draw also reads colour
    f_all = st["fragments"] / args.steps
    if scene.second_draw:
        lib.pfResetStats()
        scene.second_draw = False
        scene.frame(lib)
        lib.pfFinish()
        scene.second_draw = True
        f_opaque = stats()["fragments"]
    else:
        f_opaque = f_all
    if lib.pfGetDeviceStatus() != 0:
        raise RuntimeError(f"device status {lib.pfGetDeviceStatus():#x}")
    frags = st["fragments"]
    dev_s = st["device_ms"] / 1e3
    ms_frame = st["device_ms"] / args.steps
    fb = frame_bytes(scene)
    peak, peak_kind = _peaks()
    raster_ms = st["raster_ms"] / max(st["raster_launches"], 1)
    achieved = fb["raster"] / (raster_ms / 1e3) / 1e9
    # immediate-mode bytes: per fragment depth read + write and colour write
    # (12 B), 16 texel bytes (bilinear), colour read when blending (4 B)
    immediate = f_all * (12 + 16) + (f_all - f_opaque) * 4
    # each draw copies what it references: positions (the normals are the same
    # array, copied once), uvs, indices, texture
    h2d = 2 * (scene.pos.nbytes + scene.uv.nbytes + scene.idx.nbytes + scene.tex.nbytes)
    d2h = scene.width * scene.height * 4
    out = {
        "metric": "fragments/s",
        "value": frags / dev_s,
        "unit": "fragments/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_frame,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+u8",
        "data": "synthetic (seeded UV sphere and noise texture)",
        "config": SPHERE_CONFIG,
        "parallelism": "one GPU per rank (replicas)",
        "fragments_per_frame": frags / args.steps,
        "e2e": {"value": frags / wall, "unit": "fragments/s", "ms_per_step": wall * 1e3 / args.steps,
                "record_ms_per_step": rec * 1e3 / args.steps,
                "flush_ms_per_step": (wall - rec) * 1e3 / args.steps,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": st["kernel_launches"],
        "roofline": {"bound": "hbm", "kernel": "k_raster", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": _traffic("k_raster"),
                     "launch_share_of_frame": (st["raster_ms"] / max(st["device_ms"], 1e-9)),
                     "algorithmic_bytes_per_launch": fb["raster"], "launch_ms": raster_ms,
                     "frame_algorithmic_bytes": fb["total"],
                     "frame_frac": fb["total"] / (ms_frame / 1e3) / 1e9 / peak,
                     "frac_of_nominal_8000_gbs": achieved / 8000.0,
                     "immediate_mode_bytes_per_launch": immediate,
                     "immediate_mode_frac": immediate / (raster_ms / 1e3) / 1e9 / peak},
        "clocks": ck,
    }
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args, samples=2)
    tg.close()
    out["e2e_device_inputs"] = run_device_inputs(lib, args, l2_flush)
    # the other workloads, each in a process of its own: a failure there is
    # reported in its section and leaves the headline line intact
    for name, skip in (("soup256", args.no_soup), ("phong", args.no_phong), ("framebuffer_formats", args.no_formats),
                       ("batched", args.no_batched), ("adjoint", args.no_adjoint)):
        if not skip:
            out[name] = run_section(name)
    return out


def run_device_inputs(lib, args, l2_flush) -> dict:
    """The same frames end to end with the arrays, indices and texture
    already in device memory (the zero-copy pf*Device calls): every pf* call,
    the kernels and the device-to-host write-back of the colour into the
    caller's buffer; nothing is copied to the device."""
    import torch
    from pixelforge_gb300 import abi as A
    from pixelforge_gb300.scenes import SphereScene, Target
    sc = SphereScene(device_arrays=True)
    tg = Target(lib, sc.width, sc.height, "main")
    try:
        sc.setup(lib)
        lib.pfEnableTiming(True)
        for _ in range(args.warmup):
            sc.frame(lib)
            lib.pfFinish()
        lib.pfResetStats()
        wall = 0.0
        for _ in range(args.steps):
            l2_flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sc.frame(lib)
            lib.pfFinish()
            wall += time.perf_counter() - t0
        s = A.PFstats()
        lib.pfGetStats(s)
        status = lib.pfGetDeviceStatus()
        sc.teardown(lib)
    finally:
        tg.close()
    if status != 0:
        raise RuntimeError(f"device status {status:#x}")
    return {"value": s.fragments / wall, "unit": "fragments/s", "ms_per_step": wall * 1e3 / args.steps,
            "device_ms_per_step": s.device_ms / args.steps,
            "h2d_bytes_per_step": 0, "d2h_bytes_per_step": sc.width * sc.height * 4}


SECTION_TIMEOUT_S = 900


def run_section(name: str) -> dict:
    """Run one secondary workload (``--section NAME``) in a child process and
    return its JSON object, or {"error": ...} when the child failed."""
    import subprocess
    cmd = [sys.executable, os.path.abspath(__file__), "--section", name]
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=SECTION_TIMEOUT_S)
    except subprocess.TimeoutExpired:
        return {"error": f"timed out after {SECTION_TIMEOUT_S} s"}
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    if r.returncode != 0 or not lines:
        tail = " | ".join((r.stderr or r.stdout).strip().splitlines()[-3:])
        return {"error": f"exit code {r.returncode}: {tail}"}
    return json.loads(lines[-1])


def section_main(name: str, args) -> dict:
    from pixelforge_gb300 import load_library
    if name == "adjoint":
        return run_adjoint(args)
    lib = load_library()
    return {"soup256": run_soup, "phong": run_phong, "framebuffer_formats": run_formats,
            "batched": run_batched}[name](lib)


SPHERE_WORKLOAD = ("sphere1080: 1920x1080 textured Gouraud UV sphere 256x128, two draws "
                   "(opaque + alpha 0.5 scaled 1.05), 1024^2 bilinear repeat texture")
# identical in both arms: the same scene, frames and L2 handling
SPHERE_CONFIG = {"workload": SPHERE_WORKLOAD, "frame": "clear + opaque draw + blended draw without depth writes",
                 "l2": "flushed between frames (512 MiB device write); inputs larger than L2 on the host arm"}


def _soup_frames(lib, steps: int, warmup: int, timing: bool):
    """Frames of the 256x256 soup (immediate mode, 2,000 triangles) into a
    main buffer: the recording time (the pf* calls, made from Python), the
    flush time, and the library's statistics."""
    from pixelforge_gb300 import abi as A
    from pixelforge_gb300.scenes import SoupScene, Target
    sc = SoupScene()
    tg = Target(lib, sc.width, sc.height, "main")
    if timing:
        lib.pfEnableTiming(True)
    for _ in range(warmup):
        sc.record(lib)
        if lib.has("pfFinish"):
            lib.pfFinish()
    if lib.has("pfResetStats"):
        lib.pfResetStats()
    rec = flush = 0.0
    for _ in range(steps):
        t0 = time.perf_counter()
        sc.record(lib)
        t1 = time.perf_counter()
        if lib.has("pfFinish"):
            lib.pfFinish()
        else:
            lib.pfReadPixels(0, 0, 1, 1, A.PF_RGBA, A.PF_UNSIGNED_BYTE, tg.main.ctypes.data)
        t2 = time.perf_counter()
        rec += t1 - t0
        flush += t2 - t1
    st = None
    if lib.has("pfGetStats"):
        st = A.PFstats()
        lib.pfGetStats(st)
    status = lib.pfGetDeviceStatus() if lib.has("pfGetDeviceStatus") else 0
    tg.close()
    if status != 0:
        raise RuntimeError(f"device status {status:#x}")
    return rec, flush, st


def run_soup(lib, warmup: int = 3, steps: int = 20) -> dict:
    """The small plain workload (256x256, 2,000-triangle immediate-mode soup,
    Gouraud colours, depth LESS, the reference's default cull and
    projection): device ms/frame and fragments/s on the GPU, the recording
    and flush time through the C ABI, and the same frames on the reference's
    CPU path (the oracle port or the reference build) on the host cores."""
    rec, flush, st = _soup_frames(lib, steps, warmup, True)
    out = {"workload": "soup256: 256x256 RGBA8 + FP32 depth, 2,000-triangle seeded soup via pfBegin(PF_TRIANGLES), "
                       "default projection, Gouraud colours, depth LESS, back faces culled",
           "ms_per_frame": st.device_ms / steps, "fragments_per_frame": st.fragments / steps,
           "fragments_per_s": st.fragments / (st.device_ms / 1e3),
           "record_ms_per_frame": rec * 1e3 / steps, "flush_ms_per_frame": flush * 1e3 / steps,
           "note": "recording is 12,000 pf* calls per frame made through ctypes from Python"}
    cpu, kind = _reference_lib()
    crec, cflush, cst = _soup_frames(cpu, steps, 1, False)
    cms = (crec + cflush) * 1e3 / steps
    cfr = (cst.fragments / steps) if cst is not None else out["fragments_per_frame"]
    out["cpu"] = {"kind": kind, "ms_per_frame": cms, "fragments_per_s": cfr / (cms / 1e3),
                  "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
                  "sample": f"{steps} frames through the same Python recording loop, {platform.machine()} host"}
    return out


def run_phong(lib, warmup: int = 2, steps: int = 5) -> dict:
    """The fragment-heavy Phong workload at 1080p: 1.3M-triangle displaced
    icosphere, 8 point lights per fragment, 2048^2 nearest mirrored texture,
    30% of the triangles additive, device fog hook.  Device time of the
    frame's kernels (events), fragments counted on the device, and the end-
    to-end time of the API calls, uploads and write-back."""
    import torch
    from pixelforge_gb300 import abi as A
    from pixelforge_gb300.scenes import PhongScene, Target
    sc = PhongScene()
    tg = Target(lib, sc.width, sc.height, "main")
    sc.setup(lib)
    lib.pfEnableTiming(True)
    l2_flush = torch.empty(512 << 20, dtype=torch.uint8, device=torch.device("cuda:0"))
    for _ in range(warmup):
        sc.frame(lib)
        lib.pfFinish()
    lib.pfResetStats()
    wall = 0.0
    for _ in range(steps):
        l2_flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sc.frame(lib)
        lib.pfFinish()
        wall += time.perf_counter() - t0
    s = A.PFstats()
    lib.pfGetStats(s)
    status = lib.pfGetDeviceStatus()
    sc.teardown(lib)
    tg.close()
    if status != 0:
        raise RuntimeError(f"device status {status:#x}")
    return {"workload": f"phong1080: displaced icosphere subdiv 8 ({sc.ntris} triangles), 8 point lights per "
                        "fragment, 2048^2 nearest mirrored-repeat texture, 30% additive, device fog",
            "ms_per_frame": s.device_ms / steps, "fragments_per_frame": s.fragments / steps,
            "fragments_per_s": s.fragments / (s.device_ms / 1e3),
            "raster_ms_per_frame": s.raster_ms / steps,
            "e2e_ms_per_frame": wall * 1e3 / steps, "l2": "flushed between frames"}


def run_formats(lib, warmup: int = 2, steps: int = 5) -> dict:
    """The sphere frame into main buffers of other formats: device ms per
    frame, raster ms and end-to-end ms (the write-back moves the format's
    bytes); RGBA / unsigned byte runs the plain kernel, the others the
    generic-format raster kernel, and BGRA / unsigned byte the band-by-band
    raster (its raster time includes both kernels)."""
    import torch
    from pixelforge_gb300 import abi as A
    from pixelforge_gb300.scenes import SphereScene, Target
    l2_flush = torch.empty(512 << 20, dtype=torch.uint8, device=torch.device("cuda:0"))
    out = {}
    for name, fmt in (("RGBA8", (A.PF_RGBA, A.PF_UNSIGNED_BYTE)), ("RGB565", (A.PF_RGB, A.PF_UNSIGNED_SHORT_5_6_5)),
                      ("RGBA16F", (A.PF_RGBA, A.PF_HALF_FLOAT)), ("RGBA32F", (A.PF_RGBA, A.PF_FLOAT)),
                      ("BGRA8", (A.PF_BGRA, A.PF_UNSIGNED_BYTE))):
        sc = SphereScene()
        tg = Target(lib, sc.width, sc.height, "main", fmt=fmt)
        sc.setup(lib)
        lib.pfEnableTiming(True)
        for _ in range(warmup):
            sc.frame(lib)
            lib.pfFinish()
        lib.pfResetStats()
        wall = 0.0
        for _ in range(steps):
            l2_flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sc.frame(lib)
            lib.pfFinish()
            wall += time.perf_counter() - t0
        s = A.PFstats()
        lib.pfGetStats(s)
        status = lib.pfGetDeviceStatus()
        sc.teardown(lib)
        tg.close()
        if status != 0:
            raise RuntimeError(f"device status {status:#x}")
        out[name] = {"bytes_per_pixel": A.pixel_bytes(*fmt), "ms_per_frame": s.device_ms / steps,
                     "raster_ms_per_frame": s.raster_ms / steps, "e2e_ms_per_frame": wall * 1e3 / steps}
    return {"workload": SPHERE_WORKLOAD + ", main buffer of each format", **out}


def run_adjoint(args) -> dict:
    """One fitting iteration of the fit64 workload: forward (render 64 views
    + loss) and forward + adjoint, timed with CUDA events on torch's stream,
    on which the pfgrad calls run."""
    import torch
    from pixelforge_gb300.fit import FitScene, to_device

    fs = FitScene()
    sc = fs.build()
    with torch.no_grad():
        target = sc.render(*to_device(fs.truth(), requires_grad=False))
    params = to_device(fs.initial())
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]

    def fwd():
        img = sc.render(*params)
        return ((img - target) ** 2).mean()

    for _ in range(3):
        for p in params:
            p.grad = None
        fwd().backward()
    torch.cuda.synchronize()
    n = max(args.steps, 5)
    f_ms = b_ms = k_fwd = k_bwd = 0.0
    for _ in range(n):
        for p in params:
            p.grad = None
        ev[0].record()
        loss = fwd()
        ev[1].record()
        loss.backward()
        ev[2].record()
        torch.cuda.synchronize()
        f_ms += ev[0].elapsed_time(ev[1])
        b_ms += ev[0].elapsed_time(ev[2])
    # the two pfgrad kernels sequences alone
    img = torch.empty(sc.image_shape(), device="cuda")
    grads = [torch.empty_like(p) for p in params]
    ts = [p.detach() for p in params]
    dimg = torch.empty_like(img).fill_(1e-6)
    for _ in range(n):
        ev[0].record()
        sc.forward_raw(ts, img)
        ev[1].record()
        sc.backward_raw(ts, dimg, grads)
        ev[2].record()
        torch.cuda.synchronize()
        k_fwd += ev[0].elapsed_time(ev[1])
        k_bwd += ev[1].elapsed_time(ev[2])
    info = sc.info()
    sc.close()
    return {"workload": "fit64: icosphere subdiv 5 (20,480 triangles), 64 views of 512x512, 512^2 RGBA float "
                        "texture, bilinear repeat, Gouraud Blinn-Phong, alpha-over, MSE loss",
            "forward_ms": f_ms / n, "forward_adjoint_ms": b_ms / n, "ratio": b_ms / f_ms,
            "pfgrad_forward_ms": k_fwd / n, "pfgrad_backward_ms": k_bwd / n,
            "views_per_s_forward": fs.n_views / (f_ms / n / 1e3),
            "tile_entries": info["tileEntries"], "primitives": info["primitives"], "iterations": n}


def run_batched(lib) -> dict:
    """512 independent contexts of uneven size: one batch versus looping the
    plain path (one flush per context), on identical images."""
    import numpy as np
    from pixelforge_gb300 import abi as A
    from pixelforge_gb300.autotune import tune_batch
    from pixelforge_gb300.scenes import BatchScene

    sc = BatchScene()
    sc.create(lib)
    for c in sc.ctx:
        lib.pfMakeCurrent(c)
        lib.pfEnableTiming(True)
        lib.pfResetStats()
    # plain path: each context recorded and flushed on its own
    sc.render_loop(lib)                                  # warm-up (allocations)
    for c in sc.ctx:
        lib.pfMakeCurrent(c)
        lib.pfResetStats()
    t0 = time.perf_counter()
    loop_imgs = sc.render_loop(lib)
    loop_wall = time.perf_counter() - t0
    loop_dev_ms = 0.0
    frags = 0
    for c in sc.ctx:
        lib.pfMakeCurrent(c)
        s = A.PFstats()
        lib.pfGetStats(s)
        loop_dev_ms += s.device_ms
        frags += s.fragments
    batch = lib.pfgbBatchCreate()
    lib.pfgbBatchEnableTiming(batch, True)
    tune = tune_batch(lib, batch, lambda b: sc.render_batch(lib, b), "batch512")
    sc.render_batch(lib, batch)                          # warm-up at the tuned setting
    t0 = time.perf_counter()
    batch_imgs = sc.render_batch(lib, batch)
    batch_wall = time.perf_counter() - t0
    identical = all(np.array_equal(a, b) for a, b in zip(loop_imgs, batch_imgs))
    replay_ms = lib.pfgbBatchReplay(batch, 10)
    lib.pfgbBatchDelete(batch)
    sc.destroy(lib)
    n = sc.n
    return {"workload": "batch512: 512 contexts, sides 64..512, lognormal triangle counts "
                        f"({sc.total_tris} triangles), textured, per-context blend",
            "views_per_s_graph": n / (replay_ms / 1e3), "replay_ms": replay_ms,
            "views_per_s_batch_e2e": n / batch_wall, "batch_e2e_ms": batch_wall * 1e3,
            "views_per_s_loop_e2e": n / loop_wall, "loop_e2e_ms": loop_wall * 1e3,
            "views_per_s_loop_device": n / (loop_dev_ms / 1e3), "loop_device_ms": loop_dev_ms,
            "speedup_graph_vs_loop_device": loop_dev_ms / replay_ms,
            "speedup_batch_vs_loop_e2e": loop_wall / batch_wall,
            "fragments": frags, "images_identical": identical,
            "tuning": {k: v for k, v in tune.items() if k != "trials"}}


def _reference_lib():
    """The reference's own CPU build when it exists here, else the port."""
    from pixelforge_gb300.abi import PixelForgeLib
    asis = ROOT / "oracle" / "_ref" / "libpf_asis.so"
    if asis.exists() and platform.machine() in ("x86_64", "AMD64"):
        try:
            return PixelForgeLib(str(asis)), "reference"
        except OSError:
            pass
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "pfref"], check=True)
    return PixelForgeLib(str(ROOT / "oracle" / "_build" / "libpfref.so")), "port"


def cpu_baseline(args, samples: int = 2, warmup: int = 1) -> dict:
    """The reference's CPU path on this host's cores, on the GPU arm's scene:
    the second draw runs without depth writes through pfDepthMask, which
    the oracle port has; the reference's own build (x86-64 only) has no
    depth mask and writes depth there (same fragments, same work)."""
    from pixelforge_gb300.scenes import SphereScene, Target
    lib, kind = _reference_lib()
    scene = SphereScene(depth_mask_off=lib.has("pfDepthMask"))
    tg = Target(lib, scene.width, scene.height, "main")
    scene.setup(lib)
    for _ in range(max(1, warmup)):       # warm caches
        scene.frame(lib)
    if lib.has("pfResetStats"):
        lib.pfResetStats()
    t0 = time.perf_counter()
    for _ in range(samples):
        scene.frame(lib)
    dt = time.perf_counter() - t0
    frags = None
    if lib.has("pfGetStats") and lib.has("pfResetStats"):
        from pixelforge_gb300 import abi as A
        s = A.PFstats()
        lib.pfGetStats(s)
        frags = s.fragments / samples
    tg.close()
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    fr = frags if frags else 846563.0
    return {"value": fr * samples / dt, "unit": "fragments/s", "cores": threads, "kind": kind,
            "ms_per_frame": dt * 1e3 / samples, "fragments_per_frame": fr,
            "sample": f"{samples} frames of the sphere1080 workload after {max(1, warmup)} warm-up frame(s), "
                      f"{platform.machine()} host, OMP_NUM_THREADS={threads}"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    cb = cpu_baseline(args, samples=max(1, args.steps), warmup=max(1, args.warmup))
    return {"impl": "reference", "metric": "fragments/s", "value": cb["value"], "unit": "fragments/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": cb["ms_per_frame"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+u8", "data": "synthetic (seeded UV sphere and noise texture)",
            "config": SPHERE_CONFIG, "parallelism": "host CPU cores",
            "fragments_per_frame": cb["fragments_per_frame"],
            "cpu_baseline": {k: cb[k] for k in ("kind", "cores", "sample", "value", "unit")},
            "e2e": {"value": cb["value"], "unit": "fragments/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 512-context batch measurement")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the fitting-iteration measurement")
    ap.add_argument("--no-phong", action="store_true", help="skip the Phong 1080p measurement")
    ap.add_argument("--no-formats", action="store_true", help="skip the framebuffer-format measurement")
    ap.add_argument("--no-soup", action="store_true", help="skip the 256x256 soup measurement")
    ap.add_argument("--section", default=None,
                    choices=["soup256", "phong", "framebuffer_formats", "batched", "adjoint"],
                    help="run one secondary workload alone and print its JSON object")
    args = ap.parse_args()
    if args.section:
        print(json.dumps(section_main(args.section, args)))
        return
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    if args.impl == "reference":
        out = run_reference(args)
    else:
        rank = int(os.environ.get("RANK", "0"))
        # Replicas only: each rank renders its own frames on its own GPU; the
        # path has no exchange step.
        if args.gpus > 1:
            import torch
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        out = run_gpu(args)
        if rank != 0:
            out = None
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
