"""Batched contexts (config 3 form): many contexts rendered by one launch of
each pipeline kernel must give exactly the images of rendering each context
on its own, and match the CPU oracle (depth bit-exact, colour within 1 LSB)."""
import numpy as np
import pytest

from pixelforge_gb300 import abi as A
from pixelforge_gb300.scenes import BatchScene

pytestmark = pytest.mark.gpu


def _images_equal(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_batch_equals_per_context(gpu):
    sc = BatchScene(n=64, max_side=256, tri_clip=(100, 4000), seed=31)
    sc.create(gpu)
    try:
        loop = sc.render_loop(gpu)
        batch = gpu.pfgbBatchCreate()
        try:
            got = sc.render_batch(gpu, batch)
            s = A.PFstats()
            gpu.pfgbBatchGetStats(batch, s)
            assert s.flushes == 1, "a batch renders with one flush"
            # one launch of each pipeline kernel per attempt (a tile bin that
            # overflows its capacity makes the flush grow it and resume),
            # besides the draw-time copies of large caller arrays
            assert s.kernel_launches - s.copy_launches == 4 * (1 + s.bin_overflows)
        finally:
            gpu.pfgbBatchDelete(batch)
        assert _images_equal(loop, got)
    finally:
        sc.destroy(gpu)


def test_batch_block_shapes_and_capacities_agree(gpu):
    """Every tuning point the autotuner may pick (warps per raster CTA, bin
    capacity, CTAs per SM) renders the same images."""
    sc = BatchScene(n=24, max_side=256, tri_clip=(100, 3000), seed=33)
    sc.create(gpu)
    try:
        batch = gpu.pfgbBatchCreate()
        try:
            first = None
            for warps, cap, per in ((4, 256, 0), (2, 1024, 0), (8, 4096, 0), (4, 64, 3), (8, 256, 1)):
                gpu.pfgbBatchTune(batch, cap, per)
                gpu.pfgbBatchTuneShape(batch, warps)
                got = sc.render_batch(gpu, batch)
                if first is None:
                    first = got
                else:
                    assert _images_equal(first, got), f"{warps} warps, capacity {cap}, {per} CTAs/SM"
        finally:
            gpu.pfgbBatchDelete(batch)
    finally:
        sc.destroy(gpu)


def test_batch_vs_oracle(gpu, oracle):
    sc_g = BatchScene(n=12, max_side=192, tri_clip=(100, 900), seed=32)
    sc_o = BatchScene(n=12, max_side=192, tri_clip=(100, 900), seed=32)
    sc_g.create(gpu)
    sc_o.create(oracle)
    try:
        batch = gpu.pfgbBatchCreate()
        try:
            got = sc_g.render_batch(gpu, batch)
        finally:
            gpu.pfgbBatchDelete(batch)
        ref = sc_o.render_loop(oracle)
        for i, (g, r) in enumerate(zip(got, ref)):
            d = np.abs(g.astype(np.int32) - r.astype(np.int32))
            assert int(d.max()) <= 1, f"context {i}: colour differs by {int(d.max())}"
    finally:
        sc_g.destroy(gpu)
        sc_o.destroy(oracle)


def test_batch_mixed_framebuffer_formats_vs_oracle(gpu, oracle):
    """One batch whose contexts have main buffers of different formats (the
    raster launch takes the generic-format kernel, each target its own
    format): raw pixels bit-exact against the oracle context by context."""
    fmts = ((A.PF_RGBA, A.PF_UNSIGNED_BYTE), (A.PF_RGB, A.PF_UNSIGNED_SHORT_5_6_5), (A.PF_RGBA, A.PF_HALF_FLOAT),
            (A.PF_BGR, A.PF_UNSIGNED_BYTE), (A.PF_BGRA, A.PF_FLOAT), (A.PF_LUMINANCE_ALPHA, A.PF_HALF_FLOAT),
            (A.PF_RGBA, A.PF_UNSIGNED_SHORT_4_4_4_4))
    sc_g = BatchScene(n=14, max_side=192, tri_clip=(100, 900), seed=34, fmts=fmts)
    sc_o = BatchScene(n=14, max_side=192, tri_clip=(100, 900), seed=34, fmts=fmts)
    sc_g.create(gpu)
    sc_o.create(oracle)
    try:
        batch = gpu.pfgbBatchCreate()
        try:
            got = sc_g.render_batch(gpu, batch)
        finally:
            gpu.pfgbBatchDelete(batch)
        assert gpu.pfGetDeviceStatus() == 0
        ref = sc_o.render_loop(oracle)
        for i, (g, r) in enumerate(zip(got, ref)):
            assert g.shape == r.shape and g.shape[2] == A.pixel_bytes(*fmts[i % len(fmts)])
            nd = int((g != r).any(-1).sum())
            assert nd == 0, f"context {i} {fmts[i % len(fmts)]}: {nd} pixels differ"
    finally:
        sc_g.destroy(gpu)
        sc_o.destroy(oracle)


def test_batch_bgra8_contexts_vs_oracle(gpu, oracle):
    """A batch mixing BGRA / unsigned-byte main buffers (rasterized row by
    row after the tile raster, several targets in one launch) with RGBA8 and
    another format: raw pixels bit-exact against the oracle context by
    context; a graph replay of the batch renders the same images again."""
    fmts = ((A.PF_BGRA, A.PF_UNSIGNED_BYTE), (A.PF_RGBA, A.PF_UNSIGNED_BYTE), (A.PF_BGRA, A.PF_UNSIGNED_BYTE),
            (A.PF_RGB, A.PF_UNSIGNED_SHORT_5_6_5))
    sc_g = BatchScene(n=10, max_side=160, tri_clip=(100, 700), seed=35, fmts=fmts)
    sc_o = BatchScene(n=10, max_side=160, tri_clip=(100, 700), seed=35, fmts=fmts)
    sc_g.create(gpu)
    sc_o.create(oracle)
    try:
        batch = gpu.pfgbBatchCreate()
        try:
            got = sc_g.render_batch(gpu, batch)
            assert gpu.pfgbBatchReplay(batch, 2) > 0.0
        finally:
            gpu.pfgbBatchDelete(batch)
        assert gpu.pfGetDeviceStatus() == 0
        ref = sc_o.render_loop(oracle)
        for i, (g, r) in enumerate(zip(got, ref)):
            assert g.shape == r.shape and g.shape[2] == A.pixel_bytes(*fmts[i % len(fmts)])
            nd = int((g != r).any(-1).sum())
            assert nd == 0, f"context {i} {fmts[i % len(fmts)]}: {nd} pixels differ"
    finally:
        sc_g.destroy(gpu)
        sc_o.destroy(oracle)


def test_batch_replay_and_reuse(gpu):
    sc = BatchScene(n=24, max_side=192, tri_clip=(100, 2000), seed=33)
    sc.create(gpu)
    try:
        batch = gpu.pfgbBatchCreate()
        try:
            first = sc.render_batch(gpu, batch)
            ms = gpu.pfgbBatchReplay(batch, 3)
            assert ms > 0.0
            # rendering the batch again (recorded anew) gives the same images
            again = sc.render_batch(gpu, batch)
            assert _images_equal(first, again)
        finally:
            gpu.pfgbBatchDelete(batch)
        assert gpu.pfGetDeviceStatus() == 0
    finally:
        sc.destroy(gpu)


def test_batch512_equals_per_context(gpu):
    """The full 512-context workload: batched images equal per-context ones."""
    sc = BatchScene()
    sc.create(gpu)
    try:
        loop = sc.render_loop(gpu)
        batch = gpu.pfgbBatchCreate()
        try:
            got = sc.render_batch(gpu, batch)
        finally:
            gpu.pfgbBatchDelete(batch)
        assert _images_equal(loop, got)
    finally:
        sc.destroy(gpu)
