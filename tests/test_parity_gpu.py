"""GPU parity: libpixelforge_gb300.so against the CPU oracle, through the C ABI.

Bar (per the reference's own arithmetic): depth buffers -- hence coverage and
depth-test outcomes -- bit-exact; RGBA8 colour within 1 LSB per channel
(the only differing step is the Gouraud specular power, libm powf on the
host versus the device's pow, which can round the 8-bit specular term
differently).  Every other pixel is expected to match exactly and the tests
report how many do not.
"""
import numpy as np
import pytest

from pixelforge_gb300 import abi as A
from pixelforge_gb300.scenes import PhongScene, SoupScene, SphereScene
from fbscenes import FB_BGRA8, FB_SEEDS
from mixscenes import mix_case, run_mix

pytestmark = pytest.mark.gpu

COLOR_TOL = 1


def assert_parity(got, ref, exact_color=False, label=""):
    assert got.color.shape == ref.color.shape
    if ref.depth is not None:
        gd, rd = got.depth.view(np.uint32), ref.depth.view(np.uint32)
        nd = int((gd != rd).sum())
        assert nd == 0, f"{label}: {nd} depth values differ"
    diff = np.abs(got.color.astype(np.int32) - ref.color.astype(np.int32))
    worst = int(diff.max()) if diff.size else 0
    ndiff = int((diff.max(-1) > 0).sum())
    tol = 0 if exact_color else COLOR_TOL
    assert worst <= tol, f"{label}: colour differs by up to {worst} LSB on {ndiff} pixels"
    return ndiff


def test_soup256_config(gpu, oracle):
    sc = SoupScene()
    got, ref = sc.render(gpu), sc.render(oracle)
    assert gpu.pfGetDeviceStatus() == 0
    assert_parity(got, ref, exact_color=True, label="soup256")
    assert got.stats["fragments"] == ref.stats["fragments"]
    assert got.stats["rasterized"] == ref.stats["rasterized"]


@pytest.mark.parametrize("kw", [
    dict(cull=False), dict(shade=A.PF_FLAT), dict(depth_func=A.PF_GREATER, clear_depth=-5.0),
    dict(depth_func=A.PF_NOTEQUAL), dict(blend=A.PF_BLEND_ALPHA), dict(blend=A.PF_BLEND_SUB),
    dict(blend=A.PF_BLEND_SCREEN, cull=False), dict(width=250, height=131, ntris=500),
    dict(xy_range=(-3.0, 3.0), ntris=400),
])
def test_soup_variants(gpu, oracle, kw):
    sc = SoupScene(**kw)
    assert_parity(sc.render(gpu), sc.render(oracle), exact_color=True, label=str(kw))


@pytest.mark.parametrize("hook", [A.PF_HOOK_DITHER, A.PF_HOOK_GRAYSCALE])
def test_device_hooks_on_odd_width(gpu, oracle, hook):
    """Device post-process hooks after a soup on a 250x131 framebuffer
    (the dither hook depends on each pixel's column and row)."""
    from pixelforge_gb300.scenes import Target
    out = []
    for lib in (gpu, oracle):
        sc = SoupScene(width=250, height=131, ntris=400)
        tg = Target(lib, 250, 131, "fbo")
        try:
            sc.record(lib)
            lib.pfPostProcessDevice(hook, None, 0)
            out.append(tg.finish())
        finally:
            tg.close()
    assert gpu.pfGetDeviceStatus() == 0
    assert_parity(out[0], out[1], exact_color=True, label=f"hook {hook}")


def test_soup_main_target(gpu, oracle):
    sc = SoupScene(ntris=700)
    got, ref = sc.render(gpu, "main"), sc.render(oracle, "main")
    assert_parity(got, ref, exact_color=True, label="main target")


@pytest.mark.parametrize("filt", [A.PF_NEAREST, A.PF_BILINEAR])
def test_sphere1080(gpu, oracle, filt):
    sc = SphereScene(filt=filt)
    got, ref = sc.render(gpu), sc.render(oracle)
    n = assert_parity(got, ref, label=f"sphere1080 filter={filt}")
    assert n <= 0.001 * got.color.shape[0] * got.color.shape[1]
    assert got.stats["fragments"] == ref.stats["fragments"]


def test_phong_fog_540(gpu, oracle):
    sc = PhongScene(subdiv=6, width=960, height=540, tex_size=512)
    got, ref = sc.render(gpu), sc.render(oracle)
    assert_parity(got, ref, exact_color=True, label="phong fog")


def test_phong_fog_1080_full_size(gpu, oracle):
    """The fragment-heavy workload at its full size (1.3M triangles, tile
    bins of 2,000-3,300 entries rasterized in halves)."""
    sc = PhongScene()
    got, ref = sc.render(gpu), sc.render(oracle)
    assert gpu.pfGetDeviceStatus() == 0
    assert_parity(got, ref, exact_color=True, label="phong fog 1080")


@pytest.mark.parametrize("seed", range(60))
def test_feature_mix(gpu, oracle, seed):
    case = mix_case(seed, bilinear=True)
    assert_parity(run_mix(gpu, case), run_mix(oracle, case), label=f"mix {seed} {case}")


@pytest.mark.parametrize("seed", range(6000, 6040))
def test_feature_mix_bgra(gpu, oracle, seed):
    """Feature-mix scenes into BGRA / unsigned-byte framebuffers (k_rows:
    each 4-pixel half vector of a triangle's row takes its first pixel's
    colour, blended with that pixel's destination), main buffer and
    framebuffer object; fragment counts equal."""
    case = mix_case(seed, bilinear=True)
    for target in ("fbo", "main"):
        got, ref = run_mix(gpu, case, target, fmt=FB_BGRA8), run_mix(oracle, case, target, fmt=FB_BGRA8)
        assert gpu.pfGetDeviceStatus() == 0
        assert_parity(got, ref, label=f"bgra mix {seed} {target} {case}")
        assert got.stats["fragments"] == ref.stats["fragments"]


@pytest.mark.parametrize("case", ["far_vertices", "wide_framebuffer", "slivers"])
def test_binning_tile_test_edges(gpu, oracle, case):
    """The binning leaves out the tiles of a box where an edge function is
    negative on the whole tile, only where coordinates stay within 2^13:
    triangles whose vertices lie tens of thousands of pixels off screen
    (the 2D path, boxes clamped to the viewport: the test is off), a
    framebuffer 9,000 pixels wide (off), and long slivers crossing many
    tiles (on): colour and depth bit-exact, fragment counts equal."""
    from pixelforge_gb300.scenes import Target
    W, H = (9000, 40) if case == "wide_framebuffer" else (300, 200)
    seed = {"far_vertices": 41, "wide_framebuffer": 42, "slivers": 43}[case]
    outs = []
    for lib in (gpu, oracle):
        tg = Target(lib, W, H, "fbo")
        try:
            lib.pfDisable(A.PF_CULL_FACE)
            lib.pfEnable(A.PF_DEPTH_TEST)
            lib.pfClearDepth(1e30)
            lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
            rr = np.random.default_rng(seed)
            lib.pfBegin(A.PF_TRIANGLES)
            for k in range(300):
                lib.pfColor4ub(*[int(v) for v in rr.integers(0, 256, 3)], 255)
                if case == "far_vertices":
                    pts = rr.uniform(-120.0, 120.0, (3, 2))          # up to ~18,000 pixels off screen
                    pts[rr.integers(3)] = rr.uniform(-1.0, 1.0, 2)  # one vertex on screen
                elif case == "slivers":
                    a = rr.uniform(-1.2, 1.2, 2)
                    b = rr.uniform(-1.2, 1.2, 2)
                    pts = np.stack([a, b, b + rr.uniform(-0.02, 0.02, 2)])
                else:
                    pts = rr.uniform(-1.1, 1.1, (3, 2))
                for p in pts:
                    lib.pfVertex3f(float(p[0]), float(p[1]), float(rr.uniform(-0.9, 0.9)))
            lib.pfEnd()
            outs.append(tg.finish())
        finally:
            tg.close()
    got, ref = outs
    assert (ref.depth < 1e30).sum() > 1000
    assert_parity(got, ref, exact_color=True, label=case)
    assert got.stats["fragments"] == ref.stats["fragments"]


def test_bgra8_wide_rows(gpu, oracle):
    """A BGRA / unsigned-byte framebuffer wider than the rows k_rows keeps
    in shared memory (2,600 pixels: drawn in place), blended soup with
    culling off: bit-exact, fragment counts equal."""
    from pixelforge_gb300.scenes import Target
    sc = SoupScene(width=2600, height=40, ntris=500, blend=A.PF_BLEND_ALPHA, cull=False)
    outs = []
    for lib in (gpu, oracle):
        tg = Target(lib, sc.width, sc.height, "fbo", fmt=FB_BGRA8)
        try:
            sc.record(lib)
            outs.append(tg.finish())
        finally:
            tg.close()
    assert gpu.pfGetDeviceStatus() == 0
    assert (outs[1].depth < 1e30).sum() > 20000
    assert_parity(outs[0], outs[1], exact_color=True, label="bgra8 2600 wide")
    assert outs[0].stats["fragments"] == outs[1].stats["fragments"]


def test_bgra8_tile_bins_and_splits(gpu, oracle):
    """BGRA / unsigned byte beside RGBA8 in one flush (two framebuffer
    objects drawn alternately, the RGBA8 one rasterized by k_raster, the
    BGRA8 one by k_rows), with more triangles in a tile than a bin holds at
    first (capacity retries) and clipped triangles: both bit-exact."""
    from pixelforge_gb300.scenes import _ptr
    import ctypes as C
    W, H, n = 200, 120, 6000
    r = np.random.default_rng(31)
    pos = r.uniform(-1.3, 1.3, (n * 3, 3)).astype(np.float32) * np.float32([1, 1, 2.0])
    col = r.integers(0, 256, (n * 3, 4)).astype(np.uint8)

    def run(lib):
        buf = np.zeros((8, 8, 4), np.uint8)
        ctx = lib.pfCreateContext(_ptr(buf), 8, 8, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
        lib.pfMakeCurrent(ctx)
        fbs = [lib.pfGenFramebuffer(W, H, A.PF_RGBA, A.PF_UNSIGNED_BYTE),
               lib.pfGenFramebuffer(W, H, A.PF_BGRA, A.PF_UNSIGNED_BYTE)]
        refs = [C.pointer(f) for f in fbs]
        out = []
        try:
            lib.pfMatrixMode(A.PF_PROJECTION)
            lib.pfLoadIdentity()
            lib.pfFrustum(-0.1, 0.1, -0.06, 0.06, 0.1, 10.0)
            lib.pfMatrixMode(A.PF_MODELVIEW)
            lib.pfLoadIdentity()
            lib.pfTranslatef(0.0, 0.0, -1.5)
            lib.pfViewport(0, 0, W, H)                    # (the context's own buffer is 8x8)
            lib.pfDisable(A.PF_CULL_FACE)
            lib.pfEnable(A.PF_DEPTH_TEST)
            lib.pfEnable(A.PF_FRAMEBUFFER)
            lib.pfEnable(A.PF_VERTEX_ARRAY | A.PF_COLOR_ARRAY)
            lib.pfVertexPointer(3, A.PF_FLOAT, 0, _ptr(pos))
            lib.pfColorPointer(4, A.PF_UNSIGNED_BYTE, 0, _ptr(col))
            for k in range(4):
                lib.pfBindFramebuffer(refs[k % 2])
                if k < 2:
                    lib.pfClearColor(10, 20, 30, 255)
                    lib.pfClearDepth(1e30)
                    lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
                if k >= 2:
                    lib.pfEnable(A.PF_BLEND)
                    lib.pfBlendFunc(A.PF_BLEND_ADD)
                lib.pfDrawArrays(A.PF_TRIANGLES, 0, n * 3 // (1 + k % 2))
            if lib.has("pfFinish"):
                lib.pfFinish()
            px = lib.raw("pfGetTexturePixels")
            px.restype = C.c_void_p
            px.argtypes = [C.c_void_p] * 5
            for f in fbs:
                base = px(f.texture, None, None, None, None)
                out.append(np.ctypeslib.as_array(C.cast(base, C.POINTER(C.c_uint8)), shape=(H, W, 4)).copy())
                out.append(np.ctypeslib.as_array(f.zbuffer, shape=(H, W)).copy())
            return out
        finally:
            lib.pfDisable(A.PF_FRAMEBUFFER)
            lib.pfBindFramebuffer(None)
            for ref in refs:
                lib.pfDeleteFramebuffer(ref)
            lib.pfDeleteContext(ctx)

    got, ref = run(gpu), run(oracle)
    assert gpu.pfGetDeviceStatus() == 0
    for k, (a, b) in enumerate(zip(got, ref)):
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"buffer {k} differs in {int((a != b).sum())} values"


def test_clear_leaves_first_pixels(gpu, oracle):
    # pfClear's vector loop starts at pixel 8 and the tail copies pixel 0
    # (context.c:705-723): a 13x7 buffer (91 pixels, tail of 3).
    init = np.arange(13 * 7 * 4, dtype=np.uint32).astype(np.uint8).reshape(7, 13, 4)
    outs = []
    for lib in (gpu, oracle):
        from pixelforge_gb300.scenes import Target
        tg = Target(lib, 13, 7, "main", init=init)
        lib.pfClearColor(10, 20, 30, 40)
        lib.pfClear(A.PF_COLOR_BUFFER_BIT)
        outs.append(tg.finish().color)
        tg.close()
    assert np.array_equal(outs[0], outs[1])
    flat = outs[0].reshape(-1, 4)
    assert np.array_equal(flat[:8], init.reshape(-1, 4)[:8])
    assert (flat[8:88] == [10, 20, 30, 40]).all()
    assert np.array_equal(flat[88:], np.repeat(flat[:1], 3, 0))


def test_bin_overflow_replay(gpu, oracle):
    # thousands of full-screen triangles overflow the first tile-bin capacity;
    # the flush must grow it and replay from the failing command
    sc = SoupScene(ntris=3000, xy_range=(-6.0, 6.0), cull=False, width=64, height=64)
    got, ref = sc.render(gpu), sc.render(oracle)
    assert_parity(got, ref, exact_color=True, label="overflow")


# --- against the reference's own outputs (tests/golden) ----------------------
def _golden():
    import sys
    from pathlib import Path
    here = Path(__file__).resolve().parent / "golden"
    sys.path.insert(0, str(here))
    from cases import cases, uses_host_powf
    return np.load(here / "golden.npz"), cases(), uses_host_powf


GOLD, GOLD_CASES, GOLD_POWF = _golden()


@pytest.mark.parametrize("name", sorted(GOLD_CASES))
def test_gpu_matches_reference_golden(gpu, name):
    """Colour and depth of the GPU library against the reference build's
    (exact-reciprocal flavour) on every golden case: depth bit-exact, colour
    bit-exact except the Gouraud specular powf cases (±1 LSB)."""
    fr = GOLD_CASES[name](gpu)
    assert gpu.pfGetDeviceStatus() == 0
    gc, gd = GOLD[f"{name}.color"], GOLD[f"{name}.depth"]
    if gd.size:
        nd = int((fr.depth.view(np.uint32) != gd.view(np.uint32)).sum())
        assert nd == 0, f"{name}: {nd} depth values differ from the reference"
    diff = np.abs(fr.color.astype(np.int32) - gc.astype(np.int32))
    tol = COLOR_TOL if GOLD_POWF(name) else 0
    assert int(diff.max()) <= tol, f"{name}: colour differs by {int(diff.max())}"


@pytest.mark.parametrize("k", range(4))
def test_vertex_array_types(gpu, oracle, k):
    from mixscenes import TYPE_CASES, run_types
    assert_parity(run_types(gpu, 40 + k, TYPE_CASES[k]), run_types(oracle, 40 + k, TYPE_CASES[k]),
                  label=f"types {TYPE_CASES[k]}")


def test_tile_overfull_draw_is_split(gpu, oracle):
    """More sub-triangles in one tile than a bin can sort (16,384): the draw
    group is rendered in passes, with the same result."""
    sc = SoupScene(width=32, height=32, ntris=80000, seed=77, xy_range=(-3.0, 3.0), cull=False)
    got, ref = sc.render(gpu), sc.render(oracle)
    assert gpu.pfGetDeviceStatus() == 0
    assert got.stats["draw_splits"] >= 1
    assert_parity(got, ref, exact_color=True, label="overfull tiles")


def test_tile_overfull_draw_is_split_bgra8(gpu, oracle):
    """The same split into passes for a BGRA / unsigned-byte framebuffer
    (k_rows draws each pass on top of the previous one), alpha-blended."""
    from pixelforge_gb300.scenes import Target
    sc = SoupScene(width=32, height=24, ntris=40000, seed=78, xy_range=(-3.0, 3.0), cull=False,
                   blend=A.PF_BLEND_ALPHA)
    outs = []
    for lib in (gpu, oracle):
        tg = Target(lib, sc.width, sc.height, "fbo", fmt=FB_BGRA8)
        try:
            sc.record(lib)
            outs.append(tg.finish())
        finally:
            tg.close()
    assert gpu.pfGetDeviceStatus() == 0
    assert outs[0].stats["draw_splits"] >= 1
    assert_parity(outs[0], outs[1], exact_color=True, label="overfull tiles bgra8")


@pytest.mark.parametrize("fmt", [("BGRA", "UBYTE"), ("LUMINANCE_ALPHA", "UBYTE"), ("RGB", "HALF"), ("RGBA", "FLOAT"),
                                 ("BGRA", "S4444")])
def test_texture_formats_bilinear(gpu, oracle, fmt):
    """Non-RGBA8 textures (converted per the reference's getters when
    snapshotted) under both filters, GPU against the oracle."""
    from cases import kat_texfmt
    for filt in (A.PF_NEAREST, A.PF_BILINEAR):
        run = kat_texfmt(*fmt, filt=filt)
        assert_parity(run(gpu), run(oracle), exact_color=True, label=f"{fmt} filter {filt}")


@pytest.mark.parametrize("seed", range(0, 160))
def test_points_lines(gpu, oracle, seed):
    """Points, thin and thick lines, PF_POINT / PF_LINE polygon modes
    (immediate mode and vertex arrays): colour and depth bit-exact."""
    from lpscenes import lp_case, run_lp
    case = lp_case(seed)
    got = run_lp(gpu, case)
    assert gpu.pfGetDeviceStatus() == 0
    assert_parity(got, run_lp(oracle, case), exact_color=True, label=f"points/lines {seed} {case}")


@pytest.mark.parametrize("target", ["fbo", "main"])
def test_wireframe_1080(gpu, oracle, target):
    from lpscenes import run_wire
    got, ref = run_wire(gpu, target=target), run_wire(oracle, target=target)
    assert gpu.pfGetDeviceStatus() == 0
    assert (ref.color.reshape(-1, 4)[:, :3].any(-1)).sum() > 100000       # drawn pixels
    assert_parity(got, ref, exact_color=True, label=f"wireframe {target}")
    assert got.stats["fragments"] == ref.stats["fragments"]


@pytest.mark.parametrize("seed", range(0, 80))
def test_lists_rects_pixels_fog(gpu, oracle, seed):
    """Render lists, pfRect*, pfDrawPixels and pfFogProcess in order with
    triangles: depth bit-exact, colour exact (within 1 LSB where it goes
    through the host libm: the fog's e^x / 2^x, the lists' lit replays)."""
    from pixscenes import px_case, run_px
    case = px_case(seed)
    got = run_px(gpu, case)
    assert gpu.pfGetDeviceStatus() == 0
    assert_parity(got, run_px(oracle, case), exact_color=case["kind"] not in ("fog", "list"),
                  label=f"extras {seed} {case}")


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_lists_rects_pixels_fog_main_target(gpu, oracle, seed):
    from pixscenes import px_case, run_px
    case = px_case(seed)
    assert_parity(run_px(gpu, case, "main"), run_px(oracle, case, "main"), exact_color=case["kind"] not in ("fog", "list"),
                  label=f"extras main {seed}")


@pytest.mark.parametrize("seed", range(4))
def test_read_pixels_formats(gpu, oracle, seed):
    from pixscenes import run_readback
    a, b = run_readback(gpu, seed), run_readback(oracle, seed)
    for k in a:
        assert a[k][1] == b[k][1] == 0, k
        assert np.array_equal(a[k][0], b[k][0]), f"format/type {k}: bytes differ"


@pytest.mark.parametrize("seed,fmt", FB_SEEDS)
def test_framebuffer_formats(gpu, oracle, seed, fmt):
    """Framebuffers of every accepted format (5 seeds each, 12 for BGRA /
    unsigned byte; main buffers and framebuffer objects, odd sizes): clears
    and fills, triangles through the format's SIMD getter / setter (k_raster;
    k_rows for BGRA / unsigned byte), points, lines, rectangles and images
    through the scalar ones, linear fog and the grayscale device hook, the
    per-pixel framebuffer functions and pfReadPixels.  Raw pixels, depth and
    every read bit-exact."""
    from fbscenes import fb_case, run_fb
    case = fb_case(seed, fmt)
    a, b = run_fb(gpu, case), run_fb(oracle, case)
    assert gpu.pfGetDeviceStatus() == 0
    assert a["err"] == b["err"] == 0
    for k in ("color", "depth", "read", "get"):
        if k in b:
            x, y = a[k].view(np.uint8), b[k].view(np.uint8)
            assert np.array_equal(x, y), f"{case}: {k} differs in {int((x != y).sum())} bytes"


@pytest.mark.parametrize("fmt", [(A.PF_RGBA, A.PF_HALF_FLOAT), (A.PF_RGB, A.PF_UNSIGNED_SHORT_5_6_5),
                                 (A.PF_BGRA, A.PF_FLOAT), (A.PF_BGRA, A.PF_UNSIGNED_BYTE)])
def test_framebuffer_formats_sphere1080(gpu, oracle, fmt):
    """The textured, alpha-blended sphere at 1920x1080 (unlit: no host powf)
    into a framebuffer of another format: raw pixels and depth bit-exact
    against the oracle."""
    sc = SphereScene(filt=A.PF_NEAREST, lighting=None)
    got, ref = sc.render(gpu, "fbo", fmt=fmt), sc.render(oracle, "fbo", fmt=fmt)
    assert got.color.shape == (1080, 1920, A.pixel_bytes(*fmt))
    assert np.array_equal(got.depth.view(np.uint32), ref.depth.view(np.uint32))
    nd = int((got.color != ref.color).any(-1).sum())
    assert nd == 0, f"{fmt}: {nd} pixels differ"


def _aligned(n_bytes: int, misalign: int) -> np.ndarray:
    """A byte array whose data starts `misalign` bytes past a 64-byte boundary."""
    raw = np.zeros(n_bytes + 128, np.uint8)
    start = (-raw.ctypes.data) % 64 + misalign
    return raw[start:start + n_bytes]


@pytest.mark.parametrize("misalign", [0, 4])
def test_draw_time_snapshot_of_large_arrays(gpu, oracle, misalign):
    """Arrays of 64 KiB and more are copied during the draw call (from
    pageable memory into page-locked memory by the host workers, then by
    DMA): the caller overwrites positions, colours, texcoords, indices and
    texture right after each draw, and the image must be the one the
    reference draws from the contents at each call."""
    from pixelforge_gb300.scenes import Target, _ptr
    ntri, W, H = 20000, 256, 192
    nv = ntri * 3
    pos = _aligned(nv * 12, misalign).view(np.float32).reshape(nv, 3)
    uv = _aligned(nv * 8, misalign).view(np.float32).reshape(nv, 2)
    col = _aligned(nv * 4, misalign).reshape(nv, 4)
    idx = _aligned(nv * 4, misalign).view(np.uint32)
    tex = _aligned(256 * 256 * 4, misalign).reshape(256, 256, 4)

    def fill(seed):
        r = np.random.default_rng(seed)
        pos[...] = r.uniform(-1.1, 1.1, (nv, 3)).astype(np.float32) * np.float32([1, 1, 0.8])
        uv[...] = r.uniform(-1, 2, (nv, 2)).astype(np.float32)
        col[...] = r.integers(0, 256, (nv, 4)).astype(np.uint8)
        idx[...] = r.permutation(nv).astype(np.uint32)
        tex[...] = r.integers(0, 256, (256, 256, 4)).astype(np.uint8)

    def run(lib):
        tg = Target(lib, W, H, "fbo")
        th = None
        try:
            lib.pfDisable(A.PF_CULL_FACE)
            lib.pfEnable(A.PF_DEPTH_TEST)
            lib.pfEnable(A.PF_BLEND)
            lib.pfBlendFunc(A.PF_BLEND_ALPHA)
            lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
            th = lib.pfGenTexture(_ptr(tex), 256, 256, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
            lib.pfBindTexture(th)
            lib.pfEnable(A.PF_TEXTURE_2D)
            lib.pfEnable(A.PF_VERTEX_ARRAY | A.PF_TEXTURE_COORD_ARRAY | A.PF_COLOR_ARRAY)
            lib.pfVertexPointer(3, A.PF_FLOAT, 0, _ptr(pos))
            lib.pfTexCoordPointer(A.PF_FLOAT, 0, _ptr(uv))
            lib.pfColorPointer(4, A.PF_UNSIGNED_BYTE, 0, _ptr(col))
            for seed in (1, 2, 3):
                fill(seed)
                lib.pfDrawElements(A.PF_TRIANGLES, nv // (1 + seed % 2), A.PF_UNSIGNED_INT, _ptr(idx))
            fill(99)                                   # after the last draw, before the flush
            return tg.finish()
        finally:
            if th:
                h = C.c_void_p(th)
                lib.pfDeleteTexture(C.byref(h), False)
            tg.close()

    import ctypes as C
    got, ref = run(gpu), run(oracle)
    assert gpu.pfGetDeviceStatus() == 0
    assert (ref.depth < 1e30).sum() > 10000
    assert_parity(got, ref, exact_color=True, label=f"snapshot misalign={misalign}")


def test_draw_time_snapshot_reuse_and_pinned_texture(gpu, oracle):
    """Within one recording a later draw reuses the copy of an array it
    references again unchanged (here the indices, and positions on some
    draws) and copies again what changed; a texture of 1 MiB and more is
    page-locked on its second draw and copied by DMA from then on -- the
    caller changes it between draws too.  Every draw must see the contents
    at its own call."""
    from pixelforge_gb300.scenes import Target, _ptr
    import ctypes as C
    ntri, W, H = 20000, 256, 192
    nv = ntri * 3
    r0 = np.random.default_rng(7)
    pos = r0.uniform(-1.1, 1.1, (nv, 3)).astype(np.float32) * np.float32([1, 1, 0.8])
    uv = r0.uniform(-1, 2, (nv, 2)).astype(np.float32)
    idx = r0.permutation(nv).astype(np.uint32)
    tex = r0.integers(0, 256, (512, 512, 4)).astype(np.uint8)      # 1 MiB

    def run(lib):
        tg = Target(lib, W, H, "fbo")
        th = None
        try:
            lib.pfDisable(A.PF_CULL_FACE)
            lib.pfEnable(A.PF_DEPTH_TEST)
            lib.pfEnable(A.PF_BLEND)
            lib.pfBlendFunc(A.PF_BLEND_ALPHA)
            lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
            th = lib.pfGenTexture(_ptr(tex), 512, 512, A.PF_RGBA, A.PF_UNSIGNED_BYTE)
            lib.pfBindTexture(th)
            lib.pfEnable(A.PF_TEXTURE_2D)
            lib.pfEnable(A.PF_VERTEX_ARRAY | A.PF_TEXTURE_COORD_ARRAY)
            lib.pfVertexPointer(3, A.PF_FLOAT, 0, _ptr(pos))
            lib.pfTexCoordPointer(A.PF_FLOAT, 0, _ptr(uv))
            r = np.random.default_rng(11)
            for k in range(5):
                # indices never change; positions on draws 2 and 4; the
                # texture's top rows on every draw after the first
                if k in (2, 4):
                    pos[:, 2] = r.uniform(-0.8, 0.8, nv).astype(np.float32)
                if k > 0:
                    tex[: 16 * k] = r.integers(0, 256, (16 * k, 512, 4)).astype(np.uint8)
                lib.pfColor4ub(255, 255 - 40 * k, 255, 160)
                lib.pfDrawElements(A.PF_TRIANGLES, nv, A.PF_UNSIGNED_INT, _ptr(idx))
            return tg.finish()
        finally:
            if th:
                h = C.c_void_p(th)
                lib.pfDeleteTexture(C.byref(h), False)
            tg.close()

    saved = (pos.copy(), tex.copy())
    got = run(gpu)
    pos[...], tex[...] = saved
    ref = run(oracle)
    assert gpu.pfGetDeviceStatus() == 0
    assert (ref.depth < 1e30).sum() > 10000
    assert_parity(got, ref, exact_color=True, label="snapshot reuse and pinned texture")


def test_ragged_framebuffers(gpu, oracle):
    """Framebuffers of 1 to 165 pixels in six formats (main buffers and
    framebuffer objects): raw pixels, depth and reads bit-exact against the
    oracle."""
    from fbscenes import TINY_CASES, run_fb, tiny_case
    for k in range(TINY_CASES):
        case = tiny_case(k)
        a, b = run_fb(gpu, case), run_fb(oracle, case)
        assert gpu.pfGetDeviceStatus() == 0
        for key in ("color", "depth", "read", "get"):
            if key in b:
                x, y = a[key].view(np.uint8), b[key].view(np.uint8)
                assert np.array_equal(x, y), f"{case}: {key} differs in {int((x != y).sum())} bytes"


def test_large_framebuffer_and_empty_draws(gpu, oracle):
    """An 8192x4096 framebuffer object (524,288 tiles): clear, blended and
    depth-tested triangles, empty draws (a pfBegin/pfEnd without vertices,
    pfDrawArrays of 0 and of 2 vertices), points; colour and depth bit-exact
    against the oracle."""
    import ctypes as C
    from pixelforge_gb300.scenes import Target, _ptr

    def run(lib):
        r = np.random.default_rng(4242)
        tg = Target(lib, 8192, 4096, "fbo")
        try:
            lib.pfClearColor(10, 20, 30, 255)
            lib.pfClear(A.PF_COLOR_BUFFER_BIT | A.PF_DEPTH_BUFFER_BIT)
            lib.pfDisable(A.PF_CULL_FACE)
            lib.pfEnable(A.PF_DEPTH_TEST)
            lib.pfEnable(A.PF_BLEND)
            lib.pfBlendFunc(A.PF_BLEND_ALPHA)
            lib.pfBegin(A.PF_TRIANGLES)
            lib.pfEnd()                                        # no vertices
            pos = r.uniform(-1, 1, (6, 3)).astype(np.float32)
            lib.pfEnable(A.PF_VERTEX_ARRAY)
            lib.pfVertexPointer(3, A.PF_FLOAT, 0, _ptr(pos))
            lib.pfDrawArrays(A.PF_TRIANGLES, 0, 0)             # nothing
            lib.pfDrawArrays(A.PF_TRIANGLES, 0, 2)             # less than a triangle
            lib.pfDisable(A.PF_VERTEX_ARRAY)
            lib.pfBegin(A.PF_TRIANGLES)
            for _ in range(24):
                c = r.integers(0, 256, 4)
                lib.pfColor4ub(int(c[0]), int(c[1]), int(c[2]), int(r.integers(100, 256)))
                for _k in range(3):
                    p = r.uniform(-1.1, 1.1, 2)
                    lib.pfVertex3f(float(p[0]) * 0.6, float(p[1]) * 0.6, float(r.uniform(-0.9, 0.9)))
            lib.pfEnd()
            lib.pfPointSize(3.0)
            lib.pfBegin(A.PF_POINTS)
            for _ in range(50):
                p = r.uniform(-1, 1, 2)
                lib.pfVertex2f(float(p[0]), float(p[1]))
            lib.pfEnd()
            return tg.finish()
        finally:
            tg.close()

    got, ref = run(gpu), run(oracle)
    assert gpu.pfGetDeviceStatus() == 0
    assert (ref.depth < 1e30).sum() > 1_000_000
    assert_parity(got, ref, exact_color=True, label="8192x4096")
