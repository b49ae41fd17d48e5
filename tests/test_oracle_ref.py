"""The CPU oracle against the reference itself, live (x86-64 with the
reference sources present): bit-exact colour and depth on seeded mixed
scenes beyond the committed golden set, and on the soup workload variants.
The reference is the exact-reciprocal build (oracle/_ref/libpf_shim.so);
bilinear filtering is excluded (the reference's bilinear lerp reads an
uninitialised vector)."""
import numpy as np
import pytest

from fbscenes import FB_BGRA8, FB_SEEDS
from mixscenes import mix_case, run_mix
from pixelforge_gb300 import abi as A
from pixelforge_gb300.scenes import SoupScene


def same(a, b, label):
    assert np.array_equal(a.color, b.color), f"{label}: colour differs on {int((a.color != b.color).any(-1).sum())} pixels"
    if a.depth is not None:
        assert np.array_equal(a.depth.view(np.uint32), b.depth.view(np.uint32)), f"{label}: depth differs"


@pytest.mark.parametrize("seed", range(100, 220))
def test_oracle_equals_reference_mixed(oracle, ref_shim, seed):
    case = mix_case(seed)
    same(run_mix(oracle, case), run_mix(ref_shim, case), f"mix {seed}")


@pytest.mark.parametrize("kw", [dict(), dict(cull=False), dict(shade=A.PF_FLAT), dict(depth_func=A.PF_GREATER, clear_depth=-1.0),
                                dict(blend=A.PF_BLEND_ADD), dict(blend=A.PF_BLEND_SCREEN, cull=False)])
def test_oracle_equals_reference_soup(oracle, ref_shim, kw):
    sc = SoupScene(**kw)
    same(sc.render(oracle), sc.render(ref_shim), f"soup {kw}")


@pytest.mark.parametrize("name", ["sphere1080_nearest", "phong1080_nofog"])
def test_oracle_equals_reference_full_size(oracle, ref_shim, name):
    """The 1080p workloads at full size, without the library's extensions
    (depth writes on in the sphere's second draw, no device fog): the sphere
    with nearest filtering (the reference's bilinear lerp is unpinned) and
    the 1.3 M-triangle Phong scene with eight lights, colour and depth
    bit-exact."""
    from pixelforge_gb300.scenes import PhongScene, SphereScene
    sc = (SphereScene(filt=A.PF_NEAREST, depth_mask_off=False) if name.startswith("sphere")
          else PhongScene(fog=False))
    same(sc.render(oracle, "fbo"), sc.render(ref_shim, "fbo"), name)


@pytest.mark.parametrize("k", range(4))
def test_oracle_equals_reference_array_types(oracle, ref_shim, k):
    from mixscenes import TYPE_CASES, run_types
    a, b = run_types(oracle, 40 + k, TYPE_CASES[k]), run_types(ref_shim, 40 + k, TYPE_CASES[k])
    assert (a.depth < 1e29).sum() > 500
    same(a, b, f"types {TYPE_CASES[k]}")


@pytest.mark.parametrize("seed", range(0, 160))
def test_oracle_equals_reference_points_lines(oracle, ref_shim, seed):
    from lpscenes import lp_case, run_lp
    case = lp_case(seed)
    same(run_lp(oracle, case), run_lp(ref_shim, case), f"points/lines {seed} {case}")


@pytest.mark.parametrize("seed", range(0, 80))
def test_oracle_equals_reference_lists_rects_pixels_fog(oracle, ref_shim, seed):
    """Render lists, pfRect*, pfDrawPixels (every source format, zooms,
    depth test and blending) and pfFog* / pfFogProcess, interleaved with
    triangles."""
    from pixscenes import px_case, run_px
    case = px_case(seed)
    same(run_px(oracle, case), run_px(ref_shim, case), f"extras {seed} {case}")


@pytest.mark.parametrize("seed", range(4))
def test_oracle_equals_reference_read_pixels(oracle, ref_shim, seed):
    """pfReadPixels into every format / type with a setter, regions partly
    outside the framebuffer."""
    from pixscenes import run_readback
    a, b = run_readback(oracle, seed), run_readback(ref_shim, seed)
    for k in a:
        assert a[k][1] == b[k][1] == 0, k
        assert np.array_equal(a[k][0], b[k][0]), f"format/type {k}: bytes differ"


@pytest.mark.parametrize("seed", range(6000, 6040))
def test_oracle_equals_reference_mixed_bgra(oracle, ref_shim, seed):
    """Feature-mix scenes (projections, clipping, culling, flat / smooth,
    texture wraps, Gouraud and Phong lighting, draw modes, blending) into a
    BGRA / unsigned-byte framebuffer, whose SIMD setter writes each 4-pixel
    half vector with the value computed for its first pixel."""
    case = mix_case(seed)
    for target in ("fbo", "main"):
        a = run_mix(oracle, case, target, fmt=FB_BGRA8)
        b = run_mix(ref_shim, case, target, fmt=FB_BGRA8)
        same(a, b, f"{case} {target}")


@pytest.mark.parametrize("seed,fmt", FB_SEEDS)
def test_oracle_equals_reference_framebuffer_formats(oracle, ref_shim, seed, fmt):
    """Framebuffers of every accepted format (5 seeds each, 12 for BGRA /
    unsigned byte): clears and fills, triangles through the SIMD getter /
    setter, points, lines, rectangles and images through the scalar ones,
    fog, the per-pixel framebuffer functions and pfReadPixels; raw pixels
    bit-exact."""
    from fbscenes import fb_case, run_fb
    case = fb_case(seed, fmt)
    a, b = run_fb(oracle, case, device_hook=False), run_fb(ref_shim, case, device_hook=False)
    assert a["err"] == b["err"]
    for k in ("color", "depth", "read", "get"):
        if k in a:
            assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), f"{case}: {k} differs"


def test_oracle_equals_reference_ragged_framebuffers(oracle, ref_shim):
    """Framebuffers of 1 to 165 pixels (single rows and columns, fewer pixels
    than pfClear's 8-wide vector) in six formats: raw bytes bit-exact."""
    from fbscenes import TINY_CASES, run_fb, tiny_case
    for k in range(TINY_CASES):
        case = tiny_case(k)
        a, b = run_fb(oracle, case, device_hook=False), run_fb(ref_shim, case, device_hook=False)
        for key in ("color", "depth", "read", "get"):
            if key in a:
                assert np.array_equal(a[key].view(np.uint8), b[key].view(np.uint8)), f"{case}: {key} differs"


def _soup_then_hook(lib, hook, width=250, height=131):
    from pixelforge_gb300.scenes import Target
    sc = SoupScene(width=width, height=height, ntris=400)
    tg = Target(lib, width, height, "fbo")
    try:
        sc.record(lib)
        hook(lib)
        return tg.finish()
    finally:
        tg.close()


def test_oracle_dither_hook_equals_reference_post_process(oracle, ref_shim):
    """The dither device hook (examples/raylib/raylib_PostProcess.c:7-19)
    against the reference's own pfPostProcess driving the same per-pixel
    function: pixel order, column/row arguments and the scalar getter and
    setter around the hook."""
    import ctypes as C
    fn = C.cast(oracle.raw("pfref_dither_hook"), C.c_void_p).value
    post = ref_shim.raw("pfPostProcess")
    post.argtypes = [C.c_void_p]
    post.restype = None
    a = _soup_then_hook(oracle, lambda lib: lib.pfPostProcessDevice(A.PF_HOOK_DITHER, None, 0))
    b = _soup_then_hook(ref_shim, lambda lib: post(fn))
    assert 0 < int((a.color[..., 0] == 255).sum()) < a.color.shape[0] * a.color.shape[1]
    same(a, b, "dither")
