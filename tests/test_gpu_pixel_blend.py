"""Pixel-parallel blend (LUCID_OPT_PIXEL_BLEND) and the autotuner: the raster pass in store mode
plus the pixel-parallel blend gives the same image bits as the raster pass's own blend, for
every blend variant, colour format, deep (windowed) pixels and a store too small for the frame
(device-side fallback to the raster pass's blend); lucid_autotune keeps the image bits."""
import numpy as np
import pytest

from lucid_gb300 import scenes

pytestmark = pytest.mark.gpu


def _render(sc, flags=0, **kw):
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    r = LucidRenderer(sc.width, sc.height, max_input_quads=max(1024, sc.num_quads),
                      max_visible_quads=max(1024, sc.num_quads), flags=flags, **kw)
    img = r.render(FrameInputs.from_scene(sc)).cpu().numpy()
    info, _ = r.info()
    r.close()
    return img, info


SCENES = {
    "cpu_like": lambda: scenes.random_tris(320, 200, 6000, seed=21),
    "fp16": lambda: scenes.random_tris(256, 160, 5000, seed=22, color_format=scenes.COLOR_RGBA16F),
    "fp32_opacity": lambda: scenes.random_tris(200, 150, 4000, seed=23, color_format=scenes.COLOR_RGBA32F,
                                               tri_opacity_range=(0.1, 0.9), background=(0.3, 0.2, 0.1, 1.0)),
    "deep": lambda: scenes.random_tris(128, 96, 6000, seed=24, area_median=3000.0, area_sigma=0.5,
                                       alpha_range=(0.02, 0.05)),
    "meshes": lambda: scenes.meshes(480, 270, num_meshes=8, seed=25),
}


@pytest.mark.parametrize("name", sorted(SCENES))
@pytest.mark.parametrize("flags", [0, 2, 4])  # plain, additive, alpha threshold
def test_pixel_blend_matches_raster_blend(gpu, name, flags):
    from lucid_gb300 import _lib
    sc = SCENES[name]()
    a, ia = _render(sc, flags)
    b, ib = _render(sc, flags | _lib.OPT_PIXEL_BLEND)
    np.testing.assert_array_equal(a, b)
    assert ib.error_code == 0
    assert int(ia.num_fragments) == int(ib.num_fragments)
    assert int(ia.max_pixel_fragments) == int(ib.max_pixel_fragments)


def test_pixel_blend_store_overflow_falls_back(gpu):
    from lucid_gb300 import _lib
    sc = SCENES["cpu_like"]()
    a, _ = _render(sc)
    b, info = _render(sc, _lib.OPT_PIXEL_BLEND, grad_store_fragments=5000)
    np.testing.assert_array_equal(a, b)
    assert info.error_code == 0
    c, _ = _render(sc, _lib.OPT_PIXEL_BLEND, grad_store_fragments=-1)
    np.testing.assert_array_equal(a, c)


def test_pixel_blend_matches_oracle(gpu, oracle):
    from lucid_gb300 import _lib
    sc = SCENES["fp32_opacity"]()
    b, _ = _render(sc, _lib.OPT_PIXEL_BLEND)
    ref = oracle.run(sc)["image"]
    assert np.abs(b - ref).max() <= 1e-5


def test_autotune_keeps_image(gpu):
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    sc = scenes.random_tris(640, 360, 30000, seed=26)
    r = LucidRenderer(sc.width, sc.height, max_input_quads=sc.num_quads, max_visible_quads=sc.num_quads)
    f = FrameInputs.from_scene(sc)
    before = r.render(f).cpu().numpy()
    t = r.autotune(f)
    assert t["num_candidates"] >= 9
    assert 0.0 < t["frame_ms"] <= t["default_ms"]
    assert t["low_high_threshold"] in (256, 1024, 4096)
    assert t["light_max_pixel"] in (-1, 32, 64, 128, 256)
    after = r.render(f).cpu().numpy()
    np.testing.assert_array_equal(before, after)
    r.close()
