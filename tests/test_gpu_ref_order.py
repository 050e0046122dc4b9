"""Reference-order mode on the GPU (LUCID_OPT_REFERENCE_ORDER) against the oracle's
order_mode 1: image bits, per-pixel sample counts and order, fragment statistics and the
invalid-pixel count of the depth-4 error window, on LOW, promoted and HIGH bins, every colour
format, opacity, additive blending and a mesh scene."""
import numpy as np
import pytest

from lucid_gb300 import scenes

pytestmark = pytest.mark.gpu

VIS, ADD = 8, 2

CASES = {
    "low": (lambda: scenes.random_tris(160, 96, 1500, seed=31, area_median=150.0), 0, 1024),
    "low_errors_fp16": (lambda: scenes.random_tris(128, 96, 1200, seed=32, color_format=scenes.COLOR_RGBA16F,
                                                   area_median=200.0), VIS, 1024),
    "high_fp32_opacity": (lambda: scenes.random_tris(96, 64, 4000, seed=33, color_format=scenes.COLOR_RGBA32F,
                                                     tri_opacity_range=(0.1, 0.9), area_median=300.0,
                                                     background=(0.1, 0.2, 0.3, 1.0)), VIS, 256),
    # LOW bins by count whose densest 8x8 block holds > 256 tris: promoted to the HIGH path
    "promoted": (lambda: scenes.random_tris(64, 64, 400, seed=34, center_sigma=3.0, area_median=30.0,
                                            area_sigma=0.5), VIS, 1024),
    "additive": (lambda: scenes.random_tris(96, 64, 1500, seed=35, alpha_range=(0.02, 0.1), area_median=200.0),
                 ADD, 256),
    "meshes": (lambda: scenes.meshes(320, 180, num_meshes=6, seed=36), VIS, 1024),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_reference_order_matches_oracle(gpu, oracle, name):
    from lucid_gb300 import _lib
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    make, flags, threshold = CASES[name]
    sc = make()
    mpp = 64
    ref = oracle.run(sc, order_mode=1, max_per_pixel=mpp, flags=flags, low_high_threshold=threshold)
    r = LucidRenderer(sc.width, sc.height, max_input_quads=max(1024, sc.num_quads),
                      max_visible_quads=max(1024, sc.num_quads), flags=flags | _lib.OPT_REFERENCE_ORDER,
                      low_high_threshold=threshold)
    f = FrameInputs.from_scene(sc)
    img = r.render(f).cpu().numpy()
    info, _ = r.info()
    np.testing.assert_array_equal(img, ref["image"])
    assert info.error_code == 0
    assert int(info.num_fragments) == ref["num_fragments"]
    assert int(info.num_hblock_tris) == ref["num_hblock_tris"]
    assert int(info.stats[2]) == ref["invalid_pixels"]
    if name == "promoted":
        assert ref["bin_level_counts"][2] == 4  # all LOW by count, all promoted
    _, counts, prims = r.raster_dump(f, mpp)
    np.testing.assert_array_equal(counts, ref["frag_counts"])
    k = np.minimum(counts, mpp)
    mask = np.arange(mpp)[None, None, :] < k[..., None]
    np.testing.assert_array_equal(np.where(mask, prims, -1), np.where(mask, ref["frag_prims"], -1))
    r.close()


def test_reference_order_rejects_unsupported(gpu):
    import torch
    from lucid_gb300 import _lib
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    sc = scenes.small_scene(32, 32, 50, seed=1)
    r = LucidRenderer(32, 32, max_input_quads=1024, max_visible_quads=1024,
                      flags=_lib.OPT_REFERENCE_ORDER | _lib.OPT_ALPHA_THRESHOLD)
    with pytest.raises(_lib.LucidError) as e:
        r.render(FrameInputs.from_scene(sc))
    assert e.value.status == _lib.NOT_SUPPORTED
    r.close()
