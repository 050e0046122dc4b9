"""Textures, uv rects and vertex normals (shading.glsl:125-176) on the GPU against the oracle: the
exact-mode image (raster-pass and pixel-parallel blend), the reference-order mode (lit, vertex
normals) bit for bit, batched views, and gradients through textured colours."""
import numpy as np
import pytest

from lucid_gb300 import scenes

pytestmark = pytest.mark.gpu

CASES = {
    "rgba8_rects_normals": dict(seed=1),
    "fp16_no_rects": dict(seed=2, uv_rects=False, color_format=scenes.COLOR_RGBA16F),
    "fp32_opacity_all_transparent": dict(seed=3, opaque_fraction=0.0, color_format=scenes.COLOR_RGBA32F,
                                         tri_opacity_range=(0.2, 0.9)),
    "big_texture_no_normals": dict(seed=4, vertex_normals=False, tex_size=(256, 128)),
}


def _renderer(sc, flags=0, **kw):
    from lucid_gb300.renderer import LucidRenderer
    return LucidRenderer(sc.width, sc.height, max_input_quads=max(1024, sc.num_quads),
                         max_visible_quads=max(1024, sc.num_quads), flags=flags, **kw)


@pytest.mark.parametrize("name", sorted(CASES))
def test_textured_exact_mode(gpu, oracle, name):
    from lucid_gb300 import _lib
    from lucid_gb300.renderer import FrameInputs
    sc = scenes.textured_scene(**CASES[name])
    ref = oracle.run(sc)["image"]
    for flags in (0, _lib.OPT_PIXEL_BLEND):
        r = _renderer(sc, flags)
        img = r.render(FrameInputs.from_scene(sc)).cpu().numpy()
        r.close()
        assert np.abs(img - ref).max() <= 1e-5, (flags, np.abs(img - ref).max())


@pytest.mark.parametrize("name", sorted(CASES))
def test_textured_reference_order(gpu, oracle, name):
    from lucid_gb300 import _lib
    from lucid_gb300.renderer import FrameInputs
    sc = scenes.textured_scene(**CASES[name])
    ref = oracle.run(sc, order_mode=1, flags=8)
    r = _renderer(sc, _lib.OPT_REFERENCE_ORDER | 8)
    img = r.render(FrameInputs.from_scene(sc)).cpu().numpy()
    info, _ = r.info()
    r.close()
    np.testing.assert_array_equal(img, ref["image"])
    assert int(info.stats[2]) == ref["invalid_pixels"]


def test_textured_batch_matches_single(gpu):
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    views = [scenes.textured_scene(**CASES[n]) for n in sorted(CASES)]
    total = sum(v.num_quads for v in views)
    br = LucidRenderer(max(v.width for v in views), max(v.height for v in views), max_input_quads=total,
                       max_visible_quads=total, max_views=len(views))
    frames = [(FrameInputs.from_scene(v), v.width, v.height) for v in views]
    imgs = br.render_batch(frames)
    for v, (f, _, _), im in zip(views, frames, imgs):
        r = _renderer(v)
        np.testing.assert_array_equal(im.cpu().numpy(), r.render(f).cpu().numpy())
        r.close()
    br.close()


def test_textured_gradients(gpu, oracle):
    """Vertex-colour and opacity gradients through texture x vertex colour (the texture factor
    multiplies the vertex colour terms) against the oracle's FP64 analytic gradient."""
    import torch
    from lucid_gb300 import autograd
    from lucid_gb300.renderer import FrameInputs
    sc = scenes.textured_scene(seed=5, width=96, height=64, num_tris=300, color_format=scenes.COLOR_RGBA32F,
                               tri_opacity_range=(0.1, 0.9))
    target = np.random.default_rng(0).random((sc.height, sc.width, 4)).astype(np.float32)
    r = _renderer(sc)
    frame = FrameInputs.from_scene(sc)
    vc = torch.from_numpy(sc.colors.astype(np.float32)).cuda().requires_grad_(True)
    op = torch.from_numpy(sc.tri_opacity.astype(np.float32)).cuda().requires_grad_(True)
    img = autograd.render(vc, op, r, frame)
    ((img[..., :3] - torch.from_numpy(target).cuda()[..., :3]) ** 2).sum().backward()
    model = oracle.GradModel(sc)
    dvc, dop = model.analytic(sc.colors.astype(np.float64), sc.tri_opacity.astype(np.float64), target)
    g, ref = vc.grad.cpu().numpy().ravel().astype(np.float64), dvc.ravel()
    scale = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    assert (np.abs(g - ref) / scale).max() <= 1e-4
    go = op.grad.cpu().numpy().astype(np.float64)
    scale = np.maximum(np.abs(dop), 1e-3 * np.abs(dop).max())
    assert (np.abs(go - dop) / scale).max() <= 1e-4
    r.close()


def test_texture_kat_on_gpu(gpu, oracle):
    from tests.test_oracle import _textured_quad_scene
    from lucid_gb300.renderer import FrameInputs
    sc, _ = _textured_quad_scene()
    r = _renderer(sc)
    img = r.render(FrameInputs.from_scene(sc)).cpu().numpy()
    r.close()
    np.testing.assert_array_equal(img, oracle.run(sc)["image"])
