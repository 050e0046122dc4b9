"""Batched multi-view rendering (lucid_render_batch): every view's image and device statistics
equal those of lucid_render of that view alone (the batch runs the same per-view arithmetic),
across mixed sizes, colour formats, opacities, backgrounds, empty views and replays."""
import numpy as np
import pytest

from lucid_gb300 import scenes

pytestmark = pytest.mark.gpu


def _mixed_views():
    views = [
        scenes.random_tris(256, 256, 3000, seed=11),
        scenes.random_tris(512, 512, 20000, seed=12, color_format=scenes.COLOR_RGBA16F),
        scenes.random_tris(320, 200, 8000, seed=13, color_format=scenes.COLOR_RGBA32F,
                           tri_opacity_range=(0.1, 0.9), background=(0.2, 0.3, 0.4, 1.0)),
        scenes.random_tris(1280, 720, 40000, seed=14, center_sigma=200.0, area_median=200.0,
                           area_sigma=1.5, large_fraction=0.02),
        scenes.random_tris(96, 72, 0, seed=15),                      # no geometry
        scenes.random_tris(700, 333, 5000, seed=16, area_median=2000.0),  # ragged bins, big tris
        scenes.meshes(640, 360, num_meshes=6, seed=17),
    ]
    return views


def _single(sc):
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    r = LucidRenderer(sc.width, sc.height, max_input_quads=max(1024, sc.num_quads),
                      max_visible_quads=max(1024, sc.num_quads))
    img = r.render(FrameInputs.from_scene(sc)).cpu().numpy()
    info, _ = r.info()
    r.close()
    return img, info


def _batch_renderer(views, **kw):
    from lucid_gb300.renderer import LucidRenderer
    w = max(v.width for v in views)
    h = max(v.height for v in views)
    total = sum(max(1, v.num_quads) for v in views)
    return LucidRenderer(w, h, max_input_quads=total, max_visible_quads=total, max_views=len(views), **kw)


def _check_same(views, r, imgs):
    for i, sc in enumerate(views):
        ref, rinfo = _single(sc)
        np.testing.assert_array_equal(imgs[i].cpu().numpy(), ref, err_msg=f"view {i}")
        binfo = r.batch_info(i)
        assert binfo.error_code == 0, (i, binfo.error_code)
        assert int(binfo.num_fragments) == int(rinfo.num_fragments), i
        assert tuple(binfo.num_visible_quads) == tuple(rinfo.num_visible_quads), i
        assert int(binfo.num_bin_quad_refs) == int(rinfo.num_bin_quad_refs), i
        assert int(binfo.num_bin_tri_refs) == int(rinfo.num_bin_tri_refs), i
        assert tuple(binfo.bin_level_counts) == tuple(rinfo.bin_level_counts), i
        assert int(binfo.max_pixel_fragments) == int(rinfo.max_pixel_fragments), i


def test_batch_matches_single_views(gpu):
    from lucid_gb300.renderer import FrameInputs
    views = _mixed_views()
    r = _batch_renderer(views)
    frames = [(FrameInputs.from_scene(v), v.width, v.height) for v in views]
    imgs = r.render_batch(frames)
    _check_same(views, r, imgs)
    # replay of the recorded graph into the same outputs
    for im in imgs:
        im.fill_(-1.0)
    imgs2 = r.render_batch(frames, outs=imgs)
    _check_same(views, r, imgs2)
    r.close()


def test_batch_replay_sees_new_contents_and_configs(gpu):
    import torch
    from lucid_gb300.renderer import FrameInputs
    views = _mixed_views()[:4]
    r = _batch_renderer(views)
    frames = [(FrameInputs.from_scene(v), v.width, v.height) for v in views]
    r.render_batch(frames)
    # new colours in the same buffers (graph replay, unchanged parameters)
    rng = np.random.default_rng(5)
    new_views = []
    for (f, _, _), v in zip(frames, views):
        cols = v.colors.copy()
        if cols.dtype == np.uint32:
            cols = rng.integers(0, 2**32, size=cols.shape, dtype=np.uint64).astype(np.uint32)
        else:
            cols = rng.random(cols.shape).astype(cols.dtype)
        f.colors.copy_(torch.from_numpy(cols.view(np.int32) if cols.dtype == np.uint32 else cols))
        new_views.append(scenes.Scene(**{**v.__dict__, "colors": cols}))
    imgs = r.render_batch(frames)
    _check_same(new_views, r, imgs)
    # a new config per view (parameter change: restaged, same graph)
    cfgs = []
    for (f, _, _), v in zip(frames, new_views):
        cfg = scenes.make_config(scenes.Camera(), v.width, v.height, background=(0.5, 0.25, 0.125, 1.0))
        f.config = cfg
        cfgs.append(scenes.Scene(**{**v.__dict__, "config": cfg}))
    imgs = r.render_batch(frames)
    _check_same(cfgs, r, imgs)
    r.close()


def test_batch_topology_change_and_limits(gpu):
    from lucid_gb300 import _lib
    from lucid_gb300.renderer import FrameInputs
    views = _mixed_views()
    r = _batch_renderer(views)
    f = [(FrameInputs.from_scene(v), v.width, v.height) for v in views]
    _check_same(views[:3], r, r.render_batch(f[:3]))
    _check_same(views[2:], r, r.render_batch(f[2:]))
    with pytest.raises(_lib.LucidError) as e:
        r.render_batch(f + f)  # more views than options.max_views
    assert e.value.status == _lib.CAPACITY_EXCEEDED
    r.close()
    small = _batch_renderer(views[:2])
    with pytest.raises(_lib.LucidError) as e:
        small.render_batch(f[:1] + f[3:4])  # quads beyond the renderer's capacity / size
    assert e.value.status in (_lib.CAPACITY_EXCEEDED, _lib.INVALID_ARG)
    small.close()


def test_batch_views_match_oracle(gpu, oracle):
    """The batch against the CPU oracle directly (not only against single-view GPU renders):
    every view's image within 1e-5 and its fragment and visible-quad counts equal."""
    from lucid_gb300.renderer import FrameInputs
    views = _mixed_views()
    r = _batch_renderer(views)
    imgs = r.render_batch([(FrameInputs.from_scene(v), v.width, v.height) for v in views])
    for i, sc in enumerate(views):
        o = oracle.run(sc, max_visible_quads=max(1024, sc.num_quads), setup_outputs=False)
        assert np.abs(imgs[i].cpu().numpy() - o["image"]).max() <= 1e-5, i
        info = r.batch_info(i)
        assert int(info.num_fragments) == o["num_fragments"], i
        assert tuple(info.num_visible_quads) == tuple(o["num_visible"]), i
    r.close()


def test_batch_after_single_view_autotune(gpu):
    """A batch renderer tuned on one of its views (the bench's C3 arm) still renders every view
    exactly: the tuner leaves the pixel-parallel blend out for batch renderers."""
    from lucid_gb300.renderer import FrameInputs
    views = _mixed_views()[:4]
    r = _batch_renderer(views)
    frames = [(FrameInputs.from_scene(v), v.width, v.height) for v in views]
    full = [i for i, v in enumerate(views) if (v.width, v.height) == (r.width, r.height)]
    assert full
    tuned = r.autotune(frames[full[0]][0])
    assert tuned["pixel_blend"] == 0
    imgs = r.render_batch(frames)
    # the tuned bin size and LOW/HIGH threshold change the bin statistics, not the frame
    for i, sc in enumerate(views):
        ref, rinfo = _single(sc)
        np.testing.assert_array_equal(imgs[i].cpu().numpy(), ref, err_msg=f"view {i}")
        binfo = r.batch_info(i)
        assert binfo.error_code == 0, (i, binfo.error_code)
        assert int(binfo.num_fragments) == int(rinfo.num_fragments), i
        assert int(binfo.max_pixel_fragments) == int(rinfo.max_pixel_fragments), i
    r.close()


def test_autotune_batch(gpu):
    """lucid_autotune_batch times the batch itself; the tuned batch renders every view exactly."""
    from lucid_gb300.renderer import FrameInputs
    views = _mixed_views()
    r = _batch_renderer(views)
    frames = [(FrameInputs.from_scene(v), v.width, v.height) for v in views]
    tuned = r.autotune_batch(frames)
    assert tuned["pixel_blend"] == 0 and tuned["bin_size"] in (32, 64)
    assert tuned["num_candidates"] >= 8
    assert tuned["frame_ms"] <= tuned["default_ms"]
    imgs = r.render_batch(frames)
    for i, sc in enumerate(views):
        ref, rinfo = _single(sc)
        np.testing.assert_array_equal(imgs[i].cpu().numpy(), ref, err_msg=f"view {i}")
        binfo = r.batch_info(i)
        assert binfo.error_code == 0, (i, binfo.error_code)
        assert int(binfo.num_fragments) == int(rinfo.num_fragments), i
    r.close()
