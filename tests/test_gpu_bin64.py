"""64-pixel bins (lucid_options.bin_size = 64, the size LucidRenderer's constructor keeps as a
commented-out option, src/lucid_renderer.cpp:190): binning runs on a 64-pixel grid and the
raster pass takes each bin as its four 32x32 tiles. The exact-order image does not depend on
the bin size, so every frame must be bit-identical to the 32-pixel frame (which the parity
tests pin to the oracle) and to the oracle itself; per-pixel fragment lists and their order
must be the same; the 64-pixel small-quad lists must be exactly the union of the 32-pixel
lists of the bin's four sub-bins, and its large-tri lists a superset of theirs (the bin
scanline of bin_counter.glsl is conservative per bin row)."""
import numpy as np
import pytest

from lucid_gb300 import scenes
from tests import helpers

pytestmark = pytest.mark.gpu


def _renderer(sc, bin_size, **kw):
    from lucid_gb300.renderer import LucidRenderer
    from lucid_gb300 import _lib
    nq = max(1024, sc.num_quads)
    kw.setdefault("flags", 0)
    kw["flags"] |= _lib.OPT_SORTED_BIN_LISTS
    return LucidRenderer(sc.width, sc.height, max_input_quads=nq, max_visible_quads=nq,
                         max_bin_refs=max(1 << 16, 8 * nq), bin_size=bin_size, **kw)


def _render(sc, bin_size, dump=0, **kw):
    from lucid_gb300.renderer import FrameInputs
    from lucid_gb300 import _lib
    r = _renderer(sc, bin_size, **kw)
    frame = FrameInputs.from_scene(sc)
    res = {}
    if dump:
        img, counts, prims = r.raster_dump(frame, dump)
        res["counts"], res["prims"] = counts, prims
    else:
        img = r.render(frame)
    res["image"] = img.cpu().numpy()
    info, counters = r.info()
    res["info"], res["counters"] = info, counters
    res["verify"] = r.verify_info()
    res["bins"] = (r.bin_count_x, r.bin_count_y)
    res["bin_quads"] = r.download(_lib.BUF_BIN_QUADS, count=int(info.num_bin_quad_refs))
    res["bin_tris"] = r.download(_lib.BUF_BIN_TRIS, count=int(info.num_bin_tri_refs))
    r.close()
    return res


SCENES = {
    "random720": lambda: scenes.random_tris(1280, 720, 20000, seed=21),
    "deep_large": lambda: scenes.random_tris(640, 480, 30000, seed=22, center_sigma=120.0, area_median=300.0,
                                             area_sigma=1.5, large_fraction=0.03),
    "ragged_big_tris": lambda: scenes.random_tris(700, 333, 5000, seed=23, area_median=2000.0),
    "tiny_viewport": lambda: scenes.random_tris(40, 30, 300, seed=24),
    "fp16_meshes": lambda: scenes.meshes(640, 360, num_meshes=8, seed=25),
    "fp32_opacity": lambda: scenes.random_tris(320, 200, 8000, seed=26, color_format=scenes.COLOR_RGBA32F,
                                               tri_opacity_range=(0.1, 0.9), background=(0.2, 0.3, 0.4, 1.0)),
    "textured": lambda: scenes.textured_scene(160, 120, 800, seed=27),
}


@pytest.mark.parametrize("name", sorted(SCENES))
def test_bin64_frame_equals_bin32_frame(gpu, oracle, name):
    sc = SCENES[name]()
    a = _render(sc, 32)
    b = _render(sc, 64)
    assert a["info"].error_code == 0 and b["info"].error_code == 0
    assert b["verify"] == [], b["verify"][:4]
    assert b["bins"] == ((sc.width + 63) // 64, (sc.height + 63) // 64)
    np.testing.assert_array_equal(b["image"], a["image"])
    ref = oracle.run(sc, max_visible_quads=max(1024, sc.num_quads))
    assert helpers.max_abs_diff(b["image"], ref["image"]) <= 1e-5
    for key in ("num_fragments", "num_hblock_tris", "max_pixel_fragments"):
        assert int(getattr(b["info"], key)) == int(getattr(a["info"], key)), key
    assert tuple(b["info"].num_visible_quads) == tuple(a["info"].num_visible_quads)


@pytest.mark.parametrize("name", ["deep_large", "ragged_big_tris", "fp16_meshes"])
def test_bin64_fragment_order(gpu, name):
    sc = SCENES[name]()
    a = _render(sc, 32, dump=64)
    b = _render(sc, 64, dump=64)
    np.testing.assert_array_equal(b["counts"], a["counts"])
    np.testing.assert_array_equal(b["prims"], a["prims"])
    np.testing.assert_array_equal(b["image"], a["image"])


@pytest.mark.parametrize("name", ["random720", "deep_large", "ragged_big_tris", "tiny_viewport"])
def test_bin64_lists_cover_the_bin32_lists(gpu, name):
    sc = SCENES[name]()
    a = _render(sc, 32)
    b = _render(sc, 64)
    (ax, ay), (bx, by) = a["bins"], b["bins"]
    na, nb = ax * ay, bx * by
    qa = helpers.canonical_quad_lists(a["counters"], na, a["bin_quads"])
    qb = helpers.canonical_quad_lists(b["counters"], nb, b["bin_quads"])
    ta = helpers.canonical_tri_lists(a["counters"], na, a["bin_tris"])
    tb = helpers.canonical_tri_lists(b["counters"], nb, b["bin_tris"])
    for y in range(by):
        for x in range(bx):
            subs = [(2 * y + j) * ax + 2 * x + i for j in (0, 1) for i in (0, 1) if 2 * x + i < ax and 2 * y + j < ay]
            want_q = np.unique(np.concatenate([qa[s] for s in subs])) if subs else np.zeros(0, np.uint32)
            np.testing.assert_array_equal(np.unique(qb[y * bx + x]), want_q, err_msg=f"bin ({x}, {y}) quads")
            got_t = set(tb[y * bx + x].tolist())
            for s in subs:
                missing = set(ta[s].tolist()) - got_t
                assert not missing, f"bin ({x}, {y}) misses large tris {sorted(missing)[:5]}"
    # the 64-pixel grid needs no more references than the 32-pixel one
    assert int(b["info"].num_bin_quad_refs) <= int(a["info"].num_bin_quad_refs)


@pytest.mark.parametrize("flags", ["additive", "alpha_threshold", "pixel_blend"])
def test_bin64_blend_variants(gpu, flags):
    from lucid_gb300 import _lib
    f = {"additive": _lib.OPT_ADDITIVE_BLENDING, "alpha_threshold": _lib.OPT_ALPHA_THRESHOLD,
         "pixel_blend": _lib.OPT_PIXEL_BLEND}[flags]
    sc = SCENES["deep_large"]()
    a = _render(sc, 32, flags=f)
    b = _render(sc, 64, flags=f)
    np.testing.assert_array_equal(b["image"], a["image"])


def test_bin64_batch(gpu):
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    views = [SCENES[n]() for n in ("random720", "ragged_big_tris", "tiny_viewport", "fp16_meshes")]
    total = sum(max(1, v.num_quads) for v in views)
    r = LucidRenderer(max(v.width for v in views), max(v.height for v in views), max_input_quads=total,
                      max_visible_quads=total, max_views=len(views), bin_size=64)
    imgs = r.render_batch([(FrameInputs.from_scene(v), v.width, v.height) for v in views])
    for i, v in enumerate(views):
        want = _render(v, 32)["image"]
        np.testing.assert_array_equal(imgs[i].cpu().numpy(), want, err_msg=f"view {i}")
        assert r.batch_info(i).error_code == 0
    r.close()


def test_bin64_gradients(gpu):
    import torch
    from lucid_gb300 import autograd
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    sc = scenes.random_tris(128, 96, 4000, seed=28, color_format=scenes.COLOR_RGBA32F,
                            tri_opacity_range=(0.1, 0.9), background=(0.5, 0.5, 0.5, 1.0))
    out = {}
    for bs in (32, 64):
        r = LucidRenderer(sc.width, sc.height, max_input_quads=max(1024, sc.num_quads),
                          max_visible_quads=max(1024, sc.num_quads), bin_size=bs)
        vc = torch.from_numpy(sc.colors.astype(np.float32)).cuda().requires_grad_(True)
        op = torch.from_numpy(sc.tri_opacity.astype(np.float32)).cuda().requires_grad_(True)
        img = autograd.render(vc, op, r, FrameInputs.from_scene(sc))
        (img[..., :3] ** 2).sum().backward()
        out[bs] = (img.detach().cpu().numpy(), vc.grad.cpu().numpy(), op.grad.cpu().numpy())
        r.close()
    np.testing.assert_array_equal(out[64][0], out[32][0])
    for k in (1, 2):
        scale = max(1e-30, float(np.abs(out[32][k]).max()))
        assert float(np.abs(out[64][k] - out[32][k]).max()) <= 1e-5 * scale


def test_bin64_unsupported_combinations(gpu):
    from lucid_gb300 import _lib
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    sc = SCENES["tiny_viewport"]()
    with pytest.raises(_lib.LucidError):
        LucidRenderer(sc.width, sc.height, bin_size=48)
    r = _renderer(sc, 64, flags=_lib.OPT_REFERENCE_ORDER)
    with pytest.raises(_lib.LucidError):
        r.render(FrameInputs.from_scene(sc))
    r.close()
    r = _renderer(sc, 64)
    with pytest.raises(_lib.LucidError):
        r.raster_dump_bins(FrameInputs.from_scene(sc), [0], 8)
    r.close()


def test_autotune_searches_bin_size(gpu):
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    sc = SCENES["random720"]()
    r = LucidRenderer(sc.width, sc.height, max_input_quads=sc.num_quads, max_visible_quads=sc.num_quads)
    frame = FrameInputs.from_scene(sc)
    before = r.render(frame).cpu().numpy()
    tuned = r.autotune(frame)
    assert tuned["bin_size"] in (32, 64)
    assert r.bin_size == tuned["bin_size"]
    after = r.render(frame).cpu().numpy()
    np.testing.assert_array_equal(after, before)
    assert r.verify_info() == []
    r.close()
