"""CPU tests of the oracle: analytic known-answer cases and invariants of the reference.

The reference has no golden vectors and cannot run here (Vulkan GLSL + missing libfwk), so the
oracle is pinned by analytic cases (tests/golden/kat.npz, see make_golden.py) and by the
self-checks the reference performs at run time (LucidRenderer::verifyInfo,
src/lucid_renderer.cpp:629-707).
"""
import math

import numpy as np
import pytest

from lucid_gb300 import scenes
from tests import helpers


@pytest.mark.parametrize("name", sorted(helpers.kat_cases()))
def test_kat_coverage_and_colour(oracle, name):
    case = helpers.kat_cases()[name]
    sc = helpers.kat_scene(case)
    out = oracle.run(sc, image64=True, max_per_pixel=4)
    covered = case["covered"]          # [ntris, h, w]
    on_edge = case["on_edge"]
    expect_counts = covered.sum(0)
    got = out["frag_counts"]
    ok = ~on_edge
    np.testing.assert_array_equal(got[ok], expect_counts[ok])
    # colour: perspective-correct interpolation + front-to-back blend (float64 analytic)
    img = out["image"]
    interior = ok.copy()
    # exclude pixels next to an edge pixel: analytic centre sampling vs float scan rounding
    interior[1:] &= ok[:-1]
    interior[:-1] &= ok[1:]
    interior[:, 1:] &= ok[:, :-1]
    interior[:, :-1] &= ok[:, 1:]
    np.testing.assert_allclose(img[interior], case["image"][interior], atol=2e-4)


def test_kat_order_independent_of_input_order(oracle):
    case = helpers.kat_cases()["intersecting"]
    a = helpers.kat_scene(case)
    rev = dict(case)
    rev["tris"] = case["tris"][::-1].copy()
    rev["colors"] = case["colors"][::-1].copy()
    b = helpers.kat_scene(rev)
    ia = oracle.run(a)["image"]
    ib = oracle.run(b)["image"]
    np.testing.assert_array_equal(ia, ib)


def test_verify_info_invariants(oracle):
    sc = scenes.small_scene(160, 100, 2000, seed=11, area_median=300.0, area_sigma=1.2)
    out = oracle.run(sc, raster=False)
    n = out["bin_count"]
    c = out["bin_counters"].astype(np.int64)
    for base in (0, 3):
        cnt, off, tmp = c[n * base:n * (base + 1)], c[n * (base + 1):n * (base + 2)], c[n * (base + 2):n * (base + 3)]
        assert off[0] == 0
        np.testing.assert_array_equal(off[1:], off[:-1] + cnt[:-1])
        np.testing.assert_array_equal(tmp, off + cnt)
    levels = out["bin_level_counts"]
    assert sum(levels) == n
    assert out["num_visible"][1] > 0, "scene must exercise large quads"


def test_fp32_blend_vs_fp64(oracle):
    sc = scenes.small_scene(128, 96, 3000, seed=5, area_median=200.0)
    out = oracle.run(sc, image64=True)
    err = np.abs(out["image"].astype(np.float64) - out["image64"]).max()
    assert err < 1e-5, err


def test_fragment_lists_sorted_and_complete(oracle):
    """Per-pixel order is nearest first with ties by primitive id; lists hold every
    primitive whose triangle covers the pixel centre."""
    sc = scenes.small_scene(64, 48, 400, seed=3, area_median=150.0)
    out = oracle.run(sc, max_per_pixel=64)
    counts, prims = out["frag_counts"], out["frag_prims"]
    assert counts.max() <= 64
    # depth of primitive p at pixel (x, y) from the depth record of its tri slot
    src = out["quad_source"]
    mvq = out["max_visible_quads"]
    slots = helpers.used_slots(out["num_visible"], mvq)
    prim_to_tri = {}
    for s in slots:
        for second in (0, 1):
            prim_to_tri[int(src[s]) * 2 + second] = int(s) * 2 + second
    depth = out["tri_depth"].view(np.float32)
    for y in range(0, 48, 3):
        for x in range(0, 64, 3):
            n = counts[y, x]
            ds = []
            for p in prims[y, x, :n]:
                t = prim_to_tri[int(p)]
                dx, dy, dz = depth[t, :3]
                ds.append(np.float32(dx * np.float32(x)) + np.float32(np.float32(dy * np.float32(y)) + dz))
            ds = np.array(ds, np.float32)
            assert np.all(ds[:-1] >= ds[1:]), (x, y)
            ties = ds[:-1] == ds[1:]
            assert np.all(prims[y, x, :n][:-1][ties] < prims[y, x, :n][1:][ties])


def test_culling_and_classification(oracle):
    w, h = 256, 128
    tris = [
        [(10, 10, 5.0), (20, 10, 5.0), (10, 20, 5.0)],      # small
        [(10, 10, 5.0), (200, 15, 5.0), (30, 120, 5.0)],    # large (> 4 bins)
        [(300, 10, 5.0), (400, 10, 5.0), (350, 60, 5.0)],   # outside the right edge: frustum
        [(50.1, 50.1, 5.0), (50.3, 50.1, 5.0), (50.2, 50.3, 5.0)],  # between samples
    ]
    cols = [[(255, 255, 255, 255)] * 3] * 4
    sc = scenes.screen_triangles(tris, cols, w, h)
    out = oracle.run(sc, raster=False)
    assert out["num_visible"] == (1, 1)
    assert out["rejected"] == (0, 0, 1, 1)
    # backface culling: the same triangles wound both ways, culling on
    tris2 = [tris[0], [tris[0][0], tris[0][2], tris[0][1]]]
    sc2 = scenes.screen_triangles(tris2, cols[:2], w, h, backface_culling=True)
    out2 = oracle.run(sc2, raster=False)
    assert sum(out2["num_visible"]) == 1 and out2["rejected"][1] == 1


def test_capacity_error_is_reported(oracle):
    sc = scenes.small_scene(96, 72, 300, seed=1)
    out = oracle.run(sc, max_visible_quads=1024)
    assert out["error_code"] == 0
    small = oracle.run(sc, max_visible_quads=100)
    assert small["error_code"] == 1  # LUCID_ERR_VISIBLE_QUADS
    assert sum(small["num_visible"]) == 100


def test_bin_lists_cover_fragments(oracle):
    """Every fragment's triangle is listed in its bin (lists are conservative)."""
    sc = scenes.small_scene(128, 96, 800, seed=9, area_median=400.0, area_sigma=1.0)
    out = oracle.run(sc, max_per_pixel=32)
    n, bcx = out["bin_count"], out["bin_count_x"]
    c = out["bin_counters"]
    src = out["quad_source"]
    listed = [set() for _ in range(n)]
    qc, qo = c[:n], c[n:2 * n]
    tc, to = c[3 * n:4 * n], c[4 * n:5 * n]
    for b in range(n):
        for e in out["bin_quads"][qo[b]:qo[b] + qc[b]]:
            q = int(e) & 0x0FFFFFFF
            listed[b].update({int(src[q]) * 2, int(src[q]) * 2 + 1})
        for t in out["bin_tris"][to[b]:to[b] + tc[b]]:
            listed[b].add(int(src[int(t) >> 1]) * 2 + (int(t) & 1))
    counts, prims = out["frag_counts"], out["frag_prims"]
    for y in range(96):
        for x in range(128):
            b = (y // 32) * bcx + x // 32
            for p in prims[y, x, :min(32, counts[y, x])]:
                assert int(p) in listed[b]


def test_workload_generators_are_seeded():
    a = scenes.random_tris(320, 200, 1000, seed=4)
    b = scenes.random_tris(320, 200, 1000, seed=4)
    np.testing.assert_array_equal(a.positions, b.positions)
    np.testing.assert_array_equal(a.colors, b.colors)
    c = scenes.random_tris(320, 200, 1000, seed=5)
    assert not np.array_equal(a.positions, c.positions)
    m = scenes.meshes(640, 360, num_meshes=4, seed=1)
    assert m.quads.shape == (4 * 1250, 4) and m.num_tris == 4 * 2500
    assert m.colors.dtype == np.float16
    assert (m.instances[:, 2] <= 1024).all()


def test_fp64_gradient_model_analytic_vs_fd(oracle):
    sc = scenes.random_tris(48, 40, 300, seed=2, color_format=scenes.COLOR_RGBA32F,
                            tri_opacity_range=(0.1, 0.9), area_median=120.0,
                            background=(0.5, 0.5, 0.5, 1.0))
    model = oracle.GradModel(sc)
    vc = sc.colors.astype(np.float64)
    op = sc.tri_opacity.astype(np.float64)
    target = np.random.default_rng(1).random((40, 48, 4)).astype(np.float32)
    dvc, dop = model.analytic(vc, op, target)
    big = np.argsort(-np.abs(dvc.ravel()))[:40]
    for i in big:
        fd = model.fd(vc, op, target, 0, int(i))
        assert abs(fd - dvc.ravel()[i]) <= 1e-6 * max(1.0, abs(fd))
    for i in np.argsort(-np.abs(dop))[:20]:
        fd = model.fd(vc, op, target, 1, int(i))
        assert abs(fd - dop[i]) <= 1e-6 * max(1.0, abs(fd))
    # the FP64 model's image equals the oracle's FP64 blend of the same fragments
    out = oracle.run(sc, image64=True)
    assert model.num_fragments == out["num_fragments"]
    # the adjoint fed the loss's own upstream gradient reproduces the analytic gradient
    c64 = out["image64"]
    up = (2.0 * (np.clip(c64, 0, 1) - target)).astype(np.float32)
    bvc, bop = model.backprop(vc, op, up, c64[..., :3].astype(np.float32))
    scale = np.abs(dvc).max()
    assert np.abs(bvc - dvc).max() <= 1e-5 * scale
    assert np.abs(bop - dop).max() <= 1e-5 * np.abs(dop).max()


def _textured_quad_scene(W=16, H=8, x0=10, y0=6, z=4.0, opaque=True, uv_rect=None, levels=None):
    """One screen-aligned quad (two tris) covering W x H pixels from (x0, y0) at constant depth
    with uv (0,0)..(1,1) at its corners: pixel centres land on texel centres of level 0."""
    tris = [[(x0, y0, z), (x0 + W, y0, z), (x0 + W, y0 + H, z)], [(x0, y0, z), (x0 + W, y0 + H, z), (x0, y0 + H, z)]]
    cols = [[(255, 255, 255, 255)] * 3] * 2
    sc = scenes.screen_triangles(tris, cols, 48, 32)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 0], [1, 1], [0, 1]], np.float32)
    flags = scenes.INST_HAS_ALBEDO_TEXTURE | (scenes.INST_TEX_OPAQUE if opaque else 0)
    if uv_rect is not None:
        flags |= scenes.INST_HAS_UV_RECT
    inst, icol, _ = scenes.build_instances([(0, 2, flags, 0xFFFFFFFF)])
    tex = scenes.make_texture(W, H, seed=3, alpha_range=(0.3, 0.9), levels=levels)
    sc = scenes.Scene(**{**sc.__dict__, "instances": inst, "instance_colors": icol, "tex_coords": uv,
                         "uv_rects": None if uv_rect is None else np.array([uv_rect], np.float32),
                         "opaque_tex": tex if opaque else None, "trans_tex": None if opaque else tex})
    return sc, tex


def test_texture_kat_texel_centres(oracle):
    """Pixel centres on texel centres, one texel per pixel: the image is the texture (level 0,
    no blending between texels)."""
    W, H, x0, y0 = 16, 8, 10, 6
    sc, tex = _textured_quad_scene(W, H, x0, y0)
    img = oracle.run(sc)["image"]
    lv0 = tex.levels[0]
    want = np.stack([(lv0 >> (8 * k)) & 0xFF for k in range(3)], -1).astype(np.float32) / np.float32(255)
    np.testing.assert_allclose(img[y0:y0 + H, x0:x0 + W, :3], want, atol=2e-6)


def test_texture_transparent_and_uv_rect(oracle):
    """Transparent texture: alpha from the texture; a uv rect maps the quad onto a sub-rectangle
    (fract, then scale and offset, shading.glsl:146-150)."""
    W, H, x0, y0 = 16, 8, 10, 6
    sc, tex = _textured_quad_scene(W, H, x0, y0, opaque=False)
    img = oracle.run(sc)["image"]
    lv0 = tex.levels[0].astype(np.int64)
    rgba = np.stack([(lv0 >> (8 * k)) & 0xFF for k in range(4)], -1).astype(np.float64) / 255.0
    want = rgba[..., :3] * rgba[..., 3:]  # black background
    np.testing.assert_allclose(img[y0:y0 + H, x0:x0 + W, :3], want, atol=2e-5)
    # a uv rect of the left half: pixel x samples u = 0.5 * (x + 0.5) / W
    sc2, tex2 = _textured_quad_scene(W, H, x0, y0, uv_rect=(0.0, 0.0, 0.5, 1.0))
    img2 = oracle.run(sc2)["image"]
    assert np.abs(img2[y0:y0 + H, x0:x0 + W] - img[y0:y0 + H, x0:x0 + W]).max() > 1e-3
    assert np.isfinite(img2).all()
