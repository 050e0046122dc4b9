"""GPU parity: every pass of the CUDA path against the CPU oracle on the same inputs.

Integer outputs (setup records, bin counts, offsets, bin lists, level lists, per-pixel
fragment lists and their order) must be bit-exact; images must agree within 1e-5 per channel
(in practice they are bit-identical: both sides evaluate the same IEEE float expressions).
Bin reference lists are compared bit for bit with LUCID_OPT_SORTED_BIN_LISTS (a per-bin sort
pass puts every bin's lists in slot order, the oracle's order), and per bin as sets on
renderers without it (the dispatcher's order inside a bin follows its atomics, as in the
reference).
"""
import math

import numpy as np
import pytest

from lucid_gb300 import scenes
from tests import helpers

pytestmark = pytest.mark.gpu

IMG_TOL = 1e-5


def gpu_run(scene, max_visible_quads=None, flags=0, band_capacity=None, max_bin_refs=None,
            dump=0, renderer=None):
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    from lucid_gb300 import _lib
    mvq = max_visible_quads or max(1024, scene.num_quads)
    r = renderer or LucidRenderer(scene.width, scene.height, max_input_quads=max(1024, scene.num_quads),
                                  max_visible_quads=mvq, flags=flags | _lib.OPT_SORTED_BIN_LISTS,
                                  band_capacity=band_capacity,
                                  max_bin_refs=max_bin_refs or max(1 << 16, 8 * scene.num_quads))
    frame = FrameInputs.from_scene(scene)
    res = {}
    if dump:
        img, counts, prims = r.raster_dump(frame, dump)
        res["frag_counts"], res["frag_prims"] = counts, prims
    else:
        img = r.render(frame)
    res["image"] = img.cpu().numpy()
    info, counters = r.info()
    res["info"], res["bin_counters"] = info, counters
    n = r.options.max_visible_quads
    res["quad_aabbs"] = r.download(_lib.BUF_QUAD_AABBS)
    res["quad_source"] = r.download(_lib.BUF_QUAD_SOURCE)
    res["quad_verts"] = r.download(_lib.BUF_QUAD_VERTS).reshape(n, 4)
    res["quad_colors"] = r.download(_lib.BUF_QUAD_COLORS).reshape(n, 4)
    res["tri_bary"] = r.download(_lib.BUF_TRI_BARY).reshape(2 * n, 8)
    res["tri_scan"] = r.download(_lib.BUF_TRI_SCAN).reshape(2 * n, 8)
    res["tri_depth"] = r.download(_lib.BUF_TRI_DEPTH).reshape(2 * n, 4)
    res["tri_normals"] = r.download(_lib.BUF_TRI_NORMALS)
    res["bin_quads"] = r.download(_lib.BUF_BIN_QUADS, count=int(info.num_bin_quad_refs))
    res["bin_tris"] = r.download(_lib.BUF_BIN_TRIS, count=int(info.num_bin_tri_refs))
    res["renderer"] = r
    return res


def compare(scene, oracle, *, max_visible_quads=None, flags=0, dump=0, check_image=True,
            renderer=None, image64=True):
    mvq = max_visible_quads or max(1024, scene.num_quads)
    o = oracle.run(scene, max_visible_quads=mvq, flags=flags, max_per_pixel=dump, image64=image64)
    g = gpu_run(scene, max_visible_quads=mvq, flags=flags, dump=dump, renderer=renderer)
    info = g["info"]
    # ---- setup
    assert info.num_input_quads == o["num_input_quads"]
    assert tuple(info.num_visible_quads) == tuple(o["num_visible"])
    assert tuple(info.num_rejected_quads) == tuple(o["rejected"])
    assert info.error_code == o["error_code"]
    assert info.num_binning_dispatches[0] == o["num_binning_dispatches"]
    slots = helpers.used_slots(o["num_visible"], mvq)
    for key in ("quad_aabbs", "quad_source", "quad_verts"):
        helpers.assert_same_bits(g[key][slots], o[key][slots], key)
    if scene.color_format == scenes.COLOR_RGBA8:
        np.testing.assert_array_equal(g["quad_colors"][slots], o["quad_colors"][slots])
    tri_slots = []
    for s in slots:
        enc = int(o["quad_aabbs"][s])
        for second in (0, 1):
            if not (enc >> (30 + second)) & 1:
                tri_slots.append(2 * int(s) + second)
    tri_slots = np.array(tri_slots, np.int64)
    for key in ("tri_bary", "tri_scan", "tri_depth", "tri_normals"):
        helpers.assert_same_bits(g[key][tri_slots], o[key][tri_slots], key)
    # ---- binning
    n = o["bin_count"]
    gc, oc = g["bin_counters"], o["bin_counters"]
    np.testing.assert_array_equal(gc[:6 * n], oc[:6 * n], err_msg="bin counts/offsets")
    lv = o["bin_level_counts"]
    assert tuple(info.bin_level_counts) == tuple(lv)
    np.testing.assert_array_equal(gc[7 * n:7 * n + lv[2]], oc[7 * n:7 * n + lv[2]], err_msg="LOW bins")
    np.testing.assert_array_equal(gc[9 * n:9 * n + lv[4]], oc[9 * n:9 * n + lv[4]], err_msg="HIGH bins")
    from lucid_gb300 import _lib
    sorted_lists = bool(g["renderer"].options.flags & _lib.OPT_SORTED_BIN_LISTS)
    helpers.assert_bin_lists_equal(gc, n, g["bin_quads"], g["bin_tris"], oc, o["bin_quads"], o["bin_tris"],
                                   exact=sorted_lists)
    # ---- raster
    assert info.num_fragments == o["num_fragments"]
    assert info.num_hblock_tris == o["num_hblock_tris"]
    assert info.max_pixel_fragments == o["max_pixel_fragments"]
    if check_image:
        err = helpers.max_abs_diff(g["image"], o["image"])
        assert err <= IMG_TOL, f"image max abs error {err}"
    if dump:
        np.testing.assert_array_equal(g["frag_counts"], o["frag_counts"])
        np.testing.assert_array_equal(g["frag_prims"], o["frag_prims"])
    assert not g["renderer"].verify_info()
    return g, o


# ---------------------------------------------------------------------------------------------

@pytest.mark.parametrize("name", sorted(helpers.kat_cases()))
def test_kat(gpu, oracle, name):
    case = helpers.kat_cases()[name]
    compare(helpers.kat_scene(case), oracle, dump=8)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_small_random(gpu, oracle, seed):
    compare(scenes.small_scene(96, 72, 300, seed=seed), oracle, dump=32)


def test_many_layers_fragment_order(gpu, oracle):
    sc = scenes.random_tris(64, 64, 3000, seed=8, area_median=900.0, area_sigma=0.5)
    g, o = compare(sc, oracle, dump=256)
    assert o["max_pixel_fragments"] > 100


def test_depth_windows_early_exit(gpu, oracle):
    """Hundreds of layers per pixel: per-pixel depth windows, stop at T == 0 (image only)."""
    sc = scenes.random_tris(96, 64, 6000, seed=14, area_median=1500.0, area_sigma=0.4,
                            alpha_range=(0.05, 0.5))
    g, o = compare(sc, oracle)
    assert o["max_pixel_fragments"] > 400


def test_depth_windows_concentrated_depths(gpu, oracle):
    """Most fragments of every pixel in one depth bucket: windows overshoot their target and
    some pixels must wait for the next round (capacity deferral)."""
    rng = np.random.default_rng(5)
    tris, cols = [], []
    for i in range(420):
        d = 10.0 + 1e-4 * rng.random(3)
        x0, y0 = rng.uniform(-20, 10, 2)
        tris.append([(x0, y0, d[0]), (x0 + 120, y0 + 8, d[1]), (x0 + 10, y0 + 110, d[2])])
        cols.append([(int(c[0]), int(c[1]), int(c[2]), 40) for c in rng.integers(0, 255, (3, 3))])
    tris.append([(0, 0, 0.2), (96, 0, 0.21), (0, 64, 0.22)])
    cols.append([(255, 0, 0, 10)] * 3)
    tris.append([(96, 64, 99.0), (0, 64, 99.5), (96, 0, 98.0)])
    cols.append([(0, 255, 0, 10)] * 3)
    sc = scenes.screen_triangles(tris, cols, 96, 64)
    compare(sc, oracle, dump=512)
    compare(sc, oracle)


@pytest.mark.parametrize("slab", [8, 64, 180, 1 << 30])
def test_depth_slabs(gpu, oracle, slab):
    """The per-pixel depth histograms built one key slab at a time (small slabs force many
    slabs per group, a huge one counts every key at once): same fragment lists and image."""
    from lucid_gb300.renderer import LucidRenderer
    sc = scenes.random_tris(96, 64, 6000, seed=14, area_median=1500.0, area_sigma=0.4,
                            alpha_range=(0.05, 0.5))
    for dump in (512, 0):
        r = LucidRenderer(sc.width, sc.height, max_input_quads=max(1024, sc.num_quads),
                          max_visible_quads=max(1024, sc.num_quads),
                          max_bin_refs=max(1 << 16, 8 * sc.num_quads), slab_fragments=slab)
        g, o = compare(sc, oracle, dump=dump, renderer=r)
        assert o["max_pixel_fragments"] > 400
        r.close()


def test_large_triangles_and_high_bins(gpu, oracle):
    sc = scenes.random_tris(200, 140, 3000, seed=4, area_median=2000.0, area_sigma=1.0,
                            large_fraction=0.05, large_area=(5000.0, 20000.0))
    g, o = compare(sc, oracle, dump=16)
    assert o["num_visible"][1] > 100
    assert o["bin_level_counts"][4] > 0  # HIGH bins exercised


@pytest.mark.parametrize("w,h", [(1, 1), (33, 17), (100, 37), (257, 129)])
def test_ragged_viewports(gpu, oracle, w, h):
    sc = scenes.random_tris(w, h, 400, seed=w + h, area_median=max(4.0, w * h / 40.0))
    compare(sc, oracle, dump=8)


def test_empty_and_fully_rejected(gpu, oracle):
    empty = scenes.screen_triangles(np.zeros((0, 3, 3)), np.zeros((0, 3, 4)), 64, 64,
                                    (0.3, 0.2, 0.1, 1.0))
    g, o = compare(empty, oracle)
    np.testing.assert_allclose(g["image"][..., :3], np.broadcast_to([0.3, 0.2, 0.1], (64, 64, 3)), atol=1e-7)
    # every triangle off screen or between samples
    tris = [[(100, 100, 5.0), (120, 100.5, 5.0), (110, 130, 5.0)],
            [(10.2, 10.2, 5.0), (10.4, 10.25, 5.0), (10.3, 10.4, 5.0)]]
    sc = scenes.screen_triangles(tris, [[(255, 0, 0, 255)] * 3] * 2, 64, 64)
    g, o = compare(sc, oracle)
    assert sum(o["num_visible"]) == 0


def test_near_plane_crossing(gpu, oracle):
    sc = scenes.random_tris(160, 120, 600, seed=12, area_median=500.0, depth_range=(-3.0, 20.0))
    g, o = compare(sc, oracle, dump=16)
    assert o["num_visible"][1] > 0


def test_backface_culling(gpu, oracle):
    sc = scenes.small_scene(96, 72, 500, seed=4)
    sc.config.enable_backface_culling = 1
    g, o = compare(sc, oracle, dump=8)
    assert o["rejected"][1] > 0


@pytest.mark.parametrize("fmt", [scenes.COLOR_RGBA16F, scenes.COLOR_RGBA32F])
def test_colour_formats(gpu, oracle, fmt):
    compare(scenes.random_tris(96, 72, 400, seed=6, color_format=fmt, area_median=100.0), oracle)


def test_triangle_opacity_and_instance_colour(gpu, oracle):
    sc = scenes.random_tris(96, 72, 400, seed=13, color_format=scenes.COLOR_RGBA32F,
                            tri_opacity_range=(0.1, 0.9), area_median=100.0)
    # second draw call with an instance colour
    inst, cols, _ = scenes.build_instances([(0, 200, scenes.INST_HAS_VERTEX_COLORS, 0xFFFFFFFF),
                                            (200, 200, scenes.INST_HAS_VERTEX_COLORS, 0x8040C0FF)])
    sc.instances, sc.instance_colors = inst, cols
    compare(sc, oracle, dump=8)


def test_real_quads(gpu, oracle):
    sc = scenes.meshes(320, 200, num_meshes=6, seed=3, scale_range=(2.0, 6.0), depth_range=(10.0, 30.0))
    g, o = compare(sc, oracle, dump=8)
    culled_second = np.count_nonzero((o["quad_aabbs"][helpers.used_slots(o["num_visible"], o["max_visible_quads"])] >> 31) & 1)
    assert culled_second < sum(o["num_visible"])  # both triangles of real quads rasterised


@pytest.mark.parametrize("flags", [2, 4])
def test_blend_variants(gpu, oracle, flags):
    compare(scenes.small_scene(96, 72, 600, seed=2, area_median=200.0), oracle, flags=flags)


def test_visible_quad_capacity(gpu, oracle):
    sc = scenes.small_scene(96, 72, 300, seed=1)
    g, o = compare(sc, oracle, max_visible_quads=100)
    assert o["error_code"] == 1 and g["info"].error_code == 1


def test_band_capacity_overflow_paints_red(gpu, oracle):
    sc = scenes.random_tris(64, 64, 2000, seed=3, area_median=200.0)
    g = gpu_run(sc, band_capacity=64)
    assert g["info"].error_code == 3  # LUCID_ERR_BAND_ENTRIES
    img = g["image"]
    assert ((img[..., 0] == 1.0) & (img[..., 1] == 0.0)).any()


def test_bin_ref_capacity_overflow(gpu, oracle):
    sc = scenes.random_tris(128, 128, 2000, seed=3, area_median=400.0)
    g = gpu_run(sc, max_bin_refs=500)
    assert g["info"].error_code == 2  # LUCID_ERR_BIN_REFS
    assert np.isfinite(g["image"]).all()


def test_bad_vertex_index_is_rejected(gpu, oracle):
    sc = scenes.small_scene(64, 48, 50, seed=1)
    sc.quads = sc.quads.copy()
    sc.quads[5, 1] = 10_000_000
    g, o = compare(sc, oracle)
    assert g["info"].error_code == 7


def test_deterministic_and_renderer_reuse(gpu, oracle):
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    sc = scenes.small_scene(128, 96, 2000, seed=21, area_median=300.0)
    r = LucidRenderer(128, 96, max_input_quads=4096, max_visible_quads=4096)
    f = FrameInputs.from_scene(sc)
    a = r.render(f).cpu().numpy()
    b = r.render(f).cpu().numpy()
    np.testing.assert_array_equal(a, b)
    # a different scene on the same renderer, then the first again
    compare(scenes.small_scene(128, 96, 500, seed=22), oracle, renderer=r, max_visible_quads=4096)
    c = r.render(f).cpu().numpy()
    np.testing.assert_array_equal(a, c)


def test_cpu720_full(gpu, oracle):
    """The 1280x720 / 100k-triangle workload, every pass and every pixel."""
    sc = scenes.workload("cpu720")
    g, o = compare(sc, oracle)
    print("fragments", o["num_fragments"], "max/pixel", o["max_pixel_fragments"])


def test_largest_viewport(gpu, oracle):
    """4096x4096, the largest viewport (16384 bins): the bin counter and dispatcher keep one
    int per bin in shared memory (64 KB, above the default 48 KB limit)."""
    sc = scenes.random_tris(4096, 4096, 3000, seed=17, area_median=2000.0, area_sigma=1.0,
                            large_fraction=0.02, large_area=(50000.0, 100000.0))
    g, o = compare(sc, oracle, image64=False)
    assert o["bin_count"] == 16384 and o["num_visible"][1] > 0


@pytest.mark.parametrize("copies", [6, 40, 90])
def test_exact_depth_ties(gpu, oracle, copies):
    """Every triangle drawn several times over (identical vertices, other colours): equal depth
    keys at every pixel, ordered by input primitive id. 6 copies stay in the light path's
    single pass, 40 need its bounded passes (more than 32 fragments per pixel), 90 take the
    depth windows (more than 64)."""
    rng = np.random.default_rng(100 + copies)
    tris, cols = [], []
    for _ in range(12):
        x0, y0 = rng.uniform(-10, 60, 2)
        d = rng.uniform(1.0, 50.0, 3)
        base = [(x0, y0, d[0]), (x0 + rng.uniform(20, 60), y0 + rng.uniform(-5, 10), d[1]),
                (x0 + rng.uniform(-5, 10), y0 + rng.uniform(20, 50), d[2])]
        for _ in range(copies):
            tris.append(base)
            cols.append([(int(c[0]), int(c[1]), int(c[2]), 30) for c in rng.integers(0, 255, (3, 3))])
    order = rng.permutation(len(tris))  # copies of one triangle spread over the input order
    sc = scenes.screen_triangles([tris[i] for i in order], [cols[i] for i in order], 96, 72)
    g, o = compare(sc, oracle, dump=128)
    assert o["max_pixel_fragments"] >= copies
