"""The oracle against the reference's own shader functions, compiled from the reference tree.

oracle/ref_build.py compiles, as C++ through a GLSL-in-C++ shim:
* the reference's quad setup: processInputQuad, storeTri, storeQuad, addVisibleTri / Quad and
  their helpers (data/shaders/quad_setup.glsl, shared/funcs.glsl);
* its bin counter: countSmallQuadBins, countLargeTriBins, scanlineStep and the scanline loaders
  (bin_counter.glsl, shared/scanline.glsl);
* its low-level raster's row spans: generateRowTris with rasterBinStep (raster_low.glsl,
  shared/raster.glsl).
A harness drives them in the order of the shaders' main().

Checks:
* every setup record the oracle produces must be bit-identical to theirs (NaN payloads aside):
  the 28-bit bin AABBs with cull flags, the bary / scan / depth records, the encoded normals,
  the vertex colours, the visible and rejected counts;
* so must every per-bin quad and tri count, and every pixel's fragment count (the coverage the
  row spans give).
The GPU path is bit-exact with the oracle on all of these (tests/test_gpu_parity.py), so this
pins the GPU path to the reference's source as far as setup, binning and coverage go. The
per-pixel order and the blend are the exact-order extension (the reference keeps a 3-deep
approximate window there), checked against the FP64 blend instead.

Needs the reference tree, which only the build container has: skipped elsewhere.
"""
import numpy as np
import pytest

from lucid_gb300 import scenes
from tests import helpers


@pytest.fixture(scope="module")
def ref():
    from oracle import ref_binding
    if ref_binding.lib() is None:
        pytest.skip("the reference's shader sources are not available here")
    return ref_binding


def check(scene, oracle, ref, mvq=None, threads=1):
    mvq = mvq or max(1024, scene.num_quads)
    r = ref.quad_setup(scene, mvq)
    o = oracle.run(scene, max_visible_quads=mvq, raster=False)
    assert r["num_input_quads"] == o["num_input_quads"]
    assert r["num_visible"] == tuple(o["num_visible"])
    assert r["rejected"] == tuple(o["rejected"])
    slots = helpers.used_slots(o["num_visible"], mvq)
    helpers.assert_same_bits(r["quad_aabbs"][slots], o["quad_aabbs"][slots], "quad_aabbs")
    if scene.color_format == scenes.COLOR_RGBA8:
        helpers.assert_same_bits(r["quad_colors"][slots], o["quad_colors"][slots], "quad_colors")
    enc = o["quad_aabbs"][slots].astype(np.int64)
    tris = np.concatenate([2 * slots[((enc >> 30) & 1) == 0], 2 * slots[((enc >> 31) & 1) == 0] + 1])
    for key in ("tri_bary", "tri_scan", "tri_depth", "tri_normals"):
        helpers.assert_same_bits(r[key][tris], o[key][tris], key)
    # binning: the reference counter's per-bin counts on the reference's own records
    qc, tc = ref.bin_counts(r["quad_aabbs"], r["tri_scan"], r["num_visible"], mvq, scene.width, scene.height)
    n = o["bin_count"]
    np.testing.assert_array_equal(qc, o["bin_counters"][:n], err_msg="bin quad counts")
    np.testing.assert_array_equal(tc, o["bin_counters"][3 * n:4 * n], err_msg="bin tri counts")
    # coverage: the reference raster's row spans against the oracle's per-pixel fragment counts
    cov = ref.coverage(r["quad_aabbs"], r["tri_scan"], r["num_visible"], mvq, scene.width, scene.height)
    oc = oracle.run(scene, max_visible_quads=mvq, setup_outputs=False, threads=threads)
    np.testing.assert_array_equal(cov, oc["frag_counts"], err_msg="per-pixel fragment counts")
    return r, o


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_tris(oracle, ref, seed):
    check(scenes.small_scene(96, 72, 400, seed=seed), oracle, ref)


def test_near_plane_crossing_and_culling(oracle, ref):
    r, o = check(scenes.random_tris(160, 120, 800, seed=12, area_median=500.0, depth_range=(-3.0, 20.0)),
                 oracle, ref)
    assert o["num_visible"][1] > 0 and o["rejected"][2] > 0  # clipped AABBs and frustum rejects
    sc = scenes.small_scene(96, 72, 500, seed=4)
    sc.config.enable_backface_culling = 1
    r, o = check(sc, oracle, ref)
    assert o["rejected"][1] > 0


def test_between_samples_and_ragged_viewports(oracle, ref):
    for w, h in [(1, 1), (33, 17), (257, 129)]:
        check(scenes.random_tris(w, h, 400, seed=w + h, area_median=max(4.0, w * h / 40.0)), oracle, ref)
    r, o = check(scenes.random_tris(128, 96, 2000, seed=9, area_median=0.3), oracle, ref)
    assert o["rejected"][3] > 0  # quads that fall between samples


def test_real_quads_and_large_triangles(oracle, ref):
    check(scenes.meshes(320, 200, num_meshes=8, seed=3, scale_range=(2.0, 6.0), depth_range=(10.0, 30.0),
                        color_format=scenes.COLOR_RGBA8), oracle, ref)
    r, o = check(scenes.random_tris(200, 140, 3000, seed=4, area_median=2000.0, area_sigma=1.0,
                                    large_fraction=0.05, large_area=(5000.0, 20000.0)), oracle, ref)
    assert o["num_visible"][1] > 100


def test_workload_setup(oracle, ref):
    """The whole 1280x720 / 100k-triangle workload's setup records."""
    r, o = check(scenes.workload("cpu720"), oracle, ref)
    assert sum(o["num_visible"]) > 90_000


@pytest.mark.parametrize("name", ["heavy1080", "meshes4k"])
def test_benchmark_frames(oracle, ref, name):
    """The 1920x1080 / 1M-triangle benchmark frame and the 3840x2160 / 5M-triangle mesh frame
    (RGBA8 colours here: the reference's setup reads RGBA8 vertex colours): every setup record,
    per-bin count and per-pixel fragment count."""
    import os
    sc = scenes.workload(name)
    if sc.color_format != scenes.COLOR_RGBA8:
        sc = scenes.meshes(color_format=scenes.COLOR_RGBA8)
    r, o = check(sc, oracle, ref, threads=os.cpu_count() or 1)
    assert sum(o["num_visible"]) > 800_000
