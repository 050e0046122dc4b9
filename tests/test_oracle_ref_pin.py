"""The oracle against the reference's own shader functions, compiled from the reference tree.

oracle/ref_build.py compiles, as C++ through a GLSL-in-C++ shim:
* the reference's quad setup: processInputQuad, storeTri, storeQuad, addVisibleTri / Quad and
  their helpers (data/shaders/quad_setup.glsl, shared/funcs.glsl);
* its bin counter: countSmallQuadBins, countLargeTriBins, scanlineStep and the scanline loaders
  (bin_counter.glsl, shared/scanline.glsl);
* its low-level raster's row spans: generateRowTris with rasterBinStep (raster_low.glsl,
  shared/raster.glsl);
* its shading and reduction: shadeSample with finalShading and the sRGB conversions, and the
  3-deep window initReduceSamples / reduceSample / finishReduceSamples (shared/shading.glsl,
  shared/funcs.glsl).
A harness drives them in the order of the shaders' main().

Checks:
* every setup record the oracle produces must be bit-identical to theirs (NaN payloads aside):
  the 28-bit bin AABBs with cull flags, the bary / scan / depth records, the encoded normals,
  the vertex colours, the visible and rejected counts;
* so must every per-bin quad and tri count, and every pixel's fragment count (the coverage the
  row spans give).
* the reference-order mode's per-sample RGBA8 colour and depth must be bit-identical to
  shadeSample's, and its 3-deep window's output colour to the reference's reduction over the
  same sample sequences (GLSL's pow is implementation-defined: both sides use the oracle's
  refPow, the pow the CUDA path evaluates too).
The GPU path is bit-exact with the oracle on all of these (tests/test_gpu_parity.py,
tests/test_gpu_ref_order.py), so this pins the GPU path to the reference's source as far as
setup, binning, coverage, the reference-order shading and its reduction window go. The exact
per-pixel order and its FP32 blend are the exact-order extension (the reference keeps a 3-deep
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


# ---- shading and the 3-deep reduction window of the reference-order mode ----

def _visible_tris(o, mvq):
    slots = helpers.used_slots(o["num_visible"], mvq)
    enc = o["quad_aabbs"][slots].astype(np.int64)
    return np.concatenate([2 * slots[((enc >> 30) & 1) == 0], 2 * slots[((enc >> 31) & 1) == 0] + 1])


def _untextured_with_normals(seed):
    """Vertex colours, instance colours and per-vertex normals (textured_scene without its
    textures: the pinned shadeSample never reaches textureGrad)."""
    sc = scenes.textured_scene(160, 120, 600, seed=seed)
    sc.instances[:, 3] &= ~np.int32(scenes.INST_HAS_ALBEDO_TEXTURE | scenes.INST_HAS_UV_RECT | scenes.INST_TEX_OPAQUE)
    sc.tex_coords = sc.uv_rects = sc.opaque_tex = sc.trans_tex = None
    return sc


def _lit(sc, sun_dir, sun_power, ambient_power, ambient=(0.3, 0.35, 0.4), sun=(1.0, 0.9, 0.7)):
    c = sc.config  # lucid_config: the lighting fields are flat members of the ctypes mirror
    n = np.asarray(sun_dir, np.float64)
    n /= np.linalg.norm(n)
    for i in range(3):
        c.sun_dir[i], c.ambient_color[i], c.sun_color[i] = float(n[i]), ambient[i], sun[i]
    c.sun_power, c.ambient_power = sun_power, ambient_power
    return sc


SHADE_SCENES = {
    "flat_normals": lambda: scenes.random_tris(128, 96, 800, seed=41, area_median=200.0),
    "vertex_normals": lambda: _untextured_with_normals(42),
    "alpha_zero_and_lit": lambda: _lit(scenes.random_tris(96, 64, 600, seed=43, alpha_range=(0.0, 0.05),
                                                          area_median=300.0), (0.3, -1.0, 0.2), 2.5, 0.6),
    "vertex_normals_lit": lambda: _lit(_untextured_with_normals(44), (-0.5, -0.2, -1.0), 0.8, 1.4),
}


@pytest.mark.parametrize("name", sorted(SHADE_SCENES))
def test_reference_order_shading(oracle, ref, name):
    """The reference-order mode's shading (the oracle's shadeRef, which the GPU mode matches bit
    for bit in tests/test_gpu_ref_order.py) against the reference's own shadeSample
    (shading.glsl:107-184 with finalShading, funcs.glsl:153-164, 261-271), compiled from its
    source: RGBA8 colour and depth of every sample bit for bit, on samples inside and far
    outside their triangles (barycentrics extrapolated into the clamps). GLSL's pow is
    implementation-defined; both sides use the oracle's refPow."""
    sc = SHADE_SCENES[name]()
    mvq = max(1024, sc.num_quads)
    o = oracle.run(sc, max_visible_quads=mvq, raster=False)
    tris = _visible_tris(o, mvq)
    rng = np.random.default_rng(7)
    n = 20000
    t = tris[rng.integers(0, len(tris), n)].astype(np.uint32)
    px = rng.integers(-8, sc.width + 8, n).astype(np.int32)
    py = rng.integers(-8, sc.height + 8, n).astype(np.int32)
    want_c, want_d = ref.shade_samples(sc, px, py, t, oracle.ref_pow_address(), mvq)
    got_c, got_d = oracle.ref_shade(sc, px, py, t, mvq)
    helpers.assert_same_bits(got_d.view(np.uint32), want_d.view(np.uint32), "depth")
    np.testing.assert_array_equal(got_c, want_c, err_msg="RGBA8 colour")
    assert (want_c != 0).sum() > n // 4  # mostly visible colours, not only the alpha-0 early out


def test_reference_order_reduction(oracle, ref):
    """The oracle's 3-deep reduction window (RefReduce) against the reference's
    initReduceSamples / reduceSample / finishReduceSamples (shading.glsl:196-314), fed one
    pixel's samples in segments as shadeAndReduceSamples hands them over (raster.glsl:361-398):
    the output colour bit for bit on 4000 random sequences (equal depths, runs of increasing and
    decreasing depth, empty RGBA8 colours, opaque and transparent samples, up to 700 samples in
    up to 4 segments)."""
    rng = np.random.default_rng(11)
    for case in range(4000):
        n = int(rng.integers(0, 700 if case % 50 == 0 else 40))
        colors = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
        kind = case % 4
        if kind == 1:
            colors[rng.random(n) < 0.2] = 0  # empty samples (shadeSample's alpha-0 result)
        elif kind == 2:
            colors |= np.uint32(0xFF000000)  # opaque
        depths = rng.uniform(0.01, 10.0, n).astype(np.float32)
        if kind == 3 and n:
            depths = np.sort(depths)[::-1 if case % 8 == 3 else 1].copy()  # monotone runs
        if case % 5 == 0 and n > 2:
            depths[rng.integers(0, n, n // 3)] = depths[0]  # equal depths
        seg = np.sort(rng.integers(0, 4, n)).astype(np.int32)
        bg = rng.uniform(0.0, 1.0, 4).astype(np.float32)
        want = ref.reduce(bg, colors, depths, seg)
        got = oracle.ref_reduce(bg, colors, depths, seg)
        helpers.assert_same_bits(got.view(np.uint32), want.view(np.uint32), f"sequence {case}")
