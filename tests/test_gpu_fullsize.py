"""GPU parity on the full-size workloads, against the CPU oracle on the same inputs.

The benchmarked frames are too large for the oracle to raster whole in a test, so:

* every setup record, bin count, offset, LOW/HIGH list and bin reference list of the whole
  frame is compared (setup and binning are cheap on the CPU);
* on a seeded sample of bins (uniform, plus the bins with the most triangles) the image must
  agree within 1e-5 per channel and each pixel's fragment count and first fragments in blend
  order (input primitive ids: nearest first, ties by primitive id) must be bit-exact;
* the FP32 image's error against the FP64 blend of the same fragments (oracle ``image64``) is
  stated per workload and bounded.

The blend is the reference's front-to-back OIT accumulation (data/shaders/shared/
shading.glsl:279-280, background at :312) over the exact per-pixel order whose key is
inv_ray_pos (shading.glsl:116; the reference sorts by the same depth quantity, raster.glsl:
170-176).
"""
import os

import numpy as np
import pytest

from lucid_gb300 import scenes
from tests import helpers

pytestmark = pytest.mark.gpu

IMG_TOL = 1e-5
FP64_TOL = 1e-4


def sample_bins(counters, bin_count, n_uniform, n_dense, seed):
    rng = np.random.default_rng(seed)
    tris = 2 * counters[:bin_count].astype(np.int64) + counters[3 * bin_count:4 * bin_count]
    dense = np.argsort(-tris, kind="stable")[:n_dense]
    rest = np.setdiff1d(np.arange(bin_count), dense)
    uni = rng.choice(rest, size=min(n_uniform, rest.size), replace=False)
    return np.sort(np.concatenate([dense, uni])).astype(np.int32)


def bin_pixels(bins, bcx, w, h):
    """Pixel mask [n, 32, 32] of pixels inside the viewport and the (y, x) image slices."""
    res = []
    for b in bins:
        by, bx = divmod(int(b), bcx)
        y0, x0 = by * 32, bx * 32
        res.append((slice(y0, min(y0 + 32, h)), slice(x0, min(x0 + 32, w))))
    return res


def compare_full_frame_records(scene, g_renderer, oracle_out, info, counters):
    from lucid_gb300 import _lib
    r = g_renderer
    o = oracle_out
    n = r.options.max_visible_quads
    assert tuple(info.num_visible_quads) == tuple(o["num_visible"])
    assert tuple(info.num_rejected_quads) == tuple(o["rejected"])
    assert info.error_code == o["error_code"] == 0
    slots = helpers.used_slots(o["num_visible"], n)
    helpers.assert_same_bits(r.download(_lib.BUF_QUAD_AABBS)[slots], o["quad_aabbs"][slots], "quad_aabbs")
    helpers.assert_same_bits(r.download(_lib.BUF_QUAD_SOURCE)[slots], o["quad_source"][slots], "quad_source")
    helpers.assert_same_bits(r.download(_lib.BUF_QUAD_VERTS).reshape(n, 4)[slots], o["quad_verts"][slots],
                             "quad_verts")
    enc = o["quad_aabbs"][slots].astype(np.int64)
    tri_slots = np.concatenate([2 * slots[((enc >> 30) & 1) == 0], 2 * slots[((enc >> 31) & 1) == 0] + 1])
    for key, which, width in (("tri_bary", _lib.BUF_TRI_BARY, 8), ("tri_scan", _lib.BUF_TRI_SCAN, 8),
                              ("tri_depth", _lib.BUF_TRI_DEPTH, 4)):
        got = r.download(which).reshape(2 * n, width)
        helpers.assert_same_bits(got[tri_slots], o[key][tri_slots], key)
    bc = o["bin_count"]
    np.testing.assert_array_equal(counters[:6 * bc], o["bin_counters"][:6 * bc], err_msg="bin counts/offsets")
    lv = o["bin_level_counts"]
    assert tuple(info.bin_level_counts) == tuple(lv)
    np.testing.assert_array_equal(counters[7 * bc:7 * bc + lv[2]], o["bin_counters"][7 * bc:7 * bc + lv[2]])
    np.testing.assert_array_equal(counters[9 * bc:9 * bc + lv[4]], o["bin_counters"][9 * bc:9 * bc + lv[4]])
    bq = r.download(_lib.BUF_BIN_QUADS, count=int(info.num_bin_quad_refs))
    bt = r.download(_lib.BUF_BIN_TRIS, count=int(info.num_bin_tri_refs))
    helpers.assert_bin_lists_equal(counters, bc, bq, bt, o["bin_counters"], o["bin_quads"], o["bin_tris"])


def sampled_parity(scene, oracle, name, n_uniform=40, n_dense=8, max_per_pixel=256, seed=0):
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    nq = scene.num_quads
    from lucid_gb300 import _lib
    r = LucidRenderer(scene.width, scene.height, max_input_quads=nq, max_visible_quads=nq, max_bin_refs=8 * nq,
                      flags=_lib.OPT_SORTED_BIN_LISTS)
    frame = FrameInputs.from_scene(scene)
    # binning first (cheap on the CPU) to choose the sample
    ob = oracle.run(scene, max_visible_quads=nq, raster=False)
    bins = sample_bins(ob["bin_counters"], ob["bin_count"], n_uniform, n_dense, seed)
    threads = os.cpu_count() or 1
    o = oracle.run(scene, max_visible_quads=nq, bin_subset=bins, threads=threads, image64=True,
                   max_per_pixel=max_per_pixel, dump_by_subset=True, setup_outputs=False)
    img, counts, prims = r.raster_dump_bins(frame, bins, max_per_pixel)
    info, counters = r.info()
    compare_full_frame_records(scene, r, ob, info, counters)
    np.testing.assert_array_equal(counts, o["frag_counts"], err_msg="per-pixel fragment counts")
    np.testing.assert_array_equal(prims, o["frag_prims"], err_msg="per-pixel fragment order")
    g = img.cpu().numpy()
    # the dump run keeps shading past T == 0; the plain frame must give the same image
    plain = r.render(frame).cpu().numpy()
    np.testing.assert_array_equal(plain, g)
    err32 = err64 = 0.0
    for ys, xs in bin_pixels(bins, ob["bin_count_x"], scene.width, scene.height):
        err32 = max(err32, helpers.max_abs_diff(g[ys, xs], o["image"][ys, xs]))
        err64 = max(err64, helpers.max_abs_diff(g[ys, xs].astype(np.float64), o["image64"][ys, xs]))
    print(f"{name}: {len(bins)} bins, {int(counts.sum())} fragments, max |FP32 - oracle| {err32:.3g}, "
          f"max |FP32 - FP64 blend| {err64:.3g}")
    assert err32 <= IMG_TOL
    assert err64 <= FP64_TOL
    assert not r.verify_info()
    r.close()
    return counts


def test_heavy1080_sampled_bins(gpu, oracle):
    """1920x1080, 1M triangles (the benchmark frame): whole-frame setup and binning, and 48
    bins' images and per-pixel fragment lists (first 256 in blend order)."""
    counts = sampled_parity(scenes.workload("heavy1080"), oracle, "heavy1080")
    assert counts.max() > 1000  # the dense bins reach the deep-window and slab paths


def test_meshes4k_sampled_bins(gpu, oracle):
    """3840x2160, 5M triangles in 2000 meshes of real quads, FP16 colours, 30% translucent."""
    counts = sampled_parity(scenes.workload("meshes4k"), oracle, "meshes4k", max_per_pixel=128)
    assert counts.max() > 8


@pytest.mark.parametrize("name", ["cpu720", "grad512"])
def test_full_frame_fp64_error(gpu, oracle, name):
    """Whole frames of the 1280x720 / 100k-triangle and the 512x512 / 200k-triangle (FP32
    colours, triangle opacity) workloads: every pass against the oracle, and the FP32 image's
    error against the FP64 blend."""
    from tests.test_gpu_parity import compare
    sc = scenes.workload(name)
    g, o = compare(sc, oracle)
    err64 = helpers.max_abs_diff(g["image"].astype(np.float64), o["image64"])
    print(f"{name}: {o['num_fragments']} fragments, max |FP32 - FP64 blend| {err64:.3g}")
    assert err64 <= FP64_TOL
