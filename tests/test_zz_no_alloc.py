"""lucid_bin_noalloc: binning without any device allocation, for callers that cannot call
cudaMalloc (a host allocator owning all device memory, or recording work while allocation is
not allowed). Its scratch is a static device array shared by all calls.

The test feeds it the quad-setup records of two different scenes in a row (through the C ABI,
on caller-owned buffers) and checks both results against the regular binning passes of
lucid_render on the same records (with LUCID_OPT_SORTED_BIN_LISTS, the slot order this entry
point always produces): counts, offsets, LOW/HIGH lists and the reference lists bit-exact. A second call must not see state left by the first. This file is collected last so
that a failure here does not hide results of the other tests; it also passes alone in a fresh
process.
"""
import ctypes

import numpy as np
import pytest

from lucid_gb300 import scenes
from tests import helpers

pytestmark = pytest.mark.gpu


def regular_binning(scene, mvq, cap):
    from lucid_gb300 import _lib
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    r = LucidRenderer(scene.width, scene.height, max_input_quads=max(1024, scene.num_quads),
                      max_visible_quads=mvq, max_bin_refs=cap, flags=_lib.OPT_SORTED_BIN_LISTS)
    r.render(FrameInputs.from_scene(scene))
    info, counters = r.info()
    res = dict(info=info, counters=counters,
               aabbs=r.download(_lib.BUF_QUAD_AABBS), scan=r.download(_lib.BUF_TRI_SCAN),
               bin_quads=r.download(_lib.BUF_BIN_QUADS, count=int(info.num_bin_quad_refs)),
               bin_tris=r.download(_lib.BUF_BIN_TRIS, count=int(info.num_bin_tri_refs)))
    r.close()
    return res


def no_alloc_binning(lib, ref, scene, mvq, cap):
    import torch
    from lucid_gb300 import _lib
    bins = ((scene.width + 31) // 32) * ((scene.height + 31) // 32)
    d_aabbs = torch.from_numpy(ref["aabbs"].view(np.int32)).cuda()
    d_scan = torch.from_numpy(ref["scan"].view(np.int32)).cuda()
    # outputs start out filled with garbage: the entry point must clear what needs clearing
    d_counters = torch.full((10 * bins,), -1, dtype=torch.int32, device="cuda")
    d_bq = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
    d_bt = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
    d_info = torch.full((ctypes.sizeof(_lib.Info) // 4,), -1, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    info = ref["info"]
    st = lib.lucid_bin_noalloc(d_aabbs.data_ptr(), d_scan.data_ptr(), info.num_visible_quads[0],
                               info.num_visible_quads[1], mvq, scene.width, scene.height, 1024,
                               d_counters.data_ptr(), d_bq.data_ptr(), d_bt.data_ptr(), cap,
                               d_info.data_ptr(), stream)
    assert st == 0, lib.lucid_last_error_string()
    torch.cuda.synchronize()
    out_info = _lib.Info.from_buffer_copy(d_info.cpu().numpy().tobytes())
    return d_counters.cpu().numpy().view(np.uint32), d_bq.cpu().numpy().view(np.uint32), \
        d_bt.cpu().numpy().view(np.uint32), out_info


def check_same(ref, counters, bq, bt, info, bins):
    np.testing.assert_array_equal(counters[:6 * bins], ref["counters"][:6 * bins])
    lv = tuple(ref["info"].bin_level_counts)
    assert tuple(info.bin_level_counts) == lv
    np.testing.assert_array_equal(counters[7 * bins:7 * bins + lv[2]], ref["counters"][7 * bins:7 * bins + lv[2]])
    np.testing.assert_array_equal(counters[9 * bins:9 * bins + lv[4]], ref["counters"][9 * bins:9 * bins + lv[4]])
    assert info.error_code == 0
    helpers.assert_bin_lists_equal(counters, bins, bq, bt, ref["counters"], ref["bin_quads"], ref["bin_tris"])


def test_no_alloc_binning_matches_regular_path_twice(gpu, lucid_lib):
    mvq, cap = 8192, 1 << 17
    sc_a = scenes.random_tris(640, 360, 5000, seed=31, area_median=300.0, area_sigma=1.2,
                              large_fraction=0.03, large_area=(2000.0, 20000.0))
    sc_b = scenes.random_tris(640, 360, 3000, seed=32, area_median=800.0, area_sigma=1.0)
    for sc in (sc_a, sc_b):
        ref = regular_binning(sc, mvq, cap)
        assert ref["info"].num_visible_quads[1] > 0
        bins = ((sc.width + 31) // 32) * ((sc.height + 31) // 32)
        counters, bq, bt, info = no_alloc_binning(lucid_lib, ref, sc, mvq, cap)
        check_same(ref, counters, bq, bt, info, bins)


def test_no_alloc_reference_overflow_keeps_writes_in_bounds(gpu, lucid_lib):
    """Too small a max_bin_refs: the call still succeeds, info_out reports LUCID_ERR_BIN_REFS,
    and no reference is written past max_bin_refs (sentinels behind the lists stay intact)."""
    import torch
    from lucid_gb300 import _lib
    mvq, cap, pad = 8192, 300, 4096
    sc = scenes.random_tris(640, 360, 5000, seed=33, area_median=300.0, area_sigma=1.2,
                            large_fraction=0.03, large_area=(2000.0, 20000.0))
    ref = regular_binning(sc, mvq, 1 << 17)
    info = ref["info"]
    assert int(info.num_bin_quad_refs) > cap and int(info.num_bin_tri_refs) > cap
    bins = ((sc.width + 31) // 32) * ((sc.height + 31) // 32)
    sentinel = 0x5A5A5A5A
    d_aabbs = torch.from_numpy(ref["aabbs"].view(np.int32)).cuda()
    d_scan = torch.from_numpy(ref["scan"].view(np.int32)).cuda()
    d_counters = torch.zeros((10 * bins,), dtype=torch.int32, device="cuda")
    d_bq = torch.full((cap + pad,), sentinel, dtype=torch.int32, device="cuda")
    d_bt = torch.full((cap + pad,), sentinel, dtype=torch.int32, device="cuda")
    d_info = torch.zeros((ctypes.sizeof(_lib.Info) // 4,), dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lucid_lib.lucid_bin_noalloc(d_aabbs.data_ptr(), d_scan.data_ptr(), info.num_visible_quads[0],
                                     info.num_visible_quads[1], mvq, sc.width, sc.height, 1024,
                                     d_counters.data_ptr(), d_bq.data_ptr(), d_bt.data_ptr(), cap,
                                     d_info.data_ptr(), stream)
    assert st == 0, lucid_lib.lucid_last_error_string()
    torch.cuda.synchronize()
    out_info = _lib.Info.from_buffer_copy(d_info.cpu().numpy().tobytes())
    assert out_info.error_code == 2  # LUCID_ERR_BIN_REFS
    bq, bt = d_bq.cpu().numpy(), d_bt.cpu().numpy()
    assert (bq[cap:] == sentinel).all() and (bt[cap:] == sentinel).all()
    assert (bq[:cap] != sentinel).any() and (bt[:cap] != sentinel).any()
    # counts and offsets are still complete: they do not depend on the list capacity
    counters = d_counters.cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(counters[:2 * bins], ref["counters"][:2 * bins])
    np.testing.assert_array_equal(counters[3 * bins:5 * bins], ref["counters"][3 * bins:5 * bins])


def test_no_alloc_rejects_oversized_viewport(gpu, lucid_lib):
    from lucid_gb300 import _lib
    st = lucid_lib.lucid_bin_noalloc(None, None, 0, 0, 1024, 3840, 2160, 1024, None, None, None, 0,
                                     None, None)
    assert st == _lib.CAPACITY_EXCEEDED
    assert b"LUCID_NOALLOC_MAX_BINS" in lucid_lib.lucid_last_error_string()
