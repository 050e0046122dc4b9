"""Shared helpers of the parity tests."""
import os

import numpy as np

from lucid_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def kat_cases():
    data = np.load(os.path.join(GOLDEN, "kat.npz"))
    names = sorted({k.split("/")[0] for k in data.files})
    return {n: {k.split("/")[1]: data[k] for k in data.files if k.startswith(n + "/")} for n in names}


def kat_scene(case):
    w, h = (int(v) for v in case["size"])
    return scenes.screen_triangles(case["tris"], case["colors"], w, h, tuple(case["bg"]))


def canonical_quad_lists(counters, bin_count, lists):
    """Per-bin quad reference lists sorted by slot, keeping the cull-flag bits of every entry."""
    cnt = counters[0:bin_count]
    off = counters[bin_count:2 * bin_count]
    res = []
    for b in range(bin_count):
        seg = np.asarray(lists[int(off[b]):int(off[b]) + int(cnt[b])], np.uint32)
        order = np.argsort(seg & np.uint32(0x0FFFFFFF), kind="stable")
        res.append(seg[order])
    return res


def canonical_tri_lists(counters, bin_count, lists):
    cnt = counters[3 * bin_count:4 * bin_count]
    off = counters[4 * bin_count:5 * bin_count]
    return [np.sort(np.asarray(lists[int(off[b]):int(off[b]) + int(cnt[b])], np.uint32))
            for b in range(bin_count)]


def assert_same_bits(got, want, msg=""):
    """Bit-exact equality of u32 record arrays, except that two NaNs compare equal (the GPU's
    canonical NaN is 0x7fffffff, x86's 0x7fc00000; both behave the same in every later use)."""
    got = np.ascontiguousarray(got, np.uint32)
    want = np.ascontiguousarray(want, np.uint32)
    neq = got != want
    if neq.any():
        both_nan = np.isnan(got.view(np.float32)) & np.isnan(want.view(np.float32))
        bad = neq & ~both_nan
        if bad.any():
            idx = np.argwhere(bad)[:5]
            raise AssertionError(f"{msg}: {int(bad.sum())} mismatches, first at {idx.tolist()}: "
                                 f"got {got[bad][:5]} want {want[bad][:5]}")


def max_abs_diff(a, b):
    """Max |a-b| where NaN == NaN (and NaN vs number counts as infinite)."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    both = np.isnan(a) & np.isnan(b)
    d = np.abs(a - b)
    d[both] = 0.0
    d[np.isnan(d)] = np.inf
    return float(d.max()) if d.size else 0.0


def used_slots(nvis, mvq):
    """Quad slot indices holding visible quads (small from 0 up, large from mvq-1 down)."""
    small = np.arange(nvis[0])
    large = mvq - 1 - np.arange(nvis[1])
    return np.concatenate([small, large]).astype(np.int64)


def assert_bin_lists_equal(counters, bin_count, bin_quads, bin_tris, ref_counters, ref_quads, ref_tris,
                           exact=True):
    """The quad and tri reference lists of two binning runs are the same lists: bit for bit (the
    same offsets and, inside each bin, the same references in slot order; runs with
    LUCID_OPT_SORTED_BIN_LISTS and the oracle) or, with exact=False, the same references per bin
    in any order (the dispatcher's own order follows its atomics)."""
    n = bin_count
    np.testing.assert_array_equal(counters[:6 * n], ref_counters[:6 * n], err_msg="bin counts/offsets")
    if not exact:
        gq, rq = canonical_quad_lists(counters, n, bin_quads), canonical_quad_lists(ref_counters, n, ref_quads)
        gt, rt = canonical_tri_lists(counters, n, bin_tris), canonical_tri_lists(ref_counters, n, ref_tris)
        for b in range(n):
            np.testing.assert_array_equal(gq[b], rq[b], err_msg=f"bin {b} quads")
            np.testing.assert_array_equal(gt[b], rt[b], err_msg=f"bin {b} tris")
        return
    nq, nt = int(counters[:n].sum()), int(counters[3 * n:4 * n].sum())
    bq, rq = np.asarray(bin_quads, np.uint32)[:nq], np.asarray(ref_quads, np.uint32)[:nq]
    bt, rt = np.asarray(bin_tris, np.uint32)[:nt], np.asarray(ref_tris, np.uint32)[:nt]
    for got, want, what in ((bq, rq, "quad"), (bt, rt, "tri")):
        bad = np.nonzero(got != want)[0]
        if bad.size:
            raise AssertionError(f"bin {what} references differ at {bad.size} positions, first {bad[:5].tolist()}: "
                                 f"got {got[bad[:5]].tolist()} want {want[bad[:5]].tolist()}")
