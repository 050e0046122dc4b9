"""ctypes binding of the CPU oracle (test infrastructure only).

``run(scene, ...)`` executes quad setup, binning and (optionally) the exact raster pass on the
CPU and returns every intermediate as numpy arrays in the same layout the CUDA path uses.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


class OracleInputs(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int32), ("height", ctypes.c_int32),
        ("max_visible_quads", ctypes.c_int32), ("low_high_threshold", ctypes.c_int32),
        ("flags", ctypes.c_uint32), ("order_mode", ctypes.c_int32),
        ("positions", ctypes.c_void_p), ("colors", ctypes.c_void_p),
        ("color_format", ctypes.c_int32), ("num_verts", ctypes.c_int32),
        ("quads_ib", ctypes.c_void_p), ("num_quads", ctypes.c_int32),
        ("num_instances", ctypes.c_int32), ("instances", ctypes.c_void_p),
        ("instance_colors", ctypes.c_void_p), ("tri_opacity", ctypes.c_void_p),
        ("config", ctypes.c_void_p),
        ("tex_coords", ctypes.c_void_p), ("instance_uv_rects", ctypes.c_void_p), ("normals", ctypes.c_void_p),
        ("opaque_texture", ctypes.c_void_p), ("transparent_texture", ctypes.c_void_p),
        ("bin_subset", ctypes.c_void_p), ("num_bin_subset", ctypes.c_int32),
        ("num_threads", ctypes.c_int32),
    ]


class OracleOutputs(ctypes.Structure):
    _fields_ = [
        ("num_input_quads", ctypes.c_int32), ("num_visible", ctypes.c_int32 * 2),
        ("rejected", ctypes.c_uint32 * 4), ("error_code", ctypes.c_uint32),
        ("num_binning_dispatches", ctypes.c_uint32),
        ("quad_aabbs", ctypes.c_void_p), ("quad_source", ctypes.c_void_p),
        ("quad_colors", ctypes.c_void_p), ("quad_verts", ctypes.c_void_p),
        ("tri_bary", ctypes.c_void_p), ("tri_scan", ctypes.c_void_p),
        ("tri_depth", ctypes.c_void_p), ("tri_normals", ctypes.c_void_p),
        ("bin_count", ctypes.c_int32), ("bin_count_x", ctypes.c_int32),
        ("bin_count_y", ctypes.c_int32),
        ("bin_counters", ctypes.c_void_p), ("bin_quads", ctypes.c_void_p),
        ("bin_tris", ctypes.c_void_p), ("bin_refs_capacity", ctypes.c_int64),
        ("num_bin_quads", ctypes.c_int64), ("num_bin_tris", ctypes.c_int64),
        ("bin_level_counts", ctypes.c_int32 * 5),
        ("image", ctypes.c_void_p), ("image64", ctypes.c_void_p),
        ("frag_counts", ctypes.c_void_p), ("frag_prims", ctypes.c_void_p),
        ("max_per_pixel", ctypes.c_int32),
        ("num_fragments", ctypes.c_uint64), ("num_hblock_tris", ctypes.c_uint64),
        ("max_pixel_fragments", ctypes.c_uint32), ("invalid_pixels", ctypes.c_uint64),
        ("dump_by_subset", ctypes.c_int32),
    ]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = ctypes.CDLL(path)
        _lib.oracle_run.argtypes = [ctypes.POINTER(OracleInputs), ctypes.POINTER(OracleOutputs)]
        _lib.oracle_run.restype = ctypes.c_int
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


class _Texture(ctypes.Structure):
    _fields_ = [("texels", ctypes.c_void_p), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("num_levels", ctypes.c_int32), ("_pad", ctypes.c_int32)]


def _shading_inputs(scene, keep):
    """Pointers of the optional shading inputs (kept alive in `keep`)."""
    def arr(a, dt):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dt)
        keep.append(a)
        return a.ctypes.data

    def tex(t):
        if t is None:
            return None
        texels = t.packed()
        desc = _Texture(texels.ctypes.data, t.width, t.height, len(t.levels), 0)
        keep.extend([texels, desc])
        return ctypes.addressof(desc)

    return dict(tex_coords=arr(getattr(scene, "tex_coords", None), np.float32),
                instance_uv_rects=arr(getattr(scene, "uv_rects", None), np.float32),
                normals=arr(getattr(scene, "normals", None), np.uint32),
                opaque_texture=tex(getattr(scene, "opaque_tex", None)),
                transparent_texture=tex(getattr(scene, "trans_tex", None)))


def run(scene, max_visible_quads: int | None = None, raster: bool = True, image64: bool = False,
        bin_subset=None, threads: int = 1, max_per_pixel: int = 0, flags: int = 0,
        low_high_threshold: int = 1024, setup_outputs: bool = True, order_mode: int = 0,
        dump_by_subset: bool = False, bin_ref_capacity: int | None = None):
    """Runs the oracle on a ``lucid_gb300.scenes.Scene``; returns a dict of numpy arrays.

    With ``bin_subset`` and ``dump_by_subset`` (exact order only) the fragment counts and
    prims cover the subset's bins alone, in ascending bin order: ``frag_counts`` [n, 32, 32],
    ``frag_prims`` [n, 32, 32, max_per_pixel]; the images stay full-frame."""
    L = lib()
    mvq = max_visible_quads or max(1024, scene.num_quads)
    w, h = scene.width, scene.height
    positions = np.ascontiguousarray(scene.positions, dtype=np.float32)
    colors = np.ascontiguousarray(scene.colors)
    quads = np.ascontiguousarray(scene.quads, dtype=np.uint32)
    inst = np.ascontiguousarray(scene.instances, dtype=np.int32)
    icol = np.ascontiguousarray(scene.instance_colors, dtype=np.uint32)
    opac = None if scene.tri_opacity is None else np.ascontiguousarray(scene.tri_opacity, np.float32)
    subset = None if bin_subset is None else np.ascontiguousarray(np.sort(bin_subset), np.int32)

    bins_x, bins_y = (w + 31) // 32, (h + 31) // 32
    bins = bins_x * bins_y
    out = {}
    if setup_outputs:
        out["quad_aabbs"] = np.zeros(mvq, np.uint32)
        out["quad_source"] = np.zeros(mvq, np.uint32)
        out["quad_colors"] = np.zeros((mvq, 4), np.uint32)
        out["quad_verts"] = np.zeros((mvq, 4), np.uint32)
        out["tri_bary"] = np.zeros((2 * mvq, 8), np.uint32)
        out["tri_scan"] = np.zeros((2 * mvq, 8), np.uint32)
        out["tri_depth"] = np.zeros((2 * mvq, 4), np.uint32)
        out["tri_normals"] = np.zeros(2 * mvq, np.uint32)
    out["bin_counters"] = np.zeros(10 * bins, np.uint32)
    cap = int(8 * scene.num_quads + 1024) if bin_ref_capacity is None else int(bin_ref_capacity)
    out["bin_quads"] = np.zeros(cap, np.uint32)
    out["bin_tris"] = np.zeros(cap, np.uint32)
    compact = dump_by_subset and subset is not None and order_mode == 0
    if raster:
        out["image"] = np.zeros((h, w, 4), np.float32)
        dump_shape = (len(subset), 32, 32) if compact else (h, w)
        out["frag_counts"] = np.zeros(dump_shape, np.int32)
        if image64:
            out["image64"] = np.zeros((h, w, 4), np.float64)
        if max_per_pixel > 0:
            out["frag_prims"] = np.full(dump_shape + (max_per_pixel,), -1, np.int32)

    cfg = scene.config
    keep = []
    ins = OracleInputs(
        **_shading_inputs(scene, keep),
        width=w, height=h, max_visible_quads=mvq, low_high_threshold=low_high_threshold,
        flags=flags, order_mode=order_mode, positions=_ptr(positions), colors=_ptr(colors),
        color_format=scene.color_format, num_verts=positions.shape[0], quads_ib=_ptr(quads),
        num_quads=quads.shape[0], num_instances=inst.shape[0], instances=_ptr(inst),
        instance_colors=_ptr(icol), tri_opacity=_ptr(opac), config=ctypes.addressof(cfg),
        bin_subset=_ptr(subset), num_bin_subset=0 if subset is None else len(subset),
        num_threads=max(1, threads))
    outs = OracleOutputs()
    for k, v in out.items():
        setattr(outs, k, v.ctypes.data)
    outs.bin_refs_capacity = cap
    outs.max_per_pixel = max_per_pixel
    outs.dump_by_subset = 1 if compact else 0
    rc = L.oracle_run(ctypes.byref(ins), ctypes.byref(outs))
    if rc != 0:
        raise RuntimeError(f"oracle_run failed ({rc})")
    nbq, nbt = int(outs.num_bin_quads), int(outs.num_bin_tris)
    if nbq > cap or nbt > cap:
        if bin_ref_capacity is not None:
            raise RuntimeError("oracle bin reference capacity exceeded")
        # the counts are complete: run again with lists of the needed size
        return run(scene, max_visible_quads, raster, image64, bin_subset, threads, max_per_pixel, flags,
                   low_high_threshold, setup_outputs, order_mode, dump_by_subset, bin_ref_capacity=max(nbq, nbt))
    out["bin_quads"] = out["bin_quads"][:nbq]
    out["bin_tris"] = out["bin_tris"][:nbt]
    out.update(
        num_input_quads=outs.num_input_quads, num_visible=tuple(outs.num_visible),
        rejected=tuple(outs.rejected), error_code=outs.error_code,
        num_binning_dispatches=outs.num_binning_dispatches,
        bin_count=outs.bin_count, bin_count_x=outs.bin_count_x, bin_count_y=outs.bin_count_y,
        bin_level_counts=tuple(outs.bin_level_counts), num_fragments=int(outs.num_fragments),
        num_hblock_tris=int(outs.num_hblock_tris),
        max_pixel_fragments=int(outs.max_pixel_fragments), invalid_pixels=int(outs.invalid_pixels),
        max_visible_quads=mvq)
    return out


class GradModel:
    """FP64 gradient model of a scene (see oracle_grad_* in lucid_oracle.h)."""

    def __init__(self, scene, max_visible_quads=None):
        L = lib()
        if not hasattr(L, "_grad_bound"):
            L.oracle_grad_build.argtypes = [ctypes.POINTER(OracleInputs)]
            L.oracle_grad_build.restype = ctypes.c_void_p
            L.oracle_grad_free.argtypes = [ctypes.c_void_p]
            L.oracle_grad_loss.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
            L.oracle_grad_loss.restype = ctypes.c_double
            L.oracle_grad_analytic.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 5
            L.oracle_grad_backprop.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 6
            L.oracle_grad_fd.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_double]
            L.oracle_grad_fd.restype = ctypes.c_double
            L.oracle_grad_num_fragments.argtypes = [ctypes.c_void_p]
            L.oracle_grad_num_fragments.restype = ctypes.c_uint64
            L._grad_bound = True
        self.L = L
        self.scene = scene
        mvq = max_visible_quads or max(1024, scene.num_quads)
        self._keep = dict(
            positions=np.ascontiguousarray(scene.positions, np.float32),
            colors=np.ascontiguousarray(scene.colors),
            quads=np.ascontiguousarray(scene.quads, np.uint32),
            inst=np.ascontiguousarray(scene.instances, np.int32),
            icol=np.ascontiguousarray(scene.instance_colors, np.uint32),
            opac=None if scene.tri_opacity is None else np.ascontiguousarray(scene.tri_opacity, np.float32))
        k = self._keep
        self._shade_keep = []
        ins = OracleInputs(
            **_shading_inputs(scene, self._shade_keep),
            width=scene.width, height=scene.height, max_visible_quads=mvq, low_high_threshold=1024,
            flags=0, order_mode=0, positions=_ptr(k["positions"]), colors=_ptr(k["colors"]),
            color_format=scene.color_format, num_verts=k["positions"].shape[0], quads_ib=_ptr(k["quads"]),
            num_quads=k["quads"].shape[0], num_instances=k["inst"].shape[0], instances=_ptr(k["inst"]),
            instance_colors=_ptr(k["icol"]), tri_opacity=_ptr(k["opac"]), config=ctypes.addressof(scene.config),
            bin_subset=None, num_bin_subset=0, num_threads=1)
        self.ctx = L.oracle_grad_build(ctypes.byref(ins))
        if not self.ctx:
            raise RuntimeError("oracle_grad_build failed")

    def __del__(self):
        if getattr(self, "ctx", None):
            self.L.oracle_grad_free(self.ctx)
            self.ctx = None

    @property
    def num_fragments(self):
        return int(self.L.oracle_grad_num_fragments(self.ctx))

    def loss(self, vcolors, opacity, target):
        vc = np.ascontiguousarray(vcolors, np.float64)
        op = None if opacity is None else np.ascontiguousarray(opacity, np.float64)
        tg = np.ascontiguousarray(target, np.float32)
        return float(self.L.oracle_grad_loss(self.ctx, vc.ctypes.data, _ptr(op), tg.ctypes.data))

    def analytic(self, vcolors, opacity, target):
        vc = np.ascontiguousarray(vcolors, np.float64)
        op = None if opacity is None else np.ascontiguousarray(opacity, np.float64)
        tg = np.ascontiguousarray(target, np.float32)
        dvc = np.zeros_like(vc)
        dop = None if op is None else np.zeros_like(op)
        self.L.oracle_grad_analytic(self.ctx, vc.ctypes.data, _ptr(op), tg.ctypes.data, dvc.ctypes.data,
                                    _ptr(dop))
        return dvc, dop

    def backprop(self, vcolors, opacity, dl_dimage, color32):
        """Adjoint alone: dL/dparams for a given upstream gradient dl_dimage [h, w, 4] and the
        FP32 unclamped colour color32 [h, w, 3] (clamp mask)."""
        vc = np.ascontiguousarray(vcolors, np.float64)
        op = None if opacity is None else np.ascontiguousarray(opacity, np.float64)
        gi = np.ascontiguousarray(dl_dimage, np.float32)
        c32 = np.ascontiguousarray(color32, np.float32)
        dvc = np.zeros_like(vc)
        dop = None if op is None else np.zeros_like(op)
        rc = self.L.oracle_grad_backprop(self.ctx, vc.ctypes.data, _ptr(op), gi.ctypes.data, c32.ctypes.data,
                                         dvc.ctypes.data, _ptr(dop))
        if rc != 0:
            raise RuntimeError("oracle_grad_backprop failed")
        return dvc, dop

    def fd(self, vcolors, opacity, target, kind, index, h=1e-4):
        vc = np.ascontiguousarray(vcolors, np.float64)
        op = None if opacity is None else np.ascontiguousarray(opacity, np.float64)
        tg = np.ascontiguousarray(target, np.float32)
        return float(self.L.oracle_grad_fd(self.ctx, vc.ctypes.data, _ptr(op), tg.ctypes.data, kind, index, h))


def quadgen(positions, tris, square_weight=1.0, order=0):
    """Quad generator (oracle_quadgen): order 0 = the reference's greedy, 1 = fixed order.
    Returns (quads uint32 [n, 4], num_degenerate)."""
    L = lib()
    if not hasattr(L, "_qg_bound"):
        L.oracle_quadgen.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                                     ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                     ctypes.POINTER(ctypes.c_int32)]
        L.oracle_quadgen.restype = ctypes.c_int
        L._qg_bound = True
    pos = np.ascontiguousarray(positions, np.float32)
    tr = np.ascontiguousarray(tris, np.int32)
    out = np.zeros((max(1, tr.shape[0]), 4), np.uint32)
    n, nd = ctypes.c_int32(), ctypes.c_int32()
    rc = L.oracle_quadgen(pos.ctypes.data, pos.shape[0], tr.ctypes.data, tr.shape[0], float(square_weight), order,
                          out.ctypes.data, ctypes.byref(n), ctypes.byref(nd))
    if rc != 0:
        raise RuntimeError(f"oracle_quadgen failed ({rc})")
    return out[:n.value], nd.value


def _bind_ref(L):
    if not hasattr(L, "_ref_bound"):
        L.oracle_ref_shade.argtypes = [ctypes.POINTER(OracleInputs), ctypes.c_int32] + [ctypes.c_void_p] * 5
        L.oracle_ref_shade.restype = ctypes.c_int
        L.oracle_ref_reduce.argtypes = [ctypes.c_void_p, ctypes.c_int32] + [ctypes.c_void_p] * 4
        L.oracle_ref_reduce.restype = ctypes.c_int
        L.oracle_ref_pow.argtypes = [ctypes.c_float, ctypes.c_float]
        L.oracle_ref_pow.restype = ctypes.c_float
        L._ref_bound = True


def ref_pow_address():
    """Address of the oracle's pow (oracle_ref_pow), for the reference harness's GLSL pow."""
    L = lib()
    _bind_ref(L)
    return ctypes.cast(L.oracle_ref_pow, ctypes.c_void_p).value


def ref_shade(scene, px, py, tris, max_visible_quads=None):
    """The reference-order mode's shading (shadeRef) of samples (px[i], py[i], tris[i]) after the
    oracle's setup of `scene`: RGBA8 colours (uint32) and depths (float32)."""
    L = lib()
    _bind_ref(L)
    mvq = max_visible_quads or max(1024, scene.num_quads)
    keep = []
    positions = np.ascontiguousarray(scene.positions, dtype=np.float32)
    colors = np.ascontiguousarray(scene.colors)
    quads = np.ascontiguousarray(scene.quads, dtype=np.uint32)
    inst = np.ascontiguousarray(scene.instances, dtype=np.int32)
    icol = np.ascontiguousarray(scene.instance_colors, dtype=np.uint32)
    opac = None if scene.tri_opacity is None else np.ascontiguousarray(scene.tri_opacity, np.float32)
    keep += [positions, colors, quads, inst, icol, opac]
    ins = OracleInputs(
        **_shading_inputs(scene, keep), width=scene.width, height=scene.height, max_visible_quads=mvq,
        low_high_threshold=1024, flags=0, order_mode=1, positions=_ptr(positions), colors=_ptr(colors),
        color_format=scene.color_format, num_verts=positions.shape[0], quads_ib=_ptr(quads),
        num_quads=quads.shape[0], num_instances=inst.shape[0], instances=_ptr(inst),
        instance_colors=_ptr(icol), tri_opacity=_ptr(opac), config=ctypes.addressof(scene.config),
        bin_subset=None, num_bin_subset=0, num_threads=1)
    px = np.ascontiguousarray(px, np.int32)
    py = np.ascontiguousarray(py, np.int32)
    tris = np.ascontiguousarray(tris, np.uint32)
    out_c = np.zeros(len(tris), np.uint32)
    out_d = np.zeros(len(tris), np.float32)
    if L.oracle_ref_shade(ctypes.byref(ins), len(tris), px.ctypes.data, py.ctypes.data, tris.ctypes.data,
                          out_c.ctypes.data, out_d.ctypes.data) != 0:
        raise RuntimeError("oracle_ref_shade failed")
    return out_c, out_d


def ref_reduce(background, colors, depths, seg):
    """One pixel's samples through the reference-order mode's 3-deep window (RefReduce):
    RGBA float32[4]."""
    L = lib()
    _bind_ref(L)
    bg = np.ascontiguousarray(background, np.float32)
    c = np.ascontiguousarray(colors, np.uint32)
    d = np.ascontiguousarray(depths, np.float32)
    s = np.ascontiguousarray(seg, np.int32)
    out = np.zeros(4, np.float32)
    if L.oracle_ref_reduce(bg.ctypes.data, len(c), c.ctypes.data, d.ctypes.data, s.ctypes.data,
                           out.ctypes.data) != 0:
        raise RuntimeError("oracle_ref_reduce failed")
    return out
