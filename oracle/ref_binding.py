"""ctypes binding of oracle/_ref/libref_setup.so: the reference's quad-setup functions compiled as
C++ from its shader sources (oracle/ref_build.py). Test infrastructure only."""
from __future__ import annotations

import ctypes

import numpy as np

from . import ref_build

_lib = None


class _In(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("max_visible_quads", ctypes.c_int32),
                ("positions", ctypes.c_void_p), ("colors", ctypes.c_void_p), ("normals", ctypes.c_void_p),
                ("tex_coords", ctypes.c_void_p), ("quads_ib", ctypes.c_void_p), ("instances", ctypes.c_void_p),
                ("num_instances", ctypes.c_int32), ("config", ctypes.c_void_p)]


class _Out(ctypes.Structure):
    _fields_ = [("quad_aabbs", ctypes.c_void_p), ("tri_bary", ctypes.c_void_p), ("tri_scan", ctypes.c_void_p),
                ("tri_depth", ctypes.c_void_p), ("tri_normals", ctypes.c_void_p), ("quad_colors", ctypes.c_void_p),
                ("num_input_quads", ctypes.c_int32), ("num_visible", ctypes.c_int32 * 2),
                ("rejected", ctypes.c_uint32 * 4)]


def lib():
    """The library, or None where the reference tree is absent."""
    global _lib
    if _lib is None:
        path = ref_build.build()
        if path is None:
            return None
        _lib = ctypes.CDLL(path)
        _lib.ref_quad_setup.argtypes = [ctypes.POINTER(_In), ctypes.POINTER(_Out)]
        _lib.ref_quad_setup.restype = ctypes.c_int
    return _lib


def quad_setup(scene, max_visible_quads=None):
    """Runs the reference's setup functions on a lucid_gb300.scenes.Scene; numpy records in the
    oracle's layout (RGBA8 vertex colours only)."""
    L = lib()
    mvq = max_visible_quads or max(1024, scene.num_quads)
    keep = dict(pos=np.ascontiguousarray(scene.positions, np.float32),
                quads=np.ascontiguousarray(scene.quads, np.uint32),
                inst=np.ascontiguousarray(scene.instances, np.int32))
    if scene.colors.dtype == np.uint32:
        keep["cols"] = np.ascontiguousarray(scene.colors, np.uint32)
    nrm = getattr(scene, "normals", None)
    if nrm is not None:
        keep["nrm"] = np.ascontiguousarray(nrm, np.uint32)
    tc = getattr(scene, "tex_coords", None)
    if tc is not None:
        keep["tc"] = np.ascontiguousarray(tc, np.float32)
    out = dict(quad_aabbs=np.zeros(mvq, np.uint32), tri_bary=np.zeros((2 * mvq, 8), np.uint32),
               tri_scan=np.zeros((2 * mvq, 8), np.uint32), tri_depth=np.zeros((2 * mvq, 4), np.uint32),
               tri_normals=np.zeros(2 * mvq, np.uint32), quad_colors=np.zeros((mvq, 4), np.uint32))
    ins = _In(width=scene.width, height=scene.height, max_visible_quads=mvq,
              positions=keep["pos"].ctypes.data,
              colors=keep["cols"].ctypes.data if "cols" in keep else None,
              normals=keep["nrm"].ctypes.data if "nrm" in keep else None,
              tex_coords=keep["tc"].ctypes.data if "tc" in keep else None,
              quads_ib=keep["quads"].ctypes.data, instances=keep["inst"].ctypes.data,
              num_instances=keep["inst"].shape[0], config=ctypes.addressof(scene.config))
    o = _Out(**{k: v.ctypes.data for k, v in out.items()})
    if L.ref_quad_setup(ctypes.byref(ins), ctypes.byref(o)) != 0:
        raise RuntimeError("ref_quad_setup failed")
    out.update(num_input_quads=o.num_input_quads, num_visible=tuple(o.num_visible), rejected=tuple(o.rejected))
    return out


def _bind_more(L):
    if not hasattr(L, "_more"):
        args = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                ctypes.c_int32]
        L.ref_bin_counts.argtypes = args + [ctypes.c_void_p, ctypes.c_void_p]
        L.ref_bin_counts.restype = ctypes.c_int
        L.ref_coverage.argtypes = args + [ctypes.c_void_p]
        L.ref_coverage.restype = ctypes.c_int
        L._more = True


def bin_counts(quad_aabbs, tri_scan, num_visible, mvq, width, height):
    """The reference bin counter's per-bin quad and tri counts for the given setup records."""
    L = lib()
    _bind_more(L)
    bins = ((width + 31) // 32) * ((height + 31) // 32)
    qa = np.ascontiguousarray(quad_aabbs, np.uint32)
    ts = np.ascontiguousarray(tri_scan, np.uint32)
    qc, tc = np.zeros(bins, np.uint32), np.zeros(bins, np.uint32)
    L.ref_bin_counts(qa.ctypes.data, ts.ctypes.data, num_visible[0], num_visible[1], mvq, width, height,
                     qc.ctypes.data, tc.ctypes.data)
    return qc, tc


def coverage(quad_aabbs, tri_scan, num_visible, mvq, width, height):
    """Per-pixel fragment counts from the reference low-level raster's row spans."""
    L = lib()
    _bind_more(L)
    qa = np.ascontiguousarray(quad_aabbs, np.uint32)
    ts = np.ascontiguousarray(tri_scan, np.uint32)
    counts = np.zeros((height, width), np.int32)
    L.ref_coverage(qa.ctypes.data, ts.ctypes.data, num_visible[0], num_visible[1], mvq, width, height,
                   counts.ctypes.data)
    return counts


def _bind_shading(L):
    if not hasattr(L, "_shading"):
        L.ref_shade_samples.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32] + \
            [ctypes.c_void_p] * 5
        L.ref_shade_samples.restype = ctypes.c_int
        L.ref_reduce.argtypes = [ctypes.c_void_p, ctypes.c_int32] + [ctypes.c_void_p] * 4
        L.ref_reduce.restype = ctypes.c_int
        L._shading = True


def shade_samples(scene, px, py, tris, pow_address, max_visible_quads=None):
    """The reference's shadeSample of samples (px[i], py[i], tris[i]) on the records of its own
    setup of `scene` (run here first): RGBA8 colours and depths. pow_address: the pow that GLSL
    leaves to the implementation (the oracle's). Raises if a sample reached the texture stub."""
    L = lib()
    _bind_shading(L)
    quad_setup(scene, max_visible_quads)
    icol = np.ascontiguousarray(scene.instance_colors, np.uint32)
    px = np.ascontiguousarray(px, np.int32)
    py = np.ascontiguousarray(py, np.int32)
    tris = np.ascontiguousarray(tris, np.uint32)
    colors = np.zeros(len(tris), np.uint32)
    depths = np.zeros(len(tris), np.float32)
    tex = L.ref_shade_samples(ctypes.addressof(scene.config), icol.ctypes.data if len(icol) else None,
                              ctypes.c_void_p(pow_address), len(tris), px.ctypes.data, py.ctypes.data,
                              tris.ctypes.data, colors.ctypes.data, depths.ctypes.data)
    if tex != 0:
        raise RuntimeError(f"{tex} samples reached the texture stub")
    return colors, depths


def reduce(background, colors, depths, seg):
    """The reference's initReduceSamples / reduceSample / finishReduceSamples over one pixel's
    samples in segments `seg`: RGBA float32[4]."""
    L = lib()
    _bind_shading(L)
    bg = np.ascontiguousarray(background, np.float32)
    c = np.ascontiguousarray(colors, np.uint32)
    d = np.ascontiguousarray(depths, np.float32)
    s = np.ascontiguousarray(seg, np.int32)
    out = np.zeros(4, np.float32)
    L.ref_reduce(bg.ctypes.data, len(c), c.ctypes.data, d.ctypes.data, s.ctypes.data, out.ctypes.data)
    return out
