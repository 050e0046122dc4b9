"""ctypes declarations of the lucid_gb300 C ABI (include/lucid_gb300.h).

The shared library is the product: if it is missing this module raises instead of falling
back to anything else.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblucid_gb300.so")

c_int32, c_uint32, c_int64, c_uint64 = ctypes.c_int32, ctypes.c_uint32, ctypes.c_int64, ctypes.c_uint64
c_void_p, c_float, c_size_t = ctypes.c_void_p, ctypes.c_float, ctypes.c_size_t

# status codes
OK, INVALID_ARG, CAPACITY_EXCEEDED, CUDA_ERROR, TIMEOUT, NOT_SUPPORTED, OUT_OF_MEMORY = range(7)

# lucid_info.error_code values
ERR_NAMES = {0: "none", 1: "visible quads", 2: "bin refs", 3: "band entries",
             4: "pixel fragments", 5: "instance quads", 6: "bin count"}

# render option flags
OPT_TIMERS, OPT_ADDITIVE_BLENDING, OPT_ALPHA_THRESHOLD, OPT_VISUALIZE_ERRORS = 1, 2, 4, 8
OPT_PIXEL_BLEND, OPT_REFERENCE_ORDER, OPT_SORTED_BIN_LISTS = 16, 32, 64

# internal buffers of lucid_download_buffer
BUF_QUAD_AABBS, BUF_TRI_BARY, BUF_TRI_SCAN, BUF_TRI_DEPTH, BUF_QUAD_COLORS = 0, 1, 2, 3, 4
BUF_TRI_NORMALS, BUF_QUAD_SOURCE, BUF_BIN_QUADS, BUF_BIN_TRIS, BUF_QUAD_VERTS = 5, 6, 7, 8, 9


class Options(ctypes.Structure):
    _fields_ = [("flags", c_uint32), ("bin_size", c_int32), ("max_input_quads", c_int32),
                ("max_visible_quads", c_int32), ("max_instances", c_int32),
                ("low_high_threshold", c_int32), ("max_bin_refs", c_int32),
                ("band_capacity", c_int32), ("binning_ctas", c_int32),
                ("raster_ctas_per_sm", c_int32), ("max_views", c_int32),
                ("grad_store_fragments", c_int32), ("slab_fragments", c_int32), ("light_max_pixel", c_int32),
                ("reserved", c_int32 * 2)]


class TextureC(ctypes.Structure):
    _fields_ = [("texels", c_void_p), ("width", c_int32), ("height", c_int32), ("num_levels", c_int32),
                ("_pad", c_int32)]


class FrameInputsC(ctypes.Structure):
    _fields_ = [("positions", c_void_p), ("colors", c_void_p), ("color_format", c_int32),
                ("num_verts", c_int32), ("quads_ib", c_void_p), ("num_quads", c_int32),
                ("num_instances", c_int32), ("instances", c_void_p),
                ("instance_colors", c_void_p), ("tri_opacity", c_void_p), ("config", c_void_p),
                ("tex_coords", c_void_p), ("instance_uv_rects", c_void_p), ("normals", c_void_p),
                ("opaque_texture", c_void_p), ("transparent_texture", c_void_p)]


class Info(ctypes.Structure):
    _fields_ = [
        ("num_input_quads", c_int32), ("num_visible_quads", c_int32 * 2),
        ("num_counted_quads", c_int32 * 2), ("bin_level_counts", c_int32 * 5),
        ("a_small_bins", c_uint32), ("a_high_bins", c_uint32), ("a_setup_work_groups", c_uint32),
        ("a_dummy_counter", c_uint32), ("num_binning_dispatches", c_uint32 * 3),
        ("bin_level_dispatches", (c_uint32 * 3) * 5), ("num_rejected_quads", c_uint32 * 4),
        ("setup_timers", c_uint32 * 8), ("raster_timers", c_uint32 * 8),
        ("bin_dispatcher_timers", c_uint32 * 8), ("stats", c_uint32 * 4),
        ("dispatcher_first_batch", (c_int32 * 256) * 2),
        ("dispatcher_num_batches", (c_int32 * 256) * 2), ("temp", c_int32 * 64),
        ("error_code", c_uint32), ("error_detail", c_uint32 * 3),
        ("raster_work_counter", c_uint32), ("num_bin_quad_refs", c_uint32),
        ("num_bin_tri_refs", c_uint32), ("max_pixel_fragments", c_uint32),
        ("num_fragments", c_uint64), ("num_hblock_tris", c_uint64),
        ("num_band_entries", c_uint32), ("num_views", c_uint32),
        ("raster_windows", c_uint64), ("raster_window_fragments", c_uint64),
        ("raster_radix_windows", c_uint32), ("raster_light_bins", c_uint32),
        ("raster_blended_fragments", ctypes.c_uint64), ("ext_reserved", c_uint32 * 42)]


assert ctypes.sizeof(Info) == 1216 * 4


class DrawCall(ctypes.Structure):
    _fields_ = [("quad_offset", c_int32), ("num_quads", c_int32), ("opts", c_uint32),
                ("material_color", c_uint32)]


class CameraC(ctypes.Structure):
    _fields_ = [("position", c_float * 3), ("right", c_float * 3), ("up", c_float * 3),
                ("forward", c_float * 3), ("fov_y_radians", c_float), ("near_plane", c_float),
                ("far_plane", c_float)]


class Tuning(ctypes.Structure):
    _fields_ = [("pixel_blend", c_uint32), ("low_high_threshold", c_int32), ("binning_ctas", c_int32),
                ("num_candidates", c_int32), ("frame_ms", ctypes.c_float), ("default_ms", ctypes.c_float),
                ("light_max_pixel", c_int32), ("bin_size", c_int32)]


class ViewC(ctypes.Structure):
    _fields_ = [("width", c_int32), ("height", c_int32), ("inputs", FrameInputsC),
                ("out_rgba", c_void_p)]


# (name, restype, argtypes) of every exported entry point
SIGNATURES = [
    ("lucid_status_string", ctypes.c_char_p, [c_int32]),
    ("lucid_last_error_string", ctypes.c_char_p, []),
    ("lucid_abi_version", c_int32, []),
    ("lucid_default_options", c_int32, [ctypes.POINTER(Options)]),
    ("lucid_build_instances", c_int32, [ctypes.POINTER(DrawCall), c_int32, c_void_p, c_void_p,
                                        c_int32, ctypes.POINTER(c_int32), ctypes.POINTER(c_int32)]),
    ("lucid_make_config", c_int32, [ctypes.POINTER(CameraC), c_int32, c_int32, c_void_p, c_int32,
                                    c_void_p]),
    ("lucid_create", c_int32, [ctypes.POINTER(Options), c_int32, c_int32, ctypes.POINTER(c_void_p)]),
    ("lucid_destroy", c_int32, [c_void_p]),
    ("lucid_render", c_int32, [c_void_p, ctypes.POINTER(FrameInputsC), c_void_p, c_void_p]),
    ("lucid_quad_setup", c_int32, [c_void_p, ctypes.POINTER(FrameInputsC), c_void_p]),
    ("lucid_bin_count", c_int32, [c_void_p, c_void_p]),
    ("lucid_bin_categorize", c_int32, [c_void_p, c_void_p]),
    ("lucid_bin_dispatch", c_int32, [c_void_p, c_void_p]),
    ("lucid_raster", c_int32, [c_void_p, ctypes.POINTER(FrameInputsC), c_void_p, c_void_p]),
    ("lucid_get_info", c_int32, [c_void_p, ctypes.POINTER(Info), c_void_p, c_void_p]),
    ("lucid_download_buffer", c_int32, [c_void_p, c_int32, c_void_p, c_size_t,
                                        ctypes.POINTER(c_size_t), c_void_p]),
    ("lucid_raster_dump", c_int32, [c_void_p, ctypes.POINTER(FrameInputsC), c_void_p, c_int32,
                                    c_void_p, c_void_p, c_void_p]),
    ("lucid_raster_dump_bins", c_int32, [c_void_p, ctypes.POINTER(FrameInputsC), c_void_p, c_void_p,
                                         c_int32, c_int32, c_void_p, c_void_p, c_void_p]),
    ("lucid_render_forward_grad", c_int32, [c_void_p, ctypes.POINTER(FrameInputsC), c_void_p, c_void_p]),
    ("lucid_render_backward", c_int32, [c_void_p, ctypes.POINTER(FrameInputsC), c_void_p,
                                        c_void_p, c_void_p, c_void_p]),
    ("lucid_render_batch", c_int32, [c_void_p, ctypes.POINTER(ViewC), c_int32, c_void_p]),
    ("lucid_get_batch_info", c_int32, [c_void_p, c_int32, ctypes.POINTER(Info), c_void_p]),
    ("lucid_autotune", c_int32, [c_void_p, ctypes.POINTER(FrameInputsC), c_void_p,
                                 ctypes.POINTER(Tuning), c_void_p]),
    ("lucid_autotune_batch", c_int32, [c_void_p, ctypes.POINTER(ViewC), c_int32,
                                       ctypes.POINTER(Tuning), c_void_p]),
    ("lucid_quad_generate", c_int32, [c_void_p, c_int32, c_void_p, c_int32, ctypes.c_float, c_void_p,
                                      ctypes.POINTER(c_int32), ctypes.POINTER(c_int32), c_void_p]),
    ("lucid_bin_noalloc", c_int32, [c_void_p, c_void_p, c_int32, c_int32, c_int32, c_int32,
                                    c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_int32,
                                    c_void_p, c_void_p]),
]

_lib = None


class LucidError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


def load():
    """Loads liblucid_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run lucid_gb300.build.build() first")
        lib = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(status: int, what: str = ""):
    if status != OK:
        lib = load()
        msg = lib.lucid_last_error_string().decode() or lib.lucid_status_string(status).decode()
        raise LucidError(status, f"{what}: {msg}" if what else msg)
