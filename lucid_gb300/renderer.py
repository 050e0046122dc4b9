"""Python mirror of LucidRenderer (src/lucid_renderer.h:21-96) over the lucid_gb300 C ABI.

PyTorch only provides device memory and the current CUDA stream; every pass runs in the
hand-written CUDA kernels of liblucid_gb300.so. There is no CPU fallback: constructing a
renderer without the library or without a GPU raises.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check


def _stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _dptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _dptr_or_none(t):
    return None if t is None else t.data_ptr()


class FrameInputs:
    """Device-resident inputs of one frame (RenderContext, src/lucid_base.h:72-84)."""

    def __init__(self, positions, colors, color_format, quads, instances, instance_colors, config,
                 tri_opacity=None, num_verts=None, tex_coords=None, uv_rects=None, normals=None,
                 opaque_tex=None, trans_tex=None):
        self.positions = positions
        self.colors = colors
        self.color_format = int(color_format)
        self.quads = quads
        self.instances = instances
        self.instance_colors = instance_colors
        self.tri_opacity = tri_opacity
        self.config = config  # scenes.LucidConfig (host)
        self.num_verts = int(num_verts if num_verts is not None else positions.shape[0])
        self.tex_coords, self.uv_rects, self.normals = tex_coords, uv_rects, normals
        # textures: (texels tensor, width, height, levels); descriptors live as long as the frame
        self.opaque_tex, self.trans_tex = opaque_tex, trans_tex
        self._tex_desc = [None if t is None else _lib.TextureC(t[0].data_ptr(), t[1], t[2], t[3], 0)
                          for t in (opaque_tex, trans_tex)]

    @classmethod
    def from_scene(cls, scene, device="cuda", tri_opacity=None, colors=None):
        def up(a, dtype=None):
            t = torch.from_numpy(np.ascontiguousarray(a))
            if dtype is not None:
                t = t.view(dtype)
            return t.to(device)
        cols = scene.colors if colors is None else colors
        if cols.dtype == np.uint32:
            col_t = up(cols.view(np.int32))
        elif cols.dtype == np.float16:
            col_t = up(cols)
        else:
            col_t = up(cols.astype(np.float32))
        opac = scene.tri_opacity if tri_opacity is None else tri_opacity

        def tex(t):
            if t is None:
                return None
            return (up(t.packed().view(np.int32)), t.width, t.height, len(t.levels))

        tc = getattr(scene, "tex_coords", None)
        uvr = getattr(scene, "uv_rects", None)
        nrm = getattr(scene, "normals", None)
        return cls(up(scene.positions.astype(np.float32)), col_t, scene.color_format,
                   up(scene.quads.view(np.int32)), up(scene.instances.astype(np.int32)),
                   up(scene.instance_colors.view(np.int32)), scene.config,
                   None if opac is None else up(np.asarray(opac, np.float32)),
                   tex_coords=None if tc is None else up(np.asarray(tc, np.float32)),
                   uv_rects=None if uvr is None else up(np.asarray(uvr, np.float32)),
                   normals=None if nrm is None else up(np.asarray(nrm, np.uint32).view(np.int32)),
                   opaque_tex=tex(getattr(scene, "opaque_tex", None)),
                   trans_tex=tex(getattr(scene, "trans_tex", None)))

    def c_struct(self) -> _lib.FrameInputsC:
        return _lib.FrameInputsC(
            positions=self.positions.data_ptr(), colors=self.colors.data_ptr(),
            color_format=self.color_format, num_verts=self.num_verts,
            quads_ib=self.quads.data_ptr(), num_quads=int(self.quads.shape[0]),
            num_instances=int(self.instances.shape[0]), instances=self.instances.data_ptr(),
            instance_colors=self.instance_colors.data_ptr() if self.instance_colors is not None else None,
            tri_opacity=self.tri_opacity.data_ptr() if self.tri_opacity is not None else None,
            config=ctypes.addressof(self.config),
            tex_coords=_dptr_or_none(self.tex_coords), instance_uv_rects=_dptr_or_none(self.uv_rects),
            normals=_dptr_or_none(self.normals),
            opaque_texture=None if self._tex_desc[0] is None else ctypes.addressof(self._tex_desc[0]),
            transparent_texture=None if self._tex_desc[1] is None else ctypes.addressof(self._tex_desc[1]))


def default_options() -> _lib.Options:
    lib = _lib.load()
    o = _lib.Options()
    check(lib.lucid_default_options(ctypes.byref(o)), "lucid_default_options")
    return o


class LucidRenderer:
    """GB300 implementation of LucidRenderer's compute passes for one viewport size.

    Keyword options map to `lucid_options` (0 or None keeps the library default):

    * max_input_quads, max_visible_quads, max_bin_refs, band_capacity: buffer capacities;
    * flags: LUCID_OPT_* bits (timers, additive, alpha threshold, pixel blend, reference order);
    * low_high_threshold: tris per bin above which a bin is HIGH (work order);
    * raster_ctas_per_sm, binning_ctas: launch shapes;
    * max_views: views a batch may hold;
    * grad_store_fragments: fragment store of the differentiable frame (0 grows on demand, < 0
      none);
    * slab_fragments: fragments per unfinished pixel that a depth slab of the raster's per-pixel
      histograms aims at (0 = 165);
    * light_max_pixel: bins whose pixels have at most this many fragments take the light raster
      path (0 = 64, < 0 = off);
    * bin_size: 32 or 64 pixels per bin side (64-pixel bins are rastered as four 32x32 tiles).
    """

    def __init__(self, width: int, height: int, *, max_input_quads: int | None = None,
                 max_visible_quads: int | None = None, max_bin_refs: int | None = None,
                 band_capacity: int | None = None, flags: int = 0, low_high_threshold: int = 1024,
                 raster_ctas_per_sm: int = 0, binning_ctas: int = 0, max_views: int = 1,
                 grad_store_fragments: int = 0, slab_fragments: int = 0, light_max_pixel: int = 0,
                 bin_size: int = 32):
        if not torch.cuda.is_available():
            raise RuntimeError("lucid_gb300 needs a CUDA device")
        self.lib = _lib.load()
        o = default_options()
        if max_input_quads:
            o.max_input_quads = int(max_input_quads)
        if max_visible_quads:
            o.max_visible_quads = int(max_visible_quads)
        if max_bin_refs:
            o.max_bin_refs = int(max_bin_refs)
        if band_capacity:
            o.band_capacity = int(band_capacity)
        o.flags = int(flags)
        o.low_high_threshold = int(low_high_threshold)
        o.raster_ctas_per_sm = int(raster_ctas_per_sm)
        o.binning_ctas = int(binning_ctas)
        o.max_views = int(max_views)
        o.grad_store_fragments = int(grad_store_fragments)
        o.slab_fragments = int(slab_fragments)
        o.light_max_pixel = int(light_max_pixel)
        o.bin_size = int(bin_size)
        self.options = o
        self.width, self.height = int(width), int(height)
        self._set_bin_size(int(bin_size))
        torch.cuda.current_device()  # make sure the primary context exists
        h = ctypes.c_void_p()
        check(self.lib.lucid_create(ctypes.byref(o), self.width, self.height, ctypes.byref(h)),
              "lucid_create")
        self.handle = h

    def _set_bin_size(self, bin_size: int):
        """The bin grid of the renderer's frames (lucid_get_info's counters follow it)."""
        self.bin_size = bin_size
        self.bin_count_x = (self.width + bin_size - 1) // bin_size
        self.bin_count_y = (self.height + bin_size - 1) // bin_size
        self.num_bins = self.bin_count_x * self.bin_count_y

    # -- lifetime -------------------------------------------------------------------------
    def close(self):
        if getattr(self, "handle", None):
            self.lib.lucid_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- passes ---------------------------------------------------------------------------
    def new_image(self):
        return torch.empty((self.height, self.width, 4), dtype=torch.float32, device="cuda")

    def render(self, frame: FrameInputs, out=None, stream=None):
        out = self.new_image() if out is None else out
        fi = frame.c_struct()
        check(self.lib.lucid_render(self.handle, ctypes.byref(fi), _dptr(out), _stream_ptr(stream)),
              "lucid_render")
        return out

    def quad_setup(self, frame: FrameInputs, stream=None):
        fi = frame.c_struct()
        check(self.lib.lucid_quad_setup(self.handle, ctypes.byref(fi), _stream_ptr(stream)),
              "lucid_quad_setup")

    def bin_count(self, stream=None):
        check(self.lib.lucid_bin_count(self.handle, _stream_ptr(stream)), "lucid_bin_count")

    def bin_categorize(self, stream=None):
        check(self.lib.lucid_bin_categorize(self.handle, _stream_ptr(stream)), "lucid_bin_categorize")

    def bin_dispatch(self, stream=None):
        check(self.lib.lucid_bin_dispatch(self.handle, _stream_ptr(stream)), "lucid_bin_dispatch")

    def raster(self, frame: FrameInputs, out=None, stream=None):
        out = self.new_image() if out is None else out
        fi = frame.c_struct()
        check(self.lib.lucid_raster(self.handle, ctypes.byref(fi), _dptr(out), _stream_ptr(stream)),
              "lucid_raster")
        return out

    def raster_dump(self, frame: FrameInputs, max_per_pixel: int, stream=None):
        """Full frame in verification mode: (image, per-pixel counts, per-pixel prim ids)."""
        out = self.new_image()
        counts = np.zeros((self.height, self.width), np.int32)
        prims = np.zeros((self.height, self.width, max(1, max_per_pixel)), np.int32)
        fi = frame.c_struct()
        check(self.lib.lucid_raster_dump(self.handle, ctypes.byref(fi), _dptr(out), max_per_pixel,
                                         counts.ctypes.data, prims.ctypes.data, _stream_ptr(stream)),
              "lucid_raster_dump")
        return out, counts, prims[..., :max_per_pixel]

    def raster_dump_bins(self, frame: FrameInputs, bins, max_per_pixel: int, stream=None):
        """Full frame, recording the fragment lists of the listed bins only: (image, counts
        [n, 32, 32], prims [n, 32, 32, max_per_pixel]) with bin k's pixel (x, y) at [k, y, x]
        (pixels outside the viewport stay 0 / -1)."""
        out = self.new_image()
        b = np.ascontiguousarray(bins, np.int32)
        counts = np.zeros((len(b), 32, 32), np.int32)
        prims = np.zeros((len(b), 32, 32, max(1, max_per_pixel)), np.int32)
        fi = frame.c_struct()
        check(self.lib.lucid_raster_dump_bins(self.handle, ctypes.byref(fi), _dptr(out), b.ctypes.data, len(b),
                                              max_per_pixel, counts.ctypes.data, prims.ctypes.data,
                                              _stream_ptr(stream)),
              "lucid_raster_dump_bins")
        return out, counts, prims[..., :max_per_pixel]

    # -- info / statistics ------------------------------------------------------------------
    def autotune(self, frame: FrameInputs, stream=None) -> dict:
        """Runs lucid_autotune on `frame`; the winner stays in the renderer."""
        scratch = self.new_image()
        t = _lib.Tuning()
        fi = frame.c_struct()
        check(self.lib.lucid_autotune(self.handle, ctypes.byref(fi), _dptr(scratch), ctypes.byref(t),
                                      _stream_ptr(stream)), "lucid_autotune")
        self._set_bin_size(int(t.bin_size))
        return {k: getattr(t, k) for k in ("bin_size", "pixel_blend", "low_high_threshold", "binning_ctas",
                                           "light_max_pixel", "num_candidates", "frame_ms", "default_ms")}

    def _views(self, frames, outs):
        n = len(frames)
        if outs is None:
            outs = [torch.empty((h, w, 4), dtype=torch.float32, device="cuda") for _, w, h in frames]
        views = (_lib.ViewC * n)()
        for i, ((frame, w, h), out) in enumerate(zip(frames, outs)):
            views[i].width, views[i].height = int(w), int(h)
            views[i].inputs = frame.c_struct()
            views[i].out_rgba = out.data_ptr()
        self._batch_keep = (frames, outs)
        return views, outs

    def render_batch(self, frames, outs=None, stream=None):
        """Renders every (frame, width, height) of `frames` with lucid_render_batch; returns the
        output images (allocated unless `outs` is given)."""
        views, outs = self._views(frames, outs)
        check(self.lib.lucid_render_batch(self.handle, views, len(frames), _stream_ptr(stream)),
              "lucid_render_batch")
        return outs

    def autotune_batch(self, frames, outs=None, stream=None) -> dict:
        """Runs lucid_autotune_batch on the views of `frames` (rendered into `outs`); the winner
        stays in the renderer."""
        views, outs = self._views(frames, outs)
        t = _lib.Tuning()
        check(self.lib.lucid_autotune_batch(self.handle, views, len(frames), ctypes.byref(t),
                                            _stream_ptr(stream)), "lucid_autotune_batch")
        self._set_bin_size(int(t.bin_size))
        return {k: getattr(t, k) for k in ("bin_size", "pixel_blend", "low_high_threshold", "binning_ctas",
                                           "light_max_pixel", "num_candidates", "frame_ms", "default_ms")}

    def batch_info(self, view: int, stream=None):
        info = _lib.Info()
        check(self.lib.lucid_get_batch_info(self.handle, int(view), ctypes.byref(info), _stream_ptr(stream)),
              "lucid_get_batch_info")
        return info

    def info(self, stream=None):
        info = _lib.Info()
        counters = np.zeros(10 * self.num_bins, np.uint32)
        check(self.lib.lucid_get_info(self.handle, ctypes.byref(info), counters.ctypes.data,
                                      _stream_ptr(stream)), "lucid_get_info")
        return info, counters

    def download(self, which: int, dtype=np.uint32, count: int | None = None, stream=None):
        size = ctypes.c_size_t()
        check(self.lib.lucid_download_buffer(self.handle, which, None, 0, ctypes.byref(size), None),
              "lucid_download_buffer")
        nbytes = size.value if count is None else min(size.value, count * np.dtype(dtype).itemsize)
        arr = np.zeros(nbytes // np.dtype(dtype).itemsize, dtype)
        check(self.lib.lucid_download_buffer(self.handle, which, arr.ctypes.data, arr.nbytes, None,
                                             _stream_ptr(stream)), "lucid_download_buffer")
        return arr

    def verify_info(self, stream=None):
        """Offset consistency checks of LucidRenderer::verifyInfo (src/lucid_renderer.cpp:629-707).
        Returns a list of error strings (empty when consistent)."""
        _, c = self.info(stream)
        n = self.num_bins
        errors = []
        for base, name in ((0, "quad"), (3, "tri")):
            cnt = c[n * base:n * (base + 1)].astype(np.int64)
            off = c[n * (base + 1):n * (base + 2)].astype(np.int64)
            tmp = c[n * (base + 2):n * (base + 3)].astype(np.int64)
            bad = np.nonzero(off[1:] != off[:-1] + cnt[:-1])[0]
            errors += [f"Invalid bin {name} offset [{i + 1}]" for i in bad[:32]]
            bad = np.nonzero(tmp != off + cnt)[0]
            errors += [f"Invalid temp bin {name} offset [{i}]" for i in bad[:32]]
        return errors

    def stats(self, stream=None):
        """Counters reported by LucidRenderer::getStats (src/lucid_renderer.cpp:709-836)."""
        info, c = self.info(stream)
        n = self.num_bins
        quad_counts, tri_counts = c[:n], c[3 * n:4 * n]
        npix = self.width * self.height
        return dict(
            input_quads=info.num_input_quads,
            visible_quads=(info.num_visible_quads[0], info.num_visible_quads[1]),
            rejected_quads=tuple(info.num_rejected_quads),
            bin_levels=dict(empty=info.bin_level_counts[0], low=info.bin_level_counts[2],
                            high=info.bin_level_counts[4]),
            bin_quads=int(quad_counts.sum()), bin_tris=int(tri_counts.sum()),
            max_quads_per_bin=int(quad_counts.max()) if n else 0,
            max_tris_per_bin=int(tri_counts.max()) if n else 0,
            half_block_tris=int(info.num_hblock_tris), fragments=int(info.num_fragments),
            fragments_per_pixel=int(info.num_fragments) / npix,
            max_pixel_fragments=int(info.max_pixel_fragments),
            error=_lib.ERR_NAMES.get(info.error_code, str(info.error_code)),
            error_detail=tuple(info.error_detail))


def quad_generate(positions, tris, square_weight: float = 1.0, stream=None):
    """Pairs triangles into quads on the GPU (lucid_quad_generate). positions: (V, 3) float32 and
    tris: (T, 3) int32 CUDA tensors. Returns (quads (n, 4) uint32-as-int32 CUDA tensor,
    num_degenerate)."""
    lib = _lib.load()
    positions = positions.contiguous()
    tris = tris.contiguous()
    out = torch.empty((max(1, tris.shape[0]), 4), dtype=torch.int32, device=tris.device)
    n, nd = ctypes.c_int32(), ctypes.c_int32()
    check(lib.lucid_quad_generate(_dptr(positions), int(positions.shape[0]), _dptr(tris), int(tris.shape[0]),
                                  float(square_weight), _dptr(out), ctypes.byref(n), ctypes.byref(nd),
                                  _stream_ptr(stream)), "lucid_quad_generate")
    return out[:n.value], nd.value
