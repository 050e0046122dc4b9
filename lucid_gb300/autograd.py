"""torch.autograd.Function over the lucid_gb300 C ABI (gradient harness only).

Forward renders with lucid_render_forward_grad (the image is the FP64-accumulated colour
rounded to FP32); backward calls lucid_render_backward, which replays each pixel's exact-order
fragment list to route dL/dimage to the per-vertex RGBA colours and per-triangle opacities,
reusing the forward's bin lists. Positions are not differentiated.
"""
from __future__ import annotations

import ctypes

import torch

from ._lib import check
from .renderer import FrameInputs, LucidRenderer, _dptr, _stream_ptr


class LucidRenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vertex_rgba, tri_opacity, renderer: LucidRenderer, frame: FrameInputs):
        # the frame reads its colours / opacities from these tensors
        frame.colors = vertex_rgba.detach().contiguous()
        frame.tri_opacity = None if tri_opacity is None else tri_opacity.detach().contiguous()
        image = renderer.new_image()
        fi = frame.c_struct()
        check(renderer.lib.lucid_render_forward_grad(renderer.handle, ctypes.byref(fi), _dptr(image),
                                                     _stream_ptr()), "lucid_render_forward_grad")
        ctx.renderer, ctx.frame = renderer, frame
        ctx.has_opacity = tri_opacity is not None
        return image

    @staticmethod
    def backward(ctx, grad_image):
        r, frame = ctx.renderer, ctx.frame
        grad_image = grad_image.contiguous().float()
        dvc = torch.zeros_like(frame.colors) if ctx.needs_input_grad[0] else None
        dop = torch.zeros_like(frame.tri_opacity) if (ctx.has_opacity and ctx.needs_input_grad[1]) else None
        fi = frame.c_struct()
        check(r.lib.lucid_render_backward(r.handle, ctypes.byref(fi), _dptr(grad_image), _dptr(dvc),
                                          _dptr(dop), _stream_ptr()), "lucid_render_backward")
        return dvc, dop, None, None


def render(vertex_rgba: torch.Tensor, tri_opacity, renderer: LucidRenderer, frame: FrameInputs):
    """Differentiable render: image (H, W, 4) as a function of vertex RGBA (V, 4, float32,
    LUCID_COLOR_RGBA32F) and triangle opacity (num_quads*2, float32, or None)."""
    return LucidRenderFunction.apply(vertex_rgba, tri_opacity, renderer, frame)
