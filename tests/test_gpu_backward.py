"""Backward pass: gradients of L = sum (image - target)^2 with respect to per-vertex RGBA and
per-triangle opacity (positions frozen), computed by lucid_render_forward_grad +
lucid_render_backward through the autograd wrapper, against
 - the oracle's adjoint fed the same upstream gradient (checks the backward pass alone),
 - the oracle's FP64 analytic gradient of the FP64 loss,
 - FP64 central finite differences (h = 1e-4) of the FP64 loss on 1000 sampled parameters.

Relative error of a parameter: |g - g_ref| / max(|g_ref|, 1e-3 * max|g_ref|); the second term
keeps parameters whose gradient is ~0 (fragments hidden behind opaque layers) from dividing by
zero, so below that floor the bound is an absolute 1e-7 * max|g_ref|. Bound: 1e-4. The finite
difference checks also assert the plain relative error of the parameters above the floor.
"""
import numpy as np
import pytest

from lucid_gb300 import scenes

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel_err(g, ref):
    g, ref = np.asarray(g, np.float64), np.asarray(ref, np.float64)
    scale = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    return np.abs(g - ref) / scale


def gpu_grads(sc, target, grad_store_fragments=0):
    import torch
    from lucid_gb300 import autograd
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    r = LucidRenderer(sc.width, sc.height, max_input_quads=max(1024, sc.num_quads),
                      max_visible_quads=max(1024, sc.num_quads), grad_store_fragments=grad_store_fragments)
    frame = FrameInputs.from_scene(sc)
    vc = torch.from_numpy(sc.colors.astype(np.float32)).cuda().requires_grad_(True)
    op = torch.from_numpy(sc.tri_opacity.astype(np.float32)).cuda().requires_grad_(True)
    img = autograd.render(vc, op, r, frame)
    tgt = torch.from_numpy(target).cuda()
    loss = ((img[..., :3] - tgt[..., :3]) ** 2).sum()
    loss.backward()
    plain = r.render(frame).cpu().numpy()
    out = dict(image=img.detach().cpu().numpy(), plain=plain, loss=float(loss.detach()),
               upstream=(2.0 * (img.detach() - tgt)).cpu().numpy(),
               dvc=vc.grad.cpu().numpy().astype(np.float64), dop=op.grad.cpu().numpy().astype(np.float64))
    r.close()
    return out


def scene_and_target(w, h, n, seed, **kw):
    sc = scenes.random_tris(w, h, n, seed=seed, color_format=scenes.COLOR_RGBA32F,
                            tri_opacity_range=(0.1, 0.9), background=(0.5, 0.5, 0.5, 1.0), **kw)
    rng = np.random.default_rng(seed + 100)
    # target: the scene rendered from perturbed colours (oracle), as in the gradient workload
    pert = sc.colors.copy()
    pert[:, :3] = np.clip(pert[:, :3] + rng.normal(0, 0.1, size=pert[:, :3].shape), 0, 1)
    return sc, pert


@pytest.mark.parametrize("w,h,n,seed", [(64, 48, 400, 3), (128, 96, 4000, 5)])
def test_backward_matches_fp64_analytic_and_fd(gpu, oracle, w, h, n, seed):
    sc, pert = scene_and_target(w, h, n, seed, area_median=150.0)
    psc = scenes.Scene(**{**sc.__dict__, "colors": pert.astype(np.float32)})
    target = oracle.run(psc)["image"]
    g = gpu_grads(sc, target)
    ref = oracle.run(sc, image64=True)
    # the differentiable image is the FP64 colour rounded to FP32; the plain render's FP32 blend
    # is within the FP32 blend error of it
    img64 = ref["image64"][..., :3]
    assert np.abs(g["image"][..., :3] - np.clip(img64, 0, 1)).max() <= 1e-6
    assert np.abs(g["image"] - g["plain"]).max() <= 1e-5
    model = oracle.GradModel(sc)
    vc = sc.colors.astype(np.float64)
    op = sc.tri_opacity.astype(np.float64)
    assert abs(model.loss(vc, op, target) - g["loss"]) <= 1e-4 * max(1.0, g["loss"])
    # adjoint alone: same upstream gradient, FP64 replay (the GPU sums per-fragment terms with
    # FP32 atomics, ~2e-5 relative on gradients whose pixel terms cancel)
    bvc, bop = model.backprop(vc, op, g["upstream"], img64.astype(np.float32))
    assert rel_err(g["dvc"].ravel(), bvc.ravel()).max() <= TOL
    assert rel_err(g["dop"], bop).max() <= TOL
    dvc64, dop64 = model.analytic(vc, op, target)
    assert rel_err(g["dvc"].ravel(), dvc64.ravel()).max() <= TOL
    assert rel_err(g["dop"], dop64).max() <= TOL
    # FP64 central differences on 1000 sampled parameters (vertex colours and opacities)
    rng = np.random.default_rng(seed)
    touched_v = np.nonzero(np.abs(dvc64.ravel()) > 0)[0]
    touched_o = np.nonzero(np.abs(dop64) > 0)[0]
    iv = rng.choice(touched_v, size=min(800, len(touched_v)), replace=False)
    io = rng.choice(touched_o, size=min(200, len(touched_o)), replace=False)
    fd_v = np.array([model.fd(vc, op, target, 0, int(i)) for i in iv])
    fd_o = np.array([model.fd(vc, op, target, 1, int(i)) for i in io])
    ref = np.concatenate([fd_v, fd_o])
    got = np.concatenate([g["dvc"].ravel()[iv], g["dop"][io]])
    err = rel_err(got, ref)
    assert err.max() <= TOL, (err.max(), np.argmax(err))
    # parameters whose gradient is above the floor: the plain relative error
    above = np.abs(ref) >= 1e-3 * np.abs(ref).max()
    assert (np.abs(got - ref)[above] / np.abs(ref)[above]).max() <= TOL


@pytest.mark.parametrize("store", [-1, 1000])
def test_backward_without_fragment_store(gpu, oracle, store):
    """No fragment store (-1), or one too small for the frame (1000 fragments): the raster
    pass recomputes the fragment lists; image and gradients agree with the store path."""
    sc, pert = scene_and_target(96, 64, 1500, 8, area_median=150.0)
    psc = scenes.Scene(**{**sc.__dict__, "colors": pert.astype(np.float32)})
    target = oracle.run(psc)["image"]
    a = gpu_grads(sc, target)
    b = gpu_grads(sc, target, grad_store_fragments=store)
    np.testing.assert_array_equal(a["image"], b["image"])
    # same arithmetic per fragment; the FP32 atomic sums differ in order
    assert rel_err(b["dvc"].ravel(), a["dvc"].ravel()).max() <= TOL
    assert rel_err(b["dop"], a["dop"]).max() <= TOL


def test_backward_rejects_unsupported(gpu):
    import ctypes
    import torch
    from lucid_gb300 import _lib
    from lucid_gb300.renderer import FrameInputs, LucidRenderer
    sc = scenes.small_scene(32, 32, 50, seed=1)  # RGBA8 colours: no vertex colour gradient
    r = LucidRenderer(32, 32, max_input_quads=1024, max_visible_quads=1024)
    f = FrameInputs.from_scene(sc)
    g = torch.zeros((32, 32, 4), device="cuda")
    d = torch.zeros((sc.positions.shape[0], 4), device="cuda")
    st = r.lib.lucid_render_backward(r.handle, ctypes.byref(f.c_struct()), ctypes.c_void_p(g.data_ptr()),
                                     ctypes.c_void_p(d.data_ptr()), None, None)
    assert st == _lib.INVALID_ARG
    r.close()


def test_backward_at_workload_size(gpu, oracle):
    """The forward+backward workload itself: 512x512, 200k triangles (FP32 vertex RGBA, triangle
    opacity U[0.1, 0.9]), L2 loss to a target rendered from perturbed colours, 91 layers per
    pixel on average. GPU gradients against FP64 central differences (h = 1e-4) of the FP64
    loss on 1000 sampled parameters and against the oracle's FP64 analytic gradient.

    The relative error divides by max(|g_ref|, 1e-3 * max|g_ref|): below that floor (a gradient
    1000x smaller than the largest) the bound is an absolute 1e-7 * max|g_ref|. The largest
    relative error among parameters above the floor is asserted separately."""
    import os
    sc = scenes.workload("grad512")
    rng = np.random.default_rng(104)
    pert = sc.colors.copy()
    pert[:, :3] = np.clip(pert[:, :3] + rng.normal(0, 0.1, size=pert[:, :3].shape), 0, 1)
    psc = scenes.Scene(**{**sc.__dict__, "colors": pert.astype(np.float32)})
    target = oracle.run(psc, threads=os.cpu_count() or 1, setup_outputs=False)["image"]
    g = gpu_grads(sc, target)
    model = oracle.GradModel(sc)
    assert model.num_fragments > 20_000_000
    vc = sc.colors.astype(np.float64)
    op = sc.tri_opacity.astype(np.float64)
    assert abs(model.loss(vc, op, target) - g["loss"]) <= 1e-4 * max(1.0, g["loss"])
    dvc64, dop64 = model.analytic(vc, op, target)
    assert rel_err(g["dvc"].ravel(), dvc64.ravel()).max() <= TOL
    assert rel_err(g["dop"], dop64).max() <= TOL
    sel = np.random.default_rng(7)
    touched_v = np.nonzero(np.abs(dvc64.ravel()) > 0)[0]
    touched_o = np.nonzero(np.abs(dop64) > 0)[0]
    iv = sel.choice(touched_v, size=800, replace=False)
    io = sel.choice(touched_o, size=200, replace=False)
    fd = np.concatenate([[model.fd(vc, op, target, 0, int(i)) for i in iv],
                         [model.fd(vc, op, target, 1, int(i)) for i in io]])
    got = np.concatenate([g["dvc"].ravel()[iv], g["dop"][io]])
    err = rel_err(got, fd)
    above = np.abs(fd) >= 1e-3 * np.abs(fd).max()
    pure = np.abs(got - fd)[above] / np.abs(fd)[above]
    print(f"grad512: max rel err vs FD {err.max():.3g} ({int(above.sum())} of 1000 above the floor: "
          f"max {pure.max():.3g}); vs analytic: colours {rel_err(g['dvc'].ravel(), dvc64.ravel()).max():.3g}, "
          f"opacity {rel_err(g['dop'], dop64).max():.3g}")
    assert err.max() <= TOL
    assert pure.max() <= TOL
