"""torch.autograd binding of the path-replay adjoint (er_backward).

`render(scene, materials, env, spp, ...)` renders the scene's film with the
given per-material parameters (n, 5: albedo rgb, roughness, metallic) and
environment texels (h, w, 3) and returns the RGBA film as a tensor in the
film's output order (H*W, 4); its backward replays the same samples on the
GPU and returns d loss / d materials and d loss / d env.  The gradient is
that of the per-sample estimator with the sampling held fixed (the
estimator `er_render_replay` evaluates).  CUDA tensors are passed to the
library as device pointers; CPU tensors go through host copies.  There is
no CPU renderer behind this: without the CUDA library every call raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _abi as A
from . import _lib


def _ptr(t):
    return C.c_void_p(t.data_ptr())


class RenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, materials, env, scene, spp, max_depth, seed, sample_begin):
        L = _lib.load()
        W, H = scene.resolution
        dev = materials.is_cuda
        o = A.er_render_opts(spp, sample_begin, max_depth, 0, seed, 0, 0)
        if dev:
            m = materials.detach().float().contiguous()
            e = env.detach().float().contiguous()
            torch.cuda.current_stream(m.device).synchronize()
            _lib.check(L.er_scene_set_params(scene.h, _ptr(m), _ptr(e), A.ER_RENDER_DEVICE_OUT), "er_scene_set_params")
            beauty = torch.empty((H * W, 4), dtype=torch.float32, device=m.device)
            samples = torch.empty((H * W,), dtype=torch.int32, device=m.device)
            pc = torch.empty((H * W,), dtype=torch.int32, device=m.device)
            # keep the samples' radiance for the backward pass
            o.flags = A.ER_RENDER_DEVICE_OUT | A.ER_RENDER_KEEP_PATHS
            _lib.check(L.er_render(scene.h, C.byref(o), _ptr(beauty), None, None, None, _ptr(samples), _ptr(pc), None),
                       "er_render")
        else:
            scene.set_params(materials.detach().float().numpy(), env.detach().float().numpy())
            out = scene.render(spp, max_depth=max_depth, seed=seed, sample_begin=sample_begin,
                               flags=A.ER_RENDER_KEEP_PATHS)
            beauty = torch.from_numpy(out["beauty"])
            samples = torch.from_numpy(out["samples"].view(np.int32))
        ctx.scene = scene
        ctx.opts = (spp, max_depth, seed, sample_begin)
        ctx.save_for_backward(samples)
        ctx.shapes = (tuple(materials.shape), tuple(env.shape))
        return beauty

    @staticmethod
    def backward(ctx, grad):
        (samples,) = ctx.saved_tensors
        spp, max_depth, seed, sample_begin = ctx.opts
        scene = ctx.scene
        L = _lib.load()
        o = A.er_render_opts(spp, sample_begin, max_depth, 0, seed, 0, 0)
        if grad.is_cuda:
            g = grad.detach().float().contiguous()
            gm = torch.zeros(ctx.shapes[0], dtype=torch.float32, device=g.device)
            ge = torch.zeros(ctx.shapes[1], dtype=torch.float32, device=g.device)
            torch.cuda.current_stream(g.device).synchronize()
            o.flags = A.ER_RENDER_DEVICE_OUT
            _lib.check(L.er_backward(scene.h, C.byref(o), _ptr(g), _ptr(samples), _ptr(gm), _ptr(ge), None),
                       "er_backward")
        else:
            gm_np, ge_np, _ = scene.backward(spp, grad.detach().float().numpy(), samples.numpy().view(np.uint32),
                                             max_depth=max_depth, seed=seed, sample_begin=sample_begin)
            gm, ge = torch.from_numpy(gm_np), torch.from_numpy(ge_np)
        return gm, ge, None, None, None, None, None


def render(scene, materials, env, spp, max_depth=6, seed=0, sample_begin=0):
    """Differentiable film (H*W, 4) of `scene` with the given parameters."""
    return RenderFunction.apply(materials, env, scene, spp, max_depth, seed, sample_begin)


def l2_loss(beauty, target):
    """Sum of squared RGB differences (alpha excluded)."""
    return ((beauty[:, :3] - target[:, :3]) ** 2).sum()


def optimize(scene, target, materials, env, steps=100, lr=1e-2, spp=64, max_depth=6, seed=0, callback=None):
    """Adam on (materials, env) against a target film; each step renders
    with fresh sample numbers.  Parameters are kept in their valid ranges
    (albedo, metallic in [0, 1], roughness in [0.001, 1], env >= 0).
    Returns the final parameters and the loss history."""
    m = materials.clone().requires_grad_(True)
    e = env.clone().requires_grad_(True)
    opt = torch.optim.Adam([m, e], lr=lr)
    hist = []
    for it in range(steps):
        opt.zero_grad()
        img = render(scene, m, e, spp, max_depth=max_depth, seed=seed, sample_begin=it * spp)
        loss = l2_loss(img, target)
        loss.backward()
        opt.step()
        with torch.no_grad():
            m[:, :3].clamp_(0.0, 1.0)
            m[:, 3].clamp_(0.001, 1.0)
            m[:, 4].clamp_(0.0, 1.0)
            e.clamp_(min=0.0)
        hist.append(float(loss.detach()))
        if callback:
            callback(it, hist[-1])
    return m.detach(), e.detach(), hist
