"""Differentiable slant-stack Radon for PyTorch.

``RadonFunction`` (torch.autograd.Function): forward = slant-stack Radon
(rg_radon_slantstack), backward = its matched adjoint
(rg_radon_transpose_slantstack), not the filtered or the reference
backprojection, so gradients are exact for the discrete operator.  Inputs
are float32 CUDA tensors of shape (N, N) or (B, N, N); the geometry
(corners, nrays, nviews) is fixed per call.  Used by the TV-regularised
least-squares and unrolled-EM reconstructions.
"""
from __future__ import annotations

import math

import torch

from . import _native
from .raftypes import gpu_image, rg_image, stream_ptr, workspace

IMG = ((-1.0, 1.0), (1.0, -1.0))
SINO = ((0.0, 1.0), (math.pi, -1.0))


def _apply(fn, wsfn, src, dst, src_c, dst_c):
    L = _native.load()
    a = rg_image(gpu_image(src, *src_c))
    b = rg_image(gpu_image(dst, *dst_c))
    ws_t, ws = workspace(getattr(L, wsfn)(a, b))
    _native.check(getattr(L, fn)(a, b, ws, ws_t.numel() if ws_t is not None else 0,
                                 stream_ptr()))


def radon_forward(x, nrays, nviews, img_corners=IMG, sino_corners=SINO):
    """Slant-stack Radon of (N, N) or (B, N, N) float32 CUDA tensors."""
    xs = x.reshape(-1, x.shape[-2], x.shape[-1]).contiguous()
    out = torch.empty((xs.shape[0], nrays, nviews), device=x.device, dtype=torch.float32)
    for b in range(xs.shape[0]):
        _apply('rg_radon_slantstack', 'rg_radon_slantstack_workspace', xs[b], out[b],
               img_corners, sino_corners)
    return out.reshape(*x.shape[:-2], nrays, nviews)


def radon_adjoint(s, size, img_corners=IMG, sino_corners=SINO):
    """Matched adjoint of radon_forward."""
    ss = s.reshape(-1, s.shape[-2], s.shape[-1]).contiguous()
    out = torch.empty((ss.shape[0], size, size), device=s.device, dtype=torch.float32)
    for b in range(ss.shape[0]):
        _apply('rg_radon_transpose_slantstack', 'rg_radon_transpose_slantstack_workspace',
               ss[b], out[b], sino_corners, img_corners)
    return out.reshape(*s.shape[:-2], size, size)


class RadonFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, nrays, nviews, img_corners=IMG, sino_corners=SINO):
        ctx.geom = (x.shape[-1], img_corners, sino_corners)
        return radon_forward(x.float(), nrays, nviews, img_corners, sino_corners)

    @staticmethod
    def backward(ctx, g):
        size, ic, sc = ctx.geom
        return radon_adjoint(g.float().contiguous(), size, ic, sc), None, None, None, None


def radon(x, nrays, nviews, img_corners=IMG, sino_corners=SINO):
    """Differentiable slant-stack Radon transform."""
    return RadonFunction.apply(x, nrays, nviews, img_corners, sino_corners)
