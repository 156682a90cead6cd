"""Differentiable slant-stack Radon for PyTorch.

``RadonFunction``: forward = slant-stack Radon, backward = its matched
adjoint (not the filtered or the reference backprojection), so gradients
are exact for the discrete operator.  ``AdjointFunction`` is the transpose
pair (backward = Radon), for unrolled EM.  Inputs are CUDA tensors of shape
(N, N) or (B, N, N); the geometry (corners, nrays, nviews) is fixed per
call.

* float32 batches run as one stack launch per operator
  (rg_radon_slantstack_stack / rg_radon_transpose_slantstack_stack);
* float64 inputs use the FP64 pair (rg_radon_slantstack_f64 and its exact
  transpose), which is what torch.autograd.gradcheck needs.
"""
from __future__ import annotations

import math

import torch

from . import _native
from .raftypes import gpu_image, rg_image, stream_ptr, workspace

IMG = ((-1.0, 1.0), (1.0, -1.0))
SINO = ((0.0, 1.0), (math.pi, -1.0))


def _rg(t, corners):
    return rg_image(gpu_image(t, *corners))


def _rg64(t, corners):
    (tlx, tly), (brx, bry) = corners
    return _native.RG_IMAGE_F64(t.data_ptr(), t.shape[0], t.stride(1), t.shape[1], t.stride(0),
                                tlx, tly, brx, bry)


def radon_forward(x, nrays, nviews, img_corners=IMG, sino_corners=SINO):
    """Slant-stack Radon of (N, N) or (B, N, N) CUDA tensors (float32 or
    float64) -> (..., nrays, nviews)."""
    L = _native.load()
    xs = x.reshape(-1, x.shape[-2], x.shape[-1]).contiguous()
    B, N = xs.shape[0], xs.shape[-1]
    out = torch.empty((B, nrays, nviews), device=x.device, dtype=xs.dtype)
    if xs.dtype == torch.float64:
        for b in range(B):
            _native.check(L.rg_radon_slantstack_f64(_rg64(xs[b], img_corners),
                                                    _rg64(out[b], sino_corners), stream_ptr()))
    else:
        xs = xs.float()
        a, s = _rg(xs[0], img_corners), _rg(out[0], sino_corners)
        ws_t, ws = workspace(L.rg_radon_slantstack_stack_workspace(a, s, B))
        _native.check(L.rg_radon_slantstack_stack(a, N * N, s, nrays * nviews, B, ws,
                                                  ws_t.numel() if ws_t is not None else 0,
                                                  stream_ptr()))
    return out.reshape(*x.shape[:-2], nrays, nviews)


def radon_adjoint(s, size, img_corners=IMG, sino_corners=SINO):
    """Matched adjoint of radon_forward: (..., nrays, nviews) -> (..., N, N)."""
    L = _native.load()
    ss = s.reshape(-1, s.shape[-2], s.shape[-1]).contiguous()
    B, R, A = ss.shape
    out = torch.empty((B, size, size), device=s.device, dtype=ss.dtype)
    if ss.dtype == torch.float64:
        for b in range(B):
            _native.check(L.rg_radon_transpose_slantstack_f64(_rg64(ss[b], sino_corners),
                                                              _rg64(out[b], img_corners),
                                                              stream_ptr()))
    else:
        ss = ss.float()
        a, i = _rg(ss[0], sino_corners), _rg(out[0], img_corners)
        ws_t, ws = workspace(L.rg_radon_transpose_slantstack_stack_workspace(a, i, B))
        _native.check(L.rg_radon_transpose_slantstack_stack(
            a, R * A, i, size * size, B, ws, ws_t.numel() if ws_t is not None else 0,
            stream_ptr()))
    return out.reshape(*s.shape[:-2], size, size)


class RadonFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, nrays, nviews, img_corners=IMG, sino_corners=SINO):
        ctx.geom = (x.shape[-1], img_corners, sino_corners)
        return radon_forward(x, nrays, nviews, img_corners, sino_corners)

    @staticmethod
    def backward(ctx, g):
        size, ic, sc = ctx.geom
        return radon_adjoint(g.contiguous(), size, ic, sc), None, None, None, None


class AdjointFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, s, size, img_corners=IMG, sino_corners=SINO):
        ctx.geom = (s.shape[-2], s.shape[-1], img_corners, sino_corners)
        return radon_adjoint(s, size, img_corners, sino_corners)

    @staticmethod
    def backward(ctx, g):
        r, a, ic, sc = ctx.geom
        return radon_forward(g.contiguous(), r, a, ic, sc), None, None, None


def radon(x, nrays, nviews, img_corners=IMG, sino_corners=SINO):
    """Differentiable slant-stack Radon transform."""
    return RadonFunction.apply(x, nrays, nviews, img_corners, sino_corners)


def adjoint(s, size, img_corners=IMG, sino_corners=SINO):
    """Differentiable matched adjoint (transpose of ``radon``)."""
    return AdjointFunction.apply(s, size, img_corners, sino_corners)
