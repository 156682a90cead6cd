"""Differentiable reconstructions built on the autograd Radon pair.

* ``tv_ls``: total-variation regularised least squares,
  min_x 0.5 ||R x - y||^2 + lam * sum sqrt(|grad x|^2 + eps^2), solved with
  Adam; R and its gradient (the matched adjoint) and the TV value and
  gradient are the library's kernels, the optimiser PyTorch's Adam.
* ``unrolled_em``: MLEM x <- x * A^T(y / A x) / A^T 1 written with the
  differentiable operator pair, so gradients flow through all iterations
  (e.g. with respect to the data); the iterations are checkpointed in
  segments (torch.utils.checkpoint), keeping one iterate per segment alive
  instead of every intermediate.
Neither has a reference counterpart (pyraft has no autograd); they exercise
the operator pair the way a learned or regularised reconstruction does.
"""
from __future__ import annotations

import torch
import torch.utils.checkpoint as cp

from . import _native
from .autograd import IMG, SINO, adjoint, radon


class _TV(torch.autograd.Function):
    """TV value and gradient from one fused kernel (rg_tv); the gradient is
    computed with the value and kept for backward."""

    @staticmethod
    def forward(ctx, x, eps):
        L = _native.load()
        xc = x.detach().float().contiguous()
        n = xc.shape[-1]
        value = torch.empty((), dtype=torch.float64, device=xc.device)
        grad = torch.empty_like(xc)
        _native.check(L.rg_tv(xc.data_ptr(), xc.numel() // (n * n), n, float(eps),
                              value.data_ptr(), grad.data_ptr(),
                              torch.cuda.current_stream(xc.device).cuda_stream))
        ctx.save_for_backward(grad)
        return value.to(x.dtype)

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        return g * grad, None


def total_variation(x, eps):
    """Smoothed isotropic TV of (..., N, N) images, sum sqrt(dx^2 + dy^2 +
    eps^2) with forward differences and the last row / column replicated;
    differentiable, value and gradient from the library's fused kernel."""
    if x.shape[-1] != x.shape[-2]:
        raise ValueError("total_variation expects square images")
    return _TV.apply(x, eps)


def total_variation_reference(x, eps):
    """The same TV written with PyTorch ops (for testing the fused kernel)."""
    dx = torch.diff(x, dim=-1, append=x[..., -1:])
    dy = torch.diff(x, dim=-2, append=x[..., -1:, :])
    return torch.sqrt(dx * dx + dy * dy + eps * eps).sum()


def tv_ls(sino, size, niter=200, lam=1e-3, lr=1e-2, eps=1e-3, x0=None,
          img_corners=IMG, sino_corners=SINO):
    """sino: (B, R, A) or (R, A) float32 CUDA tensor.  Returns (x, losses)."""
    y = sino.float()
    R, A = y.shape[-2], y.shape[-1]
    x = (torch.zeros((*y.shape[:-2], size, size), device=y.device) if x0 is None
         else x0.detach().clone().float())
    x.requires_grad_(True)
    opt = torch.optim.Adam([x], lr=lr)
    losses = []
    for _ in range(niter):
        opt.zero_grad(set_to_none=True)
        r = radon(x, R, A, img_corners, sino_corners) - y
        loss = 0.5 * (r * r).sum() + lam * total_variation(x, eps)
        loss.backward()
        opt.step()
        losses.append(loss.detach())       # kept on the device: no sync per step
    return x.detach(), [float(v) for v in torch.stack(losses).cpu()] if losses else []


def _em_segment(x, y, sens_inv, steps, size, R, A, ic, sc):
    for _ in range(steps):
        ax = radon(x, R, A, ic, sc)
        ratio = torch.where(ax != 0, y / torch.where(ax != 0, ax, torch.ones_like(ax)),
                            torch.zeros_like(ax))
        x = x * adjoint(ratio, size, ic, sc) * sens_inv
    return x


def unrolled_em(sino, size, niter=20, checkpoint_every=5, x0=None,
                img_corners=IMG, sino_corners=SINO):
    """Differentiable MLEM from x0 (default ones).  sino: (..., R, A)
    tensor (float32 or float64, may require grad)."""
    y = sino
    R, A = y.shape[-2], y.shape[-1]
    x = (torch.ones((*y.shape[:-2], size, size), device=y.device, dtype=y.dtype)
         if x0 is None else x0)
    with torch.no_grad():
        sens = adjoint(torch.ones_like(y), size, img_corners, sino_corners)
        sens_inv = torch.where(sens > 0, 1.0 / torch.where(sens > 0, sens, torch.ones_like(sens)),
                               torch.zeros_like(sens))
    done = 0
    while done < niter:
        k = min(checkpoint_every, niter - done) if checkpoint_every > 0 else niter - done
        if checkpoint_every and torch.is_grad_enabled():
            x = cp.checkpoint(_em_segment, x, y, sens_inv, k, size, R, A, img_corners,
                              sino_corners, use_reentrant=False)
        else:
            x = _em_segment(x, y, sens_inv, k, size, R, A, img_corners, sino_corners)
        done += k
    return x
