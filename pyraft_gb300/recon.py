"""Differentiable reconstructions built on the autograd Radon pair.

* ``tv_ls``: total-variation regularised least squares,
  min_x 0.5 ||R x - y||^2 + lam * sum sqrt(|grad x|^2 + eps^2), solved with
  Adam; R and its gradient (the matched adjoint) are the library's kernels,
  the TV term and the optimiser are PyTorch ops on the image stack.
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

from .autograd import IMG, SINO, adjoint, radon


def total_variation(x, eps):
    """Smoothed isotropic TV of (..., N, N) images (forward differences,
    replicated last row / column)."""
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
