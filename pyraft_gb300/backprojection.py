"""Backprojections (pyraft/backprojection/backprojection.py:35-261).

* ``backprojection(sino, plan)`` with a SLANTSTACK plan:
  raft_backprojection_slantstack semantics (pixel-driven, linear in t, times
  the view spacing).
* ``radon_transpose(sino, shape, method)``: BRESENHAM is the exact transpose
  of the DDA Radon (raft_radon_transpose_bresenham); SLANTSTACK (new) is the
  exact transpose of the slant-stack Radon, i.e. the matched adjoint.
* ``backprojection(sino, plan)`` with a BRESENHAM plan: the normalised DDA
  backprojection (raft_backprojection_bresenham), sum(s sigma) / sum(sigma)
  per pixel, 0 where no ray passes.
* ``backprojection_gpu(sino, shape)``: host arrays in and out, default
  geometry, slant-stack backprojection.
The Fourier-domain families (BST, ANDERSSON, ANDERSSONPB) are not part of
this hot path and raise TypeError, as unsupported methods do in pyraft.
"""
from __future__ import annotations

import numpy

from . import _native
from .raftypes import finish, gpu_image, image, new_gpu, rg_image, stream_ptr, to_gpu, workspace
from .sinogram import method_id, radon_method


def backprojection_plan(sino_shape=(256, 180), shape=(256, 256), padding=2,
                        method=radon_method.BST):
    """Plan tuple (method, shape, padding), as pyraft returns for
    SLANTSTACK (pyraft/backprojection/backprojection.py:160-161)."""
    m = method_id(method)
    if m in (method_id(radon_method.SLANTSTACK), method_id(radon_method.BRESENHAM)):
        return (method, tuple(shape), padding)
    raise TypeError('Unsupported method for Backprojection!')


def _image_corners(kwargs):
    kw = dict(kwargs)
    kw.pop('dtype', None)
    probe = image((2, 2), **kw)
    return probe.top_left, probe.bottom_right


def _gather(fn, wsfn, sino, shape, kwargs):
    tl, br = _image_corners(kwargs)
    gs, host = to_gpu(sino, (0.0, 1.0), (numpy.pi, -1.0))
    out = new_gpu(shape, tl, br)
    a, b = rg_image(gs), rg_image(out)
    ws_t, ws = workspace(wsfn(a, b))
    _native.check(fn(a, b, ws, ws_t.numel() if ws_t is not None else 0, stream_ptr()))
    return finish(out, host)


def backprojection(sino, plan, **kwargs):
    """Backprojection of `sino` onto plan[1]-shaped image (corners from
    kwargs as pyraft.image)."""
    method, shape = plan[0], plan[1]
    L = _native.load()
    if method_id(method) == method_id(radon_method.SLANTSTACK):
        return _gather(L.rg_backprojection_slantstack, L.rg_backprojection_slantstack_workspace,
                       sino, shape, kwargs)
    if method_id(method) == method_id(radon_method.BRESENHAM):
        return _gather(L.rg_backprojection_bresenham, L.rg_backprojection_bresenham_workspace,
                       sino, shape, kwargs)
    raise TypeError('Unsupported method for Backprojection!')


def radon_transpose(sino, shape=(256, 256), method=radon_method.BRESENHAM, **kwargs):
    """Transpose of the discrete Radon transform of `method`."""
    L = _native.load()
    m = method_id(method)
    if m == method_id(radon_method.BRESENHAM):
        return _gather(L.rg_radon_transpose_bresenham, L.rg_radon_transpose_bresenham_workspace,
                       sino, shape, kwargs)
    if m == method_id(radon_method.SLANTSTACK):
        return _gather(L.rg_radon_transpose_slantstack,
                       L.rg_radon_transpose_slantstack_workspace, sino, shape, kwargs)
    raise TypeError('Unsupported method for transpose Radon!')


def backprojection_gpu(sino, shape=(256, 256), **kwargs):
    """pyraft's backprojection_gpu: (nrays, nviews) host sinogram on the
    default geometry -> (size, size) float64 array."""
    s = image(numpy.asarray(sino, dtype=numpy.float64), top_left=(0.0, 1.0),
              bottom_right=(numpy.pi, -1.0))
    out = backprojection(s, (radon_method.SLANTSTACK, (shape[0], shape[0]), 0))
    return numpy.asarray(out)
