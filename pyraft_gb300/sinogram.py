"""Radon transforms (pyraft/sinogram/sino.py:154-212,350-387).

``radon(img, shape, method, **kw)`` keeps pyraft's signature and defaults:
the result is an (nrays, nviews) sinogram image whose extent defaults to
theta in (0, pi) and t in (-1, 1); an ``image``/``gpu_image`` input gets the
discrete transform of the chosen method, a plain ndarray is read as an
(n x 6) ellipse table and gets the exact line integrals
(raft/raft_radon_fromdesc.c).
"""
from __future__ import annotations

import ctypes
import math

import numpy

from . import _native
from .raftypes import gpu_image, image, new_gpu, rg_image, stream_ptr, to_gpu, workspace, finish


class radon_method:
    """Methods for projection/backprojection (values as pyraft's, which are
    1-tuples because of trailing commas, pyraft/sinogram/sino.py:162-167)."""
    BRESENHAM = 1,
    SLANTSTACK = 2,
    HIERARCHICAL = 3,
    BST = 4,
    ANDERSSON = 5,
    ANDERSSONPB = 6


def method_id(method) -> int:
    m = method[0] if isinstance(method, tuple) else method
    return int(m)


def sinogram_corners(kwargs):
    """Resolve the sinogram extent keywords exactly as pyraft's radon()
    (pyraft/sinogram/sino.py:178-190) and return (top_left, bottom_right)."""
    kw = dict(kwargs)
    if not any(k in kw for k in ('top_left', 'bottom_right', 'x_extent', 'y_extent')):
        kw['x_extent'] = kw.pop('theta_extent', (0.0, math.pi))
        if 't_extent' in kw:
            kw['y_extent'] = kw.pop('t_extent')
    kw.pop('dtype', None)
    probe = image((2, 2), **kw)
    return probe.top_left, probe.bottom_right


def radon(img, shape=(367, 180), method=radon_method.BRESENHAM, **kwargs):
    """Discrete Radon transform of an image (or exact one of an ellipse
    table).  SLANTSTACK: raft_radon_slantstack (ray-driven, linear
    interpolation); BRESENHAM: raft_radon_bresenham (DDA walk)."""
    tl, br = sinogram_corners(kwargs)
    L = _native.load()
    if isinstance(img, (image, gpu_image)) or _is_tensor(img):
        gi, host = to_gpu(img)
        out = new_gpu(shape, tl, br)
        m = method_id(method)
        if m == method_id(radon_method.BRESENHAM):
            fn, wsfn = L.rg_radon_bresenham, L.rg_radon_bresenham_workspace
        elif m == method_id(radon_method.SLANTSTACK):
            fn, wsfn = L.rg_radon_slantstack, L.rg_radon_slantstack_workspace
        else:
            raise TypeError('Unsupported method for Radon Transform!')
        a, b = rg_image(gi), rg_image(out)
        ws_t, ws = workspace(wsfn(a, b))
        _native.check(fn(a, b, ws, ws_t.numel() if ws_t is not None else 0, stream_ptr()))
        return finish(out, host)
    if isinstance(img, numpy.ndarray):
        desc = numpy.ascontiguousarray(img, dtype=numpy.float64)
        if desc.ndim != 2 or desc.shape[1] < 6:
            raise TypeError('an ellipse table must be (n x 6)')
        desc = numpy.ascontiguousarray(desc[:, :6])
        out = new_gpu(shape, tl, br)
        _native.check(L.rg_radon_fromdesc(rg_image(out), desc.ctypes.data_as(
            ctypes.POINTER(ctypes.c_double)), desc.shape[0], stream_ptr()))
        return out.cpu()
    raise TypeError('radon expects an image, a gpu_image or an ellipse table')


def radon_gpu(*args):
    """pyraft's radon_gpu(f, rays=f.shape[0], angles=360): slant-stack Radon
    on the [-1,1]^2 grid, views on [0, pi), rays on [-1, 1]; returns a host
    image with top_left (0, 1), bottom_right (pi, -1)."""
    if len(args) == 0:
        raise TypeError('Not enough arguments!')
    f = args[0]
    rays = args[1] if len(args) > 1 else f.shape[0]
    angles = args[2] if len(args) > 2 else 360
    src = image(numpy.asarray(f, dtype=numpy.float64))
    return radon(src, (rays, angles), radon_method.SLANTSTACK)


def _is_tensor(x):
    try:
        import torch
        return isinstance(x, torch.Tensor)
    except ImportError:
        return False
