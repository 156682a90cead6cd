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


def _mesh(vol, theta, t, nstack, img_stride, sino_shape):
    """Mesh Radon of nstack slices of a device volume `vol` laid out as
    rg_image views (first slice `vol`, consecutive slices img_stride apart).
    Returns the (nstack, len(t), len(theta)) float32 device tensor."""
    import torch
    L = _native.load()
    t = numpy.ascontiguousarray(t, dtype=numpy.float64)
    theta = numpy.ascontiguousarray(theta, dtype=numpy.float64)
    out = torch.zeros((nstack,) + tuple(sino_shape), dtype=torch.float32, device='cuda')
    S = _native.RG_IMAGE(out.data_ptr(), sino_shape[0], 1, sino_shape[1], sino_shape[1],
                         -1.0, 1.0, 1.0, -1.0)
    dp = ctypes.POINTER(ctypes.c_double)
    ws_t, ws = workspace(L.rg_radon_slantstack_withmesh_workspace(vol, S, nstack))
    _native.check(L.rg_radon_slantstack_withmesh(
        vol, img_stride, S, sino_shape[0] * sino_shape[1], nstack, t.ctypes.data_as(dp),
        theta.ctypes.data_as(dp), ws, ws_t.numel() if ws_t is not None else 0, stream_ptr()))
    return out


def radon_withmesh(*args):
    """pyraft's radon_withmesh(f, theta, t=linspace over f's x extent):
    slant-stack Radon on the given t and theta vectors -> (len(t),
    len(theta)) host image (default corners, as pyraft)."""
    if len(args) == 0:
        raise TypeError('Not enough arguments!')
    f, theta = args[0], numpy.atleast_1d(numpy.asarray(args[1], dtype=numpy.float64))
    t = args[2] if len(args) > 2 else numpy.linspace(f.top_left[0], f.bottom_right[0], f.shape[1])
    g, _ = to_gpu(f)
    out = _mesh(rg_image(g), theta, t, 1, 0, (len(t), len(theta)))
    return image(out[0].double().cpu().numpy())


def radon_view(*args):
    """pyraft's radon_view(f, theta, t): one view on the mesh t -> 1-D array."""
    if len(args) < 2:
        raise TypeError('Not enough arguments!')
    f = args[0]
    t = args[2] if len(args) > 2 else numpy.linspace(f.top_left[0], f.bottom_right[0], f.shape[1])
    return numpy.asarray(radon_withmesh(f, [float(args[1])], t))[:, 0]


def _volume_slices(f):
    """Device copy of a (N, M, K) volume and the rg_image of slice f[:, 0, :]
    (slices f[:, i, :] are K floats apart), as pyraft's radon_3d_stack reads
    them (pyraft/sinogram/sino.py:307-310)."""
    import torch
    v = torch.from_numpy(numpy.ascontiguousarray(f, dtype=numpy.float32)).cuda()
    n0, n1, n2 = v.shape
    img = _native.RG_IMAGE(v.data_ptr(), n0, 1, n2, n1 * n2, -1.0, 1.0, 1.0, -1.0)
    return v, img, n2


def radon_3d_stack(*args):
    """pyraft's radon_3d_stack(f, theta, t): mesh Radon of every slice
    f[:, i, :] (i < f.shape[0]) of a cubic volume, in one launch ->
    S (len(theta), N, len(t)) with S[:, i, :] = Radon(slice i)^T."""
    if len(args) == 0:
        raise TypeError('Not enough arguments!')
    f = numpy.asarray(args[0])
    theta = numpy.asarray(args[1], numpy.float64) if len(args) > 1 else numpy.linspace(0, numpy.pi, 180)
    t = numpy.asarray(args[2], numpy.float64) if len(args) > 2 else numpy.linspace(-1, 1, f.shape[1])
    n = f.shape[0]
    v, img, step = _volume_slices(f)
    out = _mesh(img, theta, t, n, step, (len(t), len(theta)))
    return numpy.transpose(out.double().cpu().numpy(), (2, 0, 1))


def snapshot(*args):
    """pyraft's snapshot(f, theta=0, t): one view of every slice f[:, k, :]
    -> (N, len(t))."""
    if len(args) == 0:
        raise TypeError('Not enough arguments!')
    f = numpy.asarray(args[0])
    theta = float(args[1]) if len(args) > 1 else 0.0
    t = numpy.asarray(args[2], numpy.float64) if len(args) > 2 else numpy.linspace(-1.0, 1.0, f.shape[1])
    n = f.shape[0]
    v, img, step = _volume_slices(f)
    out = _mesh(img, [theta], t, n, step, (len(t), 1))
    return out[:, :, 0].double().cpu().numpy()
