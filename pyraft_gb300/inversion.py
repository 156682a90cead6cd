"""Filtered backprojection (pyraft/inversion/inversion.py:11-61).

pyraft's ``fbp`` cannot run (it asks for radon_method.ANDERSON, which does not
exist, and calls backprojection() with the wrong signature,
pyraft/inversion/inversion.py:22); here it does what its body intends:
filter with lowpassino_fbp, then slant-stack backprojection onto an N x N
image, N = number of rays.  ``fbp_gpu(s, img_size)`` keeps its signature and
returns a float32 array.  Both accept filter='lowpass' (pyraft's filter, the
default) or filter='ramlak', and run as one fused library call (filter +
backprojection, rg_fbp).
"""
from __future__ import annotations

import numpy

from . import _native
from .raftypes import finish, image, new_gpu, rg_image, stream_ptr, to_gpu, workspace

_KINDS = {'lowpass': _native.RG_FILTER_LOWPASS, 'ramlak': _native.RG_FILTER_RAMLAK}


def fbp_device(sino, shape, filter='lowpass', **kwargs):
    """Filter + slant-stack backprojection; returns the input's kind."""
    kind = _KINDS[filter]
    kw = dict(kwargs)
    probe = image((2, 2), **kw)
    gs, host = to_gpu(sino, (0.0, 1.0), (numpy.pi, -1.0))
    out = new_gpu(shape, probe.top_left, probe.bottom_right)
    L = _native.load()
    a, b = rg_image(gs), rg_image(out)
    ws_t, ws = workspace(L.rg_fbp_workspace(a, b, kind))
    _native.check(L.rg_fbp(a, b, kind, ws, ws_t.numel() if ws_t is not None else 0, stream_ptr()))
    return finish(out, host)


def fbp(*args, filter='lowpass', **kwargs):
    if len(args) == 0:
        raise TypeError('Not enough arguments!')
    sino = args[0]
    n = args[1] if len(args) > 1 else sino.shape[0]
    return fbp_device(sino, (n, n), filter=filter, **kwargs)


def fbp_gpu(*args, filter='lowpass'):
    if len(args) == 0:
        raise TypeError('Not enough arguments!')
    s = args[0]
    n = args[1] if len(args) > 1 else s.shape[0]
    src = image(numpy.asarray(s, dtype=numpy.float64), top_left=(0.0, 1.0),
                bottom_right=(numpy.pi, -1.0))
    return numpy.asarray(fbp_device(src, (n, n), filter=filter), dtype=numpy.float32)
