"""FBP filter step on the GPU, one view at a time along t.

* ``lowpassino_fbp(sino)``: pyraft's filter (pyraft/filters/filters.py:13-68,
  a cosine-windowed ramp applied by circular FFT along t).  Here it is a
  circular FFT of length R (k_filter_fft) when R is a power of two up to
  16384, else a circular convolution with its spatial kernel Re(ifft(G)),
  computed once per geometry in FP64 (k_conv_rows).
* ``ramlak(sino)``: the discrete Ram-Lak filter as a linear convolution,
  q[n] = dt * sum_k h[n-k] p[k], h[0] = 1/(4 dt^2),
  h[odd m] = -1/(pi^2 m^2 dt^2), h[even m != 0] = 0.  Up to 8192 rays it is
  evaluated by a zero-padded FFT of the first difference (k_filter_fft),
  above that by direct sums (k_ramlak_rows); both give the same linear
  convolution.
Both keep the sinogram's corners and return the input's kind (host image or
gpu_image).
"""
from __future__ import annotations

import numpy

from . import _native
from .raftypes import finish, gpu_image, new_gpu, rg_image, stream_ptr, to_gpu, workspace


def _filter(sino, kind):
    gs, host = to_gpu(sino, (0.0, 1.0), (numpy.pi, -1.0))
    out = new_gpu(gs.shape, gs.top_left, gs.bottom_right)
    L = _native.load()
    a, b = rg_image(gs), rg_image(out)
    ws_t, ws = workspace(L.rg_filter_workspace(a, kind))
    _native.check(L.rg_filter(a, b, kind, ws, ws_t.numel() if ws_t is not None else 0,
                              stream_ptr()))
    return finish(out, host)


def lowpassino_fbp(*args):
    """Filtered sinogram for FBP, pyraft's lowpassino_fbp(sino)."""
    if len(args) == 0:
        raise TypeError('Not enough arguments!')
    if len(args) > 1:
        raise TypeError('a custom t mesh is not supported; the sinogram corners define t')
    return _filter(args[0], _native.RG_FILTER_LOWPASS)


def ramlak(sino):
    """Ram-Lak filtered sinogram (linear spatial convolution along t)."""
    return _filter(sino, _native.RG_FILTER_RAMLAK)
