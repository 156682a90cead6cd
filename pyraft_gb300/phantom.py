"""Ellipse phantoms (pyraft/phantom/phantom.py:12-52,
raft/raft_image_phantom_fromdesc.c).

An ellipse table is (n x 6): [alpha, a, b, x0, y0, theta] per ellipse.
``shepplogan`` rasterises the standard table on the GPU in FP64 (bit-exact
inside/outside decisions against the reference); ``random_ellipses`` draws
the seeded synthetic tables used by the benchmarks.
"""
from __future__ import annotations

import ctypes
import math

import numpy

from . import _native
from .raftypes import gpu_image, image, new_gpu, rg_image, stream_ptr


def _shepp_logan_desc():
    """The Shepp-Logan head table as pyraft uses it
    (pyraft/phantom/phantom.py:12-26, raft/raft_matrix_phantomdesc_shepplogan.c)."""
    p10 = math.pi / 10.0
    return numpy.array([
        [1.0, 0.69, 0.92, 0.0, 0.0, 0.0],
        [-0.8, 0.6624, 0.874, 0.0, -0.0184, 0.0],
        [-0.2, 0.1100, 0.31, 0.22, 0.0, -p10],
        [-0.2, 0.1600, 0.41, -0.22, 0.0, p10],
        [0.1, 0.2100, 0.25, 0.0, 0.35, 0.0],
        [0.1, 0.0460, 0.046, 0.0, 0.1, 0.0],
        [0.1, 0.0460, 0.046, 0.0, -0.1, 0.0],
        [0.1, 0.0460, 0.023, -0.08, -0.605, 0.0],
        [0.1, 0.0230, 0.023, 0.0, -0.606, 0.0],
        [0.1, 0.0230, 0.046, 0.06, -0.605, 0.0]])


def phantom_fromdesc(shape, desc, device=False, **kwargs):
    """Rasterise an ellipse table (added on a zero image)."""
    probe = image((2, 2), **kwargs)
    out = new_gpu(shape, probe.top_left, probe.bottom_right)
    d = numpy.ascontiguousarray(numpy.asarray(desc, dtype=numpy.float64)[:, :6])
    _native.check(_native.load().rg_phantom_fromdesc(
        rg_image(out), d.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), d.shape[0],
        stream_ptr()))
    return out if device else out.cpu()


def shepplogan(shape=(256, 256), device=False, **kwargs):
    return phantom_fromdesc(shape, _shepp_logan_desc(), device=device, **kwargs)


def random_ellipses(n, rng, density=(0.0, 1.0)):
    """n random ellipses: centres uniform in the unit disk, semi-axes
    U(0.02, 0.4), orientation U(0, pi), density U(density)."""
    r = numpy.sqrt(rng.uniform(0.0, 1.0, n))
    phi = rng.uniform(0.0, 2.0 * math.pi, n)
    desc = numpy.empty((n, 6))
    desc[:, 0] = rng.uniform(density[0], density[1], n)
    desc[:, 1] = rng.uniform(0.02, 0.4, n)
    desc[:, 2] = rng.uniform(0.02, 0.4, n)
    desc[:, 3] = r * numpy.cos(phi)
    desc[:, 4] = r * numpy.sin(phi)
    desc[:, 5] = rng.uniform(0.0, math.pi, n)
    return desc
