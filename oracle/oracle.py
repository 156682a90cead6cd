"""FP64 CPU oracle for pyraft's reconstruction hot path.

TEST INFRASTRUCTURE.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module, as the checker of the
CUDA path (or as the timed CPU baseline).  ``pyraft_gb300`` never imports it.

Two back ends:

* ``liboracle.so`` -- the C restatement in ``oracle/raft_oracle.c`` (own code,
  built by ``oracle/Makefile``), used everywhere, including the GPU machine.
* ``libraft_ref.so`` -- the reference's own sources compiled in place by
  ``make -C oracle ref`` (only where the reference tree exists).  Used to pin
  the restatement and to generate ``tests/golden`` fixtures.

Array convention: numpy float64 arrays, row-major, shape (lines, columns);
corners are ``(tl_x, tl_y, br_x, br_y)`` as in ``raft_image``
(raft/raft_image.h:11-19) and ``pyraft.image.top_left/bottom_right``.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libraft_ref.so")

_dp = ctypes.POINTER(ctypes.c_double)


class OrcImg(ctypes.Structure):
    _fields_ = [("p", _dp), ("lines", ctypes.c_int), ("columns", ctypes.c_int),
                ("tl_x", ctypes.c_double), ("tl_y", ctypes.c_double),
                ("br_x", ctypes.c_double), ("br_y", ctypes.c_double)]


def build(ref_src: str | None = None) -> None:
    """Compile the oracle (and, given the reference's raft/ directory, the
    reference's own sources) with make."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref_src:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_SRC={ref_src}"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        _lib = ctypes.CDLL(ORACLE_SO)
    return _lib


def nthreads() -> int:
    return os.cpu_count() or 1


def _img(a: np.ndarray, corners) -> OrcImg:
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return OrcImg(a.ctypes.data_as(_dp), a.shape[0], a.shape[1], *map(float, corners))


IMG_CORNERS = (-1.0, 1.0, 1.0, -1.0)
SINO_CORNERS = (0.0, 1.0, math.pi, -1.0)


def radon_slantstack(img, nrays, nviews, img_corners=IMG_CORNERS,
                     sino_corners=SINO_CORNERS, threads=None):
    """restates raft/raft_radon_slantstack.c:44-214"""
    img = np.ascontiguousarray(img, dtype=np.float64)
    out = np.zeros((nrays, nviews))
    I, S = _img(img, img_corners), _img(out, sino_corners)
    lib().orc_radon_slantstack(ctypes.byref(I), ctypes.byref(S),
                               ctypes.c_int(threads or nthreads()))
    return out


def radon_slantstack_transpose(sino, size, img_corners=IMG_CORNERS,
                               sino_corners=SINO_CORNERS, threads=None):
    """Exact transpose of radon_slantstack (matched adjoint)."""
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    out = np.zeros((size, size))
    I, S = _img(out, img_corners), _img(sino, sino_corners)
    rc = lib().orc_radon_slantstack_transpose(ctypes.byref(S), ctypes.byref(I),
                                              ctypes.c_int(threads or nthreads()))
    assert rc == 0
    return out


def backprojection_slantstack(sino, size, img_corners=IMG_CORNERS,
                              sino_corners=SINO_CORNERS, threads=None):
    """restates raft/raft_backprojection_slantstack.c:43-180"""
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    out = np.zeros((size, size))
    I, S = _img(out, img_corners), _img(sino, sino_corners)
    lib().orc_backprojection_slantstack(ctypes.byref(S), ctypes.byref(I),
                                        ctypes.c_int(threads or nthreads()))
    return out


def backprojection_rows(sino, size, row0, row1, img_corners=IMG_CORNERS,
                        sino_corners=SINO_CORNERS, threads=None):
    """Rows [row0, row1) of backprojection_slantstack (CPU timing sample)."""
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    out = np.zeros((size, size))
    I, S = _img(out, img_corners), _img(sino, sino_corners)
    lib().orc_backprojection_slantstack_rows(ctypes.byref(S), ctypes.byref(I), ctypes.c_int(row0),
                                             ctypes.c_int(row1),
                                             ctypes.c_int(threads or nthreads()))
    return out


def backprojection_rowstep(sino, size, row0, step, count, img_corners=IMG_CORNERS,
                           sino_corners=SINO_CORNERS, threads=None):
    """Rows row0, row0 + step, ... (count of them) of backprojection_slantstack,
    returned as a (count, size) array: a sample spread over the image."""
    assert count >= 1 and step >= 1 and 0 <= row0 and row0 + (count - 1) * step < size
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    out = np.zeros((size, size))
    I, S = _img(out, img_corners), _img(sino, sino_corners)
    lib().orc_backprojection_slantstack_rowstep(ctypes.byref(S), ctypes.byref(I),
                                                ctypes.c_int(row0), ctypes.c_int(step),
                                                ctypes.c_int(count),
                                                ctypes.c_int(threads or nthreads()))
    return out[row0:row0 + (count - 1) * step + 1:step].copy()


def ramlak_fft(sino, dt):
    """The discrete Ram-Lak filter of `ramlak` (linear convolution along axis
    0, q[n] = dt * sum_k h[n-k] p[k]) evaluated the way pyraft filters, by
    numpy FFT (pyraft/filters/filters.py:13-68 applies its ramp by np.fft
    along t): the kernel's 2R-1 taps and each view are zero-padded to a
    power of two M >= 2R-1, multiplied in frequency and cut back to R."""
    sino = np.asarray(sino, dtype=np.float64)
    R = sino.shape[0]
    M = 1 << (2 * R - 2).bit_length()
    m = np.arange(-(R - 1), R).astype(np.float64)
    h = np.zeros(2 * R - 1)
    h[m == 0] = 1.0 / (4.0 * dt * dt)
    odd = np.abs(m) % 2 == 1
    h[odd] = -1.0 / (np.pi ** 2 * m[odd] ** 2 * dt * dt)
    hp = np.zeros(M)
    hp[:R] = h[R - 1:]                  # lags 0 .. R-1
    hp[M - (R - 1):] = h[:R - 1]        # lags -(R-1) .. -1, wrapped
    Hf = np.fft.rfft(hp)
    Sf = np.fft.rfft(sino, n=M, axis=0)
    return dt * np.fft.irfft(Sf * Hf[:, None], n=M, axis=0)[:R]


def ramlak_views(sino, dt, nv, threads=None):
    """Ram-Lak of the first nv views only (CPU timing sample)."""
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    out = np.zeros_like(sino)
    rc = lib().orc_ramlak_views(sino.ctypes.data_as(_dp), out.ctypes.data_as(_dp),
                                ctypes.c_int(sino.shape[0]), ctypes.c_int(sino.shape[1]),
                                ctypes.c_int(nv), ctypes.c_double(dt),
                                ctypes.c_int(threads or nthreads()))
    assert rc == 0
    return out


def radon_bresenham(img, nrays, nviews, img_corners=IMG_CORNERS,
                    sino_corners=SINO_CORNERS, threads=None):
    """restates raft/raft_radon_bresenham.cpp:16-105"""
    img = np.ascontiguousarray(img, dtype=np.float64)
    out = np.zeros((nrays, nviews))
    I, S = _img(img, img_corners), _img(out, sino_corners)
    lib().orc_radon_bresenham(ctypes.byref(I), ctypes.byref(S),
                              ctypes.c_int(threads or nthreads()))
    return out


def radon_transpose_bresenham(sino, shape, img_corners=IMG_CORNERS,
                              sino_corners=SINO_CORNERS, threads=None):
    """restates raft/raft_radon_transpose_bresenham.cpp:17-201"""
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    out = np.zeros(tuple(shape))
    I, S = _img(out, img_corners), _img(sino, sino_corners)
    rc = lib().orc_radon_transpose_bresenham(ctypes.byref(S), ctypes.byref(I),
                                             ctypes.c_int(threads or nthreads()))
    assert rc == 0
    return out


def dda_trace(shape, theta, t, corners=IMG_CORNERS, cap=None):
    """Pixel sequence (i, j, sigma) of one DDA ray (raft/raft_ddaiterator.c)."""
    lines, columns = shape
    cap = cap or 4 * (lines + columns) + 8
    ii = np.zeros(cap, np.int32)
    jj = np.zeros(cap, np.int32)
    ss = np.zeros(cap, np.float64)
    L = lib()
    L.orc_dda_trace.restype = ctypes.c_int
    n = L.orc_dda_trace(ctypes.c_int(lines), ctypes.c_int(columns),
                        *[ctypes.c_double(v) for v in corners],
                        ctypes.c_double(theta), ctypes.c_double(t),
                        ii.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                        jj.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                        ss.ctypes.data_as(_dp), ctypes.c_int(cap))
    n = min(n, cap)
    return ii[:n].copy(), jj[:n].copy(), ss[:n].copy()


def phantom_fromdesc(shape, desc, corners=IMG_CORNERS):
    """restates raft/raft_image_phantom_fromdesc.c:4-59"""
    desc = np.ascontiguousarray(desc, dtype=np.float64)
    out = np.zeros(tuple(shape))
    I = _img(out, corners)
    lib().orc_phantom_fromdesc(ctypes.byref(I), desc.ctypes.data_as(_dp),
                               ctypes.c_int(desc.shape[0]))
    return out


def radon_fromdesc(nrays, nviews, desc, sino_corners=SINO_CORNERS):
    """restates raft/raft_radon_fromdesc.c:4-67 (endpoint-inclusive views)"""
    desc = np.ascontiguousarray(desc, dtype=np.float64)
    out = np.zeros((nrays, nviews))
    S = _img(out, sino_corners)
    lib().orc_radon_fromdesc(ctypes.byref(S), desc.ctypes.data_as(_dp),
                             ctypes.c_int(desc.shape[0]))
    return out


def ramlak(sino, dt, threads=None):
    """FP64 direct linear convolution with the discrete Ram-Lak kernel, along
    axis 0 of an (nrays, nviews) sinogram; q[n] = dt * sum_k h[n-k] p[k]."""
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    out = np.zeros_like(sino)
    rc = lib().orc_ramlak(sino.ctypes.data_as(_dp), out.ctypes.data_as(_dp),
                          ctypes.c_int(sino.shape[0]), ctypes.c_int(sino.shape[1]),
                          ctypes.c_double(dt), ctypes.c_int(threads or nthreads()))
    assert rc == 0
    return out


def circular_filter(sino, g, threads=None):
    """out[n] = sum_k g[(n-k) mod R] in[k] along axis 0."""
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    g = np.ascontiguousarray(g, dtype=np.float64)
    out = np.zeros_like(sino)
    lib().orc_circular_filter(sino.ctypes.data_as(_dp), out.ctypes.data_as(_dp),
                              ctypes.c_int(sino.shape[0]), ctypes.c_int(sino.shape[1]),
                              g.ctypes.data_as(_dp), ctypes.c_int(threads or nthreads()))
    return out


def lowpassino_fbp(sino, corners=SINO_CORNERS):
    """numpy restatement of pyraft/filters/filters.py:13-68 (cosine-windowed
    ramp, circular FFT along t, no padding, real part kept)."""
    sino = np.asarray(sino, dtype=np.float64)
    R, V = sino.shape
    tmin, tmax = corners[3], corners[1]
    t = np.linspace(tmin, tmax, R)
    dt = (t[R - 1] - t[0]) / (R - 1)
    wc = 1 / (2 * dt)
    w = np.linspace(-wc, wc, R)
    h = np.abs(w) * np.cos(np.pi * w * dt)
    G = np.fft.fftshift(np.transpose(np.kron(np.ones((V, 1)), h)))
    return np.fft.ifft(np.fft.fft(sino, axis=0) * G, axis=0).real


def lowpass_taps(R, corners=SINO_CORNERS):
    """Spatial kernel g with lowpassino_fbp(s) == circular_filter(s, g):
    Re(ifft(s_hat * G)) = s (*) Re(ifft(G)) for real s and real G."""
    tmin, tmax = corners[3], corners[1]
    t = np.linspace(tmin, tmax, R)
    dt = (t[R - 1] - t[0]) / (R - 1)
    wc = 1 / (2 * dt)
    w = np.linspace(-wc, wc, R)
    G = np.fft.fftshift(np.abs(w) * np.cos(np.pi * w * dt))
    return np.fft.ifft(G).real


def em_guarded(sino, x0, forward, transpose, niter, weight=None):
    """MLEM x <- x * A^T(y / Ax) / A^T 1 (pyraft/iterative/em.py:109-144),
    with the division guards of the CUDA path: y/0 -> 0, x*b/0 -> 0."""
    y = np.asarray(sino, dtype=np.float64)
    x = np.asarray(x0, dtype=np.float64).copy()
    if weight is None:
        weight = transpose(np.ones_like(y))
    for _ in range(niter):
        ax = forward(x)
        ratio = np.where(ax != 0.0, y / np.where(ax != 0.0, ax, 1.0), 0.0)
        bp = transpose(ratio)
        x = np.where(weight != 0.0, x * bp / np.where(weight != 0.0, weight, 1.0), 0.0)
    return x


def osem_interleaved(sino, x0, forward_sub, transpose_sub, nsubsets, niter):
    """OSEM with interleaved angle subsets: subset s holds views s, s+S, ...
    forward_sub(x, idx) / transpose_sub(r, idx) apply the operator restricted
    to the views in idx."""
    y = np.asarray(sino, dtype=np.float64)
    x = np.asarray(x0, dtype=np.float64).copy()
    V = y.shape[1]
    subsets = [np.arange(s, V, nsubsets) for s in range(nsubsets)]
    weights = [transpose_sub(np.ones((y.shape[0], len(idx))), idx) for idx in subsets]
    for _ in range(niter):
        for idx, wgt in zip(subsets, weights):
            ax = forward_sub(x, idx)
            ys = y[:, idx]
            ratio = np.where(ax != 0.0, ys / np.where(ax != 0.0, ax, 1.0), 0.0)
            bp = transpose_sub(ratio, idx)
            x = np.where(wgt != 0.0, x * bp / np.where(wgt != 0.0, wgt, 1.0), 0.0)
    return x


SHEPP_LOGAN = np.array([
    # alpha, a, b, x0, y0, theta  (raft/raft_matrix_phantomdesc_shepplogan.c:17-46,
    # pyraft/phantom/phantom.py:12-26)
    [1.0, 0.69, 0.92, 0.0, 0.0, 0.0],
    [-0.8, 0.6624, 0.874, 0.0, -0.0184, 0.0],
    [-0.2, 0.11, 0.31, 0.22, 0.0, -math.pi / 10.0],
    [-0.2, 0.16, 0.41, -0.22, 0.0, math.pi / 10.0],
    [0.1, 0.21, 0.25, 0.0, 0.35, 0.0],
    [0.1, 0.046, 0.046, 0.0, 0.1, 0.0],
    [0.1, 0.046, 0.046, 0.0, -0.1, 0.0],
    [0.1, 0.046, 0.023, -0.08, -0.605, 0.0],
    [0.1, 0.023, 0.023, 0.0, -0.606, 0.0],
    [0.1, 0.023, 0.046, 0.06, -0.605, 0.0],
])


def shepp_logan(n):
    """Shepp-Logan rasterised like pyraft.shepplogan (top-down rows)."""
    return phantom_fromdesc((n, n), SHEPP_LOGAN)


def backprojection_bresenham(sino, shape, img_corners=IMG_CORNERS, sino_corners=SINO_CORNERS,
                             threads=None):
    """restates raft/raft_backprojection_bresenham.cpp:17-251 (0 where no
    ray passes)"""
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    out = np.zeros(tuple(shape))
    I, S = _img(out, img_corners), _img(sino, sino_corners)
    rc = lib().orc_backprojection_bresenham(ctypes.byref(S), ctypes.byref(I),
                                            ctypes.c_int(threads or nthreads()))
    assert rc == 0
    return out


def radon_slantstack_withmesh(img, t, theta, img_corners=IMG_CORNERS, threads=None):
    """restates raft/raft_radon_slantstack_withmesh.c:45-211"""
    img = np.ascontiguousarray(img, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.float64)
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    out = np.zeros((len(t), len(theta)))
    I, S = _img(img, img_corners), _img(out, SINO_CORNERS)
    lib().orc_radon_slantstack_withmesh(ctypes.byref(I), ctypes.byref(S), t.ctypes.data_as(_dp),
                                        theta.ctypes.data_as(_dp),
                                        ctypes.c_int(threads or nthreads()))
    return out


def em_transmission(raw, flat, dark, x0, forward, transpose, niter):
    """Transmission EM x <- x * A^T(b e^{-Ax}) / A^T y with y = max(raw -
    dark, 0), b = max(flat - dark, 0) (the update of raft/raft_transmission_em
    .cu:53-60 with its multiply applied once), guards 0/0 -> 0."""
    y = np.maximum(np.asarray(raw, float) - np.asarray(dark, float), 0.0)
    b = np.maximum(np.asarray(flat, float) - np.asarray(dark, float), 0.0)
    x = np.asarray(x0, dtype=np.float64).copy()
    den = transpose(y)
    for _ in range(niter):
        q = b * np.exp(-forward(x))
        num = transpose(q)
        x = np.where(den != 0.0, x * num / np.where(den != 0.0, den, 1.0), 0.0)
    return x
