"""ctypes bindings to the reference's own hot-path C/C++ compiled in place
(``make -C oracle ref REF_SRC=<checkout>/raft`` -> ``oracle/_ref/libraft_ref.so``).

TEST INFRASTRUCTURE: used only to pin the oracle restatement
(tests/test_oracle_golden.py, when the library exists) and to generate the
fixtures under tests/golden (tests/golden/make_golden.py).  The structs
mirror pyraft/raftypes.py:85-100 and are passed by value, as there.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import oracle as _o

_dp = ctypes.POINTER(ctypes.c_double)


class RAFT_MATRIX(ctypes.Structure):
    _fields_ = [("p_data", _dp), ("lines", ctypes.c_int), ("line_stride", ctypes.c_int),
                ("columns", ctypes.c_int), ("column_stride", ctypes.c_int)]


class RAFT_IMAGE(ctypes.Structure):
    _fields_ = [("data", RAFT_MATRIX), ("tl_x", ctypes.c_double), ("tl_y", ctypes.c_double),
                ("br_x", ctypes.c_double), ("br_y", ctypes.c_double)]


class RAFT_VECTOR(ctypes.Structure):
    _fields_ = [("p_data", _dp), ("size", ctypes.c_int), ("stride", ctypes.c_int)]


class RAFT_DDA(ctypes.Structure):
    """raft_ddaiterator (raft/raft_ddaiterator.h:10-47)."""
    _fields_ = [("i", ctypes.c_int), ("j", ctypes.c_int), ("sigma", ctypes.c_double),
                ("slow_move", ctypes.c_int), ("p_slow_idx", ctypes.c_void_p),
                ("p_fast_idx", ctypes.c_void_p), ("epsilon", ctypes.c_double),
                ("epsilon_update", ctypes.c_double), ("delta_x", ctypes.c_double),
                ("delta_y", ctypes.c_double), ("delta_slow", ctypes.c_double),
                ("Delta_i", ctypes.c_int), ("Delta_j", ctypes.c_int),
                ("Delta_slow", ctypes.c_int), ("Delta_fast", ctypes.c_int),
                ("sigma_tilde", ctypes.c_double), ("lines", ctypes.c_int),
                ("columns", ctypes.c_int), ("bbox_tl_x", ctypes.c_double),
                ("bbox_tl_y", ctypes.c_double), ("bbox_br_x", ctypes.c_double),
                ("bbox_br_y", ctypes.c_double), ("tl_x", ctypes.c_double),
                ("tl_y", ctypes.c_double), ("br_x", ctypes.c_double),
                ("br_y", ctypes.c_double), ("x0", ctypes.c_double), ("y0", ctypes.c_double),
                ("i_init", ctypes.c_int), ("j_init", ctypes.c_int),
                ("sin_theta", ctypes.c_double), ("cos_theta", ctypes.c_double)]


_lib = None


def available() -> bool:
    return os.path.exists(_o.REF_SO)


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_o.REF_SO)
        for name in ("raft_radon_slantstack", "raft_backprojection_slantstack",
                     "raft_radon_bresenham", "raft_radon_transpose_bresenham",
                     "raft_backprojection_bresenham"):
            getattr(_lib, name).argtypes = [RAFT_IMAGE, RAFT_IMAGE, ctypes.c_int]
            getattr(_lib, name).restype = None
        _lib.raft_radon_slantstack_withmesh.argtypes = [RAFT_IMAGE, RAFT_IMAGE, RAFT_VECTOR,
                                                        RAFT_VECTOR, ctypes.c_int]
        _lib.raft_radon_slantstack_withmesh.restype = None
        _lib.raft_image_phantom_fromdesc.argtypes = [RAFT_IMAGE, RAFT_MATRIX]
        _lib.raft_radon_fromdesc.argtypes = [RAFT_IMAGE, RAFT_MATRIX]
        _lib.raft_ddaiterator_set_image.argtypes = [ctypes.POINTER(RAFT_DDA), RAFT_IMAGE]
        _lib.raft_ddaiterator_set_theta.argtypes = [ctypes.POINTER(RAFT_DDA), ctypes.c_double]
        _lib.raft_ddaiterator_set_t.argtypes = [ctypes.POINTER(RAFT_DDA), ctypes.c_double]
        _lib.raft_ddaiterator_update.argtypes = [ctypes.POINTER(RAFT_DDA)]
        _lib.raft_ddaiterator_end.argtypes = [ctypes.POINTER(RAFT_DDA)]
        _lib.raft_ddaiterator_end.restype = ctypes.c_int
    return _lib


def _matrix(a):
    return RAFT_MATRIX(a.ctypes.data_as(_dp), a.shape[0], a.strides[1] // 8,
                       a.shape[1], a.strides[0] // 8)


def _image(a, corners):
    return RAFT_IMAGE(_matrix(a), *map(float, corners))


def _call2(name, src, src_corners, dst, dst_corners, threads):
    getattr(lib(), name)(_image(src, src_corners), _image(dst, dst_corners),
                         ctypes.c_int(threads))


def radon_slantstack(img, nrays, nviews, img_corners=_o.IMG_CORNERS,
                     sino_corners=_o.SINO_CORNERS, threads=4):
    img = np.ascontiguousarray(img, dtype=np.float64)
    out = np.zeros((nrays, nviews))
    _call2("raft_radon_slantstack", img, img_corners, out, sino_corners, threads)
    return out


def backprojection_slantstack(sino, size, img_corners=_o.IMG_CORNERS,
                              sino_corners=_o.SINO_CORNERS, threads=4):
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    out = np.zeros((size, size))
    _call2("raft_backprojection_slantstack", sino, sino_corners, out, img_corners, threads)
    return out


def radon_bresenham(img, nrays, nviews, img_corners=_o.IMG_CORNERS,
                    sino_corners=_o.SINO_CORNERS, threads=4):
    img = np.ascontiguousarray(img, dtype=np.float64)
    out = np.zeros((nrays, nviews))
    _call2("raft_radon_bresenham", img, img_corners, out, sino_corners, threads)
    return out


def radon_transpose_bresenham(sino, shape, img_corners=_o.IMG_CORNERS,
                              sino_corners=_o.SINO_CORNERS, threads=4):
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    out = np.zeros(tuple(shape))
    _call2("raft_radon_transpose_bresenham", sino, sino_corners, out, img_corners, threads)
    return out


def backprojection_bresenham(sino, shape, img_corners=_o.IMG_CORNERS,
                             sino_corners=_o.SINO_CORNERS, threads=4):
    sino = np.ascontiguousarray(sino, dtype=np.float64)
    out = np.zeros(tuple(shape))
    _call2("raft_backprojection_bresenham", sino, sino_corners, out, img_corners, threads)
    return out


def radon_slantstack_withmesh(img, t, theta, img_corners=_o.IMG_CORNERS, threads=1):
    """The reference drops the last (nrays*nviews mod nthreads) outputs; with
    threads=1 every output is computed."""
    img = np.ascontiguousarray(img, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.float64)
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    out = np.zeros((len(t), len(theta)))
    vt = RAFT_VECTOR(t.ctypes.data_as(_dp), len(t), 1)
    vth = RAFT_VECTOR(theta.ctypes.data_as(_dp), len(theta), 1)
    lib().raft_radon_slantstack_withmesh(_image(img, img_corners), _image(out, _o.SINO_CORNERS),
                                         vt, vth, ctypes.c_int(threads))
    return out


def phantom_fromdesc(shape, desc, corners=_o.IMG_CORNERS):
    desc = np.ascontiguousarray(desc, dtype=np.float64)
    out = np.zeros(tuple(shape))
    lib().raft_image_phantom_fromdesc(_image(out, corners), _matrix(desc))
    return out


def radon_fromdesc(nrays, nviews, desc, sino_corners=_o.SINO_CORNERS):
    desc = np.ascontiguousarray(desc, dtype=np.float64)
    out = np.zeros((nrays, nviews))
    lib().raft_radon_fromdesc(_image(out, sino_corners), _matrix(desc))
    return out


def dda_trace(shape, theta, t, corners=_o.IMG_CORNERS, cap=None):
    """Run the reference iterator on one ray; returns (i, j, sigma) arrays."""
    lines, columns = shape
    cap = cap or 4 * (lines + columns) + 8
    dummy = np.zeros((lines, columns))
    it = RAFT_DDA()
    L = lib()
    L.raft_ddaiterator_set_image(ctypes.byref(it), _image(dummy, corners))
    L.raft_ddaiterator_set_theta(ctypes.byref(it), ctypes.c_double(theta))
    it.sigma = float("nan")   # the axis-aligned branches leave it unset
    L.raft_ddaiterator_set_t(ctypes.byref(it), ctypes.c_double(t))
    ii, jj, ss = [], [], []
    while not L.raft_ddaiterator_end(ctypes.byref(it)) and len(ii) < cap:
        ii.append(it.i)
        jj.append(it.j)
        ss.append(it.sigma)
        L.raft_ddaiterator_update(ctypes.byref(it))
    return np.array(ii, np.int32), np.array(jj, np.int32), np.array(ss)
