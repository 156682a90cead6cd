"""ctypes binding of libraftgb.so (C ABI in include/raftgb.h).

This is the process -> native boundary, as ``libraft`` is for pyraft
(pyraft/raftypes.py:29-38,138-215).  There is no fallback: if the library is
missing or cannot be loaded, every operator raises RaftError.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libraftgb.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "raftgb.h")

RG_OK = 0
RG_EINVAL = -1
RG_ECUDA = -2
RG_ENOMEM = -3
RG_EUNSUPPORTED = -4
RG_EWORKSPACE = -5
RG_BRESENHAM = 1
RG_SLANTSTACK = 2
RG_SLANTSTACK_BP = 3
RG_FILTER_RAMLAK = 1
RG_FILTER_LOWPASS = 2

_c_double = ctypes.c_double
_c_int = ctypes.c_int
_vp = ctypes.c_void_p
_size_t = ctypes.c_size_t


class RaftError(RuntimeError):
    """A libraftgb call failed (status code and the library's message)."""

    def __init__(self, code, msg):
        super().__init__(f"{msg} (rg status {code})")
        self.code = code


class RG_IMAGE(ctypes.Structure):
    """rg_image: a raft_image (raft/raft_image.h:11-19) over device floats."""
    _fields_ = [("data", _vp), ("lines", _c_int), ("line_stride", _c_int),
                ("columns", _c_int), ("column_stride", _c_int),
                ("tl_x", _c_double), ("tl_y", _c_double),
                ("br_x", _c_double), ("br_y", _c_double)]


class RG_IMAGE_F64(ctypes.Structure):
    """rg_image_f64: rg_image over device doubles."""
    _fields_ = [("data", _vp), ("lines", _c_int), ("line_stride", _c_int),
                ("columns", _c_int), ("column_stride", _c_int),
                ("tl_x", _c_double), ("tl_y", _c_double),
                ("br_x", _c_double), ("br_y", _c_double)]


_IMG = RG_IMAGE
_IMG64 = RG_IMAGE_F64
_ll = ctypes.c_longlong
_PI = ctypes.POINTER(RG_IMAGE)
_SIGS = {
    "rg_last_error": ([], ctypes.c_char_p),
    "rg_version": ([], _c_int),
    "rg_device_status": ([], _c_int),
    "rg_radon_slantstack_workspace": ([_IMG, _IMG], _size_t),
    "rg_radon_slantstack": ([_IMG, _IMG, _vp, _size_t, _vp], _c_int),
    "rg_radon_slantstack_noalloc": ([_IMG, _IMG, _vp], _c_int),
    "rg_radon_slantstack_stack_workspace": ([_IMG, _IMG, _c_int], _size_t),
    "rg_radon_slantstack_stack": ([_IMG, _ll, _IMG, _ll, _c_int, _vp, _size_t, _vp], _c_int),
    "rg_radon_transpose_slantstack_stack_workspace": ([_IMG, _IMG, _c_int], _size_t),
    "rg_radon_transpose_slantstack_stack": ([_IMG, _ll, _IMG, _ll, _c_int, _vp, _size_t, _vp],
                                            _c_int),
    "rg_radon_slantstack_f64": ([_IMG64, _IMG64, _vp], _c_int),
    "rg_radon_transpose_slantstack_f64": ([_IMG64, _IMG64, _vp], _c_int),
    "rg_backprojection_slantstack_workspace": ([_IMG, _IMG], _size_t),
    "rg_backprojection_slantstack": ([_IMG, _IMG, _vp, _size_t, _vp], _c_int),
    "rg_radon_transpose_slantstack_workspace": ([_IMG, _IMG], _size_t),
    "rg_radon_transpose_slantstack": ([_IMG, _IMG, _vp, _size_t, _vp], _c_int),
    "rg_radon_bresenham_workspace": ([_IMG, _IMG], _size_t),
    "rg_radon_bresenham": ([_IMG, _IMG, _vp, _size_t, _vp], _c_int),
    "rg_radon_transpose_bresenham_workspace": ([_IMG, _IMG], _size_t),
    "rg_radon_transpose_bresenham": ([_IMG, _IMG, _vp, _size_t, _vp], _c_int),
    "rg_backprojection_bresenham_workspace": ([_IMG, _IMG], _size_t),
    "rg_backprojection_bresenham": ([_IMG, _IMG, _vp, _size_t, _vp], _c_int),
    "rg_radon_slantstack_withmesh_workspace": ([_IMG, _IMG, _c_int], _size_t),
    "rg_radon_slantstack_withmesh": ([_IMG, _ll, _IMG, _ll, _c_int, ctypes.POINTER(_c_double),
                                      ctypes.POINTER(_c_double), _vp, _size_t, _vp], _c_int),
    "rg_em_transmission_workspace": ([_IMG, _IMG], _size_t),
    "rg_em_transmission": ([_IMG, _IMG, _IMG, _IMG, _c_int, _vp, _size_t, _vp], _c_int),
    "rg_dda_trace": ([_c_int, _c_int, ctypes.POINTER(_c_double), ctypes.POINTER(_c_double),
                      ctypes.POINTER(_c_double), _c_int, _c_int, _vp, _vp, _vp, _vp, _vp],
                     _c_int),
    "rg_filter_workspace": ([_IMG, _c_int], _size_t),
    "rg_filter": ([_IMG, _IMG, _c_int, _vp, _size_t, _vp], _c_int),
    "rg_fbp_workspace": ([_IMG, _IMG, _c_int], _size_t),
    "rg_fbp": ([_IMG, _IMG, _c_int, _vp, _size_t, _vp], _c_int),
    "rg_em_workspace": ([_IMG, _IMG, _c_int, _c_int], _size_t),
    "rg_em": ([_IMG, _IMG, _c_int, _c_int, _c_int, _vp, _size_t, _vp], _c_int),
    "rg_em_subiterations": ([_IMG, _IMG, _c_int, _c_int, _ll, _ll, _vp, _size_t, _vp], _c_int),
    "rg_osem_batch_workspace": ([_PI, _PI, _c_int, _c_int], _size_t),
    "rg_osem_batch": ([_PI, _PI, _c_int, _c_int, _c_int, _c_int, _vp, _size_t, _vp], _c_int),
    "rg_em_plain_host": ([_vp, _vp, _c_int, _c_int, _c_int, _c_int, _c_int], _c_int),
    "rg_phantom_fromdesc": ([_IMG, ctypes.POINTER(_c_double), _c_int, _vp], _c_int),
    "rg_tv": ([_vp, _c_int, _c_int, ctypes.c_float, _vp, _vp, _vp], _c_int),
    "rg_radon_fromdesc": ([_IMG, ctypes.POINTER(_c_double), _c_int, _vp], _c_int),
    "rg_radon_slantstack_host": ([_vp, _vp, _c_int, _c_int, _c_int], _c_int),
    "rg_backprojection_slantstack_host": ([_vp, _vp, _c_int, _c_int, _c_int], _c_int),
    "rg_em_host": ([_vp, _vp, _c_int, _c_int, _c_int, _c_int], _c_int),
}

_lib = None


def header_symbols():
    """Names of every function declared in include/raftgb.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rg_\w+)\s*\(", text)))


def load(path: str = LIB_PATH):
    """Load libraftgb.so (no build, no fallback) and declare signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RaftError(-100, f"{path} is missing: build it with "
                              f"`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(path)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != RG_OK:
        raise RaftError(rc, load().rg_last_error().decode(errors="replace"))
