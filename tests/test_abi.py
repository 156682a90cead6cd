"""C-ABI checks that need no GPU: libraftgb.so builds, loads, exports every
entry point declared in include/raftgb.h, and rejects bad arguments on the
host before touching the device."""
import ctypes
import math

import pytest

from pyraft_gb300 import _native
from pyraft_gb300 import build as B


@pytest.fixture(scope="module")
def lib():
    B.build()
    return _native.load()


def test_exports_every_declared_symbol(lib):
    names = _native.header_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.rg_version() >= 100


def _img(ptr, lines, cols, tl=(-1.0, 1.0), br=(1.0, -1.0)):
    return _native.RG_IMAGE(ptr, lines, 1, cols, cols, tl[0], tl[1], br[0], br[1])


def test_rejects_bad_arguments_on_host(lib):
    null = _img(None, 8, 8)
    ok = _img(4096, 8, 8)
    sino = _img(8192, 8, 6, (0.0, 1.0), (math.pi, -1.0))
    assert lib.rg_radon_slantstack(null, sino, None, 0, None) == -1
    assert b"null" in lib.rg_last_error()
    rect = _img(4096, 8, 7)
    assert lib.rg_radon_slantstack(rect, sino, None, 0, None) == -1
    assert b"square" in lib.rg_last_error()
    tiny = _img(4096, 1, 1)
    assert lib.rg_backprojection_slantstack(sino, tiny, None, 0, None) == -1
    bad = _img(4096, 8, 8, (float("nan"), 1.0))
    assert lib.rg_radon_transpose_slantstack(sino, bad, None, 0, None) == -1
    assert lib.rg_em(sino, ok, 2, -1, 1, None, 0, None) == -1
    assert lib.rg_em(sino, ok, 2, 1, 0, None, 0, None) == -1
    assert lib.rg_em(sino, ok, 7, 1, 1, None, 0, None) == -1
    one_view = _img(8192, 8, 1, (0.0, 1.0), (math.pi, -1.0))
    assert lib.rg_radon_bresenham(ok, one_view, None, 0, None) == -1
    assert lib.rg_filter(sino, _img(4096, 7, 6), 1, None, 0, None) == -1
    assert lib.rg_filter(sino, sino, 99, None, 0, None) == -1


def _align256(n):
    return (n + 255) // 256 * 256


def test_workspace_queries_are_host_arithmetic(lib):
    img = _img(4096, 256, 256)
    sino = _img(8192, 256, 180, (0.0, 1.0), (math.pi, -1.0))
    n = lib.rg_radon_slantstack_workspace(img, sino)
    assert n >= 2 * 256 * 258 * 8 + 256 * 180 * 4
    assert lib.rg_em_workspace(sino, img, 2, 10) > lib.rg_em_workspace(sino, img, 2, 1)
    vm = _native.RG_IMAGE(8192, 256, 256, 180, 1, 0.0, 1.0, math.pi, -1.0)   # view-major
    # a view-major sinogram needs no transposed copy, only the paired
    # gathers' quads: 16 bytes per (view pair, entry), 90 pairs x 257 entries
    assert lib.rg_backprojection_slantstack_workspace(vm, img) == _align256(90 * 257 * 16)
    vm_odd = _native.RG_IMAGE(8192, 256, 256, 179, 1, 0.0, 1.0, math.pi, -1.0)
    assert lib.rg_backprojection_slantstack_workspace(vm_odd, img) == 0


def test_workspaces_hold_the_paired_gathers_quads(lib):
    """Every query whose call can run the TMA-staged paired gathers reserves
    their sample quads: 16 bytes per (view pair, entry), R + 1 entries, per
    slice, in 256-byte-aligned pieces after the call's other scratch."""
    R, A, n, S = 256, 180, 256, 4
    img = _img(4096, n, n)
    sino = _img(8192, R, A, (0.0, 1.0), (math.pi, -1.0))             # ray-major
    vm = _native.RG_IMAGE(8192, R, R, A, 1, 0.0, 1.0, math.pi, -1.0)   # view-major
    al = _align256
    quads = (A // 2) * (R + 1) * 16
    sino_b = R * A * 4
    assert lib.rg_backprojection_slantstack_workspace(sino, img) == al(sino_b) + al(quads)
    assert lib.rg_radon_transpose_slantstack_workspace(vm, img) == al(quads)
    assert lib.rg_radon_transpose_slantstack_stack_workspace(vm, img, S) == al(S * quads)
    assert (lib.rg_radon_transpose_slantstack_stack_workspace(sino, img, S) ==
            al(S * sino_b) + al(S * quads))
    assert lib.rg_fbp_workspace(sino, img, 1) == 2 * al(sino_b) + al(quads)
    # EM: the quads of the largest subset (ceil(A / nsubsets) views)
    em1, em10 = lib.rg_em_workspace(sino, img, 2, 1), lib.rg_em_workspace(sino, img, 2, 10)
    # (the subsets also carry one sensitivity image each: 9 more for 10)
    assert em1 - em10 == al(quads) - al((18 // 2) * (R + 1) * 16) - 9 * al(n * n * 4)


def test_unaligned_workspace_rejected(lib):
    img = _img(4096, 16, 16)
    sino = _img(8192, 16, 12, (0.0, 1.0), (math.pi, -1.0))
    assert lib.rg_radon_slantstack(img, sino, ctypes.c_void_p(4096 + 8), 1 << 20, None) == -1
    assert b"aligned" in lib.rg_last_error()
