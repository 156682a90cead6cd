"""DDA traversal, DDA Radon and its transpose, and the ellipse phantoms on
the GPU.  Pixel index sequences must be bit-identical to the reference's
(golden dda.npz); sums are FP32 (rel-L2 <= 1e-6 vs the FP64 oracle)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import ctypes  # noqa: E402

import pyraft_gb300 as rg  # noqa: E402
from pyraft_gb300 import _native  # noqa: E402

BRES = rg.radon_method.BRESENHAM


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_dda_sequences_bit_identical(golden):
    g = golden("dda")
    lines, cols = map(int, g["shape"])
    rays = g["rays"]
    n, cap = len(rays), 4 * (lines + cols) + 8
    oi = torch.zeros(n * cap, dtype=torch.int32, device="cuda")
    oj = torch.zeros_like(oi)
    osg = torch.zeros(n * cap, dtype=torch.float64, device="cuda")
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    th = np.ascontiguousarray(rays[:, 0])
    ts = np.ascontiguousarray(rays[:, 1])
    corners = (ctypes.c_double * 4)(-1.0, 1.0, 1.0, -1.0)
    dp = ctypes.POINTER(ctypes.c_double)
    _native.check(_native.load().rg_dda_trace(
        lines, cols, corners, th.ctypes.data_as(dp), ts.ctypes.data_as(dp), n, cap,
        oi.data_ptr(), oj.data_ptr(), osg.data_ptr(), cnt.data_ptr(), None))
    oi, oj, osg, cnt = oi.cpu().numpy(), oj.cpu().numpy(), osg.cpu().numpy(), cnt.cpu().numpy()
    off = g["offsets"]
    for r in range(n):
        lo, hi = off[r], off[r + 1]
        assert cnt[r] == hi - lo, rays[r]
        assert np.array_equal(oi[r * cap:r * cap + cnt[r]], g["i"][lo:hi]), rays[r]
        assert np.array_equal(oj[r * cap:r * cap + cnt[r]], g["j"][lo:hi]), rays[r]
        s = osg[r * cap:r * cap + cnt[r]]
        if math.sin(rays[r][0]) != 0.0 and math.cos(rays[r][0]) != 0.0:
            assert np.array_equal(s, g["sigma"][lo:hi]), rays[r]
        else:
            assert np.array_equal(s[1:], g["sigma"][lo + 1:hi]), rays[r]


def test_radon_bresenham_golden_and_oracle(orc, golden):
    g = golden("sl64")
    out = rg.radon(rg.image(g["phantom"]), (64, 48), BRES)
    assert rel(np.asarray(out)[:, 1:], g["radon_bres"][:, 1:]) <= 1e-6
    assert rel(out, orc.radon_bresenham(g["phantom"], 64, 48)) <= 1e-6
    r = golden("rect")
    out = rg.radon(rg.image(r["img"]), (37, 29), BRES)
    assert rel(np.asarray(out)[:, 1:], r["radon_bres"][:, 1:]) <= 1e-6


def test_radon_transpose_bresenham(orc, golden):
    g = golden("sl64")
    s = rg.image(g["sino_in_bres"], top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    out = rg.radon_transpose(s, (64, 64), BRES)
    assert rel(out, g["radonT_bres"]) <= 1e-6
    o = golden("odd")
    ic, sc = tuple(o["img_corners"]), tuple(o["sino_corners"])
    s = rg.image(o["sino_in"], top_left=sc[:2], bottom_right=sc[2:])
    out = rg.radon_transpose(s, (17, 17), BRES, top_left=ic[:2], bottom_right=ic[2:])
    assert rel(out, o["radonT_bres"]) <= 1e-6


def test_bresenham_adjoint_identity():
    rng = np.random.default_rng(1)
    x = rng.random((40, 52))
    y = rng.random((45, 33))
    rx = rg.radon(rg.image(x), (45, 33), BRES)
    s = rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    aty = rg.radon_transpose(s, (40, 52), BRES)
    lhs, rhs = float((np.asarray(rx) * y).sum()), float((x * np.asarray(aty)).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_phantoms(orc, golden):
    g = golden("config1")
    ph = rg.shepplogan((256, 256))
    assert np.array_equal(np.asarray(ph, np.float32), g["phantom"].astype(np.float32))
    sl = golden("sl64")
    fd = rg.radon(orc.SHEPP_LOGAN, (64, 48))
    assert rel(fd, sl["fromdesc"]) <= 1e-6


@pytest.mark.parametrize("n,r,a,corners", [
    (1024, 1024, 720, None),
    (2048, 2048, 1800, None),
    (255, 301, 181, None),
    (200, 160, 97, ((0.3, 1.0), (0.3 + math.pi, -1.0))),
])
def test_integer_walk_equals_fp64_walk(monkeypatch, n, r, a, corners):
    """The DDA kernels make the walk's decisions in 64-bit integer arithmetic
    wherever it reproduces FP64 exactly (bresenham.cu, DDAInt), and keep the
    FP64 walk elsewhere.  The Radon of an image of distinct random values
    sums every ray's visited pixels times its FP32 sigma in a fixed order, so
    one pixel or sigma off in any ray would change that ray's sum: the
    integer walk's Radon must equal the FP64 walk's (RG_DDA_FP64=1) bit for
    bit, at the benchmark sizes and on odd, offset geometries."""
    g = torch.Generator(device="cuda").manual_seed(n + a)
    x = rg.gpu_image(torch.rand((n, n), device="cuda", generator=g) + 0.5)
    kw = dict(top_left=corners[0], bottom_right=corners[1]) if corners else {}
    outs = []
    for fp64 in ("1", "0"):
        monkeypatch.setenv("RG_DDA_FP64", fp64)
        outs.append(rg.radon(x, (r, a), BRES, **kw).data.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])
    assert np.isfinite(outs[1]).all() and outs[1].any()


def test_dda_em_integer_walk_matches_fp64_walk(monkeypatch):
    """The DDA EM records each ray's walk once (k_dda_plan) and replays it;
    with the recording made by the integer walk it agrees with the FP64
    walk's to FP32 rounding (the transpose replay adds with atomics)."""
    rng = np.random.default_rng(3)
    y = rng.poisson(30.0, size=(256, 180)).astype(np.float64)
    s = rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    outs = []
    for fp64 in ("1", "0"):
        monkeypatch.setenv("RG_DDA_FP64", fp64)
        outs.append(np.asarray(rg.em(s, (256, 256), 5, method=BRES)))
    assert rel(outs[1], outs[0]) <= 1e-6


def test_normalised_backprojection_integer_walk_matches_fp64_walk(monkeypatch):
    """The normalised DDA backprojection (sum of s sigma over sum of sigma,
    FP64 sums) takes the integer walk with FP64 sigma; its sums are FP64
    atomics in a varying order, so the two walks agree to FP64 rounding
    (one pixel off in any ray would show at the 1e-3 level)."""
    rng = np.random.default_rng(5)
    n, r, a = 512, 512, 360
    s = rg.image(rng.random((r, a)) + 0.5, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    plan = rg.backprojection_plan((r, a), (n, n), 0, BRES)
    outs = []
    for fp64 in ("1", "0"):
        monkeypatch.setenv("RG_DDA_FP64", fp64)
        outs.append(np.asarray(rg.backprojection(s, plan), np.float64))
    assert rel(outs[1], outs[0]) <= 1e-12
