"""Parity at the benchmarked sizes, through the C ABI and the public API.

- FBP (Ram-Lak + slant-stack backprojection) at 2048^2 x 1800 views x 2048
  rays, the bench's headline call rg_fbp, on a random-ellipse transmission
  sinogram with Poisson noise: 64 image rows spread over the whole image
  against the FP64 oracle (direct Ram-Lak convolution, then
  raft_backprojection_slantstack's pixel sum, raft/raft_backprojection_
  slantstack.c:121-180).  Tolerance rel-L2 <= 1e-5.
- EM with 720 views (360 view pairs: the TMA-staged paired adjoint and its
  update pass) against the FP64 oracle restatement of make_em
  (pyraft/iterative/em.py:109-144): 50 iterations at 512^2 and 5 at
  1024^2 x 720 (the EM bench slice).  Tolerance rel-L2 <= 1e-4.
- The DDA Radon, its transpose and the normalised DDA backprojection
  (pyraft's default method) at the benchmarked 2048^2 image and 2048 rays,
  on 60 views: full-length rays of 2048 to 2900 pixels summed in
  compensated FP32, against the FP64 oracle.  Tolerance rel-L2 <= 1e-6.
- The batched uneven OSEM with a 2048^2 x 1800 slice among smaller ones:
  every slice against the one-slice OSEM (rg_em) on the same subsets to
  rel-L2 <= 1e-5 (FP32 atomic ray sums in both), and the smallest slice
  against the FP64 oracle's interleaved OSEM to 1e-4.

The image's first and last rows and columns are left out of the FBP
comparison: there a sample position can fall exactly on the detector's
validity limit (t = +-1 at views 0 and A/2), where the reference's decision
follows its FP64 rounding and ours exact fixed-point arithmetic.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import pyraft_gb300 as rg  # noqa: E402
from pyraft_gb300 import _native  # noqa: E402
from pyraft_gb300.raftypes import rg_image  # noqa: E402

SLANT = rg.radon_method.SLANTSTACK
SINO_C = dict(top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def emission(n, a, seed, ellipses=12):
    """Poisson counts (mean 50 per bin) of a random-ellipse activity image,
    projected by the GPU Radon; returns float64 (rays, views)."""
    rng = np.random.default_rng(seed)
    desc = rg.random_ellipses(ellipses, rng)
    ph = rg.phantom_fromdesc((n, n), desc, device=True)
    ph = rg.gpu_image(torch.flip(ph.data, dims=[0]).abs().contiguous())
    p = rg.radon(ph, (n, a), SLANT).data.double().cpu().numpy()
    return rng.poisson(np.maximum(p, 0) * 50.0 / max(p.mean(), 1e-9)).astype(np.float64)


def test_fbp_2048x1800_sampled_rows_vs_oracle(orc, monkeypatch):
    N, A, R = 2048, 1800, 2048
    rng = np.random.default_rng(1234)
    desc = rg.random_ellipses(40, rng)
    ph = np.flipud(orc.phantom_fromdesc((N, N), desc)).copy()     # bottom-up rows
    p = np.asarray(rg.radon(rg.image(ph), (R, A), SLANT), np.float64)
    mu = 3.0 / p.max()
    counts = np.maximum(rng.poisson(1e4 * np.exp(-p * mu)), 1)
    sino = (-np.log(counts / 1e4)).astype(np.float32)

    L = _native.load()
    d_s = torch.from_numpy(sino).cuda()
    d_img = torch.full((N, N), float("nan"), dtype=torch.float32, device="cuda")
    S = rg_image(rg.gpu_image(d_s, **SINO_C))
    I = rg_image(rg.gpu_image(d_img))
    wsb = L.rg_fbp_workspace(S, I, _native.RG_FILTER_RAMLAK)
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    _native.check(L.rg_fbp(S, I, _native.RG_FILTER_RAMLAK, ws.data_ptr(), wsb, sp))
    torch.cuda.synchronize()
    assert L.rg_device_status() == 0
    got = d_img.double().cpu().numpy()
    assert np.isfinite(got).all()
    # the filter writing the gather's quads (the default) and the filter's
    # rows plus the gather's prepass (RG_FBP_QUADS=0) agree to FP32 rounding
    # (the fused filter transforms each view with its partner a quarter turn
    # on instead of its neighbour)
    monkeypatch.setenv("RG_FBP_QUADS", "0")
    d_img.fill_(float("nan"))
    _native.check(L.rg_fbp(S, I, _native.RG_FILTER_RAMLAK, ws.data_ptr(), wsb, sp))
    torch.cuda.synchronize()
    assert rel(d_img.double().cpu().numpy(), got) <= 1e-6

    q = orc.ramlak(sino.astype(np.float64), 2.0 / (R - 1))
    row0, step, count = 16, 32, 64
    ref = orc.backprojection_rowstep(q, N, row0, step, count)
    rows = got[row0:row0 + (count - 1) * step + 1:step]
    assert rel(rows[:, 1:-1], ref[:, 1:-1]) <= 1e-5


def _em_vs_oracle(orc, n, a, niter, seed):
    y = emission(n, a, seed)
    fwd = lambda x: orc.radon_slantstack(x, n, a)
    adj = lambda s: orc.radon_slantstack_transpose(s, n)
    ref = orc.em_guarded(y, np.ones((n, n)), fwd, adj, niter)
    out = rg.em(rg.image(y, **SINO_C), (n, n), niter, method=SLANT)
    torch.cuda.synchronize()
    assert _native.load().rg_device_status() == 0
    return rel(out, ref)


def test_em_512x720_50_iterations_vs_oracle(orc):
    assert _em_vs_oracle(orc, 512, 720, 50, 31) <= 1e-4


def test_em_1024x720_vs_oracle(orc):
    assert _em_vs_oracle(orc, 1024, 720, 5, 32) <= 1e-4


def test_dda_operators_2048_full_length_rays_vs_oracle(orc):
    """raft/raft_radon_bresenham.cpp:16-105, raft/raft_radon_transpose_
    bresenham.cpp:17-201 and raft/raft_backprojection_bresenham.cpp:17-251 at
    a 2048^2 image and 2048 rays over 60 views of [0, pi) (view 0 included,
    as the oracle restates it)."""
    N, R, A = 2048, 2048, 60
    BRES = rg.radon_method.BRESENHAM
    rng = np.random.default_rng(2048)
    x = rng.random((N, N))
    got = np.asarray(rg.radon(rg.image(x), (R, A), BRES))
    assert rel(got, orc.radon_bresenham(x, R, A)) <= 1e-6
    y = rng.random((R, A))
    s = rg.image(y, **SINO_C)
    got = np.asarray(rg.radon_transpose(s, (N, N), BRES))
    assert rel(got, orc.radon_transpose_bresenham(y, (N, N))) <= 1e-6
    got = np.asarray(rg.backprojection(s, (BRES, (N, N), 0)))
    want = orc.backprojection_bresenham(y, (N, N))
    assert rel(got, np.where(np.isfinite(want), want, 0.0)) <= 1e-6
    assert _native.load().rg_device_status() == 0


def test_batch_with_a_2048x1800_slice(orc):
    geo = [(2048, 1800), (256, 180), (512, 777), (1024, 1001)]
    ys = [emission(n, a, 40 + k) for k, (n, a) in enumerate(geo)]
    sinos = [rg.image(y, **SINO_C) for y in ys]
    S, it = 10, 2
    out = rg.osem_batch(sinos, None, it, S)
    torch.cuda.synchronize()
    assert _native.load().rg_device_status() == 0
    for (n, a), s, o in zip(geo, sinos, out):
        assert o.shape == (n, n)
        ref = rg.osem(s, (n, n), it, S)
        assert rel(o, ref) <= 1e-5, (n, a)
    # the smallest slice against the FP64 oracle's interleaved OSEM
    n, a = geo[1]

    def fsub(x, idx):
        return orc.radon_slantstack(x, n, a)[:, idx]

    def asub(r, idx):
        full = np.zeros((n, a))
        full[:, idx] = r
        return orc.radon_slantstack_transpose(full, n)
    ref = orc.osem_interleaved(ys[1], np.ones((n, n)), fsub, asub, S, it)
    assert rel(out[1], ref) <= 1e-4
