"""Differentiable path: the autograd Radon / adjoint pair, FP64 gradcheck,
stack launches, TV-regularised least squares and unrolled EM with
checkpointing.

Tolerances: dot-product test <= 1e-6 (FP32); FP64 pair vs the FP64 oracle
rel-L2 <= 1e-8 (fixed-point sample positions); torch.autograd.gradcheck in
float64 at 64 x 64 with its default tolerances."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import pyraft_gb300 as rg  # noqa: E402
from pyraft_gb300 import autograd as AG  # noqa: E402
from pyraft_gb300 import recon  # noqa: E402


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_fp64_pair_vs_oracle(orc):
    rng = np.random.default_rng(1)
    x = rng.random((64, 64))
    x[0, :] = x[-1, :] = x[:, 0] = x[:, -1] = 0
    y = rng.random((64, 48))
    y[0, :] = y[-1, :] = 0
    fx = AG.radon_forward(torch.from_numpy(x).cuda(), 64, 48).cpu().numpy()
    assert rel(fx, orc.radon_slantstack(x, 64, 48)) <= 1e-8
    ay = AG.radon_adjoint(torch.from_numpy(y).cuda(), 64).cpu().numpy()
    assert rel(ay, orc.radon_slantstack_transpose(y, 64)) <= 1e-8


def test_gradcheck_fp64_64x64():
    rng = np.random.default_rng(2)
    x = torch.from_numpy(rng.random((64, 64))).cuda().requires_grad_()
    # the FP64 transpose scatters with atomics: allow 1e-12 run-to-run noise
    assert torch.autograd.gradcheck(lambda v: AG.radon(v, 64, 48), (x,), fast_mode=True,
                                    nondet_tol=1e-12)
    s = torch.from_numpy(rng.random((64, 48))).cuda().requires_grad_()
    assert torch.autograd.gradcheck(lambda v: AG.adjoint(v, 64), (s,), fast_mode=True,
                                    nondet_tol=1e-12)


def test_stack_equals_single_and_dot_product():
    rng = np.random.default_rng(3)
    B, n, r, a = 3, 96, 96, 80
    x = torch.from_numpy(rng.random((B, n, n), dtype=np.float32)).cuda()
    y = torch.from_numpy(rng.random((B, r, a), dtype=np.float32)).cuda()
    rx = AG.radon_forward(x, r, a)
    aty = AG.radon_adjoint(y, n)
    for b in range(B):
        one = rg.radon(rg.gpu_image(x[b].contiguous()), (r, a), rg.radon_method.SLANTSTACK)
        assert torch.equal(rx[b], one.data)
        onet = rg.radon_transpose(rg.gpu_image(y[b].contiguous(), (0.0, 1.0), (math.pi, -1.0)),
                                  (n, n), rg.radon_method.SLANTSTACK)
        assert torch.equal(aty[b], onet.data)
    lhs = float((rx.double() * y.double()).sum())
    rhs = float((x.double() * aty.double()).sum())
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs)


def test_tv_ls_reduces_error(orc):
    B, n, nv = 4, 96, 60
    rng = np.random.default_rng(4)
    xs = []
    for b in range(B):
        desc = rg.random_ellipses(8, rng)
        xs.append(np.flipud(orc.phantom_fromdesc((n, n), desc)).copy())
    x_true = torch.from_numpy(np.stack(xs).astype(np.float32)).cuda()
    y = AG.radon_forward(x_true, n, nv)
    y = y + 0.01 * float(y.max()) * torch.randn_like(y)
    x, losses = recon.tv_ls(y, n, niter=150, lam=1e-3, lr=2e-2)
    assert losses[-1] < 0.05 * losses[0]
    err = float(torch.linalg.norm(x - x_true) / torch.linalg.norm(x_true))
    assert err < 0.35, err


def test_unrolled_em_matches_library_em(orc):
    n, r, a = 64, 64, 60
    rng = np.random.default_rng(5)
    desc = np.abs(rg.random_ellipses(6, rng))
    desc[:, 1:3] *= 0.8
    xt = np.abs(np.flipud(orc.phantom_fromdesc((n, n), desc)))
    y = orc.radon_slantstack(xt, r, a) * 20.0
    yt = torch.from_numpy(y.astype(np.float32)).cuda()
    with torch.no_grad():
        x = recon.unrolled_em(yt, n, niter=20, checkpoint_every=5)
    ref = rg.em(rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0)), (n, n), 20,
                method=rg.radon_method.SLANTSTACK)
    assert rel(x.cpu().numpy(), ref) <= 1e-4


def test_unrolled_em_gradients_fp64_and_checkpointing():
    rng = np.random.default_rng(6)
    y = torch.from_numpy(rng.random((16, 10)) + 0.5).cuda().requires_grad_()

    def f(v):
        return recon.unrolled_em(v, 16, niter=3, checkpoint_every=2).sum()
    assert torch.autograd.gradcheck(lambda v: recon.unrolled_em(v, 16, niter=3,
                                                                checkpoint_every=2),
                                    (y,), fast_mode=True, nondet_tol=1e-10)
    g1, = torch.autograd.grad(f(y), y)
    g2, = torch.autograd.grad(recon.unrolled_em(y, 16, niter=3, checkpoint_every=0).sum(), y)
    assert torch.allclose(g1, g2, rtol=1e-10, atol=1e-10)


def test_fused_tv_matches_torch():
    """rg_tv (fused TV value and gradient) against the same TV written with
    PyTorch ops in FP64, on a stack with odd sizes."""
    from pyraft_gb300 import recon
    rng = np.random.default_rng(21)
    for n, b in ((37, 3), (64, 1)):
        x64 = torch.from_numpy(rng.random((b, n, n))).cuda().requires_grad_(True)
        ref = recon.total_variation_reference(x64, 1e-3)
        (gref,) = torch.autograd.grad(ref, x64)
        x32 = x64.detach().float().requires_grad_(True)
        val = recon.total_variation(x32, 1e-3)
        (g,) = torch.autograd.grad(val, x32)
        assert abs(float(val.detach()) - float(ref.detach())) <= 1e-5 * abs(float(ref.detach()))
        assert float((g.double() - gref).norm() / gref.norm()) <= 1e-5
