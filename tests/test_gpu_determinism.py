"""Repeatability of the deterministic operators: the same call on the same
input gives the same bits every time.

The TMA-staged Radon sums each ray in a fixed order (its cluster ranks are
added in rank order), the paired gathers add exactly two partial sums onto a
zeroed pixel (two adds onto zero round the same in either order), the
mirrored adjoint sums every view of a pixel in one CTA, and the FFT filter
has no atomics, so these paths, the FBP built from them and a full-plan EM
run must repeat bit for bit.  Each case runs twice into outputs filled with
NaN first, at sizes that take the TMA-staged kernels (256 or more view
pairs, adjacent-view Radon blocks) and the cluster splits.  Not covered
here, because their atomic adds land in a varying order: the tile-driven
Radon of scattered views (OSEM subsets) and the batched OSEM; both are held
to 1e-5 elsewhere.  The reference has no such check; its C paths are
deterministic by construction (raft/raft_radon_slantstack.c:44-214).
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
from pyraft_gb300.raftypes import gpu_image, rg_image  # noqa: E402

SLANT = rg.radon_method.SLANTSTACK
SINO_C = ((0.0, 1.0), (math.pi, -1.0))


def _twice(call, shape, corners=None):
    """Run call(out) twice, each time into a fresh NaN-filled output."""
    outs = []
    for _ in range(2):
        out = torch.full(shape, float("nan"), dtype=torch.float32, device="cuda")
        og = gpu_image(out, *corners) if corners else gpu_image(out)
        _native.check(call(rg_image(og), torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        outs.append(out.cpu().numpy())
    assert _native.load().rg_device_status() == 0
    assert np.isfinite(outs[0]).all()
    return outs


def _sino(n, a, seed):
    """(tensor, rg_image): the caller keeps the tensor alive while the
    rg_image's raw pointer is in use."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    t = torch.rand((n, a), device="cuda", generator=g) - 0.25
    return t, rg_image(gpu_image(t, *SINO_C))


@pytest.mark.parametrize("n,a", [(256, 720), (512, 1800)])
def test_paired_backprojection_repeats_bit_for_bit(n, a):
    L, (s, S) = _native.load(), _sino(n, a, 1)
    o1, o2 = _twice(lambda o, st: L.rg_backprojection_slantstack(S, o, None, 0, st), (n, n))
    assert np.array_equal(o1, o2)


@pytest.mark.parametrize("n,a", [(256, 720), (256, 719)])   # quarter-turn pairs / mirrored
def test_matched_adjoint_repeats_bit_for_bit(n, a):
    L, (s, S) = _native.load(), _sino(n, a, 2)
    o1, o2 = _twice(lambda o, st: L.rg_radon_transpose_slantstack(S, o, None, 0, st), (n, n))
    assert np.array_equal(o1, o2)


@pytest.mark.parametrize("n,a", [(512, 360), (256, 720)])   # strips split over clusters
def test_tma_radon_repeats_bit_for_bit(n, a):
    L = _native.load()
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.rand((n, n), device="cuda", generator=g)
    X = rg_image(gpu_image(x))
    o1, o2 = _twice(lambda o, st: L.rg_radon_slantstack(X, o, None, 0, st), (n, a), SINO_C)
    assert np.array_equal(o1, o2)


def test_fbp_repeats_bit_for_bit():
    n, a = 512, 720
    L, (s, S) = _native.load(), _sino(n, a, 4)
    o1, o2 = _twice(lambda o, st: L.rg_fbp(S, o, _native.RG_FILTER_RAMLAK, None, 0, st), (n, n))
    assert np.array_equal(o1, o2)


def test_full_plan_em_repeats_bit_for_bit():
    n, a = 256, 720
    g = torch.Generator(device="cuda").manual_seed(5)
    y = gpu_image(torch.poisson(20.0 * torch.rand((n, a), device="cuda", generator=g)), *SINO_C)
    outs = [rg.em(y, (n, n), 6, method=SLANT).data.cpu().numpy() for _ in range(2)]
    assert _native.load().rg_device_status() == 0
    assert np.isfinite(outs[0]).all()
    assert np.array_equal(outs[0], outs[1])
