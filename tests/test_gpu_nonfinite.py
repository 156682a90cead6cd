"""Non-finite inputs: a NaN sample poisons exactly the outputs whose
interpolation stencil reads it, as in the reference's FP64 loops, and
nothing else; the call still returns RG_OK with a clear device status.

The reference validates nothing and propagates NaN through its lerps
(raft/raft_radon_slantstack.c:174-211, raft/raft_backprojection_slantstack.c:163-178):
an output is NaN when one of the two samples of any of its interpolations
is NaN, even at weight 0.  The line pairs (s - d, d) and sample quads read
the same two samples per interpolation, so the set of NaN outputs must equal
the FP64 oracle's, and the finite outputs must still match it to 1e-5.  The
view grid starts at 0.013 rad so that no view is axis-aligned (positions
then never sit on an exact sample, where the oracle's FP64 floor and the
kernels' fixed-point floor could pick neighbouring stencils).  An infinite
sample comes back as NaN rather than +-Inf: the pair form subtracts it from
itself (d - d); the reference would give +-Inf.
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

SLANT = rg.radon_method.SLANTSTACK
T0 = 0.013
SINO_KW = dict(top_left=(T0, 1.0), bottom_right=(T0 + math.pi, -1.0))
IMG_C = (-1.0, 1.0, 1.0, -1.0)
SINO_C = (T0, 1.0, T0 + math.pi, -1.0)


def _check(got, ref):
    got = np.asarray(got, np.float64)
    bad = ~np.isfinite(ref)
    assert bad.any() and not bad.all()
    assert np.array_equal(np.isnan(got), bad)
    ok = ~bad
    err = np.linalg.norm(got[ok] - ref[ok]) / np.linalg.norm(ref[ok])
    assert err <= 1e-5, err
    assert _native.load().rg_device_status() == 0


@pytest.mark.parametrize("n,a", [(256, 360), (96, 40)])      # TMA-staged / direct Radon
def test_nan_pixels_poison_the_oracles_rays(orc, n, a):
    x = np.random.default_rng(11).random((n, n))
    x[0, :] = x[-1, :] = x[:, 0] = x[:, -1] = 0.0
    x[n // 3, n // 5] = x[2 * n // 3, n // 2 + 7] = np.nan
    got = rg.radon(rg.image(x), (n, a), SLANT, **SINO_KW)
    _check(got, orc.radon_slantstack(x, n, a, IMG_C, SINO_C))


@pytest.mark.parametrize("n,a", [(128, 600), (64, 60)])      # TMA-staged pairs / staged by loads
def test_nan_samples_poison_the_oracles_pixels(orc, n, a):
    s = np.random.default_rng(12).random((n, a))
    s[0, :] = s[-1, :] = 0.0
    s[n // 2 + 3, a // 7] = s[n // 4, a // 2 + 1] = np.nan
    plan = rg.backprojection_plan((n, a), (n, n), 0, SLANT)
    got = rg.backprojection(rg.image(s, **SINO_KW), plan)
    _check(got, orc.backprojection_slantstack(s, n, IMG_C, SINO_C))


def test_infinite_pixel_gives_nan_not_inf(orc):
    n, a = 96, 40
    x = np.random.default_rng(13).random((n, n))
    x[n // 2, n // 3] = np.inf
    got = np.asarray(rg.radon(rg.image(x), (n, a), SLANT, **SINO_KW))
    ref = orc.radon_slantstack(x, n, a, IMG_C, SINO_C)
    assert np.array_equal(~np.isfinite(got), ~np.isfinite(ref))
    assert np.isnan(got[~np.isfinite(ref)]).all()
