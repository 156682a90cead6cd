"""Normalised DDA backprojection, transmission EM and the mesh Radon (with
3-D stacks) on the GPU, against the golden fixtures from the reference and
the FP64 oracle.  Tolerances: rel-L2 <= 1e-5 for the projectors (1e-6 for
the DDA backprojection, FP32 atomics), <= 1e-4 after 15 transmission-EM
iterations."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import pyraft_gb300 as rg  # noqa: E402

BRES = rg.radon_method.BRESENHAM


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_normalised_bresenham_backprojection(orc, golden):
    g = golden("bres_norm")
    sc, ic = tuple(g["sino_corners"]), tuple(g["img_corners"])
    s = rg.image(g["sino_in"], top_left=sc[:2], bottom_right=sc[2:])
    plan = rg.backprojection_plan(g["sino_in"].shape, (48, 48), 0, BRES)
    out = np.asarray(rg.backprojection(s, plan))
    ref = np.where(np.isfinite(g["bp"]), g["bp"], 0.0)
    assert rel(out, ref) <= 1e-6
    out = np.asarray(rg.backprojection(s, (BRES, (31, 37), 0), top_left=ic[:2],
                                       bottom_right=ic[2:]))
    ref = np.where(np.isfinite(g["bp_odd"]), g["bp_odd"], 0.0)
    assert rel(out, ref) <= 1e-6
    # default geometry, view 0 included (its first sigma is set, as in the oracle)
    rng = np.random.default_rng(3)
    y = rng.random((50, 40))
    out = rg.backprojection(rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0)),
                            (BRES, (44, 44), 0))
    assert rel(out, orc.backprojection_bresenham(y, (44, 44))) <= 1e-6


def test_transmission_em_vs_oracle(orc):
    n, r, a = 48, 48, 40
    rng = np.random.default_rng(7)
    desc = rg.random_ellipses(6, rng)
    mu = np.abs(np.flipud(orc.phantom_fromdesc((n, n), desc))) * 0.5
    p = orc.radon_slantstack(mu, r, a)
    flat = np.full((r, a), 1e4) + rng.normal(0, 10, (r, a))
    dark = np.full((r, a), 50.0)
    raw = rng.poisson(flat * np.exp(-p)).astype(np.float64) + dark
    fwd = lambda x: orc.radon_slantstack(x, r, a)
    adj = lambda s: orc.radon_slantstack_transpose(s, n)
    ref = orc.em_transmission(raw, flat, dark, np.ones((n, n)), fwd, adj, 15)
    out = rg.em_transmission_gpu(raw, flat, dark, n, 15)
    assert out.shape == (n, n) and rel(out, ref) <= 1e-4


def test_mesh_radon_golden(golden):
    g = golden("mesh")
    img = rg.image(g["img"])
    out = rg.radon_withmesh(img, g["theta"], g["t"])
    assert out.shape == g["radon"].shape and rel(out, g["radon"]) <= 1e-5
    ic = tuple(g["img_corners"])
    out = rg.radon_withmesh(rg.image(g["img"], top_left=ic[:2], bottom_right=ic[2:]),
                            g["theta"], g["t"])
    assert rel(out, g["radon_odd"]) <= 1e-5
    v = rg.radon_view(img, float(g["theta"][3]), g["t"])
    assert rel(v, g["radon"][:, 3]) <= 1e-5


def test_radon_3d_stack_and_snapshot(orc):
    rng = np.random.default_rng(9)
    n = 40
    f = rng.random((n, n, n))
    # slices f[:, i, :]: zero their borders (the uniform mesh below has exact
    # grid ties at theta = 0, pi and t = +-1)
    f[0, :, :] = f[-1, :, :] = f[:, :, 0] = f[:, :, -1] = 0.0
    theta = np.linspace(0, np.pi, 31)
    t = np.linspace(-1, 1, 45)
    S = rg.radon_3d_stack(f, theta, t)
    assert S.shape == (31, n, 45)
    for i in (0, 17, n - 1):
        ref = orc.radon_slantstack_withmesh(f[:, i, :], t, theta)
        assert rel(S[:, i, :], ref.T) <= 1e-5
    snap = rg.snapshot(f, 0.4, t)
    assert snap.shape == (n, 45)
    for k in (0, 23):
        ref = orc.radon_slantstack_withmesh(f[:, k, :], t, [0.4])[:, 0]
        assert rel(snap[k], ref) <= 1e-5
