"""Batched uneven OSEM (persistent launches, CUDA graph) and the plain
one-slice-per-call form.

The batched path runs the same tile code as the one-slice path, so per slice
it must agree with rg_em (OSEM) to FP32 rounding (1e-5: the tile-driven
Radon adds its partial ray sums atomically, in an order that differs
between runs and between the two paths, and the gather tiles may differ in
height); against the FP64 oracle it is held to rel-L2 1e-4.  The plain form uses float positions and no
compensated sums, so it is held to 1e-3."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import pyraft_gb300 as rg  # noqa: E402

SINO_C = dict(top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def emission(orc, n, r, a, seed):
    rng = np.random.default_rng(seed)
    desc = rg.random_ellipses(6, rng)
    desc[:, 1:3] *= 0.8
    x = np.abs(np.flipud(orc.phantom_fromdesc((n, n), desc)))
    y = orc.radon_slantstack(x, r, a)
    return rng.poisson(np.maximum(y, 0) * 50.0 / max(y.mean(), 1e-9)).astype(np.float64)


@pytest.fixture(scope="module")
def slices(orc):
    geo = [(96, 96, 60), (33, 33, 25), (64, 64, 41), (128, 128, 90), (50, 50, 30)]
    return geo, [emission(orc, n, r, a, 10 + k) for k, (n, r, a) in enumerate(geo)]


@pytest.mark.parametrize("graph", [True, False])
def test_batch_matches_per_slice_osem(slices, graph):
    geo, ys = slices
    S, it = 5, 3
    sinos = [rg.image(y, **SINO_C) for y in ys]
    out = rg.osem_batch(sinos, [(n, n) for n, _, _ in geo], it, S, graph=graph)
    for (n, r, a), s, o in zip(geo, sinos, out):
        ref = rg.osem(s, (n, n), it, S)
        assert o.shape == (n, n)
        assert rel(o, ref) <= 1e-5


def test_batch_vs_oracle(orc, slices):
    geo, ys = slices
    n, r, a = geo[2]
    S, it = 4, 3

    def fsub(x, idx):
        return orc.radon_slantstack(x, r, a)[:, idx]

    def asub(s, idx):
        full = np.zeros((r, a))
        full[:, idx] = s
        return orc.radon_slantstack_transpose(full, n)
    ref = orc.osem_interleaved(ys[2], np.ones((n, n)), fsub, asub, S, it)
    out = rg.osem_batch([rg.image(y, **SINO_C) for y in ys], None, it, S)
    assert rel(out[2], ref) <= 1e-4


def test_batch_device_inputs_and_start_images(slices):
    geo, ys = slices
    sinos = [rg.image(y, **SINO_C).cuda() for y in ys[:2]]
    x0 = [rg.image(np.full((n, n), 2.0)).cuda() for n, _, _ in geo[:2]]
    out = rg.osem_batch(sinos, None, 2, 3, x0=x0)
    assert all(isinstance(o, rg.gpu_image) for o in out)
    ref = rg.osem(rg.image(ys[1], **SINO_C), rg.image(np.full((33, 33), 2.0)), 2, 3)
    assert rel(out[1].numpy(), ref) <= 1e-6


def test_plain_form_vs_oracle(orc, slices):
    geo, ys = slices
    n, r, a = geo[3]
    fwd = lambda x: orc.radon_slantstack(x, r, a)
    adj = lambda s: orc.radon_slantstack_transpose(s, n)
    ref = orc.em_guarded(ys[3], np.ones((n, n)), fwd, adj, 4)
    out = rg.em_plain(ys[3], n, 4, 1)
    assert rel(out, ref) <= 1e-3
    out5 = rg.em_plain(ys[3], n, 2, 5)
    ref5 = rg.osem(rg.image(ys[3], **SINO_C), (n, n), 2, 5)
    assert rel(out5, ref5) <= 1e-3


def test_batch_rejects_bad_arguments(slices):
    geo, ys = slices
    with pytest.raises(rg.RaftError):
        rg.osem_batch([rg.image(ys[1], **SINO_C)], None, 1, 26)   # more subsets than views
    with pytest.raises(rg.RaftError):
        rg.osem_batch([rg.image(ys[1], **SINO_C)], None, 1, 2, x0=[rg.image(np.ones((33, 32)))])


def test_batch_mirrored_tile_pairs(orc, monkeypatch):
    """Slices on the default, centred geometry whose tiles pair with their
    half-turn mirrors (N a multiple of the pair tiling) take the mirrored
    adjoint (one position and one 128-bit load serve pixel (r, c) and
    (N-1-r, N-1-c) of the same view, the EM update in the epilogue).  Each
    slice matches the tile-by-tile adjoint of RG_BATCH_MIRROR=0 and the
    one-slice OSEM to rel-L2 1e-5 (FP32 atomic ray sums in the Radon), with
    odd and even view counts and 3 subsets."""
    geo = [(256, 256, 181), (128, 128, 90), (512, 512, 300), (96, 96, 61)]
    ys = [emission(orc, n, r, a, 60 + k) for k, (n, r, a) in enumerate(geo)]
    sinos = [rg.image(y, **SINO_C) for y in ys]
    S, it = 3, 2
    out = rg.osem_batch(sinos, None, it, S)
    monkeypatch.setenv("RG_BATCH_MIRROR", "0")
    ref = rg.osem_batch(sinos, None, it, S)
    monkeypatch.delenv("RG_BATCH_MIRROR")
    for (n, r, a), s, o, q in zip(geo, sinos, out, ref):
        assert rel(o, q) <= 1e-5, (n, a)
        assert rel(o, rg.osem(s, (n, n), it, S)) <= 1e-5, (n, a)


def test_batch_mirror_sparse_rays_and_off_centre_grid(orc):
    """The mirrored adjoint with fewer rays than pixels (R < N, centred
    geometry), beside a slice whose image grid is off centre (its start
    image carries shifted corners), which must keep the tile-by-tile
    adjoint: each matches the one-slice OSEM from the same start image."""
    n, S, it = 256, 4, 2
    geo = [(200, 150), (256, 121)]
    ys = [emission(orc, n, r, a, 70 + k) for k, (r, a) in enumerate(geo)]
    sinos = [rg.image(y, **SINO_C) for y in ys]
    x0 = [rg.image(np.ones((n, n))),
          rg.image(np.ones((n, n)), top_left=(-1.0, 0.9), bottom_right=(1.0, -1.1))]
    out = rg.osem_batch(sinos, None, it, S, x0=x0)
    for s, o, x in zip(sinos, out, x0):
        assert rel(o, rg.osem(s, x, it, S)) <= 1e-5
