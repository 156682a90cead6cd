"""EM / OSEM on the GPU against the FP64 oracle restatement of pyraft's
make_em loop (pyraft/iterative/em.py:109-144) with the same division
guards.  Tolerance: rel-L2 <= 1e-4 after 50 iterations (slant-stack pair);
the DDA pair sums with FP32 atomics, held to 1e-4 after 20."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import pyraft_gb300 as rg  # noqa: E402

SLANT = rg.radon_method.SLANTSTACK
BRES = rg.radon_method.BRESENHAM


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _emission(orc, n, r, a, seed):
    rng = np.random.default_rng(seed)
    desc = rg.random_ellipses(8, rng)
    desc[:, 1:3] *= 0.8
    x = np.abs(np.flipud(orc.phantom_fromdesc((n, n), desc)))
    y = orc.radon_slantstack(x, r, a)
    y = rng.poisson(np.maximum(y, 0) * 50.0 / max(y.mean(), 1e-9)).astype(np.float64)
    return y


def test_em_slantstack_50_iterations(orc):
    n, r, a = 64, 64, 60
    y = _emission(orc, n, r, a, 1)
    fwd = lambda x: orc.radon_slantstack(x, r, a)
    adj = lambda s: orc.radon_slantstack_transpose(s, n)
    ref = orc.em_guarded(y, np.ones((n, n)), fwd, adj, 50)
    s = rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    out = rg.em(s, (n, n), 50, method=SLANT)
    assert rel(out, ref) <= 1e-4


def test_osem_interleaved_vs_oracle(orc):
    n, r, a, S = 64, 64, 60, 6
    y = _emission(orc, n, r, a, 2)

    def fsub(x, idx):
        return orc.radon_slantstack(x, r, a)[:, idx]

    def asub(s, idx):
        full = np.zeros((r, a))
        full[:, idx] = s
        return orc.radon_slantstack_transpose(full, n)
    ref = orc.osem_interleaved(y, np.ones((n, n)), fsub, asub, S, 5)
    s = rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    out = rg.osem(s, (n, n), 5, S)
    assert rel(out, ref) <= 1e-4


def test_em_dda_pair_vs_oracle(orc):
    n, r, a = 48, 48, 40
    rng = np.random.default_rng(9)
    x = orc.phantom_fromdesc((n, n), np.abs(rg.random_ellipses(6, rng)) * [1, .8, .8, .8, .8, 1])
    y = orc.radon_bresenham(x, r, a)
    fwd = lambda v: orc.radon_bresenham(v, r, a)
    adj = lambda s: orc.radon_transpose_bresenham(s, (n, n))
    ref = orc.em_guarded(y, np.ones((n, n)), fwd, adj, 20)
    s = rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    out = rg.em(s, (n, n), 20)          # pyraft's default method: the DDA pair
    assert rel(out, ref) <= 1e-4


def test_em_gpu_wrapper_and_make_em(orc):
    n, r, a = 32, 32, 30
    y = _emission(orc, n, r, a, 4)
    fwd = lambda x: orc.radon_slantstack(x, r, a)
    adj = lambda s: orc.radon_slantstack_transpose(s, n)
    bp = lambda s: orc.backprojection_slantstack(s, n)
    # em_gpu pairs the Radon with the backprojection, as raft_em_gpu does
    out = rg.em_gpu(y, n, 7)
    ref_bp = orc.em_guarded(y, np.ones((n, n)), fwd, bp, 7)
    assert out.dtype == np.float32 and rel(out, ref_bp) <= 1e-4
    ref = orc.em_guarded(y, np.ones((n, n)), fwd, adj, 7)
    s = rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    step = rg.make_em(s, (n, n), SLANT, SLANT)
    x = rg.image(np.ones((n, n)))
    for _ in range(7):
        x = step(x)
    assert rel(x, ref) <= 1e-4


def test_em_zero_data_is_guarded():
    s = rg.image(np.zeros((32, 30)), top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    out = rg.em(s, (32, 32), 3, method=SLANT)
    assert np.isfinite(np.asarray(out)).all() and np.abs(np.asarray(out)).max() == 0.0


def test_em_reference_backprojector_vs_oracle(orc):
    """reference=True: EM and OSEM with the slant-stack backprojection as the
    backprojector (the reference GPU EM's pairing), 30 iterations."""
    n, r, a = 64, 64, 60
    y = _emission(orc, n, r, a, 6)
    fwd = lambda x: orc.radon_slantstack(x, r, a)
    bp = lambda s: orc.backprojection_slantstack(s, n)
    ref = orc.em_guarded(y, np.ones((n, n)), fwd, bp, 30)
    s = rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    out = rg.em(s, (n, n), 30, method=SLANT, reference=True)
    assert rel(out, ref) <= 1e-4

    def fsub(x, idx):
        return orc.radon_slantstack(x, r, a)[:, idx]

    def bsub(t, idx):
        full = np.zeros((r, a))
        full[:, idx] = t
        return orc.backprojection_slantstack(full, n)
    ref_os = orc.osem_interleaved(y, np.ones((n, n)), fsub, bsub, 4, 5)
    out_os = rg.osem(s, (n, n), 5, 4, reference=True)
    assert rel(out_os, ref_os) <= 1e-4
    with pytest.raises(TypeError):
        rg.em(s, (n, n), 1, method=rg.radon_method.BRESENHAM, reference=True)


@pytest.mark.parametrize("S", [1, 3, 4, 5])
def test_em_quarter_turn_pairs_match_one_view_kernels(orc, monkeypatch, S):
    """EM and OSEM whose subsets pair up a quarter turn apart (S divides A/2
    = 30: S = 1, 3, 5) take the paired gathers with the update fused into
    their epilogue (N = 64 is a multiple of 32); S = 4 keeps the fused
    one-view gather.  Either way the result matches
    the one-view kernels (RG_GATHER_ROT=0) to FP32 rounding, for the matched
    adjoint and for the backprojection (reference=True)."""
    n, r, a = 64, 64, 60
    y = _emission(orc, n, r, a, 10 + S)
    s = rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    out = [rg.osem(s, (n, n), 4, S), rg.osem(s, (n, n), 4, S, reference=True)]
    monkeypatch.setenv("RG_GATHER_ROT", "0")
    ref = [rg.osem(s, (n, n), 4, S), rg.osem(s, (n, n), 4, S, reference=True)]
    for o, q in zip(out, ref):
        assert rel(o, q) <= 1e-5


@pytest.mark.parametrize("S", [1, 3])
def test_em_dda_recorded_walks_match_walking(orc, monkeypatch, S):
    """The DDA EM replays each subset's walks from a plan recorded once
    (same pixel sequences and sigmas as the walking kernels); with the plan
    off (RG_DDA_PLAN=0), or too big for its cap (RG_DDA_PLAN_MAX_GB=0), it
    walks every time.  All three agree to FP32 summation order."""
    n, r, a = 48, 48, 40
    rng = np.random.default_rng(20 + S)
    x = orc.phantom_fromdesc((n, n), np.abs(rg.random_ellipses(6, rng)) * [1, .8, .8, .8, .8, 1])
    y = orc.radon_bresenham(x, r, a)
    s = rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    planned = rg.osem(s, (n, n), 6, S, method=BRES)
    monkeypatch.setenv("RG_DDA_PLAN", "0")
    walked = rg.osem(s, (n, n), 6, S, method=BRES)
    monkeypatch.delenv("RG_DDA_PLAN")
    monkeypatch.setenv("RG_DDA_PLAN_MAX_GB", "0")
    capped = rg.osem(s, (n, n), 6, S, method=BRES)
    assert rel(planned, walked) <= 1e-5 and rel(capped, walked) <= 1e-6


@pytest.mark.parametrize("n,a,S,tma", [(128, 600, 1, None), (128, 600, 3, None),
                                       (96, 60, 1, "0"), (64, 60, 5, "0"), (64, 48, 3, "1"),
                                       (130, 64, 1, None)])
def test_em_fused_update_matches_separate_pass(orc, monkeypatch, n, a, S, tma):
    """The EM update fused into the paired gathers (the last CTA to add its
    partial sum to a 32 x 32 pixel block updates the block) against the
    same gathers writing their sums to scratch with the update as its own
    pass (RG_EM_UNFUSED=1): both compute x * (a + b) * inv from two
    partial sums added onto zero, so a full-plan EM agrees exactly; OSEM
    subsets take the tile-driven Radon, whose atomic ray sums round in a
    varying order, so they agree to 1e-5.  Checked for the matched adjoint
    and for the backprojection (reference=True), staged by TMA and by loads.
    N = 130 is not a multiple of 32 and keeps the separate pass."""
    if tma is not None:
        monkeypatch.setenv("RG_GATHER_ROT_TMA", tma)
    y = _emission(orc, n, n, a, 40 + S)
    s = rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    fused = [np.asarray(rg.osem(s, (n, n), 3, S)),
             np.asarray(rg.osem(s, (n, n), 3, S, reference=True))]
    monkeypatch.setenv("RG_EM_UNFUSED", "1")
    sep = [np.asarray(rg.osem(s, (n, n), 3, S)),
           np.asarray(rg.osem(s, (n, n), 3, S, reference=True))]
    for f, q in zip(fused, sep):
        assert rel(f, q) <= (1e-6 if S == 1 else 1e-5)


def test_em_checkpoint_resume_matches_uninterrupted_run(orc, tmp_path):
    """EM stopped after 4 of 6 sub-iterations (checkpoints every 2) and
    resumed in a second call reaches the iterate of one uninterrupted rg_em
    call bit for bit (the full-plan Radon and the paired gathers are
    deterministic); the state file records the progress."""
    import torch
    n, a = 128, 600
    y = _emission(orc, n, n, a, 50)
    s = rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    ref = np.asarray(rg.em(s, (n, n), 6, method=SLANT))
    ck = str(tmp_path / "em.pt")
    x1, st1 = rg.em_checkpointed(s, (n, n), 6, 1, checkpoint=ck, every=2, max_subiterations=4)
    assert st1["subiteration"] == 4 and not st1["done"]
    assert torch.load(ck, weights_only=True)["subiteration"] == 4
    x2, st2 = rg.em_checkpointed(s, (n, n), 6, 1, checkpoint=ck, every=2)
    assert st2["done"] and st2["subiteration"] == 6
    assert np.array_equal(np.asarray(x2), ref)


def test_osem_checkpoint_resume_mid_iteration(orc, tmp_path):
    """OSEM (5 subsets x 3 iterations) interrupted after 7 sub-iterations,
    i.e. inside an iteration, and resumed, against one uninterrupted call;
    a state saved for another sinogram is refused."""
    n, a, S = 64, 60, 5
    y = _emission(orc, n, n, a, 51)
    s = rg.image(y, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    ref = np.asarray(rg.osem(s, (n, n), 3, S))
    ck = str(tmp_path / "osem.pt")
    _, st = rg.em_checkpointed(s, (n, n), 3, S, checkpoint=ck, every=3, max_subiterations=7)
    assert st["subiteration"] == 7
    x, st = rg.em_checkpointed(s, (n, n), 3, S, checkpoint=ck, every=3)
    assert st["done"] and rel(x, ref) <= 1e-5
    other = rg.image(y * 1.5, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))
    with pytest.raises(ValueError):
        rg.em_checkpointed(other, (n, n), 3, S, checkpoint=ck)
