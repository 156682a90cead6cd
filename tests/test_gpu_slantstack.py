"""Slant-stack Radon, backprojection, matched adjoint and FBP filter on the
GPU (through the C ABI, via the public API) against the FP64 oracle and the
golden fixtures made from the reference.

Tolerance (FP32 kernels vs FP64 oracle): rel-L2 <= 1e-5 for Radon,
backprojection and adjoint; dot-product test <= 1e-6.  Random images have a
zero border and random sinograms zero first/last rays: at exact grid ties
(e.g. the ray t = 1 at view 0 sampling column N-1 exactly at the validity
limit) the reference's decision depends on its FP64 rounding, ours on
exact fixed-point arithmetic, so ties are kept where they contribute 0.
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
SINO_C = ((0.0, 1.0), (math.pi, -1.0))


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def interior_image(rng, n):
    x = rng.random((n, n))
    x[0, :] = x[-1, :] = x[:, 0] = x[:, -1] = 0.0
    return x


def inner_sino(rng, r, a):
    s = rng.random((r, a))
    s[0, :] = s[-1, :] = 0.0
    return s


def sino_img(s, tl=SINO_C[0], br=SINO_C[1]):
    return rg.image(np.asarray(s, np.float64), top_left=tl, bottom_right=br)


# ---------------------------------------------------------------- Radon
def test_radon_config1_golden(orc, golden):
    g = golden("config1")
    ph = np.flipud(g["phantom"]).copy()          # slant-stack rows are bottom-up
    out = rg.radon(rg.image(ph), (256, 256), SLANT)
    ref = orc.radon_slantstack(ph, 256, 256)
    assert rel(out, ref) <= 1e-5
    # the golden config-1 arrays are the reference's own outputs on the
    # top-down raster; check ours on that raster too
    out2 = rg.radon(rg.image(g["phantom"]), (256, 256), SLANT)
    assert rel(out2, g["radon"]) <= 1e-5


@pytest.mark.parametrize("n,r,a", [(17, 23, 9), (64, 64, 48), (100, 100, 90), (256, 256, 180),
                                   (33, 20, 31), (128, 181, 64)])
def test_radon_random_vs_oracle(orc, n, r, a):
    rng = np.random.default_rng(n * 1000 + a)
    x = interior_image(rng, n)
    out = rg.radon(rg.image(x), (r, a), SLANT)
    assert out.top_left == (0.0, 1.0) and out.bottom_right == (math.pi, -1.0)
    assert rel(out, orc.radon_slantstack(x, r, a)) <= 1e-5


def test_radon_odd_corners_golden(orc, golden):
    g = golden("odd")
    ic, sc = tuple(g["img_corners"]), tuple(g["sino_corners"])
    img = rg.image(g["img"], top_left=ic[:2], bottom_right=ic[2:])
    out = rg.radon(img, (23, 9), SLANT, top_left=sc[:2], bottom_right=sc[2:])
    # random 17x17 image with a nonzero border: compare to the oracle on the
    # same corners; ties at the validity limit do not occur for these corners
    assert rel(out, g["radon_ss"]) <= 1e-5


def test_radon_device_layouts(orc):
    """gpu_image inputs stay on the device; strided and view-major outputs."""
    rng = np.random.default_rng(7)
    n, r, a = 96, 96, 70
    x = interior_image(rng, n)
    ref = orc.radon_slantstack(x, r, a)
    gx = rg.image(x).cuda()
    out = rg.radon(gx, (r, a), SLANT)
    assert isinstance(out, rg.gpu_image)
    assert rel(out.numpy(), ref) <= 1e-5
    # transposed (column-major) input view
    xt = torch.from_numpy(np.ascontiguousarray(x.T, dtype=np.float32)).cuda().t()
    out2 = rg.radon(rg.gpu_image(xt), (r, a), SLANT)
    assert rel(out2.numpy(), ref) <= 1e-5


# ---------------------------------------------------------------- backprojection
def test_backprojection_config1_golden(orc, golden):
    g = golden("config1")
    s = sino_img(g["radon"])
    plan = rg.backprojection_plan((256, 256), (256, 256), 0, SLANT)
    bp = rg.backprojection(s, plan)
    assert rel(bp, g["bp"]) <= 1e-5


@pytest.mark.parametrize("n,r,a", [(17, 23, 9), (64, 64, 48), (255, 256, 180), (40, 80, 33)])
def test_backprojection_random_vs_oracle(orc, n, r, a):
    rng = np.random.default_rng(n + 7 * a)
    s = inner_sino(rng, r, a)
    bp = rg.backprojection(sino_img(s), (SLANT, (n, n), 0))
    assert rel(bp, orc.backprojection_slantstack(s, n)) <= 1e-5


def test_backprojection_golden_odd(golden):
    g = golden("odd")
    ic, sc = tuple(g["img_corners"]), tuple(g["sino_corners"])
    bp = rg.backprojection(sino_img(g["sino_in"], sc[:2], sc[2:]), (SLANT, (17, 17), 0),
                           top_left=ic[:2], bottom_right=ic[2:])
    assert rel(bp, g["bp_ss"]) <= 1e-5


def test_backprojection_gpu_wrapper(orc):
    rng = np.random.default_rng(3)
    s = inner_sino(rng, 128, 90)
    out = rg.backprojection_gpu(s, (128, 128))
    assert rel(out, orc.backprojection_slantstack(s, 128)) <= 1e-5


# ---------------------------------------------------------------- matched adjoint
@pytest.mark.parametrize("n,r,a,full", [(17, 17, 9, True), (64, 64, 48, False),
                                        (256, 256, 180, False), (70, 50, 37, True)])
def test_adjoint_vs_oracle_transpose(orc, n, r, a, full):
    """full: every ray nonzero, so the position-0 / N-1 validity rules of the
    border tiles are exercised.  The one exact grid tie of these geometries
    (view 0, last ray: t = 1 lands on x = 1 exactly, where the oracle's FP64
    rounding of -1 + (R-1)*dt decides validity) is zeroed."""
    rng = np.random.default_rng(n * 3 + a)
    s = rng.random((r, a)) if full else inner_sino(rng, r, a)
    s[-1, 0] = 0.0
    out = rg.radon_transpose(sino_img(s), (n, n), SLANT)
    assert rel(out, orc.radon_slantstack_transpose(s, n)) <= 1e-5


def test_adjoint_dot_product():
    rng = np.random.default_rng(11)
    n, r, a = 128, 128, 100
    x = torch.from_numpy(rng.random((n, n), dtype=np.float32)).cuda()
    y = torch.from_numpy(rng.random((r, a), dtype=np.float32)).cuda()
    from pyraft_gb300 import autograd as AG
    rx = AG.radon_forward(x, r, a).double()
    aty = AG.radon_adjoint(y, n).double()
    lhs = float((rx * y.double()).sum())
    rhs = float((x.double() * aty).sum())
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs)


def test_autograd_backward_is_adjoint():
    from pyraft_gb300 import autograd as AG
    rng = np.random.default_rng(5)
    x = torch.from_numpy(rng.random((2, 48, 48), dtype=np.float32)).cuda().requires_grad_()
    g = torch.from_numpy(rng.random((2, 48, 40), dtype=np.float32)).cuda()
    y = AG.radon(x, 48, 40)
    y.backward(g)
    ref = AG.radon_adjoint(g, 48)
    assert torch.allclose(x.grad, ref, rtol=1e-6, atol=1e-6)


# ---------------------------------------------------------------- filters / FBP
def test_ramlak_vs_oracle(orc):
    rng = np.random.default_rng(2)
    s = rng.random((200, 37))
    out = rg.ramlak(sino_img(s))
    dt = 2.0 / 199
    ref = orc.ramlak(s, dt)
    assert rel(out, ref) <= 1e-5


def _ramlak_cases(R):
    rng = np.random.default_rng(R)
    t = np.linspace(-1.0, 1.0, R)
    smooth = [2.0 * np.sqrt(np.maximum(0.25 - t * t, 0.0)), np.exp(-20.0 * t * t), 5.0 + t]
    rough = [rng.random(R), rng.poisson(50.0, R) / 50.0]
    s = np.stack(smooth + rough, axis=1).astype(np.float32).astype(np.float64)
    return s, len(smooth)


def _filter(orc, kind, s):
    R = s.shape[0]
    if kind == "ramlak":
        return (np.asarray(rg.ramlak(sino_img(s)), np.float64), orc.ramlak(s, 2.0 / (R - 1)))
    return (np.asarray(rg.lowpassino_fbp(sino_img(s)), np.float64), orc.lowpassino_fbp(s))


@pytest.mark.parametrize("kind,R", [("ramlak", R) for R in (2, 3, 5, 64, 200, 1025, 2048, 4096,
                                                              4097, 8192)] +
                         [("lowpass", R) for R in (4, 8, 64, 256, 2048, 4096, 8192)])
def test_filter_fft_vs_oracle(orc, kind, R):
    """The FFT filter kernel against the FP64 filters (the Ram-Lak
    convolution; pyraft's lowpassino_fbp by numpy FFT): Ram-Lak up to 8192
    rays, the lowpass filter (a circular convolution of length R) for R a
    power of two.  Smooth profiles are the hard case for an FFT filter (a
    ramp filter removes most of their norm), rough ones the easy case.  The
    oracle gets the FP32 inputs the kernel sees, so the bound measures the
    kernel alone.  Two views share one complex transform, so a view's error
    also carries a rounding-level share of its partner's norm: the bound
    adds 1e-7 of the largest view.  The lowpass bound is 5e-6: its circular
    difference carries the jump between a profile's two ends (2e-6 for
    5 + t at 8192 rays)."""
    s, _ = _ramlak_cases(R)
    out, ref = _filter(orc, kind, s)
    tol = 2e-6 if kind == "ramlak" else 5e-6
    big = max(np.linalg.norm(ref[:, c]) for c in range(s.shape[1]))
    for c in range(s.shape[1]):
        err = np.linalg.norm(out[:, c] - ref[:, c])
        assert err <= tol * np.linalg.norm(ref[:, c]) + 1e-7 * big, (c, err)


@pytest.mark.parametrize("kind,R", [("ramlak", 3), ("ramlak", 200), ("ramlak", 2048),
                                    ("ramlak", 4097), ("lowpass", 3), ("lowpass", 200),
                                    ("lowpass", 1025), ("lowpass", 2048)])
def test_filter_direct_vs_oracle(orc, monkeypatch, kind, R):
    """The direct-sum filter kernels (RG_FILTER_KERNEL=direct; the default
    above 8192 rays, and for the lowpass filter when R is not a power of
    two).  They sum the taps' products directly, so on smooth profiles
    their FP32 cancellation error grows with R (Ram-Lak: 1.4e-4 relative at
    4097 rays); on rough ones it stays at the 1e-7 level."""
    monkeypatch.setenv("RG_FILTER_KERNEL", "direct")
    s, ns = _ramlak_cases(R)
    out, ref = _filter(orc, kind, s)
    for c in range(s.shape[1]):
        bound = 3e-4 if c < ns else 2e-6
        assert rel(out[:, c], ref[:, c]) <= bound, (c, rel(out[:, c], ref[:, c]))


@pytest.mark.parametrize("path", ["fft", "direct"])
def test_lowpass_vs_numpy_fft(orc, monkeypatch, path):
    if path == "direct":
        monkeypatch.setenv("RG_FILTER_KERNEL", "direct")
    rng = np.random.default_rng(4)
    for R in (64, 257):
        s = rng.random((R, 21))
        out = rg.lowpassino_fbp(sino_img(s))
        assert rel(out, orc.lowpassino_fbp(s)) <= 1e-5


@pytest.mark.parametrize("path", ["fft", "direct"])
def test_lowpass_vs_reference_fixture(golden, monkeypatch, path):
    """pyraft's filter on the GPU against the reference's own lowpassino_fbp
    (pyraft/filters/filters.py:13-68, run from its source into
    tests/golden/lowpass.npz), including shifted sinogram corners.  Ray
    counts that are powers of two take the FFT kernel, the others the
    direct one (both with RG_FILTER_KERNEL=direct)."""
    if path == "direct":
        monkeypatch.setenv("RG_FILTER_KERNEL", "direct")
    g = golden("lowpass")
    for k in range(int(g["count"])):
        s, c, want = g[f"sino{k}"], g[f"corners{k}"], g[f"out{k}"]
        out = rg.lowpassino_fbp(sino_img(s, (c[0], c[1]), (c[2], c[3])))
        assert rel(out, want) <= 1e-5, k


def test_fbp_disk_density(orc):
    """Ram-Lak FBP recovers the density of a uniform disk.  pyraft's
    lowpassino_fbp filter is reproduced as is: its frequency grid
    linspace(-wc, wc, R) has no zero bin, so after fftshift the DC gain is
    wc/(R-1) = 1/(2 dt (R-1)) = 0.25 and the disk comes out ~20% high; it is
    checked against the oracle (numpy FFT filter + FP64 backprojection)."""
    n, nv = 256, 360
    desc = np.array([[1.0, 0.5, 0.5, 0.0, 0.0, 0.0]])
    sino = np.flipud(orc.radon_fromdesc(n, nv + 1, desc)[:, :nv]).copy()
    rec = rg.fbp(sino_img(sino), filter="ramlak")
    c = np.asarray(rec)[n // 2 - 20:n // 2 + 20, n // 2 - 20:n // 2 + 20]
    assert abs(c.mean() - 1.0) < 0.02, c.mean()
    q = orc.ramlak(sino, 2.0 / (n - 1))
    assert rel(rec, orc.backprojection_slantstack(q, n)) <= 1e-5
    rec = rg.fbp(sino_img(sino), filter="lowpass")
    ref = orc.backprojection_slantstack(orc.lowpassino_fbp(sino), n)
    assert rel(rec, ref) <= 1e-5
    out = rg.fbp_gpu(sino, n)
    assert out.dtype == np.float32 and rel(out, ref) <= 1e-5


# ---------------------------------------------------------------- errors
def test_errors_raise():
    with pytest.raises(rg.RaftError):
        rg.radon(rg.image(np.zeros((8, 9))), (8, 8), SLANT)   # not square
    with pytest.raises(TypeError):
        rg.radon(rg.image(np.zeros((8, 8))), (8, 8), rg.radon_method.BST)


# ---------------------------------------------------------------- cluster view split
@pytest.mark.parametrize("split", [2, 4])
def test_gather_cluster_split(orc, monkeypatch, split):
    """RG_GATHER_SPLIT forces the thread-block-cluster view split of the
    gathers (views divided over the CTAs of a cluster, partial sums reduced in
    distributed shared memory).  Backprojection, adjoint and the fused EM
    update must match the oracle as the unsplit launches do, and the split
    result must agree with the unsplit one to FP32 rounding."""
    rng = np.random.default_rng(40 + split)
    n, r, a = 200, 200, 300
    s = inner_sino(rng, r, a)
    monkeypatch.setenv("RG_GATHER_SPLIT", "1")
    bp1 = np.asarray(rg.backprojection(sino_img(s), (SLANT, (n, n), 0)))
    adj1 = np.asarray(rg.radon_transpose(sino_img(s), (n, n), SLANT))
    monkeypatch.setenv("RG_GATHER_SPLIT", str(split))
    bp = np.asarray(rg.backprojection(sino_img(s), (SLANT, (n, n), 0)))
    adj = np.asarray(rg.radon_transpose(sino_img(s), (n, n), SLANT))
    assert rel(bp, orc.backprojection_slantstack(s, n)) <= 1e-5
    assert rel(adj, orc.radon_slantstack_transpose(s, n)) <= 1e-5
    assert rel(bp, bp1) <= 1e-6 and rel(adj, adj1) <= 1e-6
    # EM: the adjoint with the fused multiplicative update
    x = interior_image(rng, n) + 0.1
    y = orc.radon_slantstack(x, r, a)
    em_split = np.asarray(rg.em(sino_img(y), (n, n), 3, method=SLANT))
    monkeypatch.setenv("RG_GATHER_SPLIT", "1")
    em_one = np.asarray(rg.em(sino_img(y), (n, n), 3, method=SLANT))
    assert rel(em_split, em_one) <= 1e-5


# ---------------------------------------------------------------- paired views
@pytest.mark.parametrize("n,r,a", [(64, 64, 48), (255, 256, 180), (97, 90, 64), (96, 120, 40)])
@pytest.mark.parametrize("rows,split", [("4", "1"), ("8", "2"), ("16", "1"), ("16", "4")])
def test_gathers_quarter_turn_pairs(orc, monkeypatch, n, r, a, rows, split):
    """The backprojection and the matched adjoint with views paired a quarter
    turn apart (an even number of views over [0, pi) on the symmetric
    default grid) against the one-view kernels (RG_GATHER_ROT=0) and the
    oracle, for each tile height and cluster split.  The adjoint's sinogram
    has every ray nonzero except the one exact grid tie (see
    test_adjoint_vs_oracle_transpose), so its edge pixels are exercised."""
    rng = np.random.default_rng(n + 3 * a)
    s = inner_sino(rng, r, a)
    sf = rng.random((r, a))
    sf[-1, 0] = 0.0
    monkeypatch.setenv("RG_GATHER_ROWS", rows)
    monkeypatch.setenv("RG_GATHER_SPLIT", split)
    adjoint = r <= n                             # the two-tap adjoint's condition
    paired = np.asarray(rg.backprojection(sino_img(s), (SLANT, (n, n), 0)))
    if adjoint:
        adj = np.asarray(rg.radon_transpose(sino_img(sf), (n, n), SLANT))
    monkeypatch.setenv("RG_GATHER_ROT", "0")
    single = np.asarray(rg.backprojection(sino_img(s), (SLANT, (n, n), 0)))
    assert rel(paired, orc.backprojection_slantstack(s, n)) <= 1e-5
    assert rel(paired, single) <= 1e-6
    if adjoint:
        adj1 = np.asarray(rg.radon_transpose(sino_img(sf), (n, n), SLANT))
        assert rel(adj, orc.radon_slantstack_transpose(sf, n)) <= 1e-5
        assert rel(adj, adj1) <= 1e-6


@pytest.mark.parametrize("n,r,a", [(64, 64, 48), (255, 256, 180), (130, 300, 64), (96, 120, 40)])
@pytest.mark.parametrize("rows,split", [("4", "1"), ("8", "2"), ("16", "4")])
def test_gathers_quarter_turn_tma_vs_staged(orc, monkeypatch, n, r, a, rows, split):
    """The paired gathers with their windows loaded by TMA from the quad
    prepass (RG_GATHER_ROT_TMA=1: any number of view pairs) against the same
    gathers staging the windows with loads (RG_GATHER_ROT_TMA=0) and the
    oracle.  At (130, 300) the 16-row windows are wider than a TMA box and
    that launch stages with loads; the 4- and 8-row ones take TMA."""
    rng = np.random.default_rng(5 * n + a)
    s = inner_sino(rng, r, a)
    sf = rng.random((r, a))
    sf[-1, 0] = 0.0
    monkeypatch.setenv("RG_GATHER_ROWS", rows)
    monkeypatch.setenv("RG_GATHER_SPLIT", split)
    monkeypatch.setenv("RG_GATHER_ROT_TMA", "1")
    adjoint = r <= n
    bp = np.asarray(rg.backprojection(sino_img(s), (SLANT, (n, n), 0)))
    if adjoint:
        adj = np.asarray(rg.radon_transpose(sino_img(sf), (n, n), SLANT))
    monkeypatch.setenv("RG_GATHER_ROT_TMA", "0")
    bp1 = np.asarray(rg.backprojection(sino_img(s), (SLANT, (n, n), 0)))
    assert rel(bp, orc.backprojection_slantstack(s, n)) <= 1e-5
    assert rel(bp, bp1) <= 1e-6
    if adjoint:
        adj1 = np.asarray(rg.radon_transpose(sino_img(sf), (n, n), SLANT))
        assert rel(adj, orc.radon_slantstack_transpose(sf, n)) <= 1e-5
        assert rel(adj, adj1) <= 1e-6


@pytest.mark.parametrize("a,tma", [(120, "1"), (600, None)])
def test_em_and_fbp_quarter_turn_tma_vs_staged(orc, monkeypatch, a, tma):
    """EM with the matched adjoint and with the backprojection, OSEM (6
    subsets: the count divides A / 2, so each subset pairs), all through
    rg_em's quad scratch, and the FBP through rg_fbp's, against the same
    calls with the windows staged by loads.  With 600 views the full-plan
    calls (300 view pairs) take TMA by default; the OSEM subsets (50 pairs)
    stage by loads either way."""
    rng = np.random.default_rng(77)
    n, r = 128, 128
    x = interior_image(rng, n) + 0.1
    y = orc.radon_slantstack(x, r, a)
    out = {}
    for mode in (tma, "0"):
        if mode is None:
            monkeypatch.delenv("RG_GATHER_ROT_TMA", raising=False)
        else:
            monkeypatch.setenv("RG_GATHER_ROT_TMA", mode)
        out[mode] = (np.asarray(rg.em(sino_img(y), (n, n), 4, method=SLANT)),
                     np.asarray(rg.em(sino_img(y), (n, n), 4, method=SLANT, reference=True)),
                     np.asarray(rg.osem(sino_img(y), (n, n), 2, nblocks=6, method=SLANT)),
                     np.asarray(rg.fbp(sino_img(y), filter="ramlak")))
    for got, ref in zip(out[tma], out["0"]):
        assert rel(got, ref) <= 1e-5


def test_paired_gathers_overwrite_the_output(orc, monkeypatch):
    """The paired gathers add two partial sums per pixel onto an output that
    the call zeroes first (for the TMA-staged backprojection, inside the quad
    prepass): an output buffer full of NaN must come back equal to the oracle,
    with the windows staged by TMA and by loads."""
    from pyraft_gb300.raftypes import rg_image
    rng = np.random.default_rng(21)
    n, r, a = 96, 96, 600                       # 300 view pairs: TMA by default
    s = inner_sino(rng, r, a)
    s[-1, 0] = 0.0                              # the adjoint's one exact grid tie
    L = _native.load()
    st = torch.cuda.current_stream().cuda_stream
    s_dev = torch.from_numpy(s.astype(np.float32)).cuda()   # rg_image keeps only its pointer
    S = rg_image(rg.gpu_image(s_dev, *SINO_C))
    cases = ((L.rg_backprojection_slantstack, orc.backprojection_slantstack(s, n)),
             (L.rg_radon_transpose_slantstack, orc.radon_slantstack_transpose(s, n)))
    for tma in ("1", "0"):
        monkeypatch.setenv("RG_GATHER_ROT_TMA", tma)
        for fn, ref in cases:
            out = torch.full((n, n), float("nan"), device="cuda")
            _native.check(fn(S, rg_image(rg.gpu_image(out)), None, 0, st))
            torch.cuda.synchronize()
            assert rel(out.cpu().numpy(), ref) <= 1e-5


@pytest.mark.parametrize("n,r,a,view_major", [(128, 128, 600, False), (96, 96, 720, True),
                                              (160, 120, 512, False), (64, 64, 300, False)])
def test_fbp_filter_writes_the_quads(orc, monkeypatch, n, r, a, view_major):
    """rg_fbp with the TMA-staged paired backprojection (>= 256 view pairs):
    the FFT filter writes the gather's quads and zeroes the image in its own
    epilogue, so the filtered rows are never stored and the gather's prepass
    does not run.  RG_FBP_QUADS=0 keeps the filter's rows and the prepass.
    The two agree to FP32 rounding (1e-6: the fused filter transforms each
    view together with its partner a quarter turn on, not with its
    neighbour, and a complex transform's rounding mixes its two real rows),
    into an output full of NaN, from a ray-major and a view-major sinogram,
    and both match the oracle's Ram-Lak backprojection inside the image's
    border (1e-5)."""
    from pyraft_gb300.raftypes import rg_image
    rng = np.random.default_rng(n + r + a)
    s = inner_sino(rng, r, a)
    L = _native.load()
    st = torch.cuda.current_stream().cuda_stream
    s_dev = torch.from_numpy(s.astype(np.float32)).cuda()
    if view_major:
        s_dev = s_dev.t().contiguous().t()        # columns (views) contiguous
    S = rg_image(rg.gpu_image(s_dev, *SINO_C))
    out = {}
    for fuse in ("1", "0"):
        monkeypatch.setenv("RG_FBP_QUADS", fuse)
        img = torch.full((n, n), float("nan"), device="cuda")
        _native.check(L.rg_fbp(S, rg_image(rg.gpu_image(img)), _native.RG_FILTER_RAMLAK,
                               None, 0, st))
        torch.cuda.synchronize()
        out[fuse] = img.cpu().numpy()
    assert L.rg_device_status() == 0
    assert np.isfinite(out["1"]).all()
    assert rel(out["1"], out["0"]) <= 1e-6
    # the filtered sinogram's first and last rays are not zero: the image's
    # border pixels meet them exactly at the detector's validity limit, where
    # the oracle's FP64 rounding decides, so the border is left out
    want = orc.backprojection_slantstack(orc.ramlak(s, 2.0 / (r - 1)), n)[1:-1, 1:-1]
    assert rel(out["1"][1:-1, 1:-1], want) <= 1e-5
    assert rel(out["0"][1:-1, 1:-1], want) <= 1e-5


@pytest.mark.parametrize("n,a", [(1000, 600), (777, 520)])
def test_backprojection_half_tile_tail(orc, monkeypatch, n, a):
    """The TMA-staged paired backprojection of one slice without a cluster
    split runs its last (tiles mod SMs) tiles as half tiles, two CTAs each,
    each summing the rows of four of the tile's eight warps.  Every pixel
    still gets exactly two partial sums (its tile's and its quarter-turned
    tile's), so the result must be the same bits as with whole tiles only
    (RG_GATHER_HALF_TILES=0), and match the oracle.  On 152 SMs: 1000^2 is
    512 tiles of 32 x 64 pixels, 56 of them in halves; 777^2 is 25 x 13 =
    325 tiles (partial ones at the right and bottom), 21 in halves."""
    rng = np.random.default_rng(n + a)
    s = inner_sino(rng, n, a)
    monkeypatch.setenv("RG_GATHER_ROWS", "8")
    monkeypatch.setenv("RG_GATHER_SPLIT", "1")
    outs = {}
    for ht in ("1", "0"):
        monkeypatch.setenv("RG_GATHER_HALF_TILES", ht)
        outs[ht] = np.asarray(rg.backprojection(sino_img(s), (SLANT, (n, n), 0)))
    assert _native.load().rg_device_status() == 0
    assert np.array_equal(outs["1"], outs["0"])
    assert rel(outs["1"], orc.backprojection_slantstack(s, n)) <= 1e-5


@pytest.mark.parametrize("n,r,a", [(2, 2, 2), (5, 5, 4), (17, 17, 10), (33, 20, 30), (40, 40, 2)])
def test_gathers_quarter_turn_small_geometries(orc, monkeypatch, n, r, a):
    """Paired gathers on images much smaller than a tile, and with a single
    view pair, against the one-view kernels and the oracle.  The views start
    1e-3 rad past 0 (the span stays pi, so they still pair): at exact
    multiples of 45 degrees these tiny grids put many samples exactly on the
    validity limits, where the oracle's FP64 rounding decides."""
    rng = np.random.default_rng(n * 7 + a)
    s = rng.random((r, a))
    tl, br = (1e-3, 1.0), (math.pi + 1e-3, -1.0)
    sc = tl + br
    monkeypatch.setenv("RG_GATHER_ROT", "1")
    bp = np.asarray(rg.backprojection(sino_img(s, tl, br), (SLANT, (n, n), 0)))
    adj = np.asarray(rg.radon_transpose(sino_img(s, tl, br), (n, n), SLANT))
    monkeypatch.setenv("RG_GATHER_ROT", "0")
    bp1 = np.asarray(rg.backprojection(sino_img(s, tl, br), (SLANT, (n, n), 0)))
    adj1 = np.asarray(rg.radon_transpose(sino_img(s, tl, br), (n, n), SLANT))
    assert rel(bp, bp1) <= 1e-6 and rel(adj, adj1) <= 1e-6
    assert rel(bp, orc.backprojection_slantstack(s, n, sino_corners=sc)) <= 1e-5
    assert rel(adj, orc.radon_slantstack_transpose(s, n, sino_corners=sc)) <= 1e-5


def test_backprojection_quarter_turn_not_applicable(orc):
    """Odd view counts, spans other than pi and off-centre grids keep the
    one-view kernel; results match the oracle either way."""
    rng = np.random.default_rng(77)
    s = inner_sino(rng, 64, 41)
    assert rel(rg.backprojection(sino_img(s), (SLANT, (64, 64), 0)),
               orc.backprojection_slantstack(s, 64)) <= 1e-5
    s = inner_sino(rng, 64, 40)
    tl, br = (0.0, 1.0), (0.75 * math.pi, -1.0)
    bp = rg.backprojection(sino_img(s, tl, br), (SLANT, (64, 64), 0))
    assert rel(bp, orc.backprojection_slantstack(s, 64, sino_corners=tl + br)) <= 1e-5
    ic = ((-1.0, 0.8), (0.8, -1.0))
    bp = rg.backprojection(sino_img(s), (SLANT, (64, 64), 0), top_left=ic[0], bottom_right=ic[1])
    ref = orc.backprojection_slantstack(s, 64, img_corners=ic[0] + ic[1])
    assert rel(bp, ref) <= 1e-5


# ---------------------------------------------------------------- TMA-staged Radon
@pytest.mark.parametrize("n,r,a", [(64, 64, 48), (255, 256, 180), (200, 300, 90), (512, 512, 360)])
def test_radon_tma_vs_direct_and_oracle(orc, monkeypatch, n, r, a):
    """The TMA-staged Radon (blocks of adjacent views, line windows streamed
    into shared memory) against the direct kernel and the oracle; no window
    check or bounded wait may have fired."""
    rng = np.random.default_rng(n + r + a)
    x = interior_image(rng, n)
    L = _native.load()
    assert L.rg_device_status() == 0
    staged = np.asarray(rg.radon(rg.image(x), (r, a), SLANT))
    monkeypatch.setenv("RG_RADON_KERNEL", "direct")
    direct = np.asarray(rg.radon(rg.image(x), (r, a), SLANT))
    assert L.rg_device_status() == 0
    assert rel(staged, orc.radon_slantstack(x, r, a)) <= 1e-5
    assert rel(staged, direct) <= 1e-6


def test_radon_tma_odd_corners_stack_and_em(orc, golden):
    """Staged Radon with off-centre corners (golden), through a stack launch
    and inside EM (ratio epilogue)."""
    g = golden("odd")
    ic, sc = tuple(g["img_corners"]), tuple(g["sino_corners"])
    img = rg.image(g["img"], top_left=ic[:2], bottom_right=ic[2:])
    out = rg.radon(img, g["radon_ss"].shape, SLANT, top_left=sc[:2], bottom_right=sc[2:])
    assert rel(out, g["radon_ss"]) <= 1e-5
    from pyraft_gb300 import autograd as AG
    rng = np.random.default_rng(5)
    xs = torch.from_numpy(rng.random((3, 96, 96), dtype=np.float32)).cuda()
    ys = AG.radon_forward(xs, 96, 120)
    for i in range(3):
        ref = orc.radon_slantstack(xs[i].double().cpu().numpy(), 96, 120)
        assert rel(ys[i].double().cpu().numpy(), ref) <= 1e-5
    assert _native.load().rg_device_status() == 0


@pytest.mark.parametrize("split", [2, 4])
def test_direct_radon_cluster_line_split(orc, monkeypatch, split):
    """The direct Radon with its lines split over a thread-block cluster
    (partials added in distributed shared memory by rank 0), forced on a
    plain geometry and inside OSEM (ratio epilogue, interleaved subsets)."""
    monkeypatch.setenv("RG_RADON_KERNEL", "direct")
    monkeypatch.setenv("RG_RADON_VIEWS", "1")
    monkeypatch.setenv("RG_RADON_SPLIT", str(split))
    rng = np.random.default_rng(70 + split)
    n, r, a = 150, 150, 70
    x = interior_image(rng, n)
    out = np.asarray(rg.radon(rg.image(x), (r, a), SLANT))
    assert rel(out, orc.radon_slantstack(x, r, a)) <= 1e-5
    y = orc.radon_slantstack(x + 0.1, r, a)
    got = np.asarray(rg.osem(sino_img(y), (n, n), 3, 5))
    monkeypatch.setenv("RG_RADON_SPLIT", "1")
    one = np.asarray(rg.osem(sino_img(y), (n, n), 3, 5))
    assert rel(got, one) <= 1e-5
    assert _native.load().rg_device_status() == 0


@pytest.mark.parametrize("n,r,a", [(64, 64, 48), (255, 256, 180), (200, 300, 90)])
def test_radon_tiles_forced_vs_oracle(orc, monkeypatch, n, r, a):
    """The tile-driven Radon (image tiles staged once by TMA, every view's
    crossing rays summed through them, partials added atomically) forced on
    plain geometries, against the oracle; no in-kernel check may fire."""
    monkeypatch.setenv("RG_RADON_KERNEL", "tiles")
    rng = np.random.default_rng(3 * n + a)
    x = interior_image(rng, n)
    out = np.asarray(rg.radon(rg.image(x), (r, a), SLANT))
    assert rel(out, orc.radon_slantstack(x, r, a)) <= 1e-5
    assert _native.load().rg_device_status() == 0


def test_osem_tiles_path_vs_oracle(orc):
    """OSEM whose subsets hold enough scattered views for the tile-driven
    Radon (48 views each), against the FP64 interleaved-subset oracle."""
    n, r, a, S = 96, 96, 192, 4
    rng = np.random.default_rng(17)
    x = interior_image(rng, n) + 0.05
    y = orc.radon_slantstack(x, r, a)

    def fsub(v, idx):
        return orc.radon_slantstack(v, r, a)[:, idx]

    def asub(t, idx):
        full = np.zeros((r, a))
        full[:, idx] = t
        return orc.radon_slantstack_transpose(full, n)
    ref = orc.osem_interleaved(y, np.ones((n, n)), fsub, asub, S, 4)
    out = np.asarray(rg.osem(sino_img(y), (n, n), 4, S))
    assert rel(out, ref) <= 1e-4
    assert _native.load().rg_device_status() == 0


@pytest.mark.parametrize("n,r,a", [(256, 256, 181), (128, 100, 45), (64, 64, 37)])
@pytest.mark.parametrize("rows,split", [("4", "1"), ("8", "2"), ("16", "4"), ("16", "1")])
def test_adjoint_half_turn_mirrored_tiles(orc, monkeypatch, n, r, a, rows, split):
    """The matched adjoint on tile pairs related by a half turn (pixel (r, c)
    and (N-1-r, N-1-c) share one position per view; odd view counts, so no
    quarter-turn pairs) against the tile-by-tile one-view kernel
    (RG_GATHER_MIRROR=0) and the oracle transpose, for each tile height and
    cluster split.  Tile heights whose pairs do not tile N take the one-view
    kernel either way.  The sinogram has every ray nonzero except the exact
    grid tie at view 0, so the edge pixels are exercised."""
    rng = np.random.default_rng(7 * n + a)
    sf = rng.random((r, a))
    sf[-1, 0] = 0.0
    monkeypatch.setenv("RG_GATHER_ROWS", rows)
    monkeypatch.setenv("RG_GATHER_SPLIT", split)
    out = np.asarray(rg.radon_transpose(sino_img(sf), (n, n), SLANT))
    monkeypatch.setenv("RG_GATHER_MIRROR", "0")
    one = np.asarray(rg.radon_transpose(sino_img(sf), (n, n), SLANT))
    assert _native.load().rg_device_status() == 0
    assert rel(out, one) <= 1e-6
    assert rel(out, orc.radon_slantstack_transpose(sf, n)) <= 1e-5


def test_em_osem_on_mirrored_tiles(orc, monkeypatch):
    """OSEM whose subsets do not pair a quarter turn apart (4 subsets of 60
    views) and EM with an odd view count take the mirrored adjoint with the
    update in its epilogue; both match the tile-by-tile kernels
    (RG_GATHER_MIRROR=0) to FP32 rounding and the OSEM the FP64 oracle."""
    n, r, a, S = 64, 64, 60, 4
    rng = np.random.default_rng(91)
    x = orc.phantom_fromdesc((n, n), np.abs(rg.random_ellipses(6, rng)) * [1, .8, .8, .8, .8, 1])
    y = orc.radon_slantstack(np.flipud(x).copy(), r, a)
    y61 = orc.radon_slantstack(np.flipud(x).copy(), r, 61)
    s, s61 = sino_img(y), sino_img(y61)
    got = [np.asarray(rg.osem(s, (n, n), 3, S)), np.asarray(rg.em(s61, (n, n), 3, method=SLANT))]
    monkeypatch.setenv("RG_GATHER_MIRROR", "0")
    ref = [np.asarray(rg.osem(s, (n, n), 3, S)), np.asarray(rg.em(s61, (n, n), 3, method=SLANT))]
    for g, q in zip(got, ref):
        assert rel(g, q) <= 1e-5

    def fsub(v, idx):
        return orc.radon_slantstack(v, r, a)[:, idx]

    def asub(t, idx):
        full = np.zeros((r, a))
        full[:, idx] = t
        return orc.radon_slantstack_transpose(full, n)
    want = orc.osem_interleaved(y, np.ones((n, n)), fsub, asub, S, 3)
    assert rel(got[0], want) <= 1e-4


@pytest.mark.parametrize("n,a", [(256, 360), (128, 200), (512, 90)])
def test_radon_tma_strip_split(orc, monkeypatch, n, a):
    """The TMA-staged Radon with its strips split over a cluster of 2 or 4
    CTAs (the partials meet in distributed shared memory, rank 0 writes the
    epilogue) against the unsplit launch (1e-6: the ranks' compensated
    partials are added in rank order) and the oracle (1e-5); also through
    EM, whose Radon carries the ratio epilogue."""
    rng = np.random.default_rng(3 * n + a)
    x = interior_image(rng, n)
    outs = {}
    for sp in ("1", "2", "4"):
        monkeypatch.setenv("RG_RADON_SPLIT_TMA", sp)
        outs[sp] = np.asarray(rg.radon(rg.image(x), (n, a), SLANT))
    assert _native.load().rg_device_status() == 0
    ref = orc.radon_slantstack(x, n, a)
    for sp in ("2", "4"):
        assert rel(outs[sp], outs["1"]) <= 1e-6
    assert rel(outs["4"], ref) <= 1e-5
    y = np.maximum(ref, 0.0) + 0.1
    em = {}
    for sp in ("1", "4"):
        monkeypatch.setenv("RG_RADON_SPLIT_TMA", sp)
        em[sp] = np.asarray(rg.em(sino_img(y), (n, n), 3, method=SLANT))
    assert rel(em["4"], em["1"]) <= 1e-5


def test_backprojection_many_rays_per_pixel(orc):
    """Four rays per pixel spacing (1024 rays over a 256^2 image): the
    16-row tiles' windows (about 640 samples) exceed what the gathers stage,
    so the first call's autotuner must skip that tile height and pick one
    that fits, and the result must still match the oracle."""
    rng = np.random.default_rng(41)
    n, r, a = 256, 1024, 90
    s = inner_sino(rng, r, a)
    plan = rg.backprojection_plan((r, a), (n, n), 0, SLANT)
    out = rg.backprojection(sino_img(s), plan)
    assert rel(out, orc.backprojection_slantstack(s, n)) <= 1e-5
    assert _native.load().rg_device_status() == 0
