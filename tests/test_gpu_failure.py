"""Failure reporting of the TMA-staged kernels, without faulting the GPU.

Every mbarrier wait in k_radon_tma and k_gather_rot_tma is bounded: a wait
that runs out sets bit 2 of the device status word, waits (bounded) for the
CTA's copies still in flight and ends the CTA's loop; a view window wider
than the staged box is skipped with bit 1.  rg_device_status() returns and
clears the word.  The test switches make those paths run on purpose:
- RG_TEST_EXPIRE_WAIT=1: the first wait of every CTA gives up at once,
  while its copies are in flight (the drain waits keep their full limit);
- RG_TEST_WINDOW_CUT=1: the gather's host under-reports its window bound by
  one 8-entry step (the TMA box and the buffers shrink with it), so the
  widest windows no longer fit.
Each case checks the status bit, then that the next normal call on the same
context reports 0 and matches the FP64 oracle (rel-L2 1e-5).  The reference
has no error reporting at all (raft/raft_filter.cpp:131-133 returns
silently).
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
SINO_C = dict(top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0))


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _sino(n, a, seed):
    s = np.random.default_rng(seed).random((n, a))
    s[0, :] = s[-1, :] = 0.0
    return s


def _image(n, seed):
    x = np.random.default_rng(seed).random((n, n))
    x[0, :] = x[-1, :] = x[:, 0] = x[:, -1] = 0.0
    return x


@pytest.fixture
def lib():
    L = _native.load()
    assert L.rg_device_status() == 0
    return L


def test_backprojection_expired_wait_reports_bit_2(orc, lib, monkeypatch):
    n, a = 128, 600                 # 300 view pairs: the TMA-staged paired gather
    s = _sino(n, a, 1)
    plan = rg.backprojection_plan((n, a), (n, n), 0, SLANT)
    sino = rg.image(s, **SINO_C)
    monkeypatch.setenv("RG_TEST_EXPIRE_WAIT", "1")
    rg.backprojection(sino, plan)
    assert lib.rg_device_status() & 2
    monkeypatch.delenv("RG_TEST_EXPIRE_WAIT")
    out = rg.backprojection(sino, plan)
    assert lib.rg_device_status() == 0
    assert rel(out, orc.backprojection_slantstack(s, n)) <= 1e-5


def test_adjoint_expired_wait_reports_bit_2(orc, lib, monkeypatch):
    n, a = 128, 600
    s = _sino(n, a, 2)
    sino = rg.image(s, **SINO_C)
    monkeypatch.setenv("RG_TEST_EXPIRE_WAIT", "1")
    rg.radon_transpose(sino, (n, n), SLANT)
    assert lib.rg_device_status() & 2
    monkeypatch.delenv("RG_TEST_EXPIRE_WAIT")
    out = rg.radon_transpose(sino, (n, n), SLANT)
    assert lib.rg_device_status() == 0
    assert rel(out, orc.radon_slantstack_transpose(s, n)) <= 1e-5


def test_radon_expired_wait_reports_bit_2(orc, lib, monkeypatch):
    n, a = 256, 360                 # adjacent views: the TMA-staged Radon
    x = _image(n, 3)
    monkeypatch.setenv("RG_TEST_EXPIRE_WAIT", "1")
    rg.radon(rg.image(x), (n, a), SLANT)
    assert lib.rg_device_status() & 2
    monkeypatch.delenv("RG_TEST_EXPIRE_WAIT")
    out = rg.radon(rg.image(x), (n, a), SLANT)
    assert lib.rg_device_status() == 0
    assert rel(out, orc.radon_slantstack(x, n, a)) <= 1e-5


def test_window_too_narrow_reports_bit_1(orc, lib, monkeypatch):
    n, a = 128, 600
    s = _sino(n, a, 4)
    plan = rg.backprojection_plan((n, a), (n, n), 0, SLANT)
    sino = rg.image(s, **SINO_C)
    monkeypatch.setenv("RG_TEST_WINDOW_CUT", "1")
    rg.backprojection(sino, plan)
    st = lib.rg_device_status()
    assert st & 1 and not st & 2
    monkeypatch.delenv("RG_TEST_WINDOW_CUT")
    out = rg.backprojection(sino, plan)
    assert lib.rg_device_status() == 0
    assert rel(out, orc.backprojection_slantstack(s, n)) <= 1e-5


def test_failed_scratch_allocation_reports_enomem(orc, lib, monkeypatch):
    """A call given no workspace takes its scratch from the stream-ordered
    pool.  RG_TEST_FAIL_ALLOC=1 makes that allocation fail as an exhausted
    pool would: the call returns RG_ENOMEM with a message and writes nothing,
    and the next call on the same context allocates and matches the oracle."""
    from pyraft_gb300.raftypes import gpu_image, rg_image
    n, a = 96, 80
    x = _image(n, 5)
    d_x = torch.from_numpy(x.astype(np.float32)).cuda()
    out = torch.full((n, a), float("nan"), dtype=torch.float32, device="cuda")
    X = rg_image(gpu_image(d_x))
    S = rg_image(gpu_image(out, (0.0, 1.0), (math.pi, -1.0)))
    stream = torch.cuda.current_stream().cuda_stream
    monkeypatch.setenv("RG_TEST_FAIL_ALLOC", "1")
    assert lib.rg_radon_slantstack(X, S, None, 0, stream) == _native.RG_ENOMEM
    assert b"allocation" in lib.rg_last_error()
    img = torch.full((n, n), float("nan"), dtype=torch.float32, device="cuda")
    I = rg_image(gpu_image(img))
    assert lib.rg_fbp(S, I, _native.RG_FILTER_RAMLAK, None, 0, stream) == _native.RG_ENOMEM
    torch.cuda.synchronize()
    assert torch.isnan(out).all() and torch.isnan(img).all()
    monkeypatch.delenv("RG_TEST_FAIL_ALLOC")
    assert lib.rg_radon_slantstack(X, S, None, 0, stream) == _native.RG_OK
    torch.cuda.synchronize()
    assert lib.rg_device_status() == 0
    assert rel(out.cpu().numpy(), orc.radon_slantstack(x, n, a)) <= 1e-5
