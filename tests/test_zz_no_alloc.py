"""The allocation-free Radon entry point, rg_radon_slantstack_noalloc.

It exists for callers that cannot allocate device memory: a process whose
device memory already belongs to another framework's pool, or an
acquisition loop that must not allocate once it runs (cudaMalloc and
cudaFree may synchronise the whole device).  Its scratch lives in a static
device array instead of a workspace or the stream-ordered pool.  This test
calls it through the C ABI twice in a row, on different inputs, and checks
each result against the regular entry point rg_radon_slantstack within the
rel-L2 1e-5 tolerance of the other Radon tests (both run the same kernels,
so they agree to the last bit in practice).  A leftover from the first call
would show up in the second.  It is collected last so that a failure here
cannot hide others.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

from pyraft_gb300 import _native  # noqa: E402
from pyraft_gb300 import build as B  # noqa: E402


def _rg(t, tl, br):
    return _native.RG_IMAGE(t.data_ptr(), t.shape[0], t.stride(1), t.shape[1], t.stride(0),
                            tl[0], tl[1], br[0], br[1])


def test_noalloc_radon_matches_regular_entry_point():
    B.build()
    lib = _native.load()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(2027)
    img_c = ((-1.0, 1.0), (1.0, -1.0))
    sino_c = ((0.0, 1.0), (math.pi, -1.0))
    for n, r, a in [(200, 200, 150), (257, 180, 97)]:      # two calls in a row
        x = rng.random((n, n)).astype(np.float32)
        x[0, :] = x[-1, :] = x[:, 0] = x[:, -1] = 0.0
        d_x = torch.from_numpy(x).cuda()
        want = torch.zeros((r, a), dtype=torch.float32, device="cuda")
        got = torch.full((r, a), float("nan"), dtype=torch.float32, device="cuda")
        rc = lib.rg_radon_slantstack(_rg(d_x, *img_c), _rg(want, *sino_c), None, 0, stream)
        _native.check(rc)
        rc = lib.rg_radon_slantstack_noalloc(_rg(d_x, *img_c), _rg(got, *sino_c), stream)
        _native.check(rc)
        torch.cuda.synchronize()
        g, w = got.double().cpu().numpy(), want.double().cpu().numpy()
        assert np.isfinite(g).all()
        assert np.linalg.norm(g - w) / np.linalg.norm(w) <= 1e-5


def test_noalloc_rejects_oversized_geometry():
    lib = _native.load()
    big = torch.zeros((8, 8), dtype=torch.float32, device="cuda")
    img = _native.RG_IMAGE(big.data_ptr(), 2048, 1, 2048, 2048, -1.0, 1.0, 1.0, -1.0)
    sino = _native.RG_IMAGE(big.data_ptr(), 2048, 1, 1800, 1800, 0.0, 1.0, math.pi, -1.0)
    assert lib.rg_radon_slantstack_noalloc(img, sino, None) == _native.RG_EINVAL
    assert b"static scratch" in lib.rg_last_error()
    # more views than the per-view table holds (4096)
    img = _native.RG_IMAGE(big.data_ptr(), 64, 1, 64, 64, -1.0, 1.0, 1.0, -1.0)
    sino = _native.RG_IMAGE(big.data_ptr(), 64, 1, 4097, 4097, 0.0, 1.0, math.pi, -1.0)
    assert lib.rg_radon_slantstack_noalloc(img, sino, None) == _native.RG_EINVAL
    assert b"4096" in lib.rg_last_error()
