"""Programmatic dependent launch keeps stream order.

The operators' kernel chains are launched with programmatic dependent
launch: each kernel's CTAs may be dispatched into its predecessor's tail and
wait there (griddepcontrol.wait) until the predecessor has completed and its
writes are visible.  A kernel that touched memory before that wait would
race with its predecessor.  This test runs the deterministic operators (the
TMA Radon, the paired backprojection and adjoint with their prepasses and
edge CTAs, the FBP with its filter and layout passes, a full-plan EM with
the fused update) in a fresh process with the attribute (the default) and in
one without it (RG_PDL=0, read once per process), and requires the same
bits.  The reference launches nothing on a GPU this way; its C operators
run in the caller's thread.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = """
import math, sys, numpy as np, torch
import pyraft_gb300 as rg
from pyraft_gb300 import _native
from pyraft_gb300.raftypes import gpu_image, rg_image
L = _native.load()
st = torch.cuda.current_stream().cuda_stream
g = torch.Generator(device="cuda").manual_seed(21)
C = ((0.0, 1.0), (math.pi, -1.0))
out = {}
x = torch.rand((512, 512), device="cuda", generator=g)              # kept alive
sino = torch.empty((512, 720), device="cuda")
_native.check(L.rg_radon_slantstack(rg_image(gpu_image(x)), rg_image(gpu_image(sino, *C)),
                                    None, 0, st))
out["radon"] = sino
s = torch.rand((512, 720), device="cuda", generator=g) - 0.25
for name, fn in (("bp", L.rg_backprojection_slantstack), ("adj", L.rg_radon_transpose_slantstack)):
    img = torch.full((512, 512), float("nan"), device="cuda")
    _native.check(fn(rg_image(gpu_image(s, *C)), rg_image(gpu_image(img)), None, 0, st))
    out[name] = img
img = torch.full((512, 512), float("nan"), device="cuda")
_native.check(L.rg_fbp(rg_image(gpu_image(s, *C)), rg_image(gpu_image(img)),
                       _native.RG_FILTER_RAMLAK, None, 0, st))
out["fbp"] = img
y = torch.poisson(20.0 * torch.rand((256, 720), device="cuda", generator=g), generator=g)
out["em_input"] = y
out["em"] = rg.em(gpu_image(y, *C), (256, 256), 6, method=rg.radon_method.SLANTSTACK).data
torch.cuda.synchronize()
assert L.rg_device_status() == 0
np.savez(sys.argv[1], **{k: v.cpu().numpy() for k, v in out.items()})
"""


def _run(tmp_path, name, **env):
    e = {k: v for k, v in os.environ.items() if k != "RG_PDL"}
    # the gathers' launch shape pinned (clusters of 2), so that the two
    # processes' autotuners cannot pick different summation orders
    e.update(RG_GATHER_ROWS="8", RG_GATHER_SPLIT="2", **env)
    e["PYTHONPATH"] = ROOT + os.pathsep + e.get("PYTHONPATH", "")
    path = str(tmp_path / f"{name}.npz")
    r = subprocess.run([sys.executable, "-c", SCRIPT, path], cwd=ROOT, env=e,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(path)


def test_chains_give_the_same_bits_with_and_without_pdl(tmp_path):
    with_pdl = _run(tmp_path, "pdl")
    without = _run(tmp_path, "nopdl", RG_PDL="0")
    for k in with_pdl.files:
        a, b = with_pdl[k], without[k]
        assert np.isfinite(a).all(), k
        assert np.array_equal(a, b), k
