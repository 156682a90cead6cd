"""The gathers' autotuner cache (RG_TUNE_CACHE).

The first backprojection or adjoint of a geometry times the gather's launch
shapes (rows per thread and cluster view split) and keeps the fastest; with
RG_TUNE_CACHE=<file> the choices are also written to a JSON file and read
back by later processes, so a deployment tunes once.  The reference has no
tuning at all (its thread count is the global nthreads = cpu_count(),
pyraft/raftypes.py:12).  Each step runs in a fresh process, since a process
reads the file when it first needs a choice:
- a tuning run writes one entry per geometry and operator;
- a run that reads an edited entry launches that shape: its output matches,
  bit for bit, a run forced to the same shape by RG_GATHER_ROWS /
  RG_GATHER_SPLIT, and differs from a run forced to another split (the
  split changes the summation order);
- a corrupt file is ignored and rewritten as valid JSON.
"""
import json
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

# One backprojection and one adjoint of a seeded 256^2 x 720 problem (360
# view pairs: the TMA-staged paired gathers); saves the backprojection.
SCRIPT = """
import math, sys, numpy as np, torch
import pyraft_gb300 as rg
from pyraft_gb300 import _native
from pyraft_gb300.raftypes import gpu_image, rg_image
L = _native.load()
g = torch.Generator(device="cuda").manual_seed(9)
s = torch.rand((256, 720), device="cuda", generator=g) - 0.25   # kept alive: S holds its pointer
S = rg_image(gpu_image(s, (0.0, 1.0), (math.pi, -1.0)))
st = torch.cuda.current_stream().cuda_stream
bp = torch.zeros((256, 256), device="cuda")
adj = torch.zeros((256, 256), device="cuda")
_native.check(L.rg_backprojection_slantstack(S, rg_image(gpu_image(bp)), None, 0, st))
_native.check(L.rg_radon_transpose_slantstack(S, rg_image(gpu_image(adj)), None, 0, st))
torch.cuda.synchronize()
assert L.rg_device_status() == 0
np.save(sys.argv[1], bp.cpu().numpy())
"""


def _run(tmp_path, name, **env):
    e = {k: v for k, v in os.environ.items()
         if k not in ("RG_TUNE_CACHE", "RG_GATHER_ROWS", "RG_GATHER_SPLIT")}
    e.update(env)
    e["PYTHONPATH"] = ROOT + os.pathsep + e.get("PYTHONPATH", "")
    out = str(tmp_path / f"{name}.npy")
    r = subprocess.run([sys.executable, "-c", SCRIPT, out], cwd=ROOT, env=e,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(out)


def _entries(path):
    with open(path) as f:
        d = json.load(f)
    assert isinstance(d, dict)
    for k, v in d.items():
        assert v["rows"] in (4, 8, 16) and v["split"] in (0, 1, 2, 4), (k, v)
    return d


def test_tuned_shapes_persist_and_are_used(tmp_path):
    cache = str(tmp_path / "tune.json")
    _run(tmp_path, "tuning", RG_TUNE_CACHE=cache)
    d = _entries(cache)
    bp_keys = [k for k in d if "|bp|N256|R256|V720|" in k]
    adj_keys = [k for k in d if "|adj|N256|R256|V720|" in k]
    assert len(bp_keys) == 1 and len(adj_keys) == 1, list(d)

    d[bp_keys[0]] = {"rows": 4, "split": 2}
    with open(cache, "w") as f:
        json.dump(d, f)
    from_cache = _run(tmp_path, "cached", RG_TUNE_CACHE=cache)
    assert _entries(cache)[bp_keys[0]] == {"rows": 4, "split": 2}
    forced = _run(tmp_path, "forced", RG_GATHER_ROWS="4", RG_GATHER_SPLIT="2")
    other = _run(tmp_path, "other", RG_GATHER_ROWS="4", RG_GATHER_SPLIT="1")
    assert np.array_equal(from_cache, forced)
    assert not np.array_equal(from_cache, other)
    rel = np.linalg.norm(from_cache - other) / np.linalg.norm(other)
    assert rel <= 1e-6, rel


def test_corrupt_cache_is_ignored_and_rewritten(tmp_path):
    cache = tmp_path / "tune.json"
    cache.write_text('{"truncated": {"rows": 8, "spl')
    _run(tmp_path, "corrupt", RG_TUNE_CACHE=str(cache))
    d = _entries(str(cache))
    assert any("|bp|N256|" in k for k in d) and "truncated" not in d
