"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own hot-path C/C++ (compiled in place by
``make -C oracle ref REF_SRC=<checkout>/raft`` into oracle/_ref/libraft_ref.so) on small seeded
inputs and saves inputs and outputs as compressed .npz files.  The tests then
pin the oracle restatement (and through it the CUDA path) to these outputs
without needing the reference tree.

Usage (in a tree where the reference sources exist):
    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
from oracle import ref as R     # noqa: E402

# Cases that use non-default corners (tl_x, tl_y, br_x, br_y).
ODD_IMG = (-1.2, 1.1, 0.8, -0.9)
ODD_SINO = (0.1, 1.2, 2.5, -1.3)

# (theta, t) pairs for DDA index sequences; theta == 0 exercises the branch
# whose first sigma the reference leaves unset (sigma is not compared there).
DDA_RAYS = [(th, t) for th in (0.0, 1e-3, 0.3, math.pi / 4, 1.0, math.pi / 2,
                               2.0, 2.9, math.pi)
            for t in (-1.0, -0.73, -0.25, 0.0, 0.31, 0.999, 1.0)]


# Read-only checkout of the reference (pyraft v0.0.8); PYRAFT_REFERENCE
# overrides the default location.
REFERENCE = os.environ.get("PYRAFT_REFERENCE", "/root/reference")


def reference_lowpassino_fbp():
    """The reference's own pyraft.filters.filters.lowpassino_fbp, loaded from
    its source file.  Its package imports the compiled libraft and pynfft,
    which cannot load here, so the two modules it star-imports are stubbed:
    ringfun (unused by this function) is empty, and raftypes provides only
    `image`, an ndarray subclass that carries top_left / bottom_right like
    pyraft's (pyraft/raftypes.py:254-358)."""
    import importlib.util
    import types

    class image(np.ndarray):
        def __new__(cls, a, top_left=(0.0, 1.0), bottom_right=(math.pi, -1.0)):
            obj = np.asarray(a, dtype=np.float64).view(cls)
            obj.top_left, obj.bottom_right = top_left, bottom_right
            return obj

        def __array_finalize__(self, obj):
            self.top_left = getattr(obj, "top_left", (0.0, 1.0))
            self.bottom_right = getattr(obj, "bottom_right", (math.pi, -1.0))

    pkg = types.ModuleType("pyraft_ref")
    pkg.__path__ = []
    sub = types.ModuleType("pyraft_ref.filters")
    sub.__path__ = []
    raftypes = types.ModuleType("pyraft_ref.raftypes")
    raftypes.image = image
    raftypes.__all__ = ["image"]
    ringfun = types.ModuleType("pyraft_ref.filters.ringfun")
    ringfun.__all__ = []
    for m in (pkg, sub, raftypes, ringfun):
        sys.modules[m.__name__] = m
    path = os.path.join(REFERENCE, "pyraft", "filters", "filters.py")
    spec = importlib.util.spec_from_file_location("pyraft_ref.filters.filters", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.lowpassino_fbp, image


def main() -> None:
    if not R.available():
        raise SystemExit("oracle/_ref/libraft_ref.so missing: run `make -C oracle ref REF_SRC=<checkout>/raft`")
    rng = np.random.default_rng(20261203)
    out = {}

    # Config-1 workload: Shepp-Logan 256^2, 256 views on [0, pi), 256 rays.
    sl256 = R.phantom_fromdesc((256, 256), O.SHEPP_LOGAN)
    sino256 = R.radon_slantstack(sl256, 256, 256, threads=1)
    bp256 = R.backprojection_slantstack(sino256, 256, threads=1)
    out["config1"] = dict(phantom=sl256, radon=sino256, bp=bp256)

    # Shepp-Logan 64^2 through every operator, default corners.
    sl64 = R.phantom_fromdesc((64, 64), O.SHEPP_LOGAN)
    s_rand = rng.random((64, 48))
    s_rand_b = s_rand.copy()
    s_rand_b[:, 0] = 0.0          # theta == 0 column: reference sigma unset
    out["sl64"] = dict(
        phantom=sl64,
        radon_ss=R.radon_slantstack(sl64, 64, 48, threads=1),
        bp_ss=R.backprojection_slantstack(s_rand, 64, threads=1),
        sino_in=s_rand,
        radon_bres=R.radon_bresenham(sl64, 64, 48, threads=3),
        sino_in_bres=s_rand_b,
        radonT_bres=R.radon_transpose_bresenham(s_rand_b, (64, 64), threads=3),
        fromdesc=R.radon_fromdesc(64, 48, O.SHEPP_LOGAN),
    )

    # Odd sizes and non-default corners.
    img17 = rng.random((17, 17))
    s_odd = rng.random((23, 9))
    s_odd_b = s_odd.copy()
    out["odd"] = dict(
        img=img17, sino_in=s_odd,
        radon_ss=R.radon_slantstack(img17, 23, 9, ODD_IMG, ODD_SINO, threads=1),
        bp_ss=R.backprojection_slantstack(s_odd, 17, ODD_IMG, ODD_SINO, threads=1),
        radon_bres=R.radon_bresenham(img17, 23, 9, ODD_IMG, ODD_SINO, threads=2),
        radonT_bres=R.radon_transpose_bresenham(s_odd_b, (17, 17), ODD_IMG, ODD_SINO,
                                                threads=2),
        img_corners=np.array(ODD_IMG), sino_corners=np.array(ODD_SINO),
    )

    # Normalised DDA backprojection (views start at 0.1: no theta == 0 ray,
    # whose first sigma the reference leaves unset, enters the weights).
    s_bn = rng.random((40, 33))
    out["bres_norm"] = dict(
        sino_in=s_bn, sino_corners=np.array(ODD_SINO),
        bp=R.backprojection_bresenham(s_bn, (48, 48), sino_corners=ODD_SINO, threads=3),
        bp_odd=R.backprojection_bresenham(s_bn, (31, 37), ODD_IMG, ODD_SINO, threads=2),
        img_corners=np.array(ODD_IMG))

    # Mesh Radon: non-uniform t and theta.
    img_m = rng.random((45, 45))
    t_m = np.sort(rng.uniform(-1.2, 1.2, 37))
    th_m = np.sort(rng.uniform(0.0, np.pi, 29))
    out["mesh"] = dict(img=img_m, t=t_m, theta=th_m,
                       radon=R.radon_slantstack_withmesh(img_m, t_m, th_m, threads=1),
                       radon_odd=R.radon_slantstack_withmesh(img_m, t_m, th_m, ODD_IMG, threads=1),
                       img_corners=np.array(ODD_IMG))

    # Rectangular image for the DDA path (the slant-stack path is square-only).
    rect = rng.random((40, 48))
    out["rect"] = dict(img=rect,
                       radon_bres=R.radon_bresenham(rect, 37, 29, threads=2))

    # DDA pixel sequences on a 32 x 40 image.
    ii, jj, ss, off, meta = [], [], [], [0], []
    for th, t in DDA_RAYS:
        a, b, s = R.dda_trace((32, 40), th, t)
        ii.append(a); jj.append(b); ss.append(s)
        off.append(off[-1] + len(a)); meta.append((th, t))
    out["dda"] = dict(i=np.concatenate(ii), j=np.concatenate(jj),
                      sigma=np.concatenate(ss), offsets=np.array(off),
                      rays=np.array(meta), shape=np.array([32, 40]))

    # pyraft's FBP filter, run from the reference's own Python source.
    lowpass, ref_image = reference_lowpassino_fbp()
    cases = {}
    for k, (r, v, tl, br) in enumerate([(64, 48, (0.0, 1.0), (math.pi, -1.0)),
                                        (97, 13, (0.0, 1.0), (math.pi, -1.0)),
                                        (256, 5, (0.2, 1.3), (2.9, -0.7)),
                                        (33, 7, (0.0, 0.5), (math.pi, -1.5))]):
        s_lp = rng.random((r, v))
        got = lowpass(ref_image(s_lp, tl, br))
        cases[f"sino{k}"] = s_lp
        cases[f"corners{k}"] = np.array([tl[0], tl[1], br[0], br[1]])
        cases[f"out{k}"] = np.asarray(got, dtype=np.float64)
    cases["count"] = np.array(4)
    out["lowpass"] = cases

    for name, arrays in out.items():
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **arrays)
        print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


if __name__ == "__main__":
    main()
