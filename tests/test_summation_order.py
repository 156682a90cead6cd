"""FP32 summation order of the paired gathers (csrc/gather_rot.cu), on the CPU.

The kernels sum each pixel's interpolated samples straight into FP32
accumulators: per cluster rank a running sum over its share of the view
pairs (the views of [0, pi/2) and, for the quarter-turned pixel, their
partners), then the ranks and the two halves are added.  This emulates that
order on a Ram-Lak-filtered Shepp-Logan sinogram with 1800 views and checks
its error against the FP64 sum, next to the alternative of FP32 partial sums
over chunks of 16 view pairs.  The terms are the FP64 interpolations of the
FP32 sinogram rounded to FP32, which is what each update adds.
"""
import math

import numpy as np

from oracle import oracle as O


def _terms(q, xs, ys, th, tmin, dt):
    X, Y = np.meshgrid(xs, ys)
    R = q.shape[0]
    out = np.empty((len(th), X.size), np.float32)
    for v, t in enumerate(th):
        u = ((X * math.cos(t) + Y * math.sin(t)) - tmin) / dt
        fl = np.floor(u).astype(np.int64)
        ok = (fl >= 0) & (fl <= R - 2)
        f = np.where(ok, fl, 0)
        s0 = q[f, v].astype(np.float64)
        s1 = q[f + 1, v].astype(np.float64)
        out[v] = np.where(ok, s0 + (u - fl) * (s1 - s0), 0.0).ravel()
    return out


def _running(t):
    return np.cumsum(t, axis=0, dtype=np.float32)[-1]


def _chunked(t, chunk=16):
    acc = np.zeros(t.shape[1], np.float32)
    for c0 in range(0, t.shape[0], chunk):
        acc = (acc + _running(t[c0:c0 + chunk])).astype(np.float32)
    return acc


def test_running_fp32_sums_stay_far_inside_parity():
    N, R, A, split = 96, 96, 1800, 2
    ph = np.flipud(O.shepp_logan(N)).copy()
    q = O.ramlak(O.radon_slantstack(ph, R, A), 2.0 / (R - 1)).astype(np.float32)
    xs, ys = np.linspace(-1, 1, N), np.linspace(1, -1, N)
    th = np.arange(A) * math.pi / A
    half, per = A // 2, A // 2 // split
    exact, run, chunked = [], [], []
    for r0 in range(0, N, 32):
        T = _terms(q, xs, ys[r0:r0 + 32], th, -1.0, 2.0 / (R - 1))
        exact.append(T.astype(np.float64).sum(axis=0))
        a = np.zeros(T.shape[1], np.float32)
        b = np.zeros(T.shape[1], np.float32)
        for lo in (0, half):                       # the views, then their partners
            ranks_a = [_running(T[lo + k * per:lo + (k + 1) * per]) for k in range(split)]
            ranks_b = [_chunked(T[lo + k * per:lo + (k + 1) * per]) for k in range(split)]
            a = (a + np.sum(ranks_a, axis=0, dtype=np.float32)).astype(np.float32)
            b = (b + np.sum(ranks_b, axis=0, dtype=np.float32)).astype(np.float32)
        run.append(a.astype(np.float64))
        chunked.append(b.astype(np.float64))
    exact, run, chunked = map(np.concatenate, (exact, run, chunked))
    rel = lambda x: np.linalg.norm(x - exact) / np.linalg.norm(exact)
    # 450-term running sums: a few 1e-7, far inside the 1e-5 parity bar
    assert rel(run) < 1e-6, rel(run)             # measured 2.9e-7 (8.8e-8 chunked)
    assert rel(chunked) <= rel(run) * 1.5
