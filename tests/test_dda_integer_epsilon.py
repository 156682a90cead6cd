"""The DDA walk's epsilon accumulator in exact integer arithmetic.

The walk (raft/raft_ddaiterator.c:196-248) decides its slow-axis moves with
FP64 arithmetic: a fast step adds epsilon_update u to epsilon, and when
epsilon exceeds delta_slow d it moves on the slow axis and subtracts d.
GB300 runs FP64 at a small fraction of its FP32 rate, so the kernels make
the same decisions with 64-bit integers (bresenham.cu, DDAInt):
- after the walk's first FP64 add, epsilon is a multiple of ulp(epsilon),
  which is at least ulp(u); so epsilon, u and d are all integer multiples of
  q = min(ulp(u), ulp(d)), a power of two;
- fl(eps + u) is then the integer sum rounded to 53 significant bits, to
  nearest, ties to even (round53 below), times q;
- while u <= d and epsilon <= d before each add, an epsilon that exceeds d
  is at most 2d, so eps - d is exact (Sterbenz) and needs no rounding;
- the sigma split at a slow move uses fl(d - eps_prev) = round53(D - E) q.
This test restates that integer walk in Python (exact integers) and checks
it against IEEE FP64 arithmetic (numpy float64, no contraction) step by
step, on random and edge-case (u, d, eps0), including the kernel's
conditions for taking the integer path.  It runs on the CPU.
"""
import math

import numpy as np
import pytest


def round53(s):
    """s > 0 (int) rounded to 53 significant bits, to nearest, ties to even."""
    n = s.bit_length()
    if n <= 53:
        return s
    sh = n - 53
    low = s & ((1 << sh) - 1)
    half = 1 << (sh - 1)
    s >>= sh
    if low > half or (low == half and (s & 1)):
        s += 1
    return s << sh


def int_path_ok(u, d, eps):
    """The kernel's conditions for the integer walk, checked after the first
    FP64 add (eps = epsilon then)."""
    if not (0.0 < u <= d) or eps > d:
        return False
    q = min(math.ulp(u), math.ulp(d))
    if q < 2.0 ** -1000:
        return False
    return (d + u) / q < 2.0 ** 61 and (eps / q).is_integer()


def fp64_steps(u, d, eps, n):
    """n fast steps of the FP64 walk: (eps after each step, slow flag,
    fl(d - eps_prev) at slow moves)."""
    u, d, eps = np.float64(u), np.float64(d), np.float64(eps)
    out = []
    for _ in range(n):
        prev = eps
        eps = eps + u
        slow = bool(eps > d)
        diff = None
        if slow:
            eps = eps - d
            diff = float(d - prev)
        out.append((float(eps), slow, diff))
    return out


def int_steps(u, d, eps, n):
    q = min(math.ulp(u), math.ulp(d))
    U, D, E = int(u / q), int(d / q), int(eps / q)
    assert U * q == u and D * q == d and E * q == eps
    out = []
    for _ in range(n):
        prev = E
        E = round53(E + U)
        slow = E > D
        diff = None
        if slow:
            E = E - D
            diff = round53(D - prev) * q if D > prev else float(D - prev) * q
        out.append((E * q, slow, diff))
    return out


def first_add(u, d, eps0):
    eps = np.float64(eps0) + np.float64(u)
    if eps > d:
        eps = eps - np.float64(d)
    return float(eps)


def _check(u, d, eps0, n=4000):
    eps1 = first_add(u, d, eps0)
    if not int_path_ok(u, d, eps1):
        return False
    assert int_steps(u, d, eps1, n) == fp64_steps(u, d, eps1, n)
    return True


def test_round53_matches_fp64_addition():
    rng = np.random.default_rng(1)
    for _ in range(20000):
        a, b = rng.random() * 10.0 ** rng.integers(-6, 3), rng.random() * 10.0 ** rng.integers(-6, 3)
        q = min(math.ulp(a), math.ulp(b))
        A, B = int(a / q), int(b / q)
        assert round53(A + B) * q == float(np.float64(a) + np.float64(b))


@pytest.mark.parametrize("n", [64, 255, 1024, 2048, 4097])
def test_integer_walk_equals_fp64_walk_on_view_grids(n):
    """u = dy |tan| and d = dx for an n x n grid on [-1, 1]^2 over views
    spread in [0, pi), with the walk's possible starting epsilons."""
    rng = np.random.default_rng(n)
    dx = 2.0 / (n - 1)
    taken = 0
    for theta in np.concatenate([np.linspace(0.0, np.pi, 181, endpoint=False)[1:],
                                 rng.random(60) * np.pi]):
        c, s = math.cos(theta), math.sin(theta)
        if abs(dx * s) <= abs(dx * c):
            u = abs(dx * s / c)
        else:
            u = abs(dx * c / s)
        for eps0 in (0.0, u / 3.0, dx * rng.random(), dx, 0.5 * dx, 1e-17):
            taken += _check(u, dx, eps0, n=2 * n)
    assert taken > 200


def test_integer_walk_edge_cases():
    d = 2.0 / 2047
    for u in (d, np.nextafter(d, 0.0), d / 2, d / 3, d * 0.999999999, d / 100.0):
        for eps0 in (0.0, np.nextafter(d, 0.0), d, u, d - u):
            assert _check(u, d, eps0, n=3000)


def test_path_conditions_reject_what_they_must():
    d = 2.0 / 1023
    assert not int_path_ok(2.0 * d, d, 0.0)          # u > d: two slow moves per step
    assert not int_path_ok(d * 2.0 ** -20, d, 0.0)   # d / q beyond 2^61: FP64 walk
    assert not int_path_ok(d / 3.0, d, 1.5 * d)      # epsilon above d
    assert int_path_ok(d / 3.0, d, 0.0)


def f32_scaled(r, kq):
    """RN_f32(r) * 2^kq built from the integer r (bresenham.cu, f32_scaled):
    r rounded to 24 bits, to nearest, ties to even, then exponent and
    mantissa assembled."""
    if r == 0:
        return np.float32(0.0)
    n = r.bit_length()
    if n > 24:
        sh = n - 24
        m = (r + (1 << (sh - 1)) - 1 + ((r >> sh) & 1)) >> sh
        if m >> 24:
            m >>= 1
            n += 1
    else:
        m = r << (24 - n)
    bits = ((n - 1 + kq + 127) << 23) | (m & 0x7FFFFF)
    return np.array([bits], dtype=np.uint32).view(np.float32)[0]


def test_split_as_float_matches_conversion():
    """The sigma split needs (float)fl(d - eps_prev): the kernels build it
    from round53(D - E_prev) with integer operations; it must equal the
    FP64 value converted to FP32."""
    rng = np.random.default_rng(7)
    vals = [1, 2, 3, (1 << 24) - 1, 1 << 24, (1 << 24) + 1, (1 << 25) - 1, (1 << 53) - 1,
            (1 << 61) + 12345]
    vals += [int(rng.integers(1, 1 << 62)) for _ in range(20000)]
    vals += [int(rng.integers(1, 1 << 30)) << int(rng.integers(0, 30)) for _ in range(5000)]
    for r in vals:
        r53 = round53(r)
        for kq in (-100, -62, -1, 0):
            want = np.float32(np.float64(float(r53) * 2.0 ** kq))
            assert f32_scaled(r53, kq) == want, (r, kq)


def test_branch_free_rounding_equals_round53():
    """The kernels round with one add and a truncation (bias = half - 1 plus
    the kept part's lowest bit); that is round53 above."""
    rng = np.random.default_rng(11)
    vals = [0, 1, (1 << 53) - 1, 1 << 53, (1 << 53) + 1, (1 << 54) + 2, (1 << 54) + 6,
            (1 << 62) - 1] + [int(rng.integers(0, 1 << 62)) for _ in range(50000)]
    for s in vals:
        sh = max(s.bit_length() - 53, 0)
        half = (1 << sh) >> 1
        bias = half - 1 + ((s >> sh) & 1) if half else 0
        assert ((s + bias) >> sh) << sh == round53(s) if s else s == 0


def round53_small(s):
    """bresenham.cu round53_small: round53 for s < 2^54 (at most one bit
    dropped): m = 1 when s has 54 bits."""
    m = s >> 53
    return (s + ((s >> 1) & m)) & ~m


def test_one_bit_rounding_equals_round53():
    rng = np.random.default_rng(13)
    vals = [0, 1, 2, (1 << 53) - 2, (1 << 53) - 1, 1 << 53, (1 << 53) + 1, (1 << 53) + 2,
            (1 << 53) + 3, (1 << 54) - 3, (1 << 54) - 2, (1 << 54) - 1]
    vals += [int(rng.integers(0, 1 << 54)) for _ in range(100000)]
    vals += [(1 << 53) + int(rng.integers(0, 1 << 20)) for _ in range(20000)]
    for s in vals:
        assert round53_small(s) == round53(s), s


def test_one_bit_walk_equals_fp64_walk():
    """The rays whose D + U < 2^54 (views more than about 18 degrees from the
    fast axis) take the one-bit rounding in the kernels: that walk, with the
    sigma split's rounding too, against IEEE FP64 step by step."""
    taken = 0
    rng = np.random.default_rng(17)
    for n in (255, 1024, 2048):
        dx = 2.0 / (n - 1)
        for theta in np.concatenate([np.linspace(0.0, np.pi / 4, 90)[1:], rng.random(40) * np.pi / 4]):
            u = abs(dx * math.tan(theta))
            for eps0 in (0.0, u / 3.0, dx * rng.random(), 0.5 * dx):
                eps1 = first_add(u, dx, eps0)
                if not int_path_ok(u, dx, eps1):
                    continue
                q = min(math.ulp(u), math.ulp(dx))
                U, D, E = int(u / q), int(dx / q), int(eps1 / q)
                if D + U >= 1 << 54:
                    continue
                want = fp64_steps(u, dx, eps1, 2 * n)
                got = []
                for _ in range(2 * n):
                    prev = E
                    E = round53_small(E + U)
                    slow = E > D
                    diff = None
                    if slow:
                        E = E - D
                        diff = round53_small(D - prev) * q
                    got.append((E * q, slow, diff))
                assert got == want, (n, theta, eps0)
                taken += 1
    assert taken > 300


def round53_top(s):
    """bresenham.cu round53 as the kernels compute it: the shift from the
    bits above bit 52, the dropped bits cleared with a mask."""
    m = s >> 53
    sh = m.bit_length()
    low = (1 << sh) - 1
    bias = (low >> 1) + (((s >> sh) & 1) if m else 0)
    return (s + bias) & ~low


def test_mask_rounding_equals_round53():
    rng = np.random.default_rng(19)
    vals = [0, 1, (1 << 53) - 1, 1 << 53, (1 << 53) + 1, (1 << 54) + 2, (1 << 54) + 6,
            (1 << 61) - 1, (1 << 61) - 256, (1 << 61) - 255, (1 << 62) + 12345, (1 << 63) - 1]
    vals += [int(rng.integers(0, 1 << 62)) for _ in range(50000)]
    vals += [int(rng.integers(1 << 53, 1 << 61)) for _ in range(50000)]
    for s in vals:
        assert round53_top(s) == round53(s), s
