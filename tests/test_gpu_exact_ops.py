"""The exact arithmetic mode's integer-pipe operations against the IEEE operations they stand
for, bit for bit (needs a GPU; the IEEE results are numpy's, computed on the host).

div6_x (x / 6.0 by the exact remainder) is checked on random values over its whole valid
range and on values made to put x / 6 close to a representable number or to a midpoint
between two (where a faithful but incorrectly rounded quotient would show); half_x and
twice_x on the range reachable from tame windows, zeros of both signs included; tame on
values at and around its thresholds; the integer-pipe IEEE additions (add_x, sub_x) and
multiplications by 3, 6 and 5/4 (mulk_x) on their whole stated range; the quotient from a
correctly rounded reciprocal (div_rcp) on tame operands.
"""
import ctypes

import numpy as np
import pytest
import torch

from apophis_gb300 import _capi, hydro
from quotient_cases import midpoint_cases

pytestmark = pytest.mark.gpu


def _run(op, x):
    xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    out = torch.empty_like(xd)
    st = _capi.load().aph_diag_exact_ops(op, ctypes.c_void_p(xd.data_ptr()),
                                          ctypes.c_void_p(out.data_ptr()), xd.numel(),
                                          hydro.stream_handle())
    assert st == 0, _capi.load().aph_last_error()
    return out.cpu().numpy()


def _bits_equal(got, want, what):
    g, w = got.view(np.int64), want.view(np.int64)
    bad = g != w
    if bad.any():
        i = int(np.argmax(bad))
        raise AssertionError("%s: %d of %d differ; first x index %d: got %r want %r" % (
            what, int(bad.sum()), bad.size, i, got[i], want[i]))


def _random_in_range(rng, n, emin, emax):
    """Random doubles with exponents uniform in [emin, emax] and random mantissas and signs."""
    mant = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    exp = rng.integers(emin + 1023, emax + 1023 + 1, n).astype(np.uint64)
    sign = rng.integers(0, 2, n).astype(np.uint64)
    return ((sign << np.uint64(63)) | (exp << np.uint64(52)) | mant).view(np.float64)


def test_div6_matches_ieee_division(cuda):
    rng = np.random.Generator(np.random.PCG64(6))
    parts = [_random_in_range(rng, 4_000_000, -999, 999)]
    # x / 6 near a representable q or a midpoint: x = RN(6 q) moved by a few ulps
    q = _random_in_range(rng, 2_000_000, -990, 990)
    x = q * 6.0
    step = rng.integers(-8, 9, x.size)
    parts.append(np.nextafter(x, np.where(step >= 0, np.inf, -np.inf)))
    xb = x.view(np.int64) + step
    parts.append(xb.view(np.float64))
    # small integers and their neighbours (exact quotients and ties in integer arithmetic)
    ints = np.arange(-3000, 3001, dtype=np.float64)
    parts += [ints, np.nextafter(ints, np.inf), np.nextafter(ints, -np.inf)]
    parts.append(np.array([0.0, -0.0, 6.0, -6.0, 2.0 ** -999, -(2.0 ** 999)]))
    x = np.concatenate(parts)
    x = x[np.isfinite(x) & ((np.abs(x) > 2.0 ** -1000) & (np.abs(x) < 2.0 ** 1000) | (x == 0))]
    _bits_equal(_run(0, x), x / 6.0, "div6_x")


def test_half_and_twice_match_ieee_scaling(cuda):
    rng = np.random.Generator(np.random.PCG64(2))
    x = np.concatenate([_random_in_range(rng, 2_000_000, -300, 300),
                        np.array([0.0, -0.0, 1.0, -1.0, 2.0 ** -300, 2.0 ** 300])])
    _bits_equal(_run(1, x), 0.5 * x, "half_x")
    _bits_equal(_run(2, x), 2.0 * x, "twice_x")


def test_tame_thresholds(cuda):
    edges = [2.0 ** -200, 2.0 ** 201]
    x = np.array([0.0, -0.0, 1.0, -3.5, edges[0], -edges[0], np.nextafter(edges[0], 0.0),
                  np.nextafter(edges[1], 0.0), edges[1], -edges[1], 5e-324, np.inf, -np.inf,
                  np.nan, 1e-300, 1e300])
    want = np.where((x == 0) | ((np.abs(x) >= edges[0]) & (np.abs(x) < edges[1])), 1.0, 0.0)
    np.testing.assert_array_equal(_run(3, x), want)


def _run2(op, x, y):
    xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    yd = torch.from_numpy(np.ascontiguousarray(y)).cuda()
    out = torch.empty_like(xd)
    st = _capi.load().aph_diag_exact_ops2(op, ctypes.c_void_p(xd.data_ptr()),
                                           ctypes.c_void_p(yd.data_ptr()),
                                           ctypes.c_void_p(out.data_ptr()), xd.numel(),
                                           hydro.stream_handle())
    assert st == 0, _capi.load().aph_last_error()
    return out.cpu().numpy()


def test_integer_pipe_add_matches_ieee(cuda):
    """add_x / sub_x against IEEE addition: random pairs with any exponent difference, near
    cancellations (b close to -a within a few ulps), equal exponents, one operand far below
    the other's ulp, and signed zeros."""
    rng = np.random.Generator(np.random.PCG64(7))
    n = 2_000_000
    a = _random_in_range(rng, n, -800, 800)
    kind = rng.integers(0, 5, n)
    b = _random_in_range(rng, n, -800, 800)
    near = -(a.view(np.int64) + rng.integers(-64, 65, n)).view(np.float64)
    b = np.where(kind == 1, near, b)
    close = (a.view(np.int64) ^ rng.integers(0, 1 << 50, n)).view(np.float64)
    b = np.where(kind == 2, np.where(rng.random(n) < 0.5, close, -close), b)
    far = a * 2.0 ** rng.integers(-70, 71, n).astype(np.float64) * (1 + rng.random(n))
    b = np.where(kind == 3, np.where(rng.random(n) < 0.5, far, -far), b)
    z = rng.random(n)
    b = np.where(z < 0.01, 0.0, np.where(z < 0.02, -0.0, b))
    a = np.where(rng.random(n) < 0.005, -0.0, a)
    ok = np.isfinite(a + b) & ((np.abs(a + b) > 2.0 ** -900) | (a + b == 0))
    a, b = a[ok], b[ok]
    _bits_equal(_run2(0, a, b), a + b, "add_x")
    _bits_equal(_run2(1, a, b), a - b, "sub_x")


def test_integer_pipe_small_multiplies_match_ieee(cuda):
    rng = np.random.Generator(np.random.PCG64(8))
    x = np.concatenate([_random_in_range(rng, 2_000_000, -800, 800), np.array([0.0, -0.0, 1.0])])
    for op, k in ((2, 3.0), (3, 6.0), (4, 1.25)):
        _bits_equal(_run2(op, x, x), k * x, "x%g" % k)


def test_quotient_from_reciprocal_matches_ieee_division(cuda):
    """x / y from y's correctly rounded reciprocal (Markstein's correction) against IEEE
    division: random tame pairs, quotients made to fall within a few ulps of a representable
    number, quotients within ~1e-14 ulp of a rounding midpoint (where a faithful but
    incorrectly rounded quotient would show), exact integer quotients and signed zeros."""
    rng = np.random.Generator(np.random.PCG64(9))
    n = 3_000_000
    a = _random_in_range(rng, n, -200, 200)
    b = _random_in_range(rng, n, -200, 200)
    q = _random_in_range(rng, n, -150, 150)
    # x near q y (and near (q + ulp(q) / 2) y), moved by a few ulps of x
    near = []
    for x0 in (q * b, q * b + (np.spacing(q) * 0.5) * b):
        x = x0.view(np.int64) + rng.integers(-3, 4, n)
        near.append(x.view(np.float64))
    # quotients within ~1e-14 ulp of a rounding midpoint (the hardest cases of division)
    ma, mb = midpoint_cases(rng, 50_000)
    ints = np.arange(-300, 301, dtype=np.float64)
    ints = ints[ints != 0]
    xs = np.concatenate([a] + near + [ma, np.repeat(ints, ints.size), np.array([0.0, -0.0, 0.0, -0.0])])
    ys = np.concatenate([b, b, b, mb, np.tile(ints, ints.size), np.array([3.0, 3.0, -3.0, -3.0])])
    keep = (np.abs(xs) >= 2.0 ** -200) & (np.abs(xs) < 2.0 ** 201) | (xs == 0)
    xs, ys = xs[keep], ys[keep]
    _bits_equal(_run2(8, xs, ys), xs / ys, "x / y by the reciprocal")
    _bits_equal(_run2(5, xs, ys), xs / ys, "x / y")
