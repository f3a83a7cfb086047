"""The algorithm behind the exact mode's shared-reciprocal quotients, on the CPU.

div_rcp (apophis_gb300/csrc/aph_math.cuh) forms a / b from y = RN(1 / b) by Markstein's
correction (P. W. Markstein, IBM J. Res. Develop. 34(1), 1990): q = RN(a y), r = a - b q
(exact, one fused multiply-add), result RN(q + r y), with q itself where a is zero.  The claim
is that this equals the IEEE quotient for every pair of tame operands (zero or normal with
2^-200 <= |x| < 2^201, b nonzero).  Here the same three operations run in C (fma from the C
library, no contraction) against C's division on 3.2e7 pairs: random exponents over the tame
range, quotients within a few ulps of a representable number, 1e5 quotients within ~1e-14 ulp
of a rounding midpoint (the hardest cases of division, where a faithful but incorrectly
rounded quotient would show), exact integer quotients and signed zeros.  tests/test_gpu_exact_ops.py checks the device's bits the same way.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

C_SRC = r"""
#include <math.h>
#include <stdint.h>
#include <string.h>
static double div_rcp(double a, double b, double y) {
  const double q = a * y;
  uint64_t ab; memcpy(&ab, &a, 8);
  if ((ab << 1) == 0) return q;
  return fma(fma(-q, b, a), y, q);
}
long long check(const double *a, const double *b, long long n, long long *first) {
  long long bad = 0;
  *first = -1;
  for (long long i = 0; i < n; ++i) {
    const double y = 1.0 / b[i];
    const double got = div_rcp(a[i], b[i], y), want = a[i] / b[i];
    if (memcmp(&got, &want, 8) != 0) {
      if (*first < 0) *first = i;
      ++bad;
    }
  }
  return bad;
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    d = tmp_path_factory.mktemp("quot")
    src, so = os.path.join(d, "q.c"), os.path.join(d, "q.so")
    with open(src, "w") as f:
        f.write(C_SRC)
    try:
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
                               src, "-o", so, "-lm"])
    except (OSError, subprocess.CalledProcessError):
        pytest.skip("no C compiler")
    L = ctypes.CDLL(so)
    dp = ctypes.POINTER(ctypes.c_double)
    L.check.argtypes = [dp, dp, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]
    L.check.restype = ctypes.c_longlong
    return L


def _tame(rng, n, emin=-200, emax=200):
    mant = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    exp = rng.integers(emin + 1023, emax + 1023 + 1, n).astype(np.uint64)
    sign = rng.integers(0, 2, n).astype(np.uint64)
    return ((sign << np.uint64(63)) | (exp << np.uint64(52)) | mant).view(np.float64)


def _check(lib, a, b):
    keep = ((np.abs(a) >= 2.0 ** -200) & (np.abs(a) < 2.0 ** 201)) | (a == 0)
    keep &= (np.abs(b) >= 2.0 ** -200) & (np.abs(b) < 2.0 ** 201)
    a, b = np.ascontiguousarray(a[keep]), np.ascontiguousarray(b[keep])
    first = ctypes.c_longlong(-1)
    dp = ctypes.POINTER(ctypes.c_double)
    bad = lib.check(a.ctypes.data_as(dp), b.ctypes.data_as(dp), a.size, ctypes.byref(first))
    assert bad == 0, (bad, a.size, a[first.value].hex(), b[first.value].hex())
    return a.size


def test_random_tame_pairs(lib):
    rng = np.random.Generator(np.random.PCG64(21))
    n = 0
    for _ in range(4):
        n += _check(lib, _tame(rng, 4_000_000), _tame(rng, 4_000_000))
    assert n > 15_000_000


def test_quotients_near_representables(lib):
    rng = np.random.Generator(np.random.PCG64(22))
    n = 0
    for _ in range(4):
        b = _tame(rng, 2_000_000, -100, 100)
        q = _tame(rng, 2_000_000, -100, 100)
        # a near q b (and near (q + ulp(q) / 2) b), moved by a few ulps of a
        for a0 in (q * b, q * b + (np.spacing(q) * 0.5) * b):
            a = (a0.view(np.int64) + rng.integers(-4, 5, b.size)).view(np.float64)
            n += _check(lib, a, b)
    assert n > 15_000_000


def test_quotients_at_midpoints(lib):
    """Quotients within ~1e-14 ulp of a rounding midpoint (tests/quotient_cases.py)."""
    from quotient_cases import midpoint_cases
    a, b = midpoint_cases(np.random.Generator(np.random.PCG64(23)), 100_000)
    assert _check(lib, a, b) == a.size


def test_exact_quotients_and_zeros(lib):
    ints = np.arange(-500, 501, dtype=np.float64)
    ints = ints[ints != 0]
    a = np.concatenate([np.repeat(ints, ints.size), [0.0, -0.0, 0.0, -0.0]])
    b = np.concatenate([np.tile(ints, ints.size), [3.0, 3.0, -3.0, -3.0]])
    _check(lib, a, b)
