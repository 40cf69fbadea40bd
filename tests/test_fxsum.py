"""The fixed-point float64 sums of the unary reductions (mgb_fxsum.h),
compiled for the host with g++ and checked against exact rational sums:
correctly rounded whenever the values lie within 10 binades of the largest
(the sum is then exact before its one rounding), within one unit in the last
place otherwise; subnormal sums, overflow to infinity, cancellation to zero,
Inf / NaN elements, and partial sums merged in any grouping."""
import ctypes
import math
import random
import shutil
import subprocess
from fractions import Fraction

import pytest

from tests.test_x96 import CSRC, same

SHIM = r'''
#include "mgb_fxsum.h"
extern "C" double fx_sum(const double *x, int n) {
    mgb::FxSum a = mgb::fx_zero();
    for (int i = 0; i < n; ++i) mgb::fx_push(a, x[i]);
    return mgb::fx_value(a);
}
extern "C" double fx_sum_parts(const double *x, int n, int k) {
    mgb::FxSum p[64];
    for (int j = 0; j < k; ++j) p[j] = mgb::fx_zero();
    for (int i = 0; i < n; ++i) mgb::fx_push(p[i % k], x[i]);
    for (int s = 1; s < k; s *= 2)  // pairwise, as a warp reduction merges
        for (int j = 0; j + s < k; j += 2 * s) mgb::fx_merge(p[j], p[j + s]);
    return mgb::fx_value(p[0]);
}
'''


@pytest.fixture(scope="module")
def fx(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("fx")
    src, so = d / "shim.cpp", d / "libfx.so"
    src.write_text(SHIM)
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I" + CSRC, str(src), "-o", str(so)], check=True)
    lib = ctypes.CDLL(str(so))
    lib.fx_sum.restype = ctypes.c_double
    lib.fx_sum.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    lib.fx_sum_parts.restype = ctypes.c_double
    lib.fx_sum_parts.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_int]

    def f(xs, parts=1):
        arr = (ctypes.c_double * max(len(xs), 1))(*xs)
        return lib.fx_sum(arr, len(xs)) if parts == 1 else lib.fx_sum_parts(arr, len(xs), parts)

    return f


def exact(xs):
    """Correctly rounded float64 of the exact sum (finite values)."""
    try:
        return float(sum((Fraction(x) for x in xs), Fraction(0)))
    except OverflowError:
        s = sum((Fraction(x) for x in xs), Fraction(0))
        return math.copysign(math.inf, s)


def window(rng, n, lo, hi, signed=True):
    out = []
    for _ in range(n):
        x = math.ldexp(rng.uniform(1.0, 2.0), rng.randint(lo, hi))
        out.append(-x if signed and rng.random() < 0.5 else x)
    return out


def test_exact_within_the_window(fx):
    rng = random.Random(1)
    for trial in range(400):
        n = rng.randint(1, 300)
        base = rng.randint(-1000, 960)
        xs = window(rng, n, base, base + rng.randint(0, 9))
        want = exact(xs)
        for parts in (1, 3, 32):
            got = fx(xs, parts)
            assert same(got, want) or (want == 0.0 and got == 0.0), (trial, parts, got, want)


def test_wide_ranges_within_one_ulp(fx):
    rng = random.Random(2)
    for trial in range(300):
        n = rng.randint(1, 200)
        xs = window(rng, n, -1070, 1000)
        want = exact(xs)
        got = fx(xs, rng.choice([1, 4, 32]))
        assert abs(got - want) <= math.ulp(want), (trial, got, want)


def test_cancellation_subnormals_and_overflow(fx):
    assert same(fx([1.0, -1.0]), 0.0)
    assert same(fx([]), 0.0)
    assert same(fx([-0.0, -0.0]), 0.0)  # an FP64 sum would keep -0.0; the sign of a zero sum is not kept
    tiny = 5e-324
    assert same(fx([tiny] * 7), 7 * tiny)
    assert same(fx([2.0**-1022, -tiny]), 2.0**-1022 - tiny)
    assert same(fx([2.0**-1022 - tiny, tiny]), 2.0**-1022)
    assert same(fx([3 * tiny, 2.0**-1074 * 0.0]), 3 * tiny)
    big = 1.7e308
    assert fx([big, big]) == math.inf and fx([-big, -big]) == -math.inf
    assert same(fx([big, big, -big]), big)  # exact in the accumulator, no intermediate overflow
    # terms more than 10 binades below the largest are truncated: the error
    # bound is relative to the largest term (2^-62 of it per term), not to a
    # sum that cancels below it
    xs = [1e308, 1e308, -1e308, -1e308, 5.0]
    assert abs(fx(xs) - 5.0) <= len(xs) * 2.0**-62 * 1e308
    assert same(fx([2.0**9, 1.0, -(2.0**9)]), 1.0)  # within the exact window
    assert same(fx([2.0**60, 1.0, -(2.0**60)]), 1.0)  # 2^-62 of 2^60 units: still kept
    xs = [1.0, 2.0**-53, 2.0**-53]  # ties and sticky bits
    assert same(fx(xs), exact(xs))
    assert same(fx([1.0, 2.0**-53]), 1.0)  # tie to even
    assert same(fx([1.0 + 2.0**-52, 2.0**-53]), 1.0 + 2.0**-51)


def test_infinities_and_nans(fx):
    assert fx([1.0, math.inf]) == math.inf
    assert fx([-math.inf, 3.0]) == -math.inf
    assert math.isnan(fx([math.inf, -math.inf]))
    assert math.isnan(fx([math.nan, 1.0]))
    assert math.isnan(fx([1.0, math.nan], parts=2))


def test_many_equal_terms(fx):
    for x in (0.1, -3.75, 1e-300, 2.0**1000):
        n = 10000
        assert same(fx([x] * n, 8), exact([x] * n))
