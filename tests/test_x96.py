"""The epilogue's 96-bit integer to float64 conversion (x96_ldexp_rn in
muscle.jl_gb300/csrc/mgb_x96.h), compiled for the host with g++ and checked
against exact rational rounding: normal, subnormal, overflow, underflow and
exact ties, for positive and negative accumulators; and the straight-line
path the epilogue runs (x96_ldexp_bits_fast), which must give the same bits
for every result that is not subnormal and flag exactly the subnormal ones."""
import ctypes
import math
import os
import random
import shutil
import subprocess
from fractions import Fraction

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "muscle.jl_gb300", "csrc")

SHIM = r'''
#include "mgb_x96.h"
extern "C" double x96_ldexp(unsigned w0, unsigned w1, unsigned w2, int e) { return mgb::x96_ldexp_rn(w0, w1, w2, e); }
extern "C" double x96_general(unsigned w0, unsigned w1, unsigned w2, int e) {
    return mgb::x96_ldexp_rn_general(w0, w1, w2, e);
}
extern "C" double x96_fast(unsigned w0, unsigned w1, unsigned w2, int e, int *slow) {
    bool s = false;
    const double d = mgb::x96_bits_to_double(mgb::x96_ldexp_bits_fast(w0, w1, w2, e, s));
    *slow = s ? 1 : 0;
    return d;
}
'''


@pytest.fixture(scope="module")
def conv(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("x96")
    src, so = d / "shim.cpp", d / "libx96.so"
    src.write_text(SHIM)
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I" + CSRC, str(src), "-o", str(so)], check=True)
    lib = ctypes.CDLL(str(so))
    args = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]
    for name in ("x96_ldexp", "x96_general"):
        getattr(lib, name).restype = ctypes.c_double
        getattr(lib, name).argtypes = args
    lib.x96_fast.restype = ctypes.c_double
    lib.x96_fast.argtypes = args + [ctypes.POINTER(ctypes.c_int)]

    def words(x):
        u = x & ((1 << 96) - 1)
        return u & 0xFFFFFFFF, (u >> 32) & 0xFFFFFFFF, (u >> 64) & 0xFFFFFFFF

    def f(x, e, which="x96_ldexp"):
        if which == "x96_fast":
            slow = ctypes.c_int(0)
            d = lib.x96_fast(*words(x), e, ctypes.byref(slow))
            return d, bool(slow.value)
        return getattr(lib, which)(*words(x), e)

    return f


def exact(x, e):
    """Correctly rounded (ties to even) float64 of x * 2^e."""
    if x == 0:
        return 0.0
    try:
        v = float(Fraction(x) * Fraction(2) ** e)
    except OverflowError:
        return math.copysign(math.inf, x)
    if v == 0.0:
        return math.copysign(0.0, x)
    return v


def same(a, b):
    return a == b and math.copysign(1.0, a) == math.copysign(1.0, b) or (math.isnan(a) and math.isnan(b))


def test_random_magnitudes_and_exponents(conv):
    rng = random.Random(7)
    for _ in range(20000):
        bits = rng.randint(1, 94)
        x = rng.getrandbits(bits) | (1 << (bits - 1))
        if rng.random() < 0.5:
            x = -x
        e = rng.choice([rng.randint(-200, 200), rng.randint(-1180, -1000), rng.randint(900, 1100),
                        rng.randint(-2200, 2200)])
        got, want = conv(x, e), exact(x, e)
        assert same(got, want), (x, e, got, want)


def test_ties_round_to_even(conv):
    for m in (2**52, 2**52 + 1, 2**53 - 1, 2**52 + 12345):
        for k in (1, 5, 31, 32, 33, 40, 41, 63, 64):
            for sticky in (0, 1):
                x = (m << k) | (1 << (k - 1)) | (sticky if k > 1 else 0)
                if x >= 2**95:
                    continue
                for sgn in (1, -1):
                    for e in (0, -k, -1074 - 60, 1023 - 52 - k):
                        got, want = conv(sgn * x, e), exact(sgn * x, e)
                        assert same(got, want), (sgn * x, e, got, want)


def test_edges(conv):
    assert same(conv(0, 5), 0.0)
    assert same(conv(1, -1074), 5e-324)
    assert same(conv(1, -1075), 0.0)  # a tie rounds to the even zero
    assert same(conv(3, -1076), 5e-324)  # 0.75 of the smallest subnormal
    assert same(conv(-1, -1075), -0.0)
    assert same(conv(2**52, -1074), 2.0**-1022)  # smallest normal
    assert same(conv(2**53 - 1, 1023 - 52), 1.7976931348623157e308)  # largest finite
    assert same(conv(2**54 - 1, 1023 - 53), math.inf)  # rounds up past the largest finite
    assert same(conv(-(2**94), 2000), -math.inf)
    assert same(conv(2**95 - 1, 0), float(2**95))
    assert same(conv(-(2**95) + 1, -95), -1.0)
    for x in range(-300, 300):
        assert same(conv(x, 0), float(x))


def test_general_routine_alone(conv):
    rng = random.Random(11)
    for _ in range(5000):
        bits = rng.randint(1, 94)
        x = rng.getrandbits(bits) | (1 << (bits - 1))
        x = -x if rng.random() < 0.5 else x
        e = rng.choice([rng.randint(-1180, -1000), rng.randint(-200, 200), rng.randint(900, 1100)])
        assert same(conv(x, e, "x96_general"), exact(x, e)), (x, e)


def test_straight_line_path(conv):
    """Same bits as exact rounding whenever the result is not subnormal; the
    slow flag is raised exactly for nonzero subnormal results."""
    rng = random.Random(13)
    tiny = 2.0 ** -1022
    cases = [(0, 0), (0, -2000), (1, 0), (-1, 0), (2**95 - 1, 0), (-(2**95) + 1, 0), (2**94, 1000)]
    for _ in range(30000):
        bits = rng.randint(1, 94)
        x = rng.getrandbits(bits) | (1 << (bits - 1))
        x = -x if rng.random() < 0.5 else x
        cases.append((x, rng.choice([rng.randint(-1200, -950), rng.randint(-300, 300), rng.randint(850, 1100)])))
    for m in (2**52, 2**53 - 1, 2**52 + 7):  # ties and carries out of the significand
        for k in (1, 11, 42, 43, 44):
            for sticky in (0, 1):
                x = (m << k) | (1 << (k - 1)) | (sticky if k > 1 else 0)
                if x < 2**95:
                    cases += [(x, 0), (-x, -k), (x, 1023 - 52 - k), (x, -1022 - 52 - k + 1)]
    for x, e in cases:
        want = exact(x, e)
        got, slow = conv(x, e, "x96_fast")
        subnormal = want != 0.0 and abs(want) < tiny
        if x != 0 and not subnormal:
            # results that round to zero are subnormal before rounding
            subnormal = abs(Fraction(x) * Fraction(2) ** e) < Fraction(tiny)
        assert slow == (subnormal and x != 0), (x, e, want, slow)
        if not slow:
            assert same(got, want), (x, e, got, want)
