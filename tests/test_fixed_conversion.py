"""The projection's integer-only fixed-point to FP64 conversion (nlchains_gb300/csrc/nlc_fixed.h,
shared by host and device) against Python's exact conversion: the value (hi 2^32 + lo) 2^(k - 64)
rounded to the nearest double, ties to even, for random and edge-case hi, lo and k."""
import ctypes
import math
import os
import random
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "nlchains_gb300", "csrc")

SRC = r'''
#include "nlc_fixed.h"
extern "C" double conv(long long hi, long long lo, int k) { return nlc::fixed128_to_double(hi, lo, k); }
'''


@pytest.fixture(scope="module")
def conv():
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    work = tempfile.mkdtemp()
    src, so = os.path.join(work, "conv.cpp"), os.path.join(work, "conv.so")
    with open(src, "w") as f:
        f.write(SRC)
    subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-I" + CSRC, src, "-o", so], check=True)
    lib = ctypes.CDLL(so)
    lib.conv.argtypes = [ctypes.c_longlong, ctypes.c_longlong, ctypes.c_int]
    lib.conv.restype = ctypes.c_double
    yield lib.conv
    shutil.rmtree(work)


def exact(hi, lo, k):
    v = hi * 2 ** 32 + lo
    if v == 0:
        return 0.0
    return math.ldexp(float(v), k - 64) if abs(k - 64) < 900 else float(v) * 2.0 ** (k - 64)


def check(conv, hi, lo, k):
    got, want = conv(hi, lo, k), exact(hi, lo, k)
    assert got == want and math.copysign(1, got) == math.copysign(1, want) or (got == 0 and want == 0), (hi, lo, k, got, want)


def test_random_values_round_to_nearest(conv):
    rng = random.Random(7)
    for _ in range(20000):
        hi = rng.randrange(-2 ** 49, 2 ** 49) >> rng.randrange(0, 49)
        lo = rng.randrange(-2 ** 57, 2 ** 57) >> rng.randrange(0, 57)
        check(conv, hi, lo, rng.randrange(-60, 60))


def test_ties_carries_and_signs(conv):
    # ties at the 53-bit boundary (even and odd mantissas, with and without bits below), carries
    # between lo and hi, opposite signs, values that round up to the next power of two
    for e in (60, 70, 80, 81):
        for low in (0, 1):
            for odd in (0, 1):
                m = (1 << 52) | odd
                v = (m << (e - 52)) + (1 << (e - 53)) + low   # exactly half an ulp, plus `low`
                hi, lo = v >> 32, v & 0xffffffff
                for s in (1, -1):
                    check(conv, s * hi, s * lo, 0)
                    check(conv, s * hi, s * lo, 17)
    for v in ((1 << 53) - 1, (1 << 54) - 1, (1 << 81) - 1, 1 << 81, 1, 2 ** 63 - 1):
        for s in (1, -1):
            hi, lo = divmod(s * v, 2 ** 32)
            check(conv, hi, lo, 3)
    check(conv, 5, -(5 << 32), 0)          # cancels to zero
    check(conv, 1, -1, 0)                  # 2^32 - 1
    check(conv, -1, 2 ** 57 - 1, 0)        # lo larger than hi's part, opposite signs
    check(conv, 2 ** 48, 2 ** 57 - 1, 0)   # carry from lo into the high word


def test_scale_and_range(conv):
    assert conv(1 << 20, 0, 64 - 52) == 2.0 ** 20 * 2 ** 32 * 2.0 ** -52
    assert conv(1, 0, 1000) == 2.0 ** (32 + 1000 - 64)
    assert conv(1, 0, -1100) == math.ldexp(1.0, 32 - 1100 - 64)   # subnormal: the slow path
    assert conv(0, 0, 5) == 0.0


SRC_SQ = r'''
#include "nlc_fixed.h"
extern "C" double sq(long long hi, long long lo, int k) { return nlc::fixed128_square_to_double(hi, lo, k); }
'''


@pytest.fixture(scope="module")
def square():
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    work = tempfile.mkdtemp()
    src, so = os.path.join(work, "sq.cpp"), os.path.join(work, "sq.so")
    with open(src, "w") as f:
        f.write(SRC_SQ)
    subprocess.run(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-I" + CSRC, src, "-o", so], check=True)
    lib = ctypes.CDLL(so)
    lib.sq.argtypes = [ctypes.c_longlong, ctypes.c_longlong, ctypes.c_int]
    lib.sq.restype = ctypes.c_double
    yield lib.sq
    shutil.rmtree(work)


def test_square_truncates_within_two_ulp(square):
    """The squared value: never above the exact square, and below it by less than 2^-51 of it."""
    from fractions import Fraction
    rng = random.Random(11)
    cases = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 5), (2 ** 48, 2 ** 57 - 1, -7), (-(2 ** 48), -(2 ** 57) + 1, 9),
             (5, -(5 << 32) + 3, 0), (0, 0, 3)]
    for _ in range(20000):
        hi = rng.randrange(-2 ** 49, 2 ** 49) >> rng.randrange(0, 49)
        lo = rng.randrange(-2 ** 57, 2 ** 57) >> rng.randrange(0, 57)
        cases.append((hi, lo, rng.randrange(-60, 60)))
    for hi, lo, k in cases:
        v = hi * 2 ** 32 + lo
        exact = Fraction(v) ** 2 * Fraction(2) ** (2 * (k - 64))
        got = Fraction(square(hi, lo, k))
        if v == 0:
            assert got == 0
            continue
        assert got <= exact and (exact - got) < exact * Fraction(1, 2 ** 51), (hi, lo, k)
